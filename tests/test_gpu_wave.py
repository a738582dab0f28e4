"""The warp-pipelined structured sweep (kernels_wave.cu) against the oracle.

* Forward and backward sweeps (the reference's division backward) of the
  oracle's ILU factor, bit for bit, for box shapes with ragged edges (x not a
  multiple of 32, the tile's other axis not a multiple of its columns, s the
  y or the z axis), several warps-per-CTA settings and start lags; each launch
  twice, so the tile dispenser, the shared-memory faces and the global face
  buffers (which the consumers reset) start over correctly.  Boxes too thin
  in x for the warp tiles (1D and 2D strips) run the CTA kernel even when the
  warp-pipelined one is asked for, with the same bits.
* Whole solves (reference-faithful, FP64 tolerance mode with the reciprocal
  diagonal, FP32-refined with FP32 sweeps) give the same bits and iteration
  counts with the warp-pipelined, the CTA and the level-scheduled kernels.
* The autotuner's choice of kernel does not change a bit.
"""
import numpy as np
import pytest

import opencslsolver_gb300 as ocsl
from opencslsolver_gb300 import workloads as W

pytestmark = pytest.mark.gpu

BOXES = [(20, 20, 20), (37, 9, 23), (70, 45, 38), (40, 36, 33), (64, 12, 8), (9, 40, 66),
         (100, 70, 30), (33, 1, 1), (9, 12, 1), (1000, 1, 1)]


def _system(dims):
    if dims[1] == 1 and dims[2] == 1:
        rp, col = W.pattern_1d(dims[0])
        rng = np.random.default_rng(2)
        val = np.where(col == W.PHANTOM, 0.0, rng.uniform(-1, 0, col.size))
        rows = np.repeat(np.arange(dims[0]), np.diff(rp.astype(np.int64)))
        val[col == rows.astype(np.uint64)] = 3.0
        return W.System(rp, col, val, rng.uniform(-1, 1, dims[0]))
    return W.hex_pprime(*dims)


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("dims", BOXES)
@pytest.mark.parametrize("warps,lag", [(1, 1), (2, 6), (4, 0), (8, 3)])
def test_wave_sweeps_bit_exact(ctx, torch_cuda, oracle, dims, warps, lag):
    torch = torch_cuda
    s = _system(dims)
    ctx.set_pattern(s.row_ptr, s.column_index)
    ctx.set_sweep_kernel(3, warps, lag)
    info = ctx.sweep_info()
    thin = dims[1] == 1 or dims[2] == 1
    assert info["kind"] == (2 if thin else 3) and info["wave"]["on"] == (not thin)
    assert thin or 1 <= info["wave"]["warps"] <= warps
    rng = np.random.default_rng(5)
    b = rng.standard_normal(s.n)
    Mh = oracle.ilu(s.row_ptr, s.column_index, s.value)
    M, B = dev(torch, Mh), dev(torch, b)
    Y, X = torch.empty_like(B), torch.empty_like(B)
    y = oracle.forsub(s.row_ptr, s.column_index, Mh, b)
    x = oracle.backsub(s.row_ptr, s.column_index, Mh, y)
    for _ in range(2):
        ctx.forsub_device(M, B, Y)
        assert np.array_equal(Y.cpu().numpy(), y)
        ctx.backsub_device(M, Y, X)
        assert np.array_equal(X.cpu().numpy(), x)


@pytest.mark.parametrize("dims", [(40, 36, 33), (24, 70, 17), (66, 20, 50)])
@pytest.mark.parametrize("method", [ocsl.BICGSTAB_REF, ocsl.ILU_BICGSTAB, ocsl.ILU_BICGSTAB_IR32])
def test_wave_solves_identical(ctx, dims, method):
    s = W.hex_pprime(*dims)
    ctx.set_pattern(s.row_ptr, s.column_index)
    out = []
    for kind, a, b in ((1, 0, 0), (2, 8, 8), (3, 1, 0), (3, 4, 0), (3, 8, 10)):
        ctx.set_sweep_kernel(kind, a, b)
        x = np.zeros(s.n)
        r = ctx.solve(method, s.value, s.b, x, tol=1e-10)
        assert r["status"] == 0, (kind, a, r)
        out.append((kind, a, x, r["iterations"], r["residual"]))
    k0, a0, x0, it0, res0 = out[0]
    for kind, a, x, it, res in out[1:]:
        assert np.array_equal(x, x0) and it == it0 and res == res0, (kind, a)


def test_autotuned_kernel_choice_keeps_bits(ctx, torch_cuda):
    torch = torch_cuda
    s = W.hex_pprime(48, 40, 36)
    ctx.set_pattern(s.row_ptr, s.column_index)
    A, B = dev(torch, s.value), dev(torch, s.b)
    X0 = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    r0 = ctx.solve_device(ocsl.ILU_BICGSTAB_IR32, A, B, X0, tol=1e-10)
    for method in (ocsl.ILU_BICGSTAB_IR32, ocsl.ILU_BICGSTAB):
        t = ctx.autotune(method, A)
        assert t["sweep_us"] > 0
    X1 = torch.zeros_like(X0)
    r1 = ctx.solve_device(ocsl.ILU_BICGSTAB_IR32, A, B, X1, tol=1e-10)
    assert torch.equal(X0, X1) and r0["iterations"] == r1["iterations"]
