"""FP32-refined solves with their control flow on the device
(ocsl_set_device_loop): the refinement loop and the inner FP32 BiCGSTAB loop
as conditional WHILE graph nodes, one graph launch per solve.

Every result -- x, iteration and refinement-step counts, relative residual,
status -- equals the host-driven loop's, bit for bit: box patterns (structured
sweeps) and tetrahedral ones (level-scheduled sweeps), zero and non-finite
right-hand sides, budgets that run out (maxit, inner_maxit), and the 128^3
system, whose solve times are printed.  On the legacy default stream (which
cannot be captured) the host loop runs instead.
"""
import numpy as np
import pytest

import opencslsolver_gb300 as ocsl
from opencslsolver_gb300 import _abi
from opencslsolver_gb300 import workloads as W

pytestmark = pytest.mark.gpu

IR32 = ocsl.ILU_BICGSTAB_IR32


def _both(ctx, torch, s, b, method=None, **opts):
    """The solve host-driven, then device-driven, on a created stream."""
    method = IR32 if method is None else method
    A = torch.from_numpy(s.value).cuda()
    B = b if isinstance(b, torch.Tensor) else torch.from_numpy(b).cuda()
    out = []
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        for dev in (False, True):
            ctx.set_device_loop(dev)
            X = torch.zeros(s.n, dtype=torch.float64, device="cuda")
            r = ctx.solve_device(method, A, B, X, **opts)
            stream.synchronize()
            out.append((X.clone(), r))
    ctx.set_device_loop(False)
    return out


def _same(out, where):
    (x0, r0), (x1, r1) = out
    assert torch_equal(x0, x1), where
    for k in ("iterations", "outer_iterations", "status", "residual"):
        assert r0[k] == r1[k], (where, k, r0, r1)


def torch_equal(a, b):
    import torch

    return bool(torch.equal(a, b)) or bool(torch.equal(torch.isnan(a), torch.isnan(b)) and
                                           torch.equal(torch.nan_to_num(a), torch.nan_to_num(b)))


@pytest.mark.parametrize("kind", ["hex", "tet"])
def test_device_loop_equals_host_loop(ctx, torch_cuda, kind):
    s = W.hex_pprime(23, 17, 13, peclet=10.0) if kind == "hex" else W.tet_pprime(9, 8, 7)
    ctx.set_pattern(s.row_ptr, s.column_index)
    for opts in ({"tol": 1e-10}, {"tol": 1e-12}, {"tol": 1e-10, "inner_maxit": 3},
                 {"tol": 1e-10, "inner_tol": 1e-2}):
        out = _both(ctx, torch_cuda, s, s.b, **opts)
        _same(out, (kind, opts))
        assert out[1][1]["status"] == 0 and out[1][1]["outer_iterations"] >= 1


def test_device_loop_edge_cases(ctx, torch_cuda):
    torch = torch_cuda
    s = W.hex_pprime(15, 13, 10, peclet=10.0)
    ctx.set_pattern(s.row_ptr, s.column_index)
    # b = 0: x = 0 at once
    out = _both(ctx, torch, s, np.zeros(s.n))
    _same(out, "b=0")
    assert out[1][1]["residual"] == 0.0 and torch.count_nonzero(out[1][0]) == 0
    # a non-finite right-hand side
    b = s.b.copy()
    b[17] = np.nan
    out = _both(ctx, torch, s, b)
    _same(out, "nan")
    assert out[1][1]["status"] == _abi.NONFINITE
    # the total budget runs out
    out = _both(ctx, torch, s, s.b, tol=1e-14, maxit=7)
    _same(out, "maxit")
    assert out[1][1]["status"] == _abi.NOT_CONVERGED
    # legacy default stream: the host loop runs, same bits
    A = torch.from_numpy(s.value).cuda()
    B = torch.from_numpy(s.b).cuda()
    ctx.set_device_loop(True)
    X = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    r = ctx.solve_device(IR32, A, B, X)
    ctx.set_device_loop(False)
    X0 = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    r0 = ctx.solve_device(IR32, A, B, X0)
    assert torch.equal(X, X0) and r["iterations"] == r0["iterations"]


def test_device_loop_full_size(ctx, torch_cuda, hex128):
    torch = torch_cuda
    s = hex128
    ctx.set_pattern(s.row_ptr, s.column_index)
    out = _both(ctx, torch, s, s.b, tol=1e-10)
    _same(out, "128^3")
    A = torch.from_numpy(s.value).cuda()
    B = torch.from_numpy(s.b).cuda()
    stream = torch.cuda.Stream()
    ms = {}
    with torch.cuda.stream(stream):
        for dev in (False, True):
            ctx.set_device_loop(dev)
            X = torch.zeros(s.n, dtype=torch.float64, device="cuda")
            ctx.solve_device(IR32, A, B, X)  # warm-up
            t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            X.zero_()
            t0.record()
            for _ in range(3):
                X.zero_()
                ctx.solve_device(IR32, A, B, X)
            t1.record()
            stream.synchronize()
            ms[dev] = t0.elapsed_time(t1) / 3
    ctx.set_device_loop(False)
    print(f"128^3 FP32-refined solve: host loop {ms[False]:.2f} ms, device loop {ms[True]:.2f} ms "
          f"({out[1][1]['iterations']} inner iterations, {out[1][1]['outer_iterations']} steps)")


def test_device_loop_small_system_replays_its_graph(ctx, torch_cuda):
    """Repeated solves of a small system (the latency-bound case, where the
    host loop's round trips cost the most): the device loop's graph is
    instantiated once and replayed; same bits; both times are printed."""
    torch = torch_cuda
    s = W.hex_pprime(16, 14, 12, peclet=10.0)
    ctx.set_pattern(s.row_ptr, s.column_index)
    A = torch.from_numpy(s.value).cuda()
    B = torch.from_numpy(s.b).cuda()
    stream = torch.cuda.Stream()
    out, ms = {}, {}
    with torch.cuda.stream(stream):
        for dev in (False, True):
            ctx.set_device_loop(dev)
            X = torch.zeros(s.n, dtype=torch.float64, device="cuda")
            ctx.solve_device(IR32, A, B, X)  # warm-up (and capture)
            import time

            stream.synchronize()
            t0 = time.perf_counter()
            for _ in range(20):
                X.zero_()
                r = ctx.solve_device(IR32, A, B, X)
            stream.synchronize()
            ms[dev] = (time.perf_counter() - t0) * 1e3 / 20
            out[dev] = (X.clone(), r)
    ctx.set_device_loop(False)
    assert torch.equal(out[False][0], out[True][0])
    assert out[False][1]["iterations"] == out[True][1]["iterations"]
    print(f"{s.n}-row FP32-refined solve: host loop {ms[False]:.3f} ms, device loop "
          f"{ms[True]:.3f} ms per solve ({out[True][1]['iterations']} inner iterations)")


@pytest.mark.parametrize("method", [ocsl.ILU_BICGSTAB, ocsl.PCG])
@pytest.mark.parametrize("kind", ["hex", "tet"])
def test_restarted_device_loop_equals_host_loop(ctx, torch_cuda, kind, method):
    """The plain FP64 ILU-BiCGSTAB and Jacobi PCG with their restart and
    Krylov loops on the device: the host loop's bits, iteration counts,
    residuals and statuses, including b = 0, a NaN and an exhausted maxit."""
    torch = torch_cuda
    pe = 0.0 if method == ocsl.PCG else 10.0
    s = W.hex_pprime(21, 17, 13, peclet=pe) if kind == "hex" else W.tet_pprime(9, 8, 7,
                                                                                 peclet=pe)
    ctx.set_pattern(s.row_ptr, s.column_index)
    for opts in ({"tol": 1e-10}, {"tol": 1e-13}, {"tol": 1e-12, "maxit": 9}):
        out = _both(ctx, torch, s, s.b, method=method, **opts)
        _same(out, (kind, method, opts))
    assert out[1][1]["status"] == _abi.NOT_CONVERGED
    out = _both(ctx, torch, s, np.zeros(s.n), method=method)
    _same(out, (kind, method, "b=0"))
    assert torch.count_nonzero(out[1][0]) == 0 and out[1][1]["status"] == 0
    b = s.b.copy()
    b[5] = np.nan
    out = _both(ctx, torch, s, b, method=method)
    _same(out, (kind, method, "nan"))
    assert out[1][1]["status"] == _abi.NONFINITE
