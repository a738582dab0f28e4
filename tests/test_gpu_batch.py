"""Several right-hand sides per matrix and batches of independent systems.

* ocsl_solve_multi_device reuses one factor for all right-hand sides and is
  bit-identical to separate solves (every method).
* ocsl_batch_solve_device runs the systems concurrently on several streams
  and is bit-identical to solving each system alone on one context; every
  solve reaches 1e-10 (true residual, long double on the host).
* A failing system reports its own status without disturbing the others.
"""
import numpy as np
import pytest

import opencslsolver_gb300 as ocsl
from opencslsolver_gb300 import _abi
from opencslsolver_gb300 import workloads as W

pytestmark = pytest.mark.gpu

METHODS = [ocsl.BICGSTAB_REF, ocsl.ILU_BICGSTAB, ocsl.ILU_BICGSTAB_IR32]


@pytest.mark.parametrize("method", METHODS + [ocsl.PCG])
def test_multi_rhs_equals_separate_solves(ctx, torch_cuda, method):
    torch = torch_cuda
    s = W.hex_pprime(14, 10, 9, peclet=0.0 if method == ocsl.PCG else 10.0)
    ctx.set_pattern(s.row_ptr, s.column_index)
    rng = np.random.default_rng(4)
    B = torch.from_numpy(rng.uniform(-1, 1, (3, s.n))).cuda()
    A = torch.from_numpy(s.value).cuda()
    X = torch.zeros_like(B)
    res = ctx.solve_multi_device(method, A, B, X)
    for r in range(3):
        x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
        one = ctx.solve_device(method, A, B[r].contiguous(), x)
        assert torch.equal(x, X[r]), r
        assert res[r]["status"] == one["status"] and res[r]["iterations"] == one["iterations"]


def _lockstep_vs_one_by_one(ctx, torch, s, B, **opts):
    """Solve B's columns with the FP32-inner solver in lockstep and one by one;
    return both results."""
    ctx.set_pattern(s.row_ptr, s.column_index)
    A = torch.from_numpy(s.value).cuda()
    X1 = torch.zeros_like(B)
    res1 = ctx.solve_multi_device(ocsl.ILU_BICGSTAB_IR32, A, B, X1, **opts)
    ctx.set_col_batching(False)
    X2 = torch.zeros_like(B)
    res2 = ctx.solve_multi_device(ocsl.ILU_BICGSTAB_IR32, A, B, X2, **opts)
    ctx.set_col_batching(True)
    return X1, res1, X2, res2


@pytest.mark.parametrize("kind,nrhs", [("hex", 2), ("hex", 3), ("hex", 4), ("hex", 6),
                                       ("tet", 3)])
def test_lockstep_columns_equal_one_by_one(ctx, oracle, torch_cuda, kind, nrhs):
    """Lockstep groups of up to four columns (structured sweeps on the box,
    one level-scheduled launch per column on tets) give every column the
    bits and iteration counts of solving it alone."""
    torch = torch_cuda
    s = W.hex_pprime(17, 12, 11, peclet=50.0) if kind == "hex" else W.tet_pprime(6, 5, 5)
    rng = np.random.default_rng(40 + nrhs)
    B = torch.from_numpy(rng.uniform(-1, 1, (nrhs, s.n))).cuda()
    X1, res1, X2, res2 = _lockstep_vs_one_by_one(ctx, torch, s, B, tol=1e-10)
    assert torch.equal(X1, X2)
    for q in range(nrhs):
        assert res1[q]["status"] == res2[q]["status"] == 0, (q, res1[q])
        assert res1[q]["iterations"] == res2[q]["iterations"], q
        assert res1[q]["outer_iterations"] == res2[q]["outer_iterations"], q
        rr = oracle.true_relres(s.row_ptr, s.column_index, s.value, B[q].cpu().numpy(),
                                X1[q].cpu().numpy())
        assert rr <= 1e-10, (q, rr)


def test_spmm_spmv_equals_per_column_spmv(ctx, torch_cuda):
    """The lockstep solve's SpMM-style box SpMV (one CTA per tile, every
    column) against one SpMV CTA per (tile, column): the same bits; the time
    of both at 128^3 x 3 right-hand sides is printed."""
    torch = torch_cuda
    for dims, timed in (((19, 13, 11), False), ((128, 128, 128), True)):
        s = W.hex_pprime(*dims, peclet=10.0)
        ctx.set_pattern(s.row_ptr, s.column_index)
        rng = np.random.default_rng(11)
        B = torch.from_numpy(rng.uniform(-1, 1, (3, s.n))).cuda()
        A = torch.from_numpy(s.value).cuda()
        out = {}
        for mode in (2, 1):
            ctx.set_col_batching(mode)
            X = torch.zeros_like(B)
            res = ctx.solve_multi_device(ocsl.ILU_BICGSTAB_IR32, A, B, X, tol=1e-10)
            ms = None
            if timed:
                t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                X2 = torch.zeros_like(B)
                torch.cuda.synchronize()
                t0.record()
                ctx.solve_multi_device(ocsl.ILU_BICGSTAB_IR32, A, B, X2, tol=1e-10)
                t1.record()
                torch.cuda.synchronize()
                ms = t0.elapsed_time(t1)
                assert torch.equal(X2, X)
            out[mode] = (X, [r["iterations"] for r in res], ms)
        ctx.set_col_batching(True)
        assert torch.equal(out[1][0], out[2][0])
        assert out[1][1] == out[2][1]
        if timed:
            print(f"128^3 x 3 rhs FP32-refined lockstep: SpMM SpMV {out[2][2]:.2f} ms, "
                  f"per-column SpMV {out[1][2]:.2f} ms (iterations {out[1][1]})")


def test_lockstep_uneven_columns(ctx, torch_cuda):
    """Columns that finish at different points: b = 0 (x = 0 at once), a tiny
    and a large right-hand side, a column with a NaN (its own status only)."""
    torch = torch_cuda
    s = W.hex_pprime(15, 13, 10, peclet=10.0)
    rng = np.random.default_rng(7)
    B = torch.from_numpy(rng.uniform(-1, 1, (4, s.n))).cuda()
    B[0].zero_()
    B[1] *= 1e-12
    B[2] *= 1e6
    X1, res1, X2, res2 = _lockstep_vs_one_by_one(ctx, torch, s, B, tol=1e-10)
    assert torch.equal(X1, X2)
    assert torch.count_nonzero(X1[0]) == 0 and res1[0]["residual"] == 0.0
    for q in range(4):
        assert res1[q]["status"] == res2[q]["status"] == 0
        assert res1[q]["iterations"] == res2[q]["iterations"]
    B[3, 17] = float("nan")
    X3 = torch.zeros_like(B)
    A = torch.from_numpy(s.value).cuda()
    res3 = ctx.solve_multi_device(ocsl.ILU_BICGSTAB_IR32, A, B, X3, tol=1e-10)
    assert res3[3]["status"] == _abi.NONFINITE
    assert all(res3[q]["status"] == 0 for q in range(3))
    assert torch.equal(X3[:3], X1[:3])


def small_batch():
    return W.batch_systems(4, min_cells=1500, max_cells=25_000)


@pytest.mark.parametrize("method", [ocsl.ILU_BICGSTAB, ocsl.ILU_BICGSTAB_IR32])
def test_batch_equals_single_solves(ctx, oracle, torch_cuda, method):
    torch = torch_cuda
    systems = small_batch()
    batch = ocsl.Batch([(b.system.row_ptr, b.system.column_index, b.rhs.shape[0])
                        for b in systems], workers=4)
    vals = [torch.from_numpy(b.system.value).cuda() for b in systems]
    Bs = [torch.from_numpy(np.ascontiguousarray(b.rhs)).cuda() for b in systems]
    Xs = [torch.zeros_like(B) for B in Bs]
    st, res = batch.solve_device(method, vals, Bs, Xs, tol=1e-10)
    assert st == 0, res
    k = 0
    for b, v, B, X in zip(systems, vals, Bs, Xs):
        ctx.set_pattern(b.system.row_ptr, b.system.column_index)
        for r in range(b.rhs.shape[0]):
            x = torch.zeros(b.system.n, dtype=torch.float64, device="cuda")
            one = ctx.solve_device(method, v, B[r].contiguous(), x, tol=1e-10)
            assert torch.equal(x, X[r]), (b.system.name, r)
            assert res[k]["iterations"] == one["iterations"]
            rr = oracle.true_relres(b.system.row_ptr, b.system.column_index, b.system.value,
                                    b.rhs[r], X[r].cpu().numpy())
            assert rr <= 1e-10, (b.system.name, r, rr)
            k += 1
    assert k == len(res) == sum(b.rhs.shape[0] for b in systems)
    batch.close()


def test_batch_reports_a_failing_system(torch_cuda):
    torch = torch_cuda
    systems = small_batch()[:3]
    batch = ocsl.Batch([(b.system.row_ptr, b.system.column_index, b.rhs.shape[0])
                        for b in systems], workers=3)
    vals = [torch.from_numpy(b.system.value).cuda() for b in systems]
    vals[1][5] = float("nan")
    Bs = [torch.from_numpy(np.ascontiguousarray(b.rhs)).cuda() for b in systems]
    Xs = [torch.zeros_like(B) for B in Bs]
    st, res = batch.solve_device(ocsl.ILU_BICGSTAB, vals, Bs, Xs)
    assert st == _abi.NONFINITE
    n0 = systems[0].rhs.shape[0]
    n1 = systems[1].rhs.shape[0]
    assert all(r["status"] == 0 for r in res[:n0])
    assert all(r["status"] == _abi.NONFINITE for r in res[n0:n0 + n1])
    assert all(r["status"] == 0 for r in res[n0 + n1:])
    batch.close()


def test_batch_workload_shape():
    dims = W.batch_boxes(64)
    cells = np.array([a * b * c for a, b, c in dims])
    assert len(dims) == 64
    assert cells.min() >= 0.6 * 10_000 and cells.max() <= 1.4 * 500_000
    assert max(max(d) / min(d) for d in dims) > 2.0


def test_batch_graph_equals_host_batch(torch_cuda):
    """ocsl_batch_set_graph: one graph launch runs every FP32-refined solve of
    the batch with its loops on the device; x, iteration and step counts,
    residuals and statuses equal the host-driven batch's, on the first call
    (capture) and on a replay; a right-hand side with a NaN reports its own
    status only."""
    torch = torch_cuda
    systems = small_batch()
    batch = ocsl.Batch([(b.system.row_ptr, b.system.column_index, b.rhs.shape[0])
                        for b in systems], workers=4)
    vals = [torch.from_numpy(b.system.value).cuda() for b in systems]
    Bs = [torch.from_numpy(np.ascontiguousarray(b.rhs)).cuda() for b in systems]
    X1 = [torch.zeros_like(B) for B in Bs]
    st1, res1 = batch.solve_device(ocsl.ILU_BICGSTAB_IR32, vals, Bs, X1, tol=1e-10)
    assert st1 == 0
    batch.set_graph(True)
    X2 = [torch.zeros_like(B) for B in Bs]
    keys = ("iterations", "outer_iterations", "status", "residual")
    for rep in range(2):
        for X in X2:
            X.zero_()
        st2, res2 = batch.solve_device(ocsl.ILU_BICGSTAB_IR32, vals, Bs, X2, tol=1e-10)
        assert st2 == 0, res2
        for i, (a, b) in enumerate(zip(X1, X2)):
            assert torch.equal(a, b), (rep, i)
        for r1, r2 in zip(res1, res2):
            assert all(r1[k] == r2[k] for k in keys), (rep, r1, r2)
    Bs[1][0, 9] = float("nan")
    for X in X2:
        X.zero_()
    st3, res3 = batch.solve_device(ocsl.ILU_BICGSTAB_IR32, vals, Bs, X2, tol=1e-10)
    assert st3 == _abi.NONFINITE
    n0 = systems[0].rhs.shape[0]
    assert res3[n0]["status"] == _abi.NONFINITE
    assert all(r["status"] == 0 for k, r in enumerate(res3) if k != n0)
    assert torch.equal(X2[0], X1[0])
    batch.close()
