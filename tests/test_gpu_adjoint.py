"""Adjoint (differentiation) path on the GPU, through the C ABI.

For x = A^-1 b and L = sum_i w_i x_i (w ~ N(0, 1), seeded):
    A^T lam = w,   dL/db = lam,   dL/dA_ij = -lam_i x_j on A's pattern.

* ocsl_solve_transpose equals the oracle's tolerance-mode solve of the
  explicitly transposed CSR bit for bit (same algorithm, rounding and
  reduction order), so the transposed pattern and its value map are exact.
* ocsl_pattern_outer_device equals -lam_i x_j exactly, with 0 on phantoms.
* A torch.autograd.Function (test harness only) wraps solve / adjoint solve;
  its gradients match central finite differences (relative step 1e-6) on 32
  random entries of b and of A on the 128^3 jittered hex p' system, in FP64
  and FP32-refined modes, within 1e-6, and an FP64 oracle gradient at 24^3.
* dL/d(inlet pressure value) through the GPU face-loop assembly of the
  pressure-correction equation on a 128^3 hex flow state: the adjoint of the
  Dirichlet inlet terms summed over the inlet faces matches central finite
  differences of the re-assembled, re-solved system within 1e-6.

The finite differences evaluate x(b +- h e_k) and x(A +- h E_ij) as
x_bar + delta with A_pert delta = b_pert - A_pert x_bar (one refinement step
from the unperturbed solution, solved to 1e-12 relative to its own right-hand
side), so the O(h) difference is not swamped by the solve tolerance.
"""
import numpy as np
import pytest

import opencslsolver_gb300 as ocsl
from opencslsolver_gb300 import _abi
from opencslsolver_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def transpose_csr(rp, col, val):
    """A^T in CSR with real entries only, rows of A ascending inside each row of A^T."""
    rp = np.asarray(rp, dtype=np.int64)
    col = np.asarray(col, dtype=np.uint64)
    n = rp.size - 1
    rows = np.repeat(np.arange(n), np.diff(rp))
    real = col < np.uint64(n)
    k = np.nonzero(real)[0]
    c = col[k].astype(np.int64)
    order = np.lexsort((rows[k], c))  # by column of A, then row of A
    perm = k[order]
    trp = np.zeros(n + 1, dtype=np.uint64)
    np.add.at(trp, c + 1, 1)
    trp = np.cumsum(trp).astype(np.uint64)
    tcol = rows[perm].astype(np.uint64)
    return trp, tcol, np.asarray(val)[perm], perm


def grad_A_reference(s, lam, x):
    n = s.n
    rows = np.repeat(np.arange(n), np.diff(s.row_ptr.astype(np.int64)))
    col = s.column_index
    g = np.zeros(col.size)
    real = col < np.uint64(n)
    g[real] = (-1.0 * lam[rows[real]]) * x[col[real].astype(np.int64)]
    return g


@pytest.mark.parametrize("kind", ["hex", "tet", "random"])
def test_transpose_solve_bit_exact_vs_oracle(ctx, oracle, kind):
    s = {"hex": W.hex_pprime(14, 11, 9, peclet=10.0), "tet": W.tet_pprime(5, peclet=50.0),
         "random": W.random_rows_system(2000, 9, seed=5)}[kind]
    ctx.set_pattern(s.row_ptr, s.column_index)
    g = np.random.default_rng(3).standard_normal(s.n)
    lam = np.zeros(s.n)
    r = ctx.solve_transpose(ocsl.ILU_BICGSTAB, s.value, g, lam, tol=1e-12)
    assert r["status"] == 0, r
    trp, tcol, tval, _ = transpose_csr(s.row_ptr, s.column_index, s.value)
    lo, rc, it, rr = oracle.bicgstab_tol(trp, tcol, tval, g, np.zeros(s.n), tol=1e-12)
    assert rc == 0
    assert np.array_equal(lam, lo) and r["iterations"] == it
    assert oracle.true_relres(trp, tcol, tval, g, lam) <= 1e-12
    # the forward solve on the same context is unaffected by the child context
    x = np.zeros(s.n)
    r = ctx.solve(ocsl.ILU_BICGSTAB, s.value, s.b, x, tol=1e-12)
    xo, _, _, _ = oracle.bicgstab_tol(s.row_ptr, s.column_index, s.value, s.b, np.zeros(s.n),
                                      tol=1e-12)
    assert np.array_equal(x, xo)


def test_transpose_solve_methods_and_edges(ctx, oracle, torch_cuda):
    torch = torch_cuda
    s = W.hex_pprime(12, peclet=10.0)
    g = np.random.default_rng(4).standard_normal(s.n)
    ctx.set_pattern(s.row_ptr, s.column_index)
    trp, tcol, tval, _ = transpose_csr(s.row_ptr, s.column_index, s.value)
    for method in (ocsl.ILU_BICGSTAB_IR32, ocsl.ILU_BICGSTAB):
        lam = np.zeros(s.n)
        r = ctx.solve_transpose(method, s.value, g, lam, tol=1e-10)
        assert r["status"] == 0
        assert oracle.true_relres(trp, tcol, tval, g, lam) <= 1e-10
    # reference-faithful methods run on A^T too, bit-identical to the oracle
    lam = np.zeros(s.n)
    ctx.solve_transpose(ocsl.BICGSTAB_REF, s.value, g, lam)
    lo, res, it = oracle.bicgstab_ref(trp, tcol, tval, g, np.zeros(s.n))
    assert np.array_equal(lam, lo)
    # device entry point agrees with the host one
    A = torch.from_numpy(s.value).cuda()
    G = torch.from_numpy(g).cuda()
    L = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    ctx.solve_transpose_device(ocsl.ILU_BICGSTAB, A, G, L, tol=1e-12)
    lam = np.zeros(s.n)
    ctx.solve_transpose(ocsl.ILU_BICGSTAB, s.value, g, lam, tol=1e-12)
    assert np.array_equal(L.cpu().numpy(), lam)


def test_transpose_without_pattern_is_an_error(ctx):
    with pytest.raises(ocsl.OcslError) as e:
        ctx.solve_transpose(ocsl.ILU_BICGSTAB, np.ones(1), np.ones(1), np.zeros(1))
    assert e.value.status == _abi.NO_PATTERN


def test_pattern_outer_exact(ctx, torch_cuda):
    torch = torch_cuda
    s = W.hex_pprime(11, 7, 5, peclet=10.0)  # has phantom columns on boundary rows
    ctx.set_pattern(s.row_ptr, s.column_index)
    rng = np.random.default_rng(8)
    lam, x = rng.standard_normal(s.n), rng.standard_normal(s.n)
    out = torch.full((s.column_index.size,), np.nan, dtype=torch.float64, device="cuda")
    ctx.pattern_outer_device(torch.from_numpy(lam).cuda(), torch.from_numpy(x).cuda(), out)
    ref = grad_A_reference(s, lam, x)
    assert np.array_equal(out.cpu().numpy(), ref)
    assert (s.column_index >= np.uint64(s.n)).any()


# ---------------------------------------------------------------- autograd harness

def make_linear_solve(ctx, method, tol):
    import torch

    class LinearSolve(torch.autograd.Function):
        """x = A^-1 b with A's values on the context's CSR pattern; backward
        solves the adjoint system (x is recomputed by the caller's forward, no
        Krylov history is kept)."""

        @staticmethod
        def forward(fctx, values, b):
            x = torch.zeros_like(b)
            r = ctx.solve_device(method, values, b, x, tol=tol)
            assert r["status"] == 0, r
            fctx.save_for_backward(values, x)
            return x

        @staticmethod
        def backward(fctx, gx):
            values, x = fctx.saved_tensors
            lam = torch.zeros_like(gx)
            r = ctx.solve_transpose_device(method, values, gx.contiguous(), lam, tol=tol)
            assert r["status"] == 0, r
            gA = torch.empty_like(values)
            ctx.pattern_outer_device(lam, x, gA, alpha=-1.0)
            return gA, lam

    return LinearSolve.apply


def fd_gradients(ctx, method, s, w, idx_b, idx_a, rel_step=1e-6):
    """Central differences of L = w . x with x_pert = x_bar + delta."""
    import torch

    dev = "cuda"
    A = torch.from_numpy(s.value).to(dev)
    B = torch.from_numpy(s.b).to(dev)
    W_ = torch.from_numpy(w).to(dev)
    xb = torch.zeros_like(B)
    assert ctx.solve_device(ocsl.ILU_BICGSTAB, A, B, xb, tol=1e-13)["status"] == 0

    def residual(vals, bvec):
        y = torch.empty_like(bvec)
        ctx.gemv_device(vals, xb, y, mode=1, z=bvec)  # y = b - A x_bar
        return y

    def delta(vals, bvec):
        d = torch.zeros_like(bvec)
        r = ctx.solve_device(method, vals, residual(vals, bvec), d, tol=1e-12)
        assert r["status"] == 0, r
        return d

    # L(+) - L(-) = w . (x_bar + d+) - w . (x_bar + d-) = w . (d+ - d-): the common
    # x_bar is cancelled before the dot product, not after it.
    fd_b = []
    for k in idx_b:
        h = rel_step * abs(s.b[k])
        Bp, Bm = B.clone(), B.clone()
        Bp[k] += h
        Bm[k] -= h
        dL = float(torch.dot(W_, delta(A, Bp) - delta(A, Bm)))
        fd_b.append(dL / (float(Bp[k]) - float(Bm[k])))
    fd_a = []
    for k in idx_a:
        h = rel_step * abs(s.value[k])
        Ap, Am = A.clone(), A.clone()
        Ap[k] += h
        Am[k] -= h
        dL = float(torch.dot(W_, delta(Ap, B) - delta(Am, B)))
        fd_a.append(dL / (float(Ap[k]) - float(Am[k])))
    return np.array(fd_b), np.array(fd_a)


def sample_entries(s, rng, count):
    real = np.nonzero(s.column_index < np.uint64(s.n))[0]
    return rng.choice(s.n, count, replace=False), rng.choice(real, count, replace=False)


def check_close(fd, adj, tol):
    floor = 1e-3 * float(np.sqrt(np.mean(adj ** 2)))
    err = np.abs(fd - adj) / np.maximum(np.abs(adj), floor)
    assert err.max() <= tol, (err.max(), fd, adj)


@pytest.mark.parametrize("method", [ocsl.ILU_BICGSTAB, ocsl.ILU_BICGSTAB_IR32])
def test_autograd_matches_finite_differences_hex128(ctx, hex128, torch_cuda, method):
    torch = torch_cuda
    s = hex128
    ctx.set_pattern(s.row_ptr, s.column_index)
    rng = np.random.default_rng(20261203 + 5)
    w = rng.standard_normal(s.n)
    solve = make_linear_solve(ctx, method, 1e-12)
    A = torch.from_numpy(s.value).cuda().requires_grad_(True)
    B = torch.from_numpy(s.b).cuda().requires_grad_(True)
    x = solve(A, B)
    L = torch.dot(torch.from_numpy(w).cuda(), x)
    L.backward()
    gA, gB = A.grad.cpu().numpy(), B.grad.cpu().numpy()
    ib, ia = sample_entries(s, rng, 32)
    fd_b, fd_a = fd_gradients(ctx, method, s, w, ib, ia)
    check_close(fd_b, gB[ib], 1e-6)
    check_close(fd_a, gA[ia], 1e-6)
    # phantom entries carry no gradient
    assert np.all(gA[s.column_index >= np.uint64(s.n)] == 0.0)


def test_gradient_matches_fp64_oracle(ctx, oracle, torch_cuda):
    torch = torch_cuda
    s = W.hex_pprime(24, peclet=10.0)
    ctx.set_pattern(s.row_ptr, s.column_index)
    w = np.random.default_rng(11).standard_normal(s.n)
    # oracle: x and lambda by the FP64 tolerance-mode solver, run tight
    xo, rc, _, _ = oracle.bicgstab_tol(s.row_ptr, s.column_index, s.value, s.b, np.zeros(s.n),
                                       tol=1e-14, maxit=5000)
    trp, tcol, tval, _ = transpose_csr(s.row_ptr, s.column_index, s.value)
    lo, rc2, _, _ = oracle.bicgstab_tol(trp, tcol, tval, w, np.zeros(s.n), tol=1e-14, maxit=5000)
    gA_o = grad_A_reference(s, lo, xo)
    for method in (ocsl.ILU_BICGSTAB, ocsl.ILU_BICGSTAB_IR32):
        solve = make_linear_solve(ctx, method, 1e-12)
        A = torch.from_numpy(s.value).cuda().requires_grad_(True)
        B = torch.from_numpy(s.b).cuda().requires_grad_(True)
        torch.dot(torch.from_numpy(w).cuda(), solve(A, B)).backward()
        gB, gA = B.grad.cpu().numpy(), A.grad.cpu().numpy()
        assert np.max(np.abs(gB - lo)) / np.max(np.abs(lo)) <= 1e-9
        assert np.max(np.abs(gA - gA_o)) / np.max(np.abs(gA_o)) <= 1e-9


@pytest.fixture(scope="module")
def hexflow128():
    return W.hex_flow_state(128, inlet_value=50.0)


@pytest.mark.parametrize("method", [ocsl.ILU_BICGSTAB, ocsl.ILU_BICGSTAB_IR32])
def test_inlet_value_gradient_through_assembly_hex128(ctx, torch_cuda, hexflow128, method):
    import assembly_cases as AC

    torch = torch_cuda
    f = hexflow128
    ctx.set_pattern(f.row_ptr, f.column_index)
    ctx.set_faces(f.left, f.right, f.bc_left)
    st = AC.to_device(torch, f.state)
    n, nnz = f.n, f.column_index.size

    def assemble(state):
        A = torch.empty(nnz, dtype=torch.float64, device="cuda")
        b, x0 = (torch.empty(n, dtype=torch.float64, device="cuda") for _ in range(2))
        ctx.assemble_device(f.eq, state, A, b, x0)
        return A, b

    A, b = assemble(st)
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    assert ctx.solve_device(method, A, b, x, tol=1e-12)["status"] == 0
    w = torch.from_numpy(np.random.default_rng(77).standard_normal(n)).cuda()
    lam = torch.zeros(n, dtype=torch.float64, device="cuda")
    assert ctx.solve_transpose_device(method, A, w, lam, tol=1e-12)["status"] == 0
    g = torch.empty(f.bc_left.size, dtype=torch.float64, device="cuda")
    ctx.bc_value_grad_device(f.eq, st, lam, g)
    inlet = torch.from_numpy(f.inlet).cuda()
    adj = float(g[inlet].sum())
    # central differences of L = w . x(p_in): the inlet value moves only b
    p_in = 50.0
    h = 1e-6 * p_in
    deltas = []
    for sgn in (1.0, -1.0):
        bv = st["bc_value"].clone()
        bv[inlet] = p_in + sgn * h
        A2, b2 = assemble(dict(st, bc_value=bv))
        assert torch.equal(A2, A)
        r = torch.empty_like(b2)
        ctx.gemv_device(A, x, r, mode=1, z=b2)  # b(p_in +- h) - A x
        d = torch.zeros_like(r)
        assert ctx.solve_device(method, A, r, d, tol=1e-12)["status"] == 0
        deltas.append(d)
    fd = float(torch.dot(w, deltas[0] - deltas[1])) / (2 * h)
    assert abs(fd - adj) <= 1e-6 * abs(adj), (fd, adj)
    assert f.inlet.size == 128 * 128
