"""GPU parity of the solvers through the C ABI.

* Reference-faithful methods (CG_solve, ILU_BICGSTAB_solve semantics) are
  bit-identical to the oracle -- x, returned residual and iteration count --
  and within 1e-12 of the reference's own recorded outputs (its solver
  unit-test system, solve calls captured from its SIMPLE loop, seeded
  systems).
* Tolerance-mode methods reach ||b - A x|| / ||b|| <= tol (checked on the host
  in long double) and agree with the oracle's solution.
* Edge cases: empty system, b = 0, non-finite input, iteration cap, bad and
  missing patterns, host- vs device-buffer entry points, the CMatrix_solver
  mirror.
"""
import numpy as np
import pytest

import opencslsolver_gb300 as ocsl
from opencslsolver_gb300 import _abi
from opencslsolver_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def rel(a, b):
    den = max(float(np.max(np.abs(b))), 1e-300)
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b)))) / den


def gen_systems():
    return [W.hex_pprime(16, peclet=10.0), W.hex_pprime(12, 10, 9, peclet=0.0),
            W.tet_pprime(5, peclet=50.0), W.random_rows_system(2500, 11, seed=21)]


def run(ctx, method, s, x0, **opts):
    x = np.array(x0, dtype=np.float64, copy=True)
    r = ctx.solve(method, s.value, s.b, x, **opts)
    return x, r


@pytest.mark.parametrize("k", range(4))
def test_reference_methods_bit_exact(ctx, oracle, k):
    s = gen_systems()[k]
    ctx.set_pattern(s.row_ptr, s.column_index)
    for x0 in (np.zeros(s.n), np.random.default_rng(k).uniform(-1, 1, s.n)):
        x, r = run(ctx, ocsl.CG_REF, s, x0)
        xo, res, it = oracle.cg_ref(s.row_ptr, s.column_index, s.value, s.b, x0)
        assert r["status"] == 0
        assert np.array_equal(x, xo) and r["residual"] == res and r["iterations"] == it
        x, r = run(ctx, ocsl.BICGSTAB_REF, s, x0)
        xo, res, it = oracle.bicgstab_ref(s.row_ptr, s.column_index, s.value, s.b, x0)
        assert r["status"] == 0
        assert np.array_equal(x, xo) and r["residual"] == res and r["iterations"] == it


def test_reference_unit_test_system(ctx, golden_kat):
    z = golden_kat
    ctx.set_pattern(z["row_ptr"], z["column_index"])
    s = W.System(z["row_ptr"], z["column_index"], z["value"], z["b"])
    x, r = run(ctx, ocsl.CG_REF, s, z["x0"])
    assert r["iterations"] == 4 and rel(x, z["cg_x"]) <= 1e-14
    assert abs(r["residual"] - float(z["cg_res"])) <= 1e-12 * float(z["cg_res"])
    x, r = run(ctx, ocsl.BICGSTAB_REF, s, z["x0"])
    assert r["iterations"] == 3 and rel(x, z["bicg_x"]) <= 1e-14
    assert abs(r["residual"] - float(z["bicg_res"])) <= 1e-9 * float(z["bicg_res"])


def test_shocktube_calls(ctx, oracle, golden_shocktube):
    """Every solve call recorded from the reference's SIMPLE loop."""
    z = golden_shocktube
    ctx.set_pattern(z["row_ptr"], z["column_index"])
    for k in range(z["meta"].shape[0]):
        eq = int(z["meta"][k, 2])
        s = W.System(z["row_ptr"], z["column_index"], z["value"][k], z["b"][k])
        method = ocsl.CG_REF if eq < 3 else ocsl.BICGSTAB_REF
        x, r = run(ctx, method, s, z["x0"][k])
        fn = oracle.cg_ref if eq < 3 else oracle.bicgstab_ref
        xo, res, it = fn(z["row_ptr"], z["column_index"], s.value, s.b, z["x0"][k])
        assert np.array_equal(x, xo) and r["residual"] == res and r["iterations"] == it
        assert rel(x, z["x"][k]) <= 1e-12, (k, eq)


def test_seeded_systems_vs_reference(ctx, golden_small):
    for c in golden_small:
        ctx.set_pattern(c["row_ptr"], c["column_index"])
        s = W.System(c["row_ptr"], c["column_index"], c["value"], c["b"])
        x, r = run(ctx, ocsl.CG_REF, s, c["x0"])
        assert rel(x, c["cg_x"]) <= 1e-12
        x, r = run(ctx, ocsl.BICGSTAB_REF, s, c["x0"])
        assert rel(x, c["bicg_x"]) <= 1e-10


@pytest.mark.parametrize("k", range(4))
def test_tolerance_bicgstab_fp64(ctx, oracle, k):
    s = gen_systems()[k]
    ctx.set_pattern(s.row_ptr, s.column_index)
    x0 = np.zeros(s.n)
    x, r = run(ctx, ocsl.ILU_BICGSTAB, s, x0, tol=1e-10)
    assert r["status"] == 0, r
    assert oracle.true_relres(s.row_ptr, s.column_index, s.value, s.b, x) <= 1e-10
    xo, rc, it, rr = oracle.bicgstab_tol(s.row_ptr, s.column_index, s.value, s.b, x0, tol=1e-10)
    # same algorithm, same rounding, same reduction order: same iterates
    assert np.array_equal(x, xo) and r["iterations"] == it


@pytest.mark.parametrize("k", range(4))
def test_tolerance_ir32(ctx, oracle, k):
    s = gen_systems()[k]
    ctx.set_pattern(s.row_ptr, s.column_index)
    x0 = np.zeros(s.n)
    x, r = run(ctx, ocsl.ILU_BICGSTAB_IR32, s, x0, tol=1e-10)
    assert r["status"] == 0, r
    assert r["outer_iterations"] >= 1
    rr = oracle.true_relres(s.row_ptr, s.column_index, s.value, s.b, x)
    assert rr <= 1e-10
    xo, _, _, _ = oracle.bicgstab_tol(s.row_ptr, s.column_index, s.value, s.b, x0, tol=1e-12)
    assert rel(x, xo) <= 1e-7


def test_tolerance_pcg_symmetric(ctx, oracle):
    s = W.hex_pprime(14, peclet=0.0)
    ctx.set_pattern(s.row_ptr, s.column_index)
    x0 = np.zeros(s.n)
    x, r = run(ctx, ocsl.PCG, s, x0, tol=1e-10)
    assert r["status"] == 0
    xo, rc, it, rr = oracle.pcg_tol(s.row_ptr, s.column_index, s.value, s.b, x0, tol=1e-10)
    assert np.array_equal(x, xo) and r["iterations"] == it
    assert oracle.true_relres(s.row_ptr, s.column_index, s.value, s.b, x) <= 1e-10


def test_host_and_device_entry_points_agree(ctx, torch_cuda):
    s = W.hex_pprime(10)
    ctx.set_pattern(s.row_ptr, s.column_index)
    for method in (ocsl.BICGSTAB_REF, ocsl.ILU_BICGSTAB, ocsl.ILU_BICGSTAB_IR32):
        xh, _ = run(ctx, method, s, np.zeros(s.n))
        A = torch_cuda.from_numpy(s.value).cuda()
        B = torch_cuda.from_numpy(s.b).cuda()
        X = torch_cuda.zeros(s.n, dtype=torch_cuda.float64, device="cuda")
        r = ctx.solve_device(method, A, B, X)
        assert r["status"] == 0 and np.array_equal(X.cpu().numpy(), xh)


def test_empty_system(ctx):
    ctx.set_pattern(np.zeros(1, np.uint64), np.zeros(0, np.uint64))
    x = np.zeros(0)
    for m in range(5):
        r = ctx.solve(m, np.zeros(0), np.zeros(0), x)
        assert r["status"] == 0


def test_zero_rhs(ctx, oracle):
    s = W.hex_pprime(6)
    ctx.set_pattern(s.row_ptr, s.column_index)
    z = W.System(s.row_ptr, s.column_index, s.value, np.zeros(s.n))
    for m in (ocsl.ILU_BICGSTAB, ocsl.ILU_BICGSTAB_IR32, ocsl.PCG):
        x, r = run(ctx, m, z, np.ones(s.n))
        assert r["status"] == 0 and np.all(x == 0.0)
    # reference-faithful CG divides by norm(b, b) nowhere: it runs as the oracle does
    x, r = run(ctx, ocsl.CG_REF, z, np.ones(s.n))
    xo, res, it = oracle.cg_ref(s.row_ptr, s.column_index, s.value, z.b, np.ones(s.n))
    assert np.array_equal(x, xo) and r["residual"] == res


def test_nonfinite_rhs_reported(ctx):
    s = W.hex_pprime(6)
    ctx.set_pattern(s.row_ptr, s.column_index)
    b = s.b.copy()
    b[7] = np.nan
    x, r = run(ctx, ocsl.ILU_BICGSTAB, W.System(s.row_ptr, s.column_index, s.value, b),
               np.zeros(s.n))
    assert r["status"] == _abi.NONFINITE


def test_iteration_cap_reported(ctx, oracle):
    s = W.tet_pprime(5)
    ctx.set_pattern(s.row_ptr, s.column_index)
    x, r = run(ctx, ocsl.ILU_BICGSTAB, s, np.zeros(s.n), tol=1e-14, maxit=2)
    assert r["status"] == _abi.NOT_CONVERGED and r["iterations"] <= 2
    # the context stays usable
    x, r = run(ctx, ocsl.ILU_BICGSTAB, s, np.zeros(s.n), tol=1e-10)
    assert r["status"] == 0


def test_bad_and_missing_pattern(ctx):
    s = W.hex_pprime(4)
    with pytest.raises(ocsl.OcslError) as e:
        ctx.solve(ocsl.CG_REF, s.value, s.b, np.zeros(s.n))
    assert e.value.status == _abi.NO_PATTERN
    rp = np.array([0, 2, 4], np.uint64)
    col = np.array([0, 1, 0, 5], np.uint64)
    with pytest.raises(ocsl.OcslError) as e:
        ctx.set_pattern(rp, col)
    assert e.value.status == _abi.BAD_PATTERN


def test_cmatrix_solver_mirror(lib_built, torch_cuda, golden_kat):
    """The reference class's call protocol: fill members, call, read x_vector."""
    z = golden_kat
    s = ocsl.CMatrix_solver(10, 10, 28)
    s.matrix.row_ptr = z["row_ptr"].copy()
    s.matrix.column_index = z["column_index"].copy()
    s.matrix.value = z["value"].copy()
    s.b_vector.value = z["b"].copy()
    s.x_vector.value = z["x0"].copy()
    res = s.CG_solve()
    assert rel(s.x_vector.value, z["cg_x"]) <= 1e-14
    assert abs(res - float(z["cg_res"])) <= 1e-12 * float(z["cg_res"])
    s.x_vector.value = z["x0"].copy()
    res = s.ILU_BICGSTAB_solve()
    assert rel(s.x_vector.value, z["bicg_x"]) <= 1e-14
    s.x_vector.value = np.zeros(10)
    r = s.solve("ilu_bicgstab", tol=1e-12)
    assert r["status"] == 0 and r["residual"] <= 1e-12


def test_full_size_solves(ctx, oracle, hex128):
    """128^3 jittered hex p' system: FP64 and FP32-refined ILU-BiCGSTAB reach
    1e-10 (true residual recomputed on the host); the reference-faithful
    ILU_BICGSTAB_solve is bit-identical to the oracle at full size."""
    s = hex128
    ctx.set_pattern(s.row_ptr, s.column_index)
    x0 = np.zeros(s.n)
    x64, r64 = run(ctx, ocsl.ILU_BICGSTAB, s, x0, tol=1e-10)
    assert r64["status"] == 0
    assert oracle.true_relres(s.row_ptr, s.column_index, s.value, s.b, x64) <= 1e-10
    x32, r32 = run(ctx, ocsl.ILU_BICGSTAB_IR32, s, x0, tol=1e-10)
    assert r32["status"] == 0
    assert oracle.true_relres(s.row_ptr, s.column_index, s.value, s.b, x32) <= 1e-10
    assert rel(x32, x64) <= 1e-7
    xr, rr = run(ctx, ocsl.BICGSTAB_REF, s, x0)
    xo, res, it = oracle.bicgstab_ref(s.row_ptr, s.column_index, s.value, s.b, x0)
    assert np.array_equal(xr, xo) and rr["residual"] == res


def test_misaligned_device_pointer_rejected(ctx, torch_cuda):
    """A device pointer that is not 8-byte aligned is refused on the host,
    before any kernel runs."""
    s = W.hex_pprime(4)
    ctx.set_pattern(s.row_ptr, s.column_index)
    A = torch_cuda.from_numpy(s.value).cuda()
    X = torch_cuda.zeros(s.n + 1, dtype=torch_cuda.float64, device="cuda")
    Y = torch_cuda.zeros(s.n, dtype=torch_cuda.float64, device="cuda")
    with pytest.raises(ocsl.OcslError) as e:
        ctx.gemv_device(A, X.data_ptr() + 4, Y)
    assert e.value.status == _abi.BAD_ARGUMENT
    ctx.gemv_device(A, X[1:], Y)  # element-aligned offsets are fine


@pytest.mark.parametrize("method", [ocsl.BICGSTAB_REF, ocsl.ILU_BICGSTAB, ocsl.ILU_BICGSTAB_IR32])
def test_sweep_kernels_give_identical_solves(ctx, method):
    """Level-scheduled and structured sweeps produce the same bits end to
    end (FP64 and FP32 sweeps)."""
    s = W.hex_pprime(40, 36, 33)
    ctx.set_pattern(s.row_ptr, s.column_index)
    out = []
    for kind in (1, 2):
        ctx.set_sweep_kernel(kind)
        assert ctx.sweep_info()["kind"] == kind
        x, r = run(ctx, method, s, np.zeros(s.n), tol=1e-10)
        assert r["status"] == 0
        out.append((x, r["iterations"]))
    for x, it in out[1:]:
        assert np.array_equal(out[0][0], x) and out[0][1] == it


@pytest.mark.parametrize("method", [ocsl.BICGSTAB_REF, ocsl.ILU_BICGSTAB, ocsl.ILU_BICGSTAB_IR32])
def test_clustered_sweeps_give_identical_solves(ctx, torch_cuda, method):
    """Sweeps with tiles in thread-block clusters give the bits and
    iteration counts of single-tile sweeps, on the legacy stream (direct
    launches) and on a created stream (graph replay), and for lockstep
    right-hand sides."""
    torch = torch_cuda
    s = W.hex_pprime(40, 36, 33)
    ctx.set_pattern(s.row_ptr, s.column_index)
    A = torch.from_numpy(s.value).cuda()
    rng = np.random.default_rng(21)
    B = torch.from_numpy(rng.uniform(-1, 1, (3, s.n))).cuda()
    side = torch.cuda.Stream()
    out = {}
    for cl in [(1, 1), (2, 2), (4, 4), (2, 4)]:
        ctx.set_sweep_kernel(2, 8, 8)
        ctx.set_sweep_cluster(*cl)
        assert ctx.sweep_info()["cluster"] == cl
        X = torch.zeros(s.n, dtype=torch.float64, device="cuda")
        r = ctx.solve_device(method, A, B[0], X, tol=1e-10)
        assert r["status"] == 0, r
        with torch.cuda.stream(side):
            X2 = torch.zeros(s.n, dtype=torch.float64, device="cuda")
            r2 = ctx.solve_device(method, A, B[0], X2, tol=1e-10)
            XM = torch.zeros_like(B)
            rm = ctx.solve_multi_device(method, A, B, XM, tol=1e-10) \
                if method != ocsl.BICGSTAB_REF else None
        torch.cuda.synchronize()
        assert torch.equal(X, X2) and r["iterations"] == r2["iterations"]
        out[cl] = (X, r["iterations"], XM if rm is not None else None)
    X0, it0, XM0 = out[(1, 1)]
    for cl, (X, it, XM) in out.items():
        assert torch.equal(X, X0) and it == it0, cl
        if XM0 is not None:
            assert torch.equal(XM, XM0), cl
            assert torch.equal(XM[0], X0), cl


@pytest.mark.parametrize("method", [ocsl.PCG, ocsl.ILU_BICGSTAB, ocsl.ILU_BICGSTAB_IR32])
def test_graph_replay_gives_identical_solves(ctx, torch_cuda, method):
    """Iteration batches replayed from CUDA graphs give the same bits as
    direct launches, over several solves with changing matrices and right-hand
    sides (new device buffers each time, as a finite-difference loop does)."""
    torch = torch_cuda
    s = W.hex_pprime(30, 26, 22, peclet=0.0 if method == ocsl.PCG else 10.0)
    ctx.set_pattern(s.row_ptr, s.column_index)
    rng = np.random.default_rng(12)
    cases = []
    for k in range(4):
        val = s.value.copy()
        val[rng.integers(0, val.size, 5)] *= 1.0 + 1e-3 * (k + 1)
        cases.append((val, rng.uniform(-1, 1, s.n)))
    out = {}
    side = torch.cuda.Stream()  # graphs need a created stream, not the legacy default one
    with torch.cuda.stream(side):
        for graphs in (True, False):
            ctx.set_graphs(graphs)
            res = []
            for val, b in cases:
                A = torch.from_numpy(val).cuda()
                B = torch.from_numpy(b).cuda()
                X = torch.zeros(s.n, dtype=torch.float64, device="cuda")
                r = ctx.solve_device(method, A, B, X, tol=1e-11)
                assert r["status"] == 0, r
                res.append((X.cpu().numpy(), r["iterations"]))
            out[graphs] = res
    for (x1, i1), (x2, i2) in zip(out[True], out[False]):
        assert i1 == i2 and np.array_equal(x1, x2)


def test_new_pattern_drops_captured_graph(ctx, torch_cuda):
    """A context that replayed iteration graphs for one box and then gets a
    box of the same size but another shape (same buffer sizes, so the
    allocator may hand back the same addresses) solves the new system exactly
    as a fresh context does: captured graphs go with the old pattern."""
    torch = torch_cuda
    s1, s2 = W.hex_pprime(40, 36, 33), W.hex_pprime(33, 40, 36)
    assert s1.n == s2.n and s1.value.size == s2.value.size
    side = torch.cuda.Stream()
    fresh = ocsl.Context(0)
    with torch.cuda.stream(side):
        out = []
        for c, systems in ((ctx, (s1, s2)), (fresh, (s2,))):
            for s in systems:
                c.set_pattern(s.row_ptr, s.column_index)
                A = torch.from_numpy(s.value).cuda()
                B = torch.from_numpy(s.b).cuda()
                X = torch.zeros(s.n, dtype=torch.float64, device="cuda")
                r = c.solve_device(ocsl.ILU_BICGSTAB_IR32, A, B, X, tol=1e-10)
                assert r["status"] == 0, r
            out.append((X, r["iterations"]))
    torch.cuda.synchronize()
    fresh.close()
    assert torch.equal(out[0][0], out[1][0]) and out[0][1] == out[1][1]


@pytest.mark.parametrize("method", [ocsl.BICGSTAB_REF, ocsl.PCG, ocsl.ILU_BICGSTAB,
                                    ocsl.ILU_BICGSTAB_IR32])
def test_spmv_lanes_give_identical_solves(ctx, torch_cuda, method):
    """Every CSR SpMV shape (lanes per row) gives the same solve, bit for bit,
    on the tet system, whose SpMVs carry the fused dots of every method; the
    SpMV autotuner keeps one of them."""
    torch = torch_cuda
    s = W.tet_pprime(9, 8, 7, peclet=0.0 if method == ocsl.PCG else 50.0)
    ctx.set_pattern(s.row_ptr, s.column_index)
    A = torch.from_numpy(s.value).cuda()
    B = torch.from_numpy(s.b).cuda()
    out = {}
    for lanes in (1, 4, 16):
        ctx.set_spmv_lanes(lanes)
        X = torch.zeros(s.n, dtype=torch.float64, device="cuda")
        r = ctx.solve_device(method, A, B, X)
        out[lanes] = (X, r["iterations"], r["status"])
    for lanes in (4, 16):
        assert torch.equal(out[lanes][0], out[1][0]), lanes
        assert out[lanes][1:] == out[1][1:], lanes
    t = ctx.autotune_spmv(method, A)
    assert t["lanes"] in (1, 4, 16) and t["spmv_us"] > 0 and ctx.spmv_lanes() == t["lanes"]
    X = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    ctx.solve_device(method, A, B, X)
    assert torch.equal(X, out[1][0])


@pytest.mark.parametrize("method", [ocsl.ILU_BICGSTAB_IR32, ocsl.ILU_BICGSTAB, ocsl.BICGSTAB_REF])
def test_autotuned_tile_gives_identical_solves(ctx, torch_cuda, method):
    """ocsl_autotune_device picks one of its candidate tiles, keeps it for the
    next solves, and the solve's bits do not depend on it."""
    torch = torch_cuda
    s = W.hex_pprime(40, 36, 33)
    ctx.set_pattern(s.row_ptr, s.column_index)
    A = torch.from_numpy(s.value).cuda()
    B = torch.from_numpy(s.b).cuda()
    X0 = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    r0 = ctx.solve_device(method, A, B, X0)
    t = ctx.autotune(method, A)
    assert t["sweep_us"] > 0 and t["tiles"][0] * t["tiles"][1] <= 256, t
    sfx = "32" if method == ocsl.ILU_BICGSTAB_IR32 else ""
    info = ctx.sweep_info()
    assert info["tiles" + sfx] == t["tiles"] and info["cluster" + sfx] == t["cluster"], (info, t)
    X1 = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    r1 = ctx.solve_device(method, A, B, X1)
    assert torch.equal(X0, X1) and r0["iterations"] == r1["iterations"]
    # the other precision's geometry is tuned on its own
    other = ocsl.ILU_BICGSTAB if method == ocsl.ILU_BICGSTAB_IR32 else ocsl.ILU_BICGSTAB_IR32
    t2 = ctx.autotune(other, A)
    info2 = ctx.sweep_info()
    assert info2["tiles" + sfx] == t["tiles"] and info2["cluster" + sfx] == t["cluster"]
    X2 = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    r2 = ctx.solve_device(method, A, B, X2)
    assert torch.equal(X0, X2) and r0["iterations"] == r2["iterations"]
    assert t2["sweep_us"] > 0
    # nothing to tune: Jacobi PCG, level-scheduled sweeps
    assert ctx.autotune(ocsl.PCG, A)["tiles"] == (0, 0)
    ctx.set_sweep_kernel(1)
    assert ctx.autotune(method, A)["tiles"] == (0, 0)
