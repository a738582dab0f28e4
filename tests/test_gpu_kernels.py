"""GPU parity of the kernel-level entry points (gemv, dot, ILU factor,
triangular sweeps) against the CPU oracle -- bit for bit -- and against the
reference's own outputs recorded in tests/golden (tight relative tolerance).

Device buffers come from torch; every call goes through the C ABI."""
import numpy as np
import pytest

import opencslsolver_gb300 as ocsl
from opencslsolver_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def host(t):
    return t.cpu().numpy()


def rel(a, b):
    den = max(float(np.max(np.abs(b))), 1e-300) if np.size(b) else 1.0
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b)))) / den if np.size(b) else 0.0


def systems():
    return [W.hex_pprime(20, peclet=10.0), W.hex_pprime(9, 13, 7, peclet=0.0),
            W.tet_pprime(6, peclet=50.0), W.random_rows_system(3000, 14, seed=4),
            W.random_rows_system(700, 40, seed=9)]


@pytest.mark.parametrize("k", range(5))
def test_gemv_bit_exact(ctx, torch_cuda, oracle, k):
    s = systems()[k]
    rng = np.random.default_rng(k)
    x, z = rng.standard_normal(s.n), rng.standard_normal(s.n)
    ctx.set_pattern(s.row_ptr, s.column_index)
    A, X, Z = dev(torch_cuda, s.value), dev(torch_cuda, x), dev(torch_cuda, z)
    Y = torch_cuda.empty_like(X)
    for mode, a in ((0, 0.0), (1, 0.0), (2, -0.731)):
        ctx.gemv_device(A, X, Y, mode=mode, a=a, z=Z if mode else None)
        want = oracle.gemv(s.row_ptr, s.column_index, s.value, x, mode, a, z)
        assert np.array_equal(host(Y), want), (s.name, mode)


@pytest.mark.parametrize("k", range(5))
def test_gemv_lanes_per_row_bit_exact(ctx, torch_cuda, oracle, k):
    """The CSR SpMV with 4 and 16 lanes per row (ocsl_set_spmv_lanes): the
    oracle's bits for rows of 5 to 40 entries, phantoms included."""
    s = systems()[k]
    rng = np.random.default_rng(100 + k)
    x, z = rng.standard_normal(s.n), rng.standard_normal(s.n)
    ctx.set_pattern(s.row_ptr, s.column_index)
    A, X, Z = dev(torch_cuda, s.value), dev(torch_cuda, x), dev(torch_cuda, z)
    Y = torch_cuda.empty_like(X)
    for lanes in (4, 16):
        ctx.set_spmv_lanes(lanes)
        assert ctx.spmv_lanes() == lanes
        for mode, a in ((0, 0.0), (1, 0.0), (2, -0.731)):
            ctx.gemv_device(A, X, Y, mode=mode, a=a, z=Z if mode else None)
            want = oracle.gemv(s.row_ptr, s.column_index, s.value, x, mode, a, z)
            assert np.array_equal(host(Y), want), (s.name, lanes, mode)
    with pytest.raises(ocsl.OcslError):
        ctx.set_spmv_lanes(3)
    ctx.set_pattern(s.row_ptr, s.column_index)
    assert ctx.spmv_lanes() == 1  # a new pattern starts from the default


def test_gemv_matches_reference_golden(ctx, torch_cuda, golden_small):
    for c in golden_small:
        ctx.set_pattern(c["row_ptr"], c["column_index"])
        A, X, Z = dev(torch_cuda, c["value"]), dev(torch_cuda, c["xin"]), dev(torch_cuda, c["z"])
        Y = torch_cuda.empty_like(X)
        ctx.gemv_device(A, X, Y, mode=0)
        assert rel(host(Y), c["gemv0"]) <= 1e-15
        ctx.gemv_device(A, X, Y, mode=1, z=Z)
        assert rel(host(Y), c["gemv1"]) <= 1e-15
        ctx.gemv_device(A, X, Y, mode=2, a=-0.37, z=Z)
        assert rel(host(Y), c["gemv2"]) <= 1e-15


@pytest.mark.parametrize("n", [1, 255, 2047, 2048, 2049, 100_003, 3_000_001])
def test_dot_bit_exact(ctx, torch_cuda, oracle, n):
    rng = np.random.default_rng(n)
    x, y = rng.standard_normal(n), rng.standard_normal(n)
    got = ctx.dot_device(dev(torch_cuda, x), dev(torch_cuda, y))
    assert got == oracle.dot(x, y)


@pytest.mark.parametrize("k", range(5))
@pytest.mark.parametrize("sweeps", [0, 1, 3, 5])
def test_ilu_bit_exact(ctx, torch_cuda, oracle, k, sweeps):
    s = systems()[k]
    ctx.set_pattern(s.row_ptr, s.column_index)
    A = dev(torch_cuda, s.value)
    M = torch_cuda.empty_like(A)
    ctx.ilu_device(A, M, sweeps)
    assert np.array_equal(host(M), oracle.ilu(s.row_ptr, s.column_index, s.value, sweeps))


@pytest.mark.parametrize("k", range(5))
def test_sweeps_bit_exact(ctx, torch_cuda, oracle, k):
    s = systems()[k]
    rng = np.random.default_rng(10 + k)
    b = rng.standard_normal(s.n)
    ctx.set_pattern(s.row_ptr, s.column_index)
    Mh = oracle.ilu(s.row_ptr, s.column_index, s.value)
    M, B = dev(torch_cuda, Mh), dev(torch_cuda, b)
    Y = torch_cuda.empty_like(B)
    X = torch_cuda.empty_like(B)
    ctx.forsub_device(M, B, Y)
    y = oracle.forsub(s.row_ptr, s.column_index, Mh, b)
    assert np.array_equal(host(Y), y)
    ctx.backsub_device(M, Y, X)
    assert np.array_equal(host(X), oracle.backsub(s.row_ptr, s.column_index, Mh, y))


def test_factor_and_sweeps_match_reference_golden(ctx, torch_cuda, golden_small):
    for c in golden_small:
        ctx.set_pattern(c["row_ptr"], c["column_index"])
        A = dev(torch_cuda, c["value"])
        M = torch_cuda.empty_like(A)
        ctx.ilu_device(A, M, 3)
        assert rel(host(M), c["ilu"]) <= 1e-15, str(c["name"])
        Mref, Z = dev(torch_cuda, c["ilu"]), dev(torch_cuda, c["z"])
        Y = torch_cuda.empty_like(Z)
        ctx.forsub_device(Mref, Z, Y)
        assert rel(host(Y), c["forsub"]) <= 1e-14
        ctx.backsub_device(Mref, Z, Y)
        assert rel(host(Y), c["backsub"]) <= 1e-14


def test_full_size_spmv_and_sweeps(ctx, torch_cuda, oracle, hex128):
    """128^3 jittered hex p' system (n = 2,097,152): SpMV and both sweeps are
    bit-identical to the oracle at full size."""
    s = hex128
    ctx.set_pattern(s.row_ptr, s.column_index)
    info = ctx.pattern_info()
    assert info["n"] == 2_097_152 and info["nnz_real"] == 14_581_760
    assert info["fw_levels"] == 382 and info["bw_levels"] == 382
    rng = np.random.default_rng(1)
    x = rng.standard_normal(s.n)
    A, X = dev(torch_cuda, s.value), dev(torch_cuda, x)
    Y = torch_cuda.empty_like(X)
    ctx.gemv_device(A, X, Y)
    assert np.array_equal(host(Y), oracle.gemv(s.row_ptr, s.column_index, s.value, x))
    Mh = oracle.ilu(s.row_ptr, s.column_index, s.value)
    M = torch_cuda.empty_like(A)
    ctx.ilu_device(A, M, 3)
    assert np.array_equal(host(M), Mh)
    ctx.forsub_device(M, X, Y)
    y = oracle.forsub(s.row_ptr, s.column_index, Mh, x)
    assert np.array_equal(host(Y), y)
    Z = torch_cuda.empty_like(X)
    ctx.backsub_device(M, Y, Z)
    assert np.array_equal(host(Z), oracle.backsub(s.row_ptr, s.column_index, Mh, y))


BOXES = [(20, 20, 20), (13, 7, 9), (5, 17, 3), (33, 1, 1), (9, 12, 1), (1000, 1, 1)]


@pytest.mark.parametrize("dims", BOXES)
@pytest.mark.parametrize("tiles", [(0, 0), (4, 8), (3, 5), (32, 8)])
def test_structured_sweeps_bit_exact(ctx, torch_cuda, oracle, dims, tiles):
    kind = 2
    """The structured (box) sweep kernel against the oracle and against the
    level-scheduled kernel, for several box shapes and column tiles."""
    if dims[1] == 1:
        rp, col = W.pattern_1d(dims[0])
        rng = np.random.default_rng(2)
        val = np.where(col == W.PHANTOM, 0.0, rng.uniform(-1, 0, col.size))
        rows = np.repeat(np.arange(dims[0]), np.diff(rp.astype(np.int64)))
        val[col == rows.astype(np.uint64)] = 3.0
        s = W.System(rp, col, val, rng.uniform(-1, 1, dims[0]))
    else:
        s = W.hex_pprime(*dims)
    ctx.set_pattern(s.row_ptr, s.column_index)
    ctx.set_sweep_kernel(kind, *tiles)
    info = ctx.sweep_info()
    assert info["kind"] == kind
    rng = np.random.default_rng(7)
    b = rng.standard_normal(s.n)
    Mh = oracle.ilu(s.row_ptr, s.column_index, s.value)
    M, B = dev(torch_cuda, Mh), dev(torch_cuda, b)
    Y, X = torch_cuda.empty_like(B), torch_cuda.empty_like(B)
    ctx.forsub_device(M, B, Y)
    y = oracle.forsub(s.row_ptr, s.column_index, Mh, b)
    assert np.array_equal(host(Y), y)
    ctx.backsub_device(M, Y, X)
    assert np.array_equal(host(X), oracle.backsub(s.row_ptr, s.column_index, Mh, y))
    ctx.set_sweep_kernel(1)
    assert ctx.sweep_info()["kind"] == 1
    X2 = torch_cuda.empty_like(B)
    ctx.backsub_device(M, Y, X2)
    assert torch_cuda.equal(X, X2)


CLUSTER_CASES = [
    ((20, 20, 20), (4, 4), (2, 2)),
    ((20, 20, 20), (4, 4), (4, 4)),
    ((20, 20, 20), (3, 5), (4, 2)),
    ((13, 7, 9), (2, 2), (4, 1)),
    ((13, 7, 9), (2, 2), (1, 4)),
    ((64, 48, 40), (8, 8), (4, 4)),   # partial clusters: 6 x 5 tiles in 4 x 4 clusters
    ((64, 48, 40), (16, 8), (2, 4)),
    ((9, 12, 1), (4, 1), (2, 2)),     # one tile row: the cluster is clipped to 2 x 1
]


def _box_system(dims, seed=2):
    """A box-stencil system; a 1-cell-wide box is the reference's 1D mesh."""
    if dims[1] == 1 and dims[2] == 1:
        rp, col = W.pattern_1d(dims[0])
        rng = np.random.default_rng(seed)
        val = np.where(col == W.PHANTOM, 0.0, rng.uniform(-1, 0, col.size))
        rows = np.repeat(np.arange(dims[0]), np.diff(rp.astype(np.int64)))
        val[col == rows.astype(np.uint64)] = 3.0
        return W.System(rp, col, val, rng.uniform(-1, 1, dims[0]))
    return W.hex_pprime(*dims)


SERIAL = [(33, 1, 1), (1000, 1, 1), (5120, 1, 1), (2000, 2, 1), (1500, 2, 1)]


@pytest.mark.parametrize("dims", SERIAL)
def test_serial_sweeps_bit_exact(ctx, torch_cuda, oracle, dims):
    """Tiny systems whose schedule is about as deep as they are long take the
    one-warp serial sweep in automatic mode (kind 4): sweeps and whole solves
    equal the oracle bit for bit, FP64 and FP32."""
    import opencslsolver_gb300 as ocsl

    s = _box_system(dims)
    ctx.set_pattern(s.row_ptr, s.column_index)
    assert ctx.sweep_info()["kind"] == 4
    rng = np.random.default_rng(3)
    b = rng.standard_normal(s.n)
    Mh = oracle.ilu(s.row_ptr, s.column_index, s.value)
    M, B = dev(torch_cuda, Mh), dev(torch_cuda, b)
    Y, X = torch_cuda.empty_like(B), torch_cuda.empty_like(B)
    ctx.forsub_device(M, B, Y)
    y = oracle.forsub(s.row_ptr, s.column_index, Mh, b)
    assert np.array_equal(host(Y), y)
    ctx.backsub_device(M, Y, X)
    assert np.array_equal(host(X), oracle.backsub(s.row_ptr, s.column_index, Mh, y))
    x0 = np.zeros(s.n)
    for method, fn in ((ocsl.BICGSTAB_REF, oracle.bicgstab_ref), (ocsl.CG_REF, oracle.cg_ref)):
        x = x0.copy()
        r = ctx.solve(method, s.value, s.b, x)
        xo, res_o, it_o = fn(s.row_ptr, s.column_index, s.value, s.b, x0)
        assert np.array_equal(x, xo) and r["residual"] == res_o and r["iterations"] == it_o
    x = x0.copy()
    r = ctx.solve(ocsl.ILU_BICGSTAB, s.value, s.b, x, tol=1e-10)
    xo, rc, it, _ = oracle.bicgstab_tol(s.row_ptr, s.column_index, s.value, s.b, x0, tol=1e-10)
    assert r["status"] == 0 and np.array_equal(x, xo) and r["iterations"] == it
    x = x0.copy()
    r = ctx.solve(ocsl.ILU_BICGSTAB_IR32, s.value, s.b, x, tol=1e-10)
    assert r["status"] == 0
    assert oracle.true_relres(s.row_ptr, s.column_index, s.value, s.b, x) <= 1e-10
    # the other kernels give the same bits
    ctx.set_sweep_kernel(1)
    assert ctx.sweep_info()["kind"] == 1
    Y2 = torch_cuda.empty_like(B)
    ctx.forsub_device(M, B, Y2)
    assert torch_cuda.equal(Y, Y2)


def _random_doubles(rng, size, emin, emax):
    """Random signs, exponents in [emin, emax] and 52-bit mantissas, with a
    share of mantissas near all ones or all zeros (binade edges)."""
    mant = rng.integers(0, 1 << 52, size, dtype=np.uint64)
    edge = rng.random(size)
    mant[edge < 0.1] = np.uint64((1 << 52) - 1) - rng.integers(0, 64, int((edge < 0.1).sum()),
                                                               dtype=np.uint64)
    mant[(edge >= 0.1) & (edge < 0.2)] = rng.integers(0, 64, int(((edge >= 0.1) & (edge < 0.2)).sum()),
                                                      dtype=np.uint64)
    exp = (rng.integers(emin, emax + 1, size) + 1023).astype(np.uint64)
    sign = rng.integers(0, 2, size, dtype=np.uint64)
    return ((sign << np.uint64(63)) | (exp << np.uint64(52)) | mant).view(np.float64)


def test_serial_backsub_division_is_correctly_rounded(ctx, torch_cuda):
    """The serial backward sweep divides by the pivot with Markstein's method
    (a two-term reciprocal + one residual correction) in the safe exponent range and by
    the IEEE division elsewhere: on a 1D system whose off-diagonal entries are
    0, x = y / M_ii must be the correctly rounded quotient, bit for bit, for
    12M operand pairs -- exponents within +-260 (the fast path), pairs beyond
    +-500 with a moderate quotient, subnormals and zeros (the IEEE path),
    mantissas at binade edges.  Quotients stay finite, so no row poisons the
    next through 0 * inf."""
    n = 5120
    rp, col = W.pattern_1d(n)
    ctx.set_pattern(rp, col)
    assert ctx.sweep_info()["kind"] == 4
    rows = np.repeat(np.arange(n), np.diff(rp.astype(np.int64))).astype(np.uint64)
    on_diag = col == rows
    rng = np.random.default_rng(12)
    specials = [(0.0, 3.0), (-0.0, 3.0), (5e-324, 0.5), (5e-324, 3.0), (-2.2250738585072014e-308, 3.0),
                (1.7976931348623157e308, 2.0), (1.7976931348623157e308, np.inf), (1.0, -np.inf),
                (2.0 ** -500, 2.0 ** 500), (2.0 ** 500, 2.0 ** -500), (1.0, 3.0), (-1.0, 3.0)]
    val = np.zeros(col.size)
    Y = torch_cuda.empty(n, dtype=torch_cuda.float64, device="cuda")
    X = torch_cuda.empty_like(Y)
    Mt = torch_cuda.empty(col.size, dtype=torch_cuda.float64, device="cuda")
    bad = 0
    for it in range(2000):
        if it % 2 == 0:
            a = _random_doubles(rng, n, -260, 260)
            b = _random_doubles(rng, n, -260, 260)
        else:  # large or small operands, quotient near 1
            ea = rng.integers(-1020, 1021, n)
            a = _random_doubles(rng, n, 0, 0) * np.exp2(ea.astype(np.float64))
            b = _random_doubles(rng, n, 0, 0) * np.exp2((ea + rng.integers(-20, 21, n)).clip(-1022, 1023))
        if it % 10 == 0:
            a[:len(specials)] = [p[0] for p in specials]
            b[:len(specials)] = [p[1] for p in specials]
        val[on_diag] = b
        Mt.copy_(torch_cuda.from_numpy(val))
        Y.copy_(torch_cuda.from_numpy(a))
        ctx.backsub_device(Mt, Y, X)
        got = X.cpu().numpy()
        want = a / b
        assert np.all(np.isfinite(want))
        bad += int(np.count_nonzero(got.view(np.uint64) != want.view(np.uint64)))
    assert bad == 0


def test_serial_sweep_limits(ctx):
    """Larger or shallow patterns keep the level-scheduled / structured kernels."""
    for dims, kind in (((5121, 1, 1), 2), ((20, 20, 20), 2), ((64, 8, 1), 2)):
        s = _box_system(dims)
        ctx.set_pattern(s.row_ptr, s.column_index)
        assert ctx.sweep_info()["kind"] == kind, dims


@pytest.mark.parametrize("dims,tiles,cluster", CLUSTER_CASES)
def test_clustered_sweeps_bit_exact(ctx, torch_cuda, oracle, dims, tiles, cluster):
    """Structured sweeps whose tiles run in thread-block clusters (faces
    through distributed shared memory) equal the oracle bit for bit."""
    s = W.hex_pprime(*dims)
    ctx.set_pattern(s.row_ptr, s.column_index)
    ctx.set_sweep_kernel(2, *tiles)
    ctx.set_sweep_cluster(*cluster)
    info = ctx.sweep_info()
    assert info["kind"] == 2 and info["tiles"] == tiles
    cx, cy = info["cluster"]
    assert 1 <= cx <= cluster[0] and 1 <= cy <= cluster[1]
    rng = np.random.default_rng(11)
    b = rng.standard_normal(s.n)
    Mh = oracle.ilu(s.row_ptr, s.column_index, s.value)
    M, B = dev(torch_cuda, Mh), dev(torch_cuda, b)
    Y, X = torch_cuda.empty_like(B), torch_cuda.empty_like(B)
    for _ in range(2):  # the tickets and counters of the first launches reset
        ctx.forsub_device(M, B, Y)
        y = oracle.forsub(s.row_ptr, s.column_index, Mh, b)
        assert np.array_equal(host(Y), y)
        ctx.backsub_device(M, Y, X)
        assert np.array_equal(host(X), oracle.backsub(s.row_ptr, s.column_index, Mh, y))


def test_cluster_shape_is_clipped(ctx):
    import opencslsolver_gb300 as ocsl

    s = W.hex_pprime(20, 20, 20)
    ctx.set_pattern(s.row_ptr, s.column_index)
    ctx.set_sweep_kernel(2, 16, 16)          # 2 x 2 tiles
    ctx.set_sweep_cluster(4, 4)
    assert ctx.sweep_info()["cluster"] == (2, 2)
    ctx.set_sweep_cluster(1, 1)
    assert ctx.sweep_info()["cluster"] == (1, 1)
    ctx.set_sweep_cluster(0, 0)                   # automatic: 4 tiles, no clusters
    assert ctx.sweep_info()["cluster"] == (1, 1)
    big = W.hex_pprime(40, 36, 33)                 # 16 x 8 tiles: 3 x 5, still below 64
    ctx.set_pattern(big.row_ptr, big.column_index)
    ctx.set_sweep_kernel(2, 8, 4)                 # 5 x 9 = 45 tiles
    assert ctx.sweep_info()["cluster"] == (1, 1)
    ctx.set_sweep_kernel(2, 4, 4)                 # 9 x 9 = 81 tiles: 2 x 4 clusters
    assert ctx.sweep_info()["cluster"] == (2, 4)
    for bad in [(0, 1), (1, 0), (4, 5), (17, 1)]:
        with pytest.raises(ocsl.OcslError):
            ctx.set_sweep_cluster(*bad)


def test_structured_kernel_refused_for_unstructured(ctx):
    s = W.tet_pprime(3)
    ctx.set_pattern(s.row_ptr, s.column_index)
    assert ctx.sweep_info()["kind"] == 1
    import opencslsolver_gb300 as ocsl

    with pytest.raises(ocsl.OcslError):
        ctx.set_sweep_kernel(2)


AXPY_CASES = [(1.0, 1.0), (-1.0, 1.0), (0.3, 1.0), (1.0, -1.0), (-1.0, -1.0), (0.3, -1.0),
              (0.3, 0.7), (2.5, None)]


@pytest.mark.parametrize("n", [1, 2047, 2048, 100003, 3_000_000])
def test_vector_routines_bit_exact(ctx, torch_cuda, oracle, n):
    """sum / ABSsum / product / axpy entry points against the oracle."""
    rng = np.random.default_rng(n)
    x, y = rng.standard_normal(n), rng.standard_normal(n)
    X, Y = dev(torch_cuda, x), dev(torch_cuda, y)
    assert ctx.sum_device(X) == oracle.sum(x)
    assert ctx.sum_device(X, absolute=True) == oracle.sum(x, absolute=True)
    O = torch_cuda.empty_like(X)
    ctx.product_device(X, Y, O)
    assert np.array_equal(host(O), oracle.product(x, y))
    for a, b in AXPY_CASES:
        if b is None:
            ctx.axpy_device(a, X, O)
            want = oracle.axpy(a, x)
        else:
            ctx.axpy_device(a, X, O, b, Y)
            want = oracle.axpy(a, x, b, y)
        assert np.array_equal(host(O), want), (a, b)
