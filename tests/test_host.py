"""CPU tests of the C-ABI library: it loads, exports every symbol include/ocsl.h
declares, refuses to run without a device (no CPU fallback), and its host-side
pattern analysis (validation + level schedules) behaves as documented."""
import ctypes as C

import numpy as np
import pytest

import opencslsolver_gb300 as ocsl
from opencslsolver_gb300 import _abi
from opencslsolver_gb300 import workloads as W


def test_library_exports_every_header_symbol(lib_built):
    names = _abi.header_symbols()
    assert len(names) >= 18
    missing = [n for n in names if not hasattr(lib_built, n)]
    assert not missing, missing
    assert set(_abi._PROTOS) == set(names), set(_abi._PROTOS) ^ set(names)


def test_version_and_status_strings(lib_built):
    assert b"sm_103a" in lib_built.ocsl_version()
    assert _abi.status_string(0) == "OCSL_OK"
    assert _abi.status_string(5) == "OCSL_TIMEOUT"
    assert _abi.status_string(99) == "OCSL_UNKNOWN"
    o = _abi.default_opts()
    assert o.tol == 1e-10 and o.ilu_sweeps == 3 and o.maxit > 0


def test_no_device_is_an_error_not_a_fallback(lib_built):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    assert lib_built.ocsl_create(C.byref(h), 0) == _abi.NO_DEVICE
    assert not h.value
    with pytest.raises(ocsl.OcslError):
        ocsl.Context(0)


def test_null_context_arguments(lib_built):
    assert lib_built.ocsl_destroy(None) == _abi.BAD_ARGUMENT
    assert lib_built.ocsl_set_pattern(None, 0, None, None) == _abi.BAD_ARGUMENT
    r = _abi.Result()
    assert lib_built.ocsl_solve(None, 0, None, None, None, None, C.byref(r)) == _abi.BAD_ARGUMENT


def test_hex_levels_and_counts():
    for nx, ny, nz in ((4, 4, 4), (7, 5, 3), (16, 1, 1)):
        rp, col = W.hex_pattern(nx, ny, nz)
        st, info = ocsl.check_pattern(rp, col)
        assert st == 0, info
        # natural ordering of a 7-point box: wavefronts i + j + k
        assert info["fw_levels"] == nx + ny + nz - 2
        assert info["bw_levels"] == nx + ny + nz - 2
        n = nx * ny * nz
        inner = max(nx - 2, 0) * max(ny - 2, 0) * max(nz - 2, 0)
        assert np.count_nonzero(col == W.PHANTOM) == n - inner
        assert info["nnz_real"] == col.size - (n - inner)


def _hex_counts(m):
    n = m**3
    real = n + 6 * m * m * (m - 1)      # diagonal + two entries per interior face
    return n, real, n - (m - 2) ** 3    # rows, real nonzeros, boundary rows (phantoms)


def test_config_scale_counts():
    """The 128^3 hex p' pattern has 2,097,152 rows, 14,581,760 real nonzeros and
    one phantom on each of the 128^3 - 126^3 boundary rows; the generator and
    the analysis reproduce the same formulas at 40^3 (the full size runs in the
    GPU suite)."""
    assert _hex_counts(128) == (2_097_152, 14_581_760, 96_776)
    rp, col = W.hex_pattern(40, 40, 40)
    n, real, phantoms = _hex_counts(40)
    assert rp.size - 1 == n and np.count_nonzero(col == W.PHANTOM) == phantoms
    st, info = ocsl.check_pattern(rp, col)
    assert st == 0 and info["nnz_real"] == real and info["fw_levels"] == 3 * 40 - 2


def test_reference_1d_pattern(golden_shocktube):
    z = golden_shocktube
    rp, col = W.pattern_1d(1000)
    assert np.array_equal(rp, z["row_ptr"]) and np.array_equal(col, z["column_index"])
    st, info = ocsl.check_pattern(rp, col)
    assert st == 0 and info["fw_levels"] == 1000 and info["nnz_real"] == 2998


def test_tet_pattern_valid():
    s = W.tet_pprime(3)
    st, info = ocsl.check_pattern(s.row_ptr, s.column_index)
    assert st == 0, info
    lens = np.diff(s.row_ptr.astype(np.int64))
    assert lens.min() >= 3 and lens.max() <= 6


def test_empty_pattern():
    st, info = ocsl.check_pattern(np.zeros(1, np.uint64), np.zeros(0, np.uint64))
    assert st == 0 and info["fw_levels"] == 0


@pytest.mark.parametrize("case", ["no_diag", "out_of_range", "unsorted", "rp_decreasing",
                                  "rp0", "phantom_before_diag"])
def test_bad_patterns_rejected(case):
    rp = np.array([0, 2, 4, 6], np.uint64)
    col = np.array([0, 1, 0, 1, 1, 2], np.uint64)
    if case == "no_diag":
        col = np.array([0, 1, 0, 2, 1, 2], np.uint64)  # row 1 lacks (1, 1)
        col[2:4] = [0, 2]
        col = np.array([0, 1, 0, 2, 1, 2], np.uint64)
    elif case == "out_of_range":
        col = np.array([0, 7, 0, 1, 1, 2], np.uint64)
    elif case == "unsorted":
        col = np.array([0, 1, 1, 0, 1, 2], np.uint64)  # row 1: (1, 0) after the diagonal
    elif case == "rp_decreasing":
        rp = np.array([0, 2, 1, 6], np.uint64)
    elif case == "rp0":
        rp = np.array([1, 2, 4, 6], np.uint64)
    elif case == "phantom_before_diag":
        col = np.array([0, 1, int(W.PHANTOM), 1, 1, 2], np.uint64)
    st, info = ocsl.check_pattern(rp, col)
    assert st == _abi.BAD_PATTERN and info["error"], (case, info)


def test_random_ragged_patterns_valid():
    for seed in range(5):
        s = W.random_rows_system(300, 12, seed=seed)
        st, info = ocsl.check_pattern(s.row_ptr, s.column_index)
        assert st == 0, info


def test_workload_properties():
    s = W.hex_pprime(8)
    n = s.n
    rows = np.repeat(np.arange(n), np.diff(s.row_ptr.astype(np.int64)))
    real = s.column_index != W.PHANTOM
    assert np.all(s.value[~real] == 0.0)
    diag = s.value[real & (s.column_index == rows.astype(np.uint64))]
    off = np.zeros(n)
    np.add.at(off, rows[real], np.abs(s.value[real]))
    off -= np.abs(diag)
    ratio = diag / off
    assert ratio.min() >= 1.01 - 1e-12 and ratio.max() <= 1.1 + 1e-12
    # Peclet scaling: max |F| / D == 10 by construction -> nonsymmetric
    import scipy.sparse as sp

    A = sp.csr_matrix((s.value[real], (rows[real], s.column_index[real].astype(np.int64))),
                      shape=(n, n))
    assert abs(A - A.T).max() > 0
    sym = W.hex_pprime(8, peclet=0.0)
    A = sp.csr_matrix((sym.value[real], (rows[real], sym.column_index[real].astype(np.int64))),
                      shape=(n, n))
    assert abs(A - A.T).max() == 0


def test_box_detection():
    for dims in ((4, 4, 4), (7, 5, 3), (16, 1, 1), (9, 6, 1), (2, 2, 2)):
        rp, col = W.hex_pattern(*dims)
        st, info = ocsl.check_pattern(rp, col)
        assert st == 0
        nx, ny, nz = dims
        want = (nx, ny, nz) if ny > 1 else (nx, 1, 1)
        if ny > 1 and nz == 1:
            want = (nx, ny, 1)
        assert info["box"] == want, (dims, info["box"])
    # the reference's 1D shock-tube pattern is a 1000 x 1 x 1 box
    rp, col = W.pattern_1d(1000)
    assert ocsl.check_pattern(rp, col)[1]["box"] == (1000, 1, 1)
    # unstructured patterns are not
    s = W.tet_pprime(3)
    assert ocsl.check_pattern(s.row_ptr, s.column_index)[1]["box"] == (0, 0, 0)
    s = W.random_rows_system(200, 8)
    assert ocsl.check_pattern(s.row_ptr, s.column_index)[1]["box"] == (0, 0, 0)
    # a box pattern with one stencil entry dropped is not a box
    rp, col = W.hex_pattern(5, 5, 5)
    rp2 = rp.copy()
    col2 = np.delete(col, int(rp[62]) + 1)  # row 62 loses an entry (sorted order kept)
    rp2[63:] -= 1
    st, info = ocsl.check_pattern(rp2, col2)
    assert st == 0 and info["box"] == (0, 0, 0)


def test_build_pattern_matches_reference_patterns(lib_built):
    """ocsl_build_pattern (O(n + faces)) reproduces the matrix structure the
    reference builds with insert_element (cfvm.cpp:74-98) on every recorded
    mesh: 1000-cell shock tube, 200-cell channel and steady cases, heat."""
    import assembly_cases as AC
    import opencslsolver_gb300 as ocsl

    for case in AC.CASES:
        c = AC.load(case)[0]
        rp, col = ocsl.build_pattern(c.n, c.left, c.right, c.bc_left)
        assert np.array_equal(rp, c.row_ptr) and np.array_equal(col, c.column_index), case


def test_build_pattern_hex_box_and_errors(lib_built):
    import opencslsolver_gb300 as ocsl

    f = W.hex_flow_state(9, 7, 5)
    rp, col = ocsl.build_pattern(f.n, f.left, f.right, f.bc_left)
    assert np.array_equal(rp, f.row_ptr) and np.array_equal(col, f.column_index)
    with pytest.raises(ocsl.OcslError):
        ocsl.build_pattern(f.n, f.left, np.full_like(f.right, f.n), f.bc_left)
    rp, col = ocsl.build_pattern(4, [], [], [])  # isolated cells: diagonal only
    assert rp.tolist() == [0, 1, 2, 3, 4] and col.tolist() == [0, 1, 2, 3]


def test_dot_noalloc_refuses_bad_pointers_before_any_cuda_call(lib_built):
    # null and misaligned pointers are refused on the host, so no kernel could
    # fault on them; this runs (and must pass) without a GPU
    L = lib_built
    buf = (C.c_double * 4)()
    base = C.addressof(buf)
    good = C.c_void_p(base)
    odd = C.c_void_p(base + 4)
    assert L.ocsl_dot_noalloc(4, None, good, good, None) == _abi.BAD_ARGUMENT
    assert b"null" in L.ocsl_noalloc_last_error()
    assert L.ocsl_dot_noalloc(4, good, good, None, None) == _abi.BAD_ARGUMENT
    for x, y, r in ((odd, good, good), (good, odd, good), (good, good, odd)):
        assert L.ocsl_dot_noalloc(4, x, y, r, None) == _abi.BAD_ARGUMENT
        assert b"aligned" in L.ocsl_noalloc_last_error()
    # with n = 0 the inputs are not read, only the result pointer is checked
    assert L.ocsl_dot_noalloc(0, odd, odd, odd, None) == _abi.BAD_ARGUMENT


def test_new_entry_points_refuse_null_handles(lib_built):
    """Host-side argument checks of the device-loop, batch-graph, SpMV-shape and
    VTK entry points: null handles are OCSL_BAD_ARGUMENT, before any CUDA call."""
    L = lib_built
    assert L.ocsl_set_device_loop(None, 1) == _abi.BAD_ARGUMENT
    assert L.ocsl_batch_set_graph(None, 1) == _abi.BAD_ARGUMENT
    assert L.ocsl_set_spmv_lanes(None, 4) == _abi.BAD_ARGUMENT
    lanes = C.c_int(-1)
    assert L.ocsl_spmv_lanes(None, C.byref(lanes)) == _abi.BAD_ARGUMENT
    us = C.c_double()
    assert L.ocsl_autotune_spmv_device(None, 0, None, C.byref(lanes), C.byref(us)) == \
        _abi.BAD_ARGUMENT
    err = C.create_string_buffer(64)
    assert L.ocsl_vtk_write(None, None, None, None, err, 64) == _abi.BAD_ARGUMENT
    assert b"null" in err.value
