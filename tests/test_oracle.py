"""Pins the CPU oracle against the reference's own golden vectors.

The fixtures under tests/golden/ were produced by the reference itself
(tests/golden/make_golden.py): its solver unit-test system, solve calls
captured from its SIMPLE loop on the 1000-cell shock tube, and seeded small
systems with the outputs of gemv, ILU_decompose, ILU_forsub/backsub,
CG_solve and ILU_BICGSTAB_solve.  The reference was compiled with its own
-O3 -ffast-math -march=native, so its rounding can differ from the oracle's
explicit one in the last bits: tolerances here are relative and tight.
"""
import math

import numpy as np
import pytest

from opencslsolver_gb300 import workloads as W


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    den = max(np.max(np.abs(b)), 1e-300)
    return float(np.max(np.abs(a - b)) / den) if a.size else 0.0


def test_kat_matches_reference_unit_tests(oracle, golden_kat):
    """cmatrix_solver_supply.h:29-114, values recorded from the reference."""
    z = golden_kat
    x, res, it = oracle.cg_ref(z["row_ptr"], z["column_index"], z["value"], z["b"], z["x0"])
    assert it == 4
    assert abs(res - float(z["cg_res"])) <= 1e-12 * abs(float(z["cg_res"]))
    assert rel(x, z["cg_x"]) <= 1e-14
    x, res, it = oracle.bicgstab_ref(z["row_ptr"], z["column_index"], z["value"], z["b"], z["x0"])
    assert it == 3
    assert abs(res - float(z["bicg_res"])) <= 1e-9 * abs(float(z["bicg_res"]))
    assert rel(x, z["bicg_x"]) <= 1e-14
    # the printed values of the reference's own run
    assert f"{float(z['cg_res']):.6g}" == "6.08031e-06"
    assert f"{float(z['bicg_res']):.6e}"[:6] == "3.3577"


def test_shocktube_calls_match_reference(oracle, golden_shocktube):
    z = golden_shocktube
    rp, col = z["row_ptr"], z["column_index"]
    assert rp.size - 1 == 1000 and np.count_nonzero(col == W.PHANTOM) == 1000
    for k in range(z["meta"].shape[0]):
        eq = int(z["meta"][k, 2])
        fn = oracle.cg_ref if eq < 3 else oracle.bicgstab_ref
        x, res, _ = fn(rp, col, z["value"][k], z["b"][k], z["x0"][k])
        assert rel(x, z["x"][k]) <= 1e-12, (k, eq)
        ref_res = float(z["residual"][k])
        # below ~1e-26 (relative, squared) a residual is round-off noise
        floor = 1e-26 * (float(np.dot(z["b"][k], z["b"][k])) if eq < 3 else 1.0)
        assert abs(res - ref_res) <= 1e-6 * abs(ref_res) + floor, (k, eq, res, ref_res)


@pytest.mark.parametrize("k", range(5))
def test_small_systems_match_reference(oracle, golden_small, k):
    c = golden_small[k]
    rp, col, val = c["row_ptr"], c["column_index"], c["value"]
    assert rel(oracle.gemv(rp, col, val, c["xin"]), c["gemv0"]) <= 1e-15
    assert rel(oracle.gemv(rp, col, val, c["xin"], 1, 0.0, c["z"]), c["gemv1"]) <= 1e-15
    assert rel(oracle.gemv(rp, col, val, c["xin"], 2, -0.37, c["z"]), c["gemv2"]) <= 1e-15
    M = oracle.ilu(rp, col, val)
    assert rel(M, c["ilu"]) <= 1e-15
    assert rel(oracle.forsub(rp, col, c["ilu"], c["z"]), c["forsub"]) <= 1e-14
    assert rel(oracle.backsub(rp, col, c["ilu"], c["z"]), c["backsub"]) <= 1e-14
    x, res, _ = oracle.cg_ref(rp, col, val, c["b"], c["x0"])
    assert rel(x, c["cg_x"]) <= 1e-12
    assert abs(res - float(c["cg_res"])) <= 1e-9 * abs(float(c["cg_res"]))
    x, res, _ = oracle.bicgstab_ref(rp, col, val, c["b"], c["x0"])
    assert rel(x, c["bicg_x"]) <= 1e-10
    assert abs(res - float(c["bicg_res"])) <= 1e-8 * abs(float(c["bicg_res"]))


def test_dot_orders(oracle):
    rng = np.random.default_rng(3)
    for n in (0, 1, 255, 2048, 2049, 100_003):
        x, y = rng.standard_normal(n), rng.standard_normal(n)
        exact = math.fsum(x * y) if n else 0.0
        assert abs(oracle.dot(x, y) - exact) <= 1e-13 * (np.abs(x * y).sum() + 1e-300)
        assert abs(oracle.dot_seq(x, y) - exact) <= 1e-12 * (np.abs(x * y).sum() + 1e-300)


def test_oracle_thread_count_invariant(oracle):
    s = W.hex_pprime(10)
    outs = []
    for t in (1, 4):
        oracle.set_threads(t)
        outs.append(oracle.bicgstab_ref(s.row_ptr, s.column_index, s.value, s.b, np.zeros(s.n)))
    oracle.set_threads(1)
    assert np.array_equal(outs[0][0], outs[1][0]) and outs[0][1] == outs[1][1]


@pytest.mark.parametrize("gen", ["hex", "hex_sym", "tet", "random"])
def test_tolerance_mode_oracle_converges(oracle, gen):
    s = {"hex": lambda: W.hex_pprime(10), "hex_sym": lambda: W.hex_pprime(10, peclet=0.0),
         "tet": lambda: W.tet_pprime(4), "random": lambda: W.random_rows_system(400, 8)}[gen]()
    x0 = np.zeros(s.n)
    x, rc, it, rr = oracle.bicgstab_tol(s.row_ptr, s.column_index, s.value, s.b, x0, tol=1e-10)
    assert rc == 0 and rr <= 1e-10 and it > 0
    x2, rc, it2, out, rr2 = oracle.bicgstab_ir32(s.row_ptr, s.column_index, s.value, s.b, x0,
                                                 tol=1e-10)
    assert rc == 0 and rr2 <= 1e-10 and out >= 1
    assert rel(x2, x) <= 1e-8
    if gen == "hex_sym":
        x3, rc, it3, rr3 = oracle.pcg_tol(s.row_ptr, s.column_index, s.value, s.b, x0, tol=1e-10)
        assert rc == 0 and rr3 <= 1e-10
        assert rel(x3, x) <= 1e-8


def test_live_reference_agrees_with_oracle(oracle, reference):
    """Where the reference was built here: random ragged systems, 1 thread."""
    for seed in range(3):
        s = W.random_rows_system(150, 7, seed=100 + seed)
        x0 = np.zeros(s.n)
        xr, rr = reference.bicgstab_solve(s.row_ptr, s.column_index, s.value, s.b, x0)
        xo, ro, _ = oracle.bicgstab_ref(s.row_ptr, s.column_index, s.value, s.b, x0)
        assert rel(xo, xr) <= 1e-11
        xr, rr = reference.cg_solve(s.row_ptr, s.column_index, s.value, s.b, x0)
        xo, ro, _ = oracle.cg_ref(s.row_ptr, s.column_index, s.value, s.b, x0)
        assert rel(xo, xr) <= 1e-12


AXPY_CASES = [(1.0, 1.0), (-1.0, 1.0), (0.3, 1.0), (1.0, -1.0), (-1.0, -1.0), (0.3, -1.0),
              (0.3, 0.7), (2.5, None)]


def test_vector_routines_match_reference(oracle, reference):
    """sum / ABSsum / product / axpy (cmatrix_solver.cpp:244-335) against the
    reference built from its sources: elementwise results bit for bit (every
    axpy branch), sums to the reordering bound (the reference adds in index
    order, the oracle in tile order)."""
    rng = np.random.default_rng(1)
    for n in (0, 1, 1000, 5000, 100003):
        x, y = rng.standard_normal(n), rng.standard_normal(n)
        for absolute in (False, True):
            so, sr = oracle.sum(x, absolute), reference.sum(x, absolute)
            assert abs(so - sr) <= 1e-12 * max(np.sum(np.abs(x)), 1e-300)
        assert np.array_equal(oracle.product(x, y), reference.product(x, y))
        for a, b in AXPY_CASES:
            yy = None if b is None else y
            bb = 0.0 if b is None else b
            assert np.array_equal(oracle.axpy(a, x, bb, yy), reference.axpy(a, x, bb, yy)), (a, b)


def test_tile_order_sum_is_exact_on_integers(oracle):
    x = np.arange(-5000, 7001, dtype=np.float64)
    assert oracle.sum(x) == float(x.sum())
    assert oracle.sum(x, absolute=True) == float(np.abs(x).sum())
