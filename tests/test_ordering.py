"""The multicolour ordering on the host (ocsl_colour_pattern, no device):
the library's permutation against the numpy restatement in
tests/ordering_cases.py, and the property the ordering exists for -- the
permuted pattern's triangular sweeps have one level per colour."""
import numpy as np
import pytest

import opencslsolver_gb300 as ocsl
from opencslsolver_gb300 import workloads as W

import ordering_cases as OC


def _systems():
    return {"hex": W.hex_pprime(9, 7, 6), "tet": W.tet_pprime(4),
            "flow1d": W.System(*W.pattern_1d(40), None, None)}


@pytest.mark.parametrize("name", ["hex", "tet", "flow1d"])
def test_colouring_matches_restatement(name):
    s = _systems()[name]
    st, perm, colours, err = ocsl.colour_pattern(s.row_ptr, s.column_index)
    assert st == 0, err
    want, k = OC.colour_order(s.row_ptr, s.column_index)
    assert np.array_equal(perm, want) and colours == k
    assert np.array_equal(np.sort(perm), np.arange(perm.size))
    if name in ("hex", "flow1d"):
        assert colours == 2  # the parity colouring of a box / chain


@pytest.mark.parametrize("name", ["hex", "tet", "flow1d"])
def test_permuted_pattern_sweeps_one_level_per_colour(name):
    s = _systems()[name]
    _, perm, colours, _ = ocsl.colour_pattern(s.row_ptr, s.column_index)
    rp, col, slot = OC.permuted_pattern(s.row_ptr, s.column_index, perm)
    assert np.array_equal(np.sort(slot), np.arange(np.asarray(s.column_index).size))
    st, info = ocsl.check_pattern(rp, col)
    assert st == 0, info["error"]
    assert info["fw_levels"] == colours and info["bw_levels"] == colours
    st, natural = ocsl.check_pattern(s.row_ptr, s.column_index)
    assert natural["fw_levels"] > colours


def test_colouring_rejects_unsymmetric_and_bad_patterns():
    PH = ocsl.PHANTOM
    # entry (0, 1) without (1, 0): rows 0 and 1 would share colour 0
    rp = np.array([0, 2, 3, 4], dtype=np.uint64)
    col = np.array([0, 1, 1, 2], dtype=np.uint64)
    st, _, _, err = ocsl.colour_pattern(rp, col)
    assert st == 4 and "symmetric" in err
    # no diagonal in row 1: rejected by the pattern check first
    col = np.array([0, 1, 0, 2], dtype=np.uint64)
    st, _, _, err = ocsl.colour_pattern(np.array([0, 2, 3, 4], dtype=np.uint64), col)
    assert st == 4 and "diagonal" in err
    # phantom columns are not neighbours
    rp = np.array([0, 2, 4], dtype=np.uint64)
    col = np.array([0, PH, 1, PH], dtype=np.uint64)
    st, perm, colours, _ = ocsl.colour_pattern(rp, col)
    assert st == 0 and colours == 1 and list(perm) == [0, 1]
