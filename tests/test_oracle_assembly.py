"""The oracle's face-loop assembly against the reference's own assembled
systems (recorded from its SIMPLE loop on one thread, tests/golden/assembly_*):
matrix values, b, x0 and the side outputs ap_vec / total_mdot.

The reference is compiled with -ffast-math; the oracle fixes one contraction
choice per expression, so entries agree to a few ulps rather than bitwise.
"""
import numpy as np
import pytest

from oracle import oracle as orc

import assembly_cases as AC


def relerr(a, b):
    scale = max(float(np.max(np.abs(b))), 1e-300)
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b)))) / scale


@pytest.mark.parametrize("case", AC.CASES)
def test_oracle_assembly_matches_reference(oracle, case):
    for c in AC.load(case):
        value, b, x0, ap, tm = orc.assemble(c.row_ptr, c.column_index, c.left, c.right,
                                            c.bc_left, c.eq, c.state)
        assert relerr(value, c.value) <= 1e-14, (case, c.name, relerr(value, c.value))
        assert relerr(b, c.b) <= 1e-13, (case, c.name, relerr(b, c.b))
        assert np.array_equal(x0, c.x0), (case, c.name)
        phantom = c.column_index >= np.uint64(c.n)
        assert np.all(value[phantom] == 0.0)
        if c.eq["equation"] == 0 and c.ap_vec is not None:
            assert relerr(ap, c.ap_expected) <= 1e-14
        if c.eq["equation"] == 1 and c.total_mdot is not None:
            assert relerr(tm, c.total_mdot) <= 1e-14


def test_assembly_cases_cover_the_boundary_kinds():
    kinds = set()
    for case in AC.CASES:
        if case == "heat":
            continue
        for c in AC.load(case):
            kinds |= set(np.unique(c.state["bc_type"]).tolist())
            if c.eq["equation"] == 0 and c.eq["viscous"]:
                assert (c.state["bc_wall"][c.state["bc_type"] == 2] >= 0).all()
        if c.name == "heat":
            continue
    kinds.discard(None)
    assert kinds == {0, 2, 3, 4, 5}  # empty, wall, velocity inlet, supersonic inlet, outlet


def test_bc_value_gradient_is_linear_in_b(oracle):
    """dL/d(bc_value) = lambda_P * D: the change of b when the Dirichlet values
    of the pressure-correction faces move, contracted with lambda."""
    c = [c for c in AC.load("steady") if c.name == "pressure"][0]
    rng = np.random.default_rng(2)
    lam = rng.standard_normal(c.n)
    g = orc.bc_value_grad(c.row_ptr, c.bc_left, c.eq, c.state, lam)
    nb = c.bc_left.size
    st0 = dict(c.state, bc_value=np.zeros(nb))
    _, b0, _, _, _ = orc.assemble(c.row_ptr, c.column_index, c.left, c.right, c.bc_left, c.eq, st0)
    hit = np.nonzero(g)[0]
    assert hit.size > 0
    for k in hit[:4]:
        v = np.zeros(nb)
        v[k] = 1.0
        _, b1, _, _, _ = orc.assemble(c.row_ptr, c.column_index, c.left, c.right, c.bc_left,
                                      c.eq, dict(c.state, bc_value=v))
        assert np.isclose(float(np.dot(lam, b1 - b0)), g[k], rtol=1e-12, atol=0)
