"""The initial flow state of opencslsolver_gb300.flow.initial_state against
the state the reference wrote right after CFlow_solver::initialize
(cflow_solver.cpp:33-195) for its four recorded cases (setup records of
tests/golden/flow_<case>.npz): cells, boundary faces of every kind and the
first face and boundary mass fluxes, to a few ulps (numpy here, -ffast-math
there); boundary kinds, wall kinds and supersonic flags exactly."""
import numpy as np
import pytest

from opencslsolver_gb300 import _abi
from opencslsolver_gb300 import flow as F

import flow_cases as FC


@pytest.mark.parametrize("case", FC.CASES)
def test_initial_state_matches_reference(case):
    g = FC.Golden(case)
    c = F.initial_state(FC.mesh_from_setup(g.setup), **FC.CONFIGS[case])
    want = FC.make_case(g.setup, g.setup)
    walls = want["state"]["bc_type"] == _abi.BC_WALL
    for group in ("state", "arrays"):
        for k, w in want[group].items():
            got = c[group][k]
            if k in ("bc_wall", "bc_thermal"):
                assert np.array_equal(got[walls], w[walls]), (case, k)
            elif k in _abi.INT_FIELDS:
                assert np.array_equal(got, w), (case, k)
            else:
                assert got.shape == w.shape, (case, k)
                err = FC.relerr(got, w)
                assert err <= 1e-14, (case, k, err)
    for k in ("viscous", "blended", "transient"):
        assert c["eq"][k] == want["eq"][k], (case, k)
    assert c["eq"]["R_specific"] == want["eq"]["R_specific"]
    assert c["constants"] == pytest.approx(want["constants"], rel=0, abs=0)
