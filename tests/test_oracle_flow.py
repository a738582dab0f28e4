"""The oracle's SIMPLE inner iteration (oracle/ocsl_oracle_flow.c) against the
reference's own recorded shock-tube run (tests/golden/flow_shocktube.npz).

* Stages: each recorded inner iteration is replayed from the reference's
  state before it, with the reference's own solutions in place of the five
  solves; the assembled systems and every field the iteration writes must
  agree to a few ulps (the first iteration bit for bit).  The remaining
  differences are the face-loop assembly's contraction choices, which the
  reference's -ffast-math build makes per expression.
* Trajectory: 200 time steps x 5 inner iterations with the oracle's own
  reference-faithful solves (CG_solve / ILU_BICGSTAB_solve restated, tile-order
  dot products) against the reference's final fields, for both solver
  choices of the recorder: every field within 1e-11 relative (the parity bar
  for fields is 1e-9).
"""
import numpy as np
import pytest

from opencslsolver_gb300 import _abi
from oracle import oracle as orc

import flow_cases as FC

STAGE_TOL = 1e-14


@pytest.fixture(scope="module")
def golden():
    return FC.Golden()


@pytest.mark.parametrize("tag", FC.ITERATIONS)
def test_oracle_iteration_stages_match_reference(oracle, golden, tag):
    case = golden.case(golden.start(tag))
    sy = golden.systems(tag)
    r = orc.flow_iterate(case, [_abi.BICGSTAB_REF] * 3, given_x=list(sy["x"]), capture=True)
    for key in ("value", "b", "x0"):
        for e in range(5):
            err = FC.relerr(r[key][e], sy[key][e])
            assert err <= STAGE_TOL, (tag, key, e, err)
    post = golden.record(f"post_{tag}")
    errs = FC.field_errors(FC.written(case), FC.recorded(golden.setup, post))
    assert max(errs.values()) <= STAGE_TOL, (tag, errs)
    if tag == "0_0":
        assert all(v == 0.0 for v in errs.values()), errs
        assert np.array_equal(r["x0"], sy["x0"])
    # the residual sums: tile order here, serial in the reference
    res = post["residuals"]
    for k in (0, 3, 4):
        assert abs(r["residual"][k] - res[k]) <= 1e-13 * abs(res[k]), (tag, k, r["residual"], res)


@pytest.mark.parametrize("mode", ["bicg", "cg"])
def test_oracle_trajectory_matches_reference(oracle, golden, mode):
    case = golden.case()
    momentum = _abi.CG_REF if mode == "cg" else _abi.BICGSTAB_REF
    methods = [momentum, _abi.BICGSTAB_REF, _abi.BICGSTAB_REF]
    for _ in range(FC.STEPS):
        for _ in range(FC.INNER):
            orc.flow_iterate(case, methods)
        orc.flow_end_step(case)
    errs = FC.field_errors(FC.written(case), FC.recorded(golden.setup, golden.record(f"final_{mode}")))
    print(mode, {k: f"{v:.1e}" for k, v in errs.items()})
    assert max(errs.values()) <= 1e-11, errs


def test_oracle_iteration_rejects_other_methods(oracle, golden):
    case = golden.case()
    with pytest.raises(ValueError):
        orc.flow_iterate(case, [_abi.ILU_BICGSTAB_IR32] * 3)
