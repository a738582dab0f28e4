"""The oracle's SIMPLE inner iteration (oracle/ocsl_oracle_flow.c) against the
reference's own recorded runs (tests/golden/flow_<case>.npz): the 1000-cell
inviscid shock tube (walls, empty sides), the 200-cell viscous channel
(velocity inlet, no-slip walls, pressure outlet; transient, upwind) and the
200-cell viscous steady case (supersonic inlet, slip walls, pressure outlet;
implicit under-relaxation ramp, blended) and a 3D viscous channel on a
240-cell jittered hex mesh the reference read from an SU2 file (velocity
inlet with transverse components, no-slip walls, outlet; blended).

* Stages: each recorded inner iteration is replayed from the reference's
  state before it, with the reference's own solutions in place of the five
  solves; the assembled systems and every field the iteration writes must
  agree to a few ulps.  The remaining differences are contraction choices
  the reference's -ffast-math build makes per expression.
* Trajectory: the whole recorded run with the oracle's own
  reference-faithful solves (CG_solve / ILU_BICGSTAB_solve restated,
  tile-order dot products) against the reference's final fields: the state
  (p, u, T, rho, h, mass fluxes) within 1e-12 relative, every field within
  1e-8 -- pressure gradients, p' and the cell mass balance are differences
  of nearly equal pressures (measured at most 5.2e-9 on the channel).
"""
import numpy as np
import pytest

from opencslsolver_gb300 import _abi
from oracle import oracle as orc

import flow_cases as FC

STAGE_TOL = 1e-14
STATE = ("velocity", "pressure", "temperature", "density_c", "enthalpy", "mdot", "density",
         "bc_mdot", "bc_density", "bc_enthalpy", "bc_temperature", "bc_velocity", "bc_pressure")

_golden = {}


def golden(case):
    if case not in _golden:
        _golden[case] = FC.Golden(case)
    return _golden[case]


def _end_step(c):
    FC.end_step(c, orc.flow_end_step)


@pytest.mark.parametrize("case,tag", [(c, t) for c in FC.CASES for t in FC.ITERATIONS[c]])
def test_oracle_iteration_stages_match_reference(oracle, case, tag):
    g = golden(case)
    c = g.start_case(tag, _end_step)
    sy = g.systems(tag)
    r = orc.flow_iterate(c, [_abi.BICGSTAB_REF] * 3, given_x=list(sy["x"]), capture=True)
    for key in ("value", "b", "x0"):
        for e in range(5):
            err = FC.relerr(r[key][e], sy[key][e])
            assert err <= STAGE_TOL, (case, tag, key, e, err)
    post = g.record(f"post_{tag}")
    errs = FC.field_errors(FC.written(c), FC.recorded(g.setup, post))
    assert max(errs.values()) <= STAGE_TOL, (case, tag, errs)
    if tag == "0_0":
        assert np.array_equal(r["x0"], sy["x0"])
    # the residual sums: tile order here, serial in the reference
    res = post["residuals"]
    for k in (0, 3, 4):
        assert abs(r["residual"][k] - res[k]) <= 1e-13 * abs(res[k]), (case, tag, k)


@pytest.mark.parametrize("case,mode", [("shocktube", "bicg"), ("shocktube", "cg"),
                                       ("channel", "bicg"), ("steady", "bicg"),
                                       ("box3d", "bicg")])
def test_oracle_trajectory_matches_reference(oracle, case, mode):
    g = golden(case)
    c = g.case()
    momentum = _abi.CG_REF if mode == "cg" else _abi.BICGSTAB_REF
    methods = [momentum, _abi.BICGSTAB_REF, _abi.BICGSTAB_REF]
    for _ in range(g.steps):
        for _ in range(g.inner):
            orc.flow_iterate(c, methods)
        _end_step(c)
    errs = FC.field_errors(FC.written(c), FC.recorded(g.setup, g.record(f"final_{mode}")))
    print(case, mode, {k: f"{v:.1e}" for k, v in errs.items() if v})
    for k in STATE:
        assert errs[k] <= 1e-12, (case, k, errs)
    assert max(errs.values()) <= 1e-8, errs


def test_steady_ramp_follows_reference(oracle):
    """The host-side under-relaxation ramp of update_timestep reproduces the
    values the reference used step by step."""
    g = golden("steady")
    c = g.case()
    for _ in range(10):
        _end_step(c)
    assert c["eq"]["implicit_underrelaxation"] == float(g._z["relax_10_0"][0])


def test_oracle_iteration_rejects_other_methods(oracle):
    c = golden("shocktube").case()
    with pytest.raises(ValueError):
        orc.flow_iterate(c, [_abi.ILU_BICGSTAB_IR32] * 3)
