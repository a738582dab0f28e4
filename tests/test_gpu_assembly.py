"""The GPU face-loop assembly through the C ABI, on the systems recorded from
the reference's own SIMPLE loop (tests/golden/assembly_*.npz):

* bit-identical to the oracle restatement (same summation order, same
  contraction choices) -- values, b, x0, ap and total_mdot;
* within a few ulps of the reference's assembled systems (the reference is
  compiled with -ffast-math and uses pow(T, 1.5));
* the adjoint of the p' boundary values equals the oracle's;
* argument checking: faces before pattern, pairs missing from the pattern,
  NULL state fields.
"""
import numpy as np
import pytest

import opencslsolver_gb300 as ocsl
from opencslsolver_gb300 import _abi
from oracle import oracle as orc

import assembly_cases as AC

pytestmark = pytest.mark.gpu


to_device = AC.to_device


def relerr(a, b):
    scale = max(float(np.max(np.abs(b))), 1e-300)
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b)))) / scale


@pytest.mark.parametrize("case", AC.CASES)
def test_assembly_bit_exact_vs_oracle_and_close_to_reference(ctx, torch_cuda, case):
    torch = torch_cuda
    calls = AC.load(case)
    c0 = calls[0]
    ctx.set_pattern(c0.row_ptr, c0.column_index)
    ctx.set_faces(c0.left, c0.right, c0.bc_left)
    n, nnz = c0.n, c0.column_index.size
    for c in calls:
        st = to_device(torch, c.state)
        value = torch.full((nnz,), np.nan, dtype=torch.float64, device="cuda")
        b, x0, ap, tm = (torch.full((n,), np.nan, dtype=torch.float64, device="cuda")
                         for _ in range(4))
        ctx.assemble_device(c.eq, st, value, b, x0, ap, tm)
        v, bb, xx, aa, mm = (t.cpu().numpy() for t in (value, b, x0, ap, tm))
        ov, ob, ox, oa, om = orc.assemble(c.row_ptr, c.column_index, c.left, c.right, c.bc_left,
                                          c.eq, c.state)
        for got, want, what in ((v, ov, "value"), (bb, ob, "b"), (xx, ox, "x0"), (aa, oa, "ap"),
                                (mm, om, "total_mdot")):
            assert np.array_equal(got, want), (case, c.name, what)
        assert relerr(v, c.value) <= 1e-14, (case, c.name)
        assert relerr(bb, c.b) <= 1e-13, (case, c.name)
        assert np.array_equal(xx, c.x0)


def test_bc_value_gradient_matches_oracle(ctx, torch_cuda):
    torch = torch_cuda
    for case in ("steady", "channel"):
        c = [c for c in AC.load(case) if c.name == "pressure"][0]
        ctx.set_pattern(c.row_ptr, c.column_index)
        ctx.set_faces(c.left, c.right, c.bc_left)
        lam = np.random.default_rng(9).standard_normal(c.n)
        st = to_device(torch, c.state)
        g = torch.full((c.bc_left.size,), np.nan, dtype=torch.float64, device="cuda")
        ctx.bc_value_grad_device(c.eq, st, torch.from_numpy(lam).cuda(), g)
        want = orc.bc_value_grad(c.row_ptr, c.bc_left, c.eq, c.state, lam)
        assert np.array_equal(g.cpu().numpy(), want)


def test_assembly_argument_errors(ctx, torch_cuda):
    torch = torch_cuda
    c = AC.load("channel")[0]
    with pytest.raises(ocsl.OcslError) as e:
        ctx.set_faces(c.left, c.right, c.bc_left)
    assert e.value.status == _abi.NO_PATTERN
    ctx.set_pattern(c.row_ptr, c.column_index)
    st = to_device(torch, c.state)
    out = [torch.zeros(c.column_index.size, dtype=torch.float64, device="cuda")] + [
        torch.zeros(c.n, dtype=torch.float64, device="cuda") for _ in range(2)]
    with pytest.raises(ocsl.OcslError) as e:  # faces not set yet
        ctx.assemble_device(c.eq, st, *out)
    assert "set_faces" in str(e.value)
    bad_right = c.right.copy()
    bad_right[3] = (c.left[3] + 7) % c.n  # a pair the pattern does not store
    with pytest.raises(ocsl.OcslError) as e:
        ctx.set_faces(c.left, bad_right, c.bc_left)
    assert e.value.status == _abi.BAD_ARGUMENT
    ctx.set_faces(c.left, c.right, c.bc_left)
    st.pop("velocity")
    with pytest.raises(ocsl.OcslError) as e:
        ctx.assemble_device(c.eq, st, *out)
    assert "velocity" in str(e.value)
