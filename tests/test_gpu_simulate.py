"""The simulator action through the C ABI (cafe_simulate) against the
compiled reference's simulate_processes (tests/golden/ref_simulations.json):
with the same seed and root sizes the simulated families must be the
reference's. The draws use the GPU-built transition matrices, which agree
with the reference's to ~1e-12 relative, so a draw could only differ if its
uniform variate fell within ~1e-12 of a cumulative-probability boundary;
the test requires every size to be equal."""
import numpy as np
import pytest

from golden_cases import load_simulation_cases

pytestmark = pytest.mark.gpu

CASES = load_simulation_cases()


@pytest.fixture(scope="module")
def ctx():
    from cafe5_gb300.engine import Context
    c = Context()
    yield c
    c.close()


@pytest.mark.parametrize("case", CASES, ids=[c.name for c in CASES])
def test_simulation_matches_reference(ctx, case):
    from cafe5_gb300.inputs import discrete_gamma
    tid = ctx.upload_tree(case.tree, case.lambda_of_node)
    sid = ctx.upload_families(tid, np.zeros((1, len(case.tree.leaves)), np.int32))
    kw = dict(S=case.S, R=case.R, seed=case.seed, lambda_kind=case.lambda_kind)
    if case.K:
        probs, mult = discrete_gamma(case.alpha, case.K)
        kw.update(model=1, multipliers=mult, cat_probs=probs)
    if case.err is not None:
        ctx.set_error_model(case.err.table())
        kw.update(use_error_model=True)
    else:
        ctx.set_error_model(None)
    sizes, lam = ctx.simulate(tid, sid, case.lambdas, case.roots, **kw)
    assert np.array_equal(sizes, case.sizes)
    assert np.array_equal(lam, case.lambda_used)


def test_simulation_error_model_bound_is_enforced(ctx):
    """A leaf size past the error model's rows is an error (the reference
    throws)."""
    from cafe5_gb300._lib import CafeError
    case = [c for c in CASES if c.err is not None][0]
    tid = ctx.upload_tree(case.tree, case.lambda_of_node)
    sid = ctx.upload_families(tid, np.zeros((1, len(case.tree.leaves)), np.int32))
    ctx.set_error_model(np.array([[0.0, 0.95, 0.05], [0.05, 0.9, 0.05]]))
    with pytest.raises(CafeError) as e:
        ctx.simulate(tid, sid, case.lambdas, [6] * 10, S=case.S, R=case.R, seed=1, lambda_kind=case.lambda_kind,
                     use_error_model=True)
    assert e.value.code == 6
    ctx.set_error_model(None)
