"""GPU parameter search through the library (cafe_optimize) against the
reference's own searches (optimizer scorers + fminsearch_min, committed in
tests/golden/ref_optimizer.json).

Every vertex the search proposes is computed from earlier vertices by the
same host arithmetic as the reference, so the two searches take identical
steps as long as every comparison of two scores comes out the same. The
FP64 path agrees with the reference's -lnL to 1e-10 relative, far below the
gaps the simplex compares, so the bar is: the same iteration and
evaluation counts, the same best point bit for bit, and the best -lnL
within 1e-10 relative."""
import numpy as np
import pytest

from golden_cases import load_searches, prior_from_spec

pytestmark = pytest.mark.gpu

SEARCHES = load_searches()


@pytest.fixture(scope="module")
def ctx():
    from cafe5_gb300.engine import Context
    c = Context()
    yield c
    c.close()


def build(ctx, raw, case):
    from cafe5_gb300 import engine
    from cafe5_gb300.families import FamilySet
    from cafe5_gb300.inputs import ErrorModel
    from cafe5_gb300.tree import parse_newick
    fams = FamilySet(raw["ids"], case.counts)
    if raw["lambda_newick"]:
        lam = engine.MultipleLambda(parse_newick(raw["lambda_newick"], lambda_tree=True), case.lambdas)
    else:
        lam = engine.SingleLambda(case.lambdas[0])
    em = ErrorModel.parse(raw["error_model"]) if raw["error_model"] else None
    prior = prior_from_spec(raw["prior"], case.R)
    if raw["model"] == "gamma":
        model = engine.GammaModel(lam, case.tree, fams, case.S, case.R, n_gamma_cats=raw["K"],
                                  fixed_alpha=raw["alpha"], error_model=em, ctx=ctx)
    else:
        model = engine.BaseModel(lam, case.tree, fams, case.S, case.R, error_model=em, ctx=ctx)
    longest = max(case.tree.branch_length[v] for v in range(case.tree.n_nodes) if case.tree.parent[v] >= 0)
    kind = raw["optimize"]
    if kind == "lambda":
        sc = engine.LambdaOptimizerScorer(lam, model, prior, longest)
    elif kind == "alpha":
        sc = engine.GammaOptimizerScorer(lam, model, prior)
    elif kind == "lambda_alpha":
        sc = engine.GammaLambdaOptimizerScorer(lam, model, prior, longest)
    else:
        sc = engine.LambdaEpsilonOptimizerScorer(lam, model, prior, longest, em)
    return model, sc


@pytest.mark.parametrize("raw,case", SEARCHES, ids=[c.name for _, c in SEARCHES])
def test_search_matches_reference(ctx, raw, case):
    from cafe5_gb300 import engine
    model, sc = build(ctx, raw, case)
    ref = raw["search"]
    initial = [float.fromhex(x) for x in raw["initial"]]
    first = sc.calculate_score(initial)
    assert abs(first - float.fromhex(ref["first_hex"])) <= 1e-10 * abs(first)
    r = engine.Optimizer(sc).optimize(initial=initial)
    assert r.num_iterations == ref["iters"]
    assert r.evaluations == ref["evals"]      # both count the initial-point check
    assert [v.hex() for v in r.values] == [float.fromhex(h).hex() for h in ref["best_hex"]]
    ref_score = float.fromhex(ref["score_hex"])
    assert abs(r.score - ref_score) <= 1e-10 * abs(ref_score)
    assert r.converged
    # the scorer's finalize leaves the model at the optimum
    sc.finalize(r.values)
    again = model.infer_family_likelihoods(sc.prior, sc.lam)
    assert abs(again - ref_score) <= 1e-10 * abs(ref_score)


def test_search_in_mixed_precision_lands_on_the_same_optimum(ctx):
    """The tensor-core path changes -lnL by < 1e-6 relative; the search it
    drives ends within the simplex tolerance of the FP64 optimum."""
    from cafe5_gb300 import engine
    raw, case = [s for s in SEARCHES if s[1].name == "opt_lambda_alpha_gamma_24taxa"][0]
    model, sc = build(ctx, raw, case)
    model.precision = "mixed_tf32x3"
    initial = [float.fromhex(x) for x in raw["initial"]]
    r = engine.Optimizer(sc).optimize(initial=initial)
    ref_best = [float.fromhex(h) for h in raw["search"]["best_hex"]]
    ref_score = float.fromhex(raw["search"]["score_hex"])
    assert abs(r.score - ref_score) <= 1e-6 * abs(ref_score)
    assert np.allclose(r.values, ref_best, rtol=2e-3)


def test_search_refuses_an_infinite_start(ctx):
    from cafe5_gb300 import engine
    from cafe5_gb300._lib import CafeError
    raw, case = SEARCHES[0]
    model, sc = build(ctx, raw, case)
    with pytest.raises(CafeError) as e:
        engine.Optimizer(sc).optimize(initial=[-0.01])     # lambda < 0 scores +inf
    assert e.value.code == 6
