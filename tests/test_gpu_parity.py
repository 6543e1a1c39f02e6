"""GPU parity through the C ABI: the FP64 path against the reference's own
outputs (committed fixtures) and against the CPU oracle.

Tolerances (stated per test):
  * transition matrices: relative 1e-12 per entry >= 1e-280 up to side 260,
    4e-12 above. The GPU builds them with an O(S^2) recurrence, the reference
    with per-term exp/pow whose own error grows with the lgamma magnitudes
    (measured against 40-digit arithmetic at side 601: reference up to
    5.6e-13, recurrence up to 1.8e-13, so they differ by up to 1.8e-12);
  * -lnL and per-family lnL: relative 1e-10 (the parity bar for the plain
    FP64 path).
"""
import math

import numpy as np
import pytest

import oracle
from golden_cases import load_cases, load_json

pytestmark = pytest.mark.gpu

CASES = load_cases()
# subsets of the larger shapes: two lambdas + error model at the reference's
# global bound S = 488 (bins up to 512), 48 taxa with K = 8
CONFIG_CASES = load_cases("ref_configs.json")
REL = 1e-10


@pytest.fixture(scope="module")
def ctx():
    from cafe5_gb300.engine import Context
    c = Context()
    yield c
    c.close()


def rel_err(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-300)


def test_matrices_match_reference_bits(ctx):
    d = load_json("ref_matrices.json")
    for m in d["matrices"]:
        ctx.matrices_build([m["lambda"]], [m["t"]], m["size"])
        ours = ctx.matrix_get(m["lambda"], m["t"], m["size"])
        ref = np.array([[float.fromhex(x) for x in row] for row in m["hex"]])
        mask = ref >= 1e-280
        assert np.all(rel_err(ours[mask], ref[mask]) <= 1e-12), (m["lambda"], m["t"])
        assert np.all(np.abs(ours[~mask]) <= 1e-270)


@pytest.mark.parametrize("lam,t,size", [(0.002, 1.0, 200), (0.0005, 150.0, 257), (0.01, 68.71, 150),
                                         (0.0113, 44.0, 96), (0.3, 1.5, 40), (0.0025, 0.001, 64),
                                         (0.05, 25.0, 12), (0.02, 0.5, 601)])
def test_matrix_build_vs_oracle(ctx, lam, t, size):
    ctx.matrices_build([lam], [t], size)
    ours = ctx.matrix_get(lam, t, size)
    ref = oracle.fill_matrix(lam, t, size)
    mask = ref >= 1e-280
    tol = 1e-12 if size <= 260 else 4e-12
    assert np.all(rel_err(ours[mask], ref[mask]) <= tol)
    assert np.all(ours[~mask] <= 1e-270)
    assert ours[0, 0] == 1.0 and np.all(ours[0, 1:] == 0)


def test_missing_matrix_is_reported(ctx):
    from cafe5_gb300._lib import CafeError
    with pytest.raises(CafeError) as e:
        ctx.matrix_get(0.123456, 9.87, 17)
    assert e.value.code == 2


def _score_case(ctx, case, precision="fp64_ref", prior=None, **kw):
    tid = ctx.upload_tree(case.tree, case.lambda_of_node)
    sid = ctx.upload_families(tid, case.counts)
    ctx.set_prior(case.prior if prior is None else prior)
    ctx.set_error_model(case.err_rows)
    r = ctx.score(tid, sid, case.lambdas, model=case.model, lambda_kind=case.lambda_kind,
                  multipliers=case.multipliers, cat_probs=case.cat_probs, use_error_model=case.err_rows is not None,
                  S=case.S if precision == "fp64_ref" else 0, R=case.R if precision == "fp64_ref" else 0,
                  precision=precision, want_categories=True, **kw)
    ctx.free_families(sid)
    return r


@pytest.mark.parametrize("case", CASES + CONFIG_CASES, ids=[c.name for c in CASES + CONFIG_CASES])
@pytest.mark.parametrize("dedupe", [False, True])
def test_fp64_ref_matches_reference(ctx, case, dedupe):
    """Plain FP64 path vs the reference's own -lnL and per-family lnL
    (tolerance: 1e-10 relative)."""
    r = _score_case(ctx, case, dedupe=dedupe)
    if math.isinf(case.total):
        assert r.total == math.inf
        return
    assert abs(r.total - case.total) <= REL * abs(case.total), (r.total, case.total)
    if case.model == 0:
        exp = np.array(case.fam_lnl)
        fin = np.isfinite(exp)
        assert np.all(rel_err(r.family_lnl[fin], exp[fin]) <= REL)
        assert np.all(r.family_lnl[~fin] == exp[~fin])
    else:
        for f, cats in enumerate(case.cat):
            fam_lh = float.fromhex(cats[0]["fam_lh"])
            assert abs(r.family_lnl[f] - math.log(fam_lh)) <= REL * abs(math.log(fam_lh))
            for k, c in enumerate(cats):
                lc = math.log(float.fromhex(c["cat_lh"]))
                assert abs(r.category_lnl[f, k] - lc) <= REL * abs(lc)


@pytest.mark.parametrize("case", [c for c in CASES + CONFIG_CASES
                                  if not math.isinf(c.total) or c.name in ("syn_base_underflow",
                                                                           "cfg3_gamma_k8_48taxa_underflow")],
                         ids=lambda c: c.name)
def test_fp64_binned_matches_scaled_oracle(ctx, case):
    """Per-family S-bins with power-of-two rescale vs the rescaled oracle at
    the same bins (tolerance: 1e-10 relative)."""
    from cafe5_gb300.families import FamilySet, bin_families
    fams = FamilySet([str(i) for i in range(len(case.counts))], case.counts)
    W, S, R = bin_families(fams)
    ta = oracle.TreeArrays.from_tree(case.tree, case.lambda_of_node)
    prior = np.zeros(int(W.max()) + 8)
    prior[:len(case.prior)] = case.prior[:len(prior)]
    tot, fam, cat = oracle.score(ta, case.counts, case.lambdas, lambda_kind=case.lambda_kind, model=case.model,
                                 multipliers=case.multipliers, cat_probs=case.cat_probs, prior=prior,
                                 err_rows=case.err_rows, fam_S=S, fam_R=R, scaled=True, dedupe=False)
    r = _score_case(ctx, case, precision="fp64_binned", prior=prior)
    if math.isinf(tot):
        assert r.total == math.inf
        return
    assert abs(r.total - tot) <= REL * abs(tot)
    assert np.all(rel_err(r.family_lnl, fam) <= REL)


def test_reference_config0_workload_vs_oracle(ctx):
    """1,000 families, 12 taxa: FP64_REF vs the oracle with the reference's
    global bounds."""
    from cafe5_gb300.families import global_bounds
    from cafe5_gb300.inputs import RootPrior
    from cafe5_gb300.synth import workload
    w = workload(0)
    S, R = global_bounds(w.families)
    prior = RootPrior.uniform(R).vector()
    ta = oracle.TreeArrays.from_tree(w.tree)
    tot, fam, _ = oracle.score(ta, w.families.counts, [0.0025], prior=prior, S=S, R=R)
    tid = ctx.upload_tree(w.tree)
    sid = ctx.upload_families(tid, w.families.counts)
    ctx.set_prior(prior)
    ctx.set_error_model(None)
    r = ctx.score(tid, sid, [0.0025], S=S, R=R, precision="fp64_ref")
    assert abs(r.total - tot) <= REL * abs(tot)
    assert np.all(rel_err(r.family_lnl, fam) <= REL)


def test_rejections_are_scores(ctx):
    """Invalid lambda and gamma saturation return +inf (base_model.cpp:56-60,
    gamma_core.cpp:174-178) without an error."""
    case = [c for c in CASES if c.name == "syn_base_12taxa"][0]
    tid = ctx.upload_tree(case.tree)
    sid = ctx.upload_families(tid, case.counts)
    ctx.set_prior(case.prior)
    ctx.set_error_model(None)
    r = ctx.score(tid, sid, [0.0], S=case.S, R=case.R)
    assert r.total == math.inf
    r = ctx.score(tid, sid, [-1.0], S=case.S, R=case.R)
    assert r.total == math.inf
    r = ctx.score(tid, sid, [5.0], model=1, multipliers=[0.5, 1.5], cat_probs=[0.5, 0.5], S=case.S, R=case.R)
    assert r.total == math.inf and r.status == 3


def test_invalid_arguments_fail_loudly(ctx):
    from cafe5_gb300._lib import CafeError
    case = [c for c in CASES if c.name == "syn_base_12taxa"][0]
    tid = ctx.upload_tree(case.tree)
    with pytest.raises(CafeError):
        ctx.upload_families(tid, case.counts[:, :5])        # wrong column count
    sid = ctx.upload_families(tid, case.counts)
    with pytest.raises(CafeError):
        ctx.score(tid, sid, [0.01], S=3, R=30)             # a count exceeds S
    with pytest.raises(CafeError):
        ctx.score(tid, 999, [0.01], S=case.S, R=case.R)    # unknown set


def test_serving_results_equal_alone_and_in_the_mix(ctx):
    """Requests from several 'optimizers' submitted together give the same
    results as the same requests scored alone."""
    from cafe5_gb300.synth import workload
    from cafe5_gb300.families import global_bounds
    from cafe5_gb300.inputs import RootPrior
    w = workload(0, n_families=300, seed=11)
    S, R = global_bounds(w.families)
    tid = ctx.upload_tree(w.tree)
    sid = ctx.upload_families(tid, w.families.counts)
    ctx.set_prior(RootPrior.uniform(R).vector())
    ctx.set_error_model(None)
    lams = [0.001 * (1 + i) for i in range(12)]
    alone = [ctx.score(tid, sid, [l], S=S, R=R) for l in lams]
    handles = [ctx.submit(tid, sid, [l], S=S, R=R) for l in lams]
    mixed = [ctx.poll(h, -1) for h in handles]
    for a, m in zip(alone, mixed):
        assert m.total == a.total
        assert np.array_equal(m.family_lnl, a.family_lnl)
    st = ctx.serving_stats()
    assert st["completed"] >= len(lams) and st["p99_ms"] >= st["p50_ms"] > 0


# ---------------------------------------------------------------- tensor cores
MIXED_REL = 1e-6    # |dlnL| / |lnL| per family against FP64 at the same bins


def _both(ctx, tree, counts, lambdas, lam_idx=None, kind=0, model=0, mult=(1.0,), probs=(1.0,), err=None, prior=None):
    tid = ctx.upload_tree(tree, lam_idx)
    sid = ctx.upload_families(tid, counts)
    if prior is None:
        from cafe5_gb300.inputs import RootPrior
        prior = RootPrior.uniform(1100).vector()
    ctx.set_prior(prior)
    ctx.set_error_model(err)
    kw = dict(model=model, lambda_kind=kind, multipliers=list(mult), cat_probs=list(probs),
              use_error_model=err is not None, want_categories=True)
    a = ctx.score(tid, sid, lambdas, precision="fp64_binned", **kw)
    b = ctx.score(tid, sid, lambdas, precision="mixed_tf32x3", **kw)
    ctx.free_families(sid)
    return a, b


def _scaled_oracle_binned(tree, counts, lambdas, lam_idx=None, kind=0, model=0, mult=(1.0,), probs=(1.0,), err=None,
                          prior=None):
    """The rescaled FP64 oracle at the GPU's per-family bins: (total, fam)."""
    from cafe5_gb300.families import FamilySet, bin_families
    from cafe5_gb300.inputs import RootPrior
    W, Sb, Rb = bin_families(FamilySet([str(i) for i in range(len(counts))], counts))
    if prior is None:
        prior = RootPrior.uniform(1100).vector()
    ta = oracle.TreeArrays.from_tree(tree, lam_idx)
    tot, fam, _ = oracle.score(ta, counts, lambdas, lambda_kind=kind, model=model, multipliers=list(mult),
                               cat_probs=list(probs), prior=prior, err_rows=err, fam_S=Sb, fam_R=Rb, scaled=True,
                               dedupe=False)
    return tot, fam


def _check_vs_oracle(b, ref_total, ref_fam):
    """The tensor-core path against the FP64 oracle, family by family."""
    fin = np.isfinite(ref_fam)
    assert np.array_equal(fin, np.isfinite(b.family_lnl))
    rel = np.abs(b.family_lnl[fin] - ref_fam[fin]) / np.abs(ref_fam[fin])
    assert rel.max() <= MIXED_REL, f"max rel dlnL vs oracle {rel.max():.3e}"
    if math.isfinite(ref_total):
        assert abs(b.total - ref_total) <= MIXED_REL * abs(ref_total)


def _check_mixed(a, b):
    fin = np.isfinite(a.family_lnl)
    assert np.array_equal(fin, np.isfinite(b.family_lnl))
    rel = np.abs(b.family_lnl[fin] - a.family_lnl[fin]) / np.abs(a.family_lnl[fin])
    assert rel.max() <= MIXED_REL, f"max rel dlnL {rel.max():.3e}"
    if math.isfinite(a.total):
        assert abs(b.total - a.total) <= MIXED_REL * abs(a.total)
    else:
        assert b.total == a.total


@pytest.mark.parametrize("lam", [0.002, 0.0007, 0.0035])
def test_mixed_gamma_config1_shape(ctx, lam):
    """3,000 families of the config-1 shape (24 taxa, K = 4): the tensor-core
    path against the rescaled FP64 oracle and against FP64_BINNED, 1e-6
    relative per family."""
    from cafe5_gb300.synth import workload
    w = workload(1, n_families=3000, seed=21)
    a, b = _both(ctx, w.tree, w.families.counts, [lam], model=1, mult=w.multipliers, probs=w.cat_probs)
    _check_mixed(a, b)
    _check_vs_oracle(b, *_scaled_oracle_binned(w.tree, w.families.counts, [lam], model=1, mult=w.multipliers,
                                               probs=w.cat_probs))


@pytest.mark.parametrize("lam", [0.001, 0.002])
def test_mixed_config3_shape_vs_oracle(ctx, lam):
    """2,000 families of the config-3 shape (48 taxa, K = 8, alpha = 0.5).
    The reference's own FP64 underflows on 3,995 of its first 4,000 such
    families; the rescaled oracle does not. The tree's longest branch is 180,
    so at lambda = 0.002 the largest category saturates (lambda m t > 1) and
    every family with a gene under that branch fails in every path (NaN, a
    total of +inf as the reference's); at 0.001 every family is finite. The
    tensor-core path within 1e-6 of the oracle on every finite family."""
    from cafe5_gb300.synth import workload
    w = workload(3, n_families=2000, seed=0)
    a, b = _both(ctx, w.tree, w.families.counts, [lam], model=1, mult=w.multipliers, probs=w.cat_probs)
    tot, fam = _scaled_oracle_binned(w.tree, w.families.counts, [lam], model=1, mult=w.multipliers,
                                     probs=w.cat_probs)
    if lam == 0.001:
        assert np.isfinite(fam).all() and math.isfinite(tot)
    _check_vs_oracle(b, tot, fam)
    _check_mixed(a, b)


def test_mixed_config2_wide_bins_vs_oracle(ctx):
    """The two-lambda + error-model families of ref_configs.json (the
    largest counts of the 50,000-family set: bins up to 512) on the mixed
    path against the rescaled oracle at the same bins."""
    case = [c for c in CONFIG_CASES if c.name == "cfg2_two_lambdas_error_S600"][0]
    a, b = _both(ctx, case.tree, case.counts, case.lambdas, lam_idx=case.lambda_of_node, kind=1, err=case.err_rows)
    _check_vs_oracle(b, *_scaled_oracle_binned(case.tree, case.counts, case.lambdas, lam_idx=case.lambda_of_node,
                                               kind=1, err=case.err_rows))
    _check_mixed(a, b)


def test_mixed_base_config0(ctx):
    from cafe5_gb300.synth import workload
    w = workload(0, seed=22)
    a, b = _both(ctx, w.tree, w.families.counts, [0.0025])
    _check_mixed(a, b)
    assert b.n_fallback == 0


def test_mixed_error_model_two_lambdas(ctx):
    case = [c for c in CASES if c.name == "syn_multilambda_error_32taxa"][0]
    a, b = _both(ctx, case.tree, case.counts, case.lambdas, lam_idx=case.lambda_of_node, kind=1, err=case.err_rows)
    _check_mixed(a, b)
    _check_vs_oracle(b, *_scaled_oracle_binned(case.tree, case.counts, case.lambdas, lam_idx=case.lambda_of_node,
                                               kind=1, err=case.err_rows))


def _wide_error_model(ndev, max_count=1100):
    """An error model with deviations -h .. +h (ndev = 2h + 1): weight 0.9
    at 0 and the rest shared, halving per step away; deviations below zero
    count are left out of the first rows, as the reference's files do."""
    h = (ndev - 1) // 2
    base = np.array([0.5 ** abs(d) for d in range(-h, h + 1)])
    base[h] = 0.0
    base *= 0.1 / base.sum()
    base[h] = 0.9
    rows = np.tile(base, (max_count + 1, 1))
    for n in range(h):
        rows[n, :h - n] = 0.0
        rows[n] /= rows[n].sum()
    return rows


@pytest.mark.parametrize("ndev", [5, 19])
def test_mixed_wide_error_models(ctx, ndev):
    """Error models of 5 and 19 deviations on the two-lambda tree. Up to
    +-8 deviations the conversion folds the model into each leaf's row of
    the transposed matrix: the tensor-core path within 1e-6 of the rescaled
    oracle; wider models take the FP64 path (every family counted as
    recomputed in FP64)."""
    case = [c for c in CASES if c.name == "syn_multilambda_error_32taxa"][0]
    err = _wide_error_model(ndev)
    a, b = _both(ctx, case.tree, case.counts, case.lambdas, lam_idx=case.lambda_of_node, kind=1, err=err)
    tot, fam = _scaled_oracle_binned(case.tree, case.counts, case.lambdas, lam_idx=case.lambda_of_node, kind=1,
                                     err=err)
    fin = np.isfinite(fam)
    assert fin.all()
    assert np.allclose(a.family_lnl, fam, rtol=1e-10, atol=0)
    if ndev <= 17:
        _check_vs_oracle(b, tot, fam)
        _check_mixed(a, b)
    else:
        assert b.n_fallback == len(case.counts)
        _check_mixed(a, b)


def test_mixed_polytomy_and_underflow_cases(ctx):
    for name in ["syn_polytomy", "syn_base_underflow", "syn_base_zero_family", "syn_gamma_24taxa_k4"]:
        case = [c for c in CASES if c.name == name][0]
        a, b = _both(ctx, case.tree, case.counts, case.lambdas, model=case.model, mult=case.multipliers,
                     probs=case.cat_probs)
        _check_mixed(a, b)


def _check_saturated(a, b):
    """Saturated keys: the same families end (-inf / NaN) on both paths,
    the rest agree to MIXED_REL."""
    fa, fb = a.family_lnl, b.family_lnl
    assert np.array_equal(np.isnan(fa), np.isnan(fb))
    assert np.array_equal(np.isneginf(fa), np.isneginf(fb))
    fin = np.isfinite(fa)
    assert np.array_equal(fin, np.isfinite(fb))
    if fin.any():
        assert np.max(np.abs(fb[fin] - fa[fin]) / np.abs(fa[fin])) <= MIXED_REL
    assert (a.total == b.total) if not math.isfinite(a.total) else abs(b.total - a.total) <= MIXED_REL * abs(a.total)


def test_mixed_saturated_category_matches_fp64(ctx):
    """The largest K=8 category saturates (can_infer tests the raw lambda
    only, so the reference scores it): on the tensor cores a family that is
    exactly zero through a saturated branch ends there; both paths agree on
    every family and on +inf."""
    case = [c for c in CASES if c.name == "syn_gamma_24taxa_k8_small_cat"][0]
    a, b = _both(ctx, case.tree, case.counts, case.lambdas, model=1, mult=case.multipliers, probs=case.cat_probs)
    assert a.total == b.total == math.inf
    _check_saturated(a, b)


@pytest.mark.parametrize("lam,err", [(0.01, False), (0.004, False), (0.01, True)])
def test_mixed_saturated_branches_base_model(ctx, lam, err):
    """Base model with lambda * t > 1 on the long branches of a 8-taxon tree
    (root age 224): families with a nonzero count under a saturated branch
    have lnL = -inf, the others stay finite; with the error model the zero
    test does not apply and the tensor-core pass sends such families to
    FP64."""
    from cafe5_gb300.inputs import ErrorModel
    from cafe5_gb300.synth import _keep_nonzero, _poisson_ge1, simulate_families, yule_tree
    rng = np.random.default_rng(4)
    tree = yule_tree(8, 224.4, 12)
    root = _poisson_ge1(rng, 5.0, 3000)
    c = _keep_nonzero(simulate_families(tree, len(root), np.full(len(root), 0.0025), root, 40))[:2000]
    em = ErrorModel.symmetric(0.05, 200).table() if err else None
    a, b = _both(ctx, tree, c, [lam], err=em)
    _check_saturated(a, b)
    if lam == 0.01 and not err:
        assert np.isneginf(a.family_lnl).any()


def test_mixed_saturated_gamma_many_families_stays_on_tensor_cores(ctx):
    """A saturated category on 20,000 families: the per-family FP64
    recompute covers only families that are not exactly zero."""
    from cafe5_gb300.synth import workload
    w = workload(1, n_families=20000, seed=9)
    from cafe5_gb300.inputs import discrete_gamma
    probs, mult = discrete_gamma(0.5, 8)
    a, b = _both(ctx, w.tree, w.families.counts, [0.006], model=1, mult=mult, probs=probs)
    _check_saturated(a, b)
    assert b.n_fallback < w.families.n_families // 2


def test_mixed_wide_bins_hybrid(ctx):
    """Families needing more than 256 states (bin 384: a pair of CTAs per
    tile) in the same request as families of the single-CTA bins."""
    from cafe5_gb300.synth import workload
    w = workload(0, n_families=600, seed=23)
    counts = w.families.counts.copy()
    counts[:7] += 230            # bins 384 (counts ~240-260)
    a, b = _both(ctx, w.tree, counts, [0.0025])
    _check_mixed(a, b)


def test_mixed_pair_tiles_vs_oracle_and_tile_walk(ctx):
    """Bins 384 and 512 on the tensor cores: each 128-family tile is shared by
    a cluster of two CTAs, each computing half the states and exchanging the
    per-family statistics. 160 gamma (K = 4) families of the config-1 tree
    with counts of 230-400 against the rescaled FP64 oracle at 1e-6; then the
    same families tiled 40 times (200 tiles per bin, more than the pairs the
    GPU holds, so every pair walks several tiles) give the same bits. The
    range bound must leave most families on the tensor cores."""
    from cafe5_gb300.synth import workload
    w = workload(1, n_families=400, seed=31)
    counts = w.families.counts[w.families.counts.max(axis=1) < 40][:160].copy()
    counts[:80] += 230                  # bin 384
    counts[80:] += 330                  # bin 512
    mult, probs = w.multipliers, w.cat_probs
    a, b = _both(ctx, w.tree, counts, [0.002], model=1, mult=mult, probs=probs)
    assert b.n_fallback < len(counts) // 4, f"{b.n_fallback} of {len(counts)} families recomputed in FP64"
    _check_mixed(a, b)
    _check_vs_oracle(b, *_scaled_oracle_binned(w.tree, counts, [0.002], model=1, mult=mult, probs=probs))
    big = np.tile(counts, (40, 1))
    c, d = _both(ctx, w.tree, big, [0.002], model=1, mult=mult, probs=probs)
    for r in range(40):
        assert np.array_equal(d.family_lnl[r * len(counts):(r + 1) * len(counts)], b.family_lnl), r


def test_mixed_results_do_not_depend_on_batch_composition(ctx):
    """Per-family results are identical whether a family is scored with
    10,000 others or with 100."""
    from cafe5_gb300.synth import workload
    w = workload(1, n_families=4000, seed=24)
    a, b = _both(ctx, w.tree, w.families.counts, [0.002], model=1, mult=w.multipliers, probs=w.cat_probs)
    sub = w.families.counts[:300]
    c, d = _both(ctx, w.tree, sub, [0.002], model=1, mult=w.multipliers, probs=w.cat_probs)
    assert np.array_equal(d.family_lnl, b.family_lnl[:300])


def test_mixed_term_recompute_is_per_family_and_exact(ctx):
    """Config-3 families (48 taxa, K = 8): the smallest categories' nearly
    diagonal matrices push some families' FP32 range bound over budget, and
    the FP64 pass recomputes only the flagged (family, category) terms,
    sharing 32-family tiles with families whose terms it must not write.
    Every family's result is the same bits in a batch of 2,000 and in
    subsets that change which families share its tiles, and within 1e-6 of
    the rescaled oracle."""
    from cafe5_gb300.synth import workload
    w = workload(3, n_families=2000, seed=0)
    lam = [0.001]
    a, b = _both(ctx, w.tree, w.families.counts, lam, model=1, mult=w.multipliers, probs=w.cat_probs)
    assert b.n_fallback > 0, "no family was flagged: the case does not reach the per-term recompute"
    rng = np.random.default_rng(5)
    for take in (np.arange(0, 2000, 3), np.sort(rng.choice(2000, 400, replace=False))):
        c, d = _both(ctx, w.tree, w.families.counts[take], lam, model=1, mult=w.multipliers, probs=w.cat_probs)
        assert np.array_equal(d.family_lnl, b.family_lnl[take], equal_nan=True)
        # (a category term whose product is zero everywhere is NaN, as in FP64)
        assert np.array_equal(d.category_lnl, b.category_lnl[take], equal_nan=True)
    _check_vs_oracle(b, *_scaled_oracle_binned(w.tree, w.families.counts, lam, model=1, mult=w.multipliers,
                                               probs=w.cat_probs))


@pytest.mark.parametrize("wl,model", [(2, 0), (0, 1)], ids=["two_lambda_error_model", "gamma_k4"])
def test_sparse_fp64_bins_walk_one_family_per_cluster(ctx, wl, model):
    """FP64 bins too sparse to fill the GPU with 32-family tiles are walked
    one family per thread-block cluster; their families get the same bits as
    in a bin full enough for the 32-family tile walk in fp64_binned, and
    mixed_tf32x3 (bins 384 and 512 on the tensor cores, in CTA pairs) gives
    the same bits in both sets as well. The small golden
    cases of test_fp64_binned_matches_scaled_oracle run on the cluster walk
    (every bin sparse) against the oracle."""
    from cafe5_gb300.families import FamilySet, bin_families
    from cafe5_gb300.inputs import ErrorModel, RootPrior
    from cafe5_gb300.synth import workload
    w = workload(wl, n_families=160, seed=41)
    counts = w.families.counts.copy()
    counts = counts[counts.max(axis=1) < 60]
    counts[:3] += 230                        # bin 384
    counts[3:6] += 330                       # bin 512
    fams = FamilySet([str(i) for i in range(len(counts))], counts)
    W, _, _ = bin_families(fams)
    assert sorted(set(int(x) for x in W[:6])) == [384, 512]
    K = 4 if model else 1
    mult = [0.2, 0.6, 1.1, 2.1] if model else [1.0]
    probs = [0.25] * 4 if model else [1.0]
    reps = -(-(100 * 32) // K)               # 100 tiles per category: a bin this full takes the tile walk
    wide = [np.tile(counts[i:i + 3], (reps // 3 + 1, 1))[:reps] for i in (0, 3)]
    big = np.concatenate([wide[0], wide[1], counts[6:]])
    pos_big = [0, 1, 2, reps, reps + 1, reps + 2]
    err = ErrorModel.symmetric(0.05, 1100).table() if wl == 2 else None
    prior = RootPrior.uniform(1100).vector()
    lam_idx = w.lambda_of_node if wl == 2 else None
    kw = dict(model=model, lambda_kind=1 if wl == 2 else 0, multipliers=mult, cat_probs=probs,
              use_error_model=err is not None)
    tid = ctx.upload_tree(w.tree, lam_idx)
    ctx.set_prior(prior)
    ctx.set_error_model(err)
    small_sid = ctx.upload_families(tid, counts)
    big_sid = ctx.upload_families(tid, big)
    for precision in ("fp64_binned", "mixed_tf32x3"):
        a = ctx.score(tid, small_sid, w.lambdas, precision=precision, **kw)
        b = ctx.score(tid, big_sid, w.lambdas, precision=precision, **kw)
        assert np.array_equal(a.family_lnl[:6], b.family_lnl[pos_big]), precision
        assert np.array_equal(a.family_lnl[6:], b.family_lnl[2 * reps:]), precision
    ctx.free_families(small_sid)
    ctx.free_families(big_sid)
