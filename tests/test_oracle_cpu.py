"""Pins the CPU oracle (oracle/cafe_oracle.c) before anything is checked
against it:

* the known-answer values of the reference's own unit tests (test.cpp),
* bit patterns produced by the reference itself, compiled from its own
  sources (tests/golden/ref_*.json, made by tests/golden/make_golden.py).
"""
import math

import numpy as np
import pytest

import oracle
from cafe5_gb300.inputs import ErrorModel, RootPrior, discrete_gamma
from cafe5_gb300.tree import parse_newick
from golden_cases import load_cases, load_json

KAT = load_json("reference_kats.json")
CASES = load_cases()
CONFIG_CASES = load_cases("ref_configs.json")


def approx5(a, b, rel=1.1920929e-5):
    """doctest::Approx's default rule (epsilon = 100 * FLT_EPSILON, scale 1):
    |a - b| < eps * (1 + max(|a|, |b|)). The test.cpp values are printed to
    5-6 digits, so these checks pin about 5 significant digits; bit-exact
    parity comes from the reference-generated fixtures below."""
    return abs(a - b) < rel * (1.0 + max(abs(a), abs(b)))


def test_transition_kats():
    # the test prints 5-6 significant digits (truncated): one unit in the
    # last printed place
    for k in KAT["transition"]:
        assert abs(oracle.transition(k["lambda"], k["t"], k["s"], k["c"]) - k["value"]) <= 1e-5, k


def test_cached_matrix_entry_uses_quantized_keys():
    for k in KAT["cached_matrix_entry"]:
        m = oracle.fill_matrix(k["lambda"], k["t"], 8)       # quantized lambda / t
        assert approx5(m[k["s"], k["c"]], k["value"], k["rel"]), k
    # 68.7105 is computed as 68.710 (matrix_cache.h:49-62)
    assert oracle.quantize(0.006335, 68.7105) == (0.006335, 68.71)


def test_matrix_5x5():
    k = KAT["matrix_5x5"]
    m = oracle.fill_matrix(k["lambda"], k["t"], 5)
    assert np.max(np.abs(m - np.asarray(k["values"]))) < k["abs"]


def test_bd_rate_kats():
    for k in KAT["bd_rate_log"]:
        assert approx5(math.log(oracle.bd_rate(k["s"], k["c"], k["log_alpha"], k["coeff"])), k["log_value"]), k
    for k in KAT["bd_rate"]:
        assert approx5(oracle.bd_rate(k["s"], k["c"], k["log_alpha"], k["coeff"]), k["value"]), k


def test_multiply_subrange():
    k = KAT["multiply"]
    m = np.asarray(k["matrix"], dtype=np.float64)
    v = np.asarray(k["v"], dtype=np.float64)
    out = np.zeros(3)
    lib = oracle.lib()
    lib.oracle_multiply(m.ctypes.data, 3, v.ctypes.data, 0, 2, 0, 2, out.ctypes.data)
    assert out.tolist() == k["result"]
    big = np.zeros((8, 8))
    big[3:6, 3:6] = m
    lib.oracle_multiply(big.ctypes.data, 8, v.ctypes.data, 3, 5, 3, 5, out.ctypes.data)
    assert out.tolist() == k["result"]


def test_saturation():
    for k in KAT["saturation"]:
        assert bool(oracle.lib().oracle_is_saturated(k["t"], k["lambda"])) == k["saturated"]


def test_cache_key_quantization():
    k = KAT["cache_key_quantization"]
    keys = set()
    lam = 0.0
    for _ in range(k["n_accumulated"]):
        lam += k["step"]
        keys.add((int(lam * 1000000000), int(k["t"] * 1000)))
    assert len(keys) == k["distinct"]
    assert (int(k["probe_lambda"] * 1000000000), int(k["t"] * 1000)) in keys


def _tree_mats(newick, lam, size):
    t = parse_newick(newick)
    ta = oracle.TreeArrays.from_tree(t)
    mats = [None if t.parent[v] < 0 else oracle.fill_matrix(lam, t.branch_length[v], size) for v in range(t.n_nodes)]
    return t, ta, mats


def test_prune_root_vector_kat():
    k = KAT["prune_root_log"]
    t, ta, mats = _tree_mats(k["newick"], k["lambda"] * k["multiplier"], k["matrix_size"])
    counts = [k["counts"][n] for n in t.leaf_names]
    root, _ = oracle.prune(ta, counts, mats, k["matrix_size"], k["S"], k["R"])
    for a, b in zip(np.log(root), k["log_expected"]):
        assert approx5(a, b), (a, b)
    k = KAT["root_vector_log"]
    t, ta, mats = _tree_mats(k["newick"], k["lambda"], k["matrix_size"])
    root, _ = oracle.prune(ta, [k["counts"][n] for n in t.leaf_names], mats, k["matrix_size"], k["S"], k["R"])
    for a, b in zip(np.log(root), k["log_expected"]):
        assert approx5(a, b), (a, b)


def test_leaf_vectors_through_identity_branch():
    """A root with one leaf child on an identity matrix exposes the leaf
    vector as root[j] = leaf[j + 1] (test.cpp:1685-1727, 1765-1804)."""
    t = parse_newick("(A:1);")
    ta = oracle.TreeArrays.from_tree(t)
    eye = np.eye(22)
    mats = [None if t.parent[v] < 0 else eye for v in range(t.n_nodes)]
    k = KAT["leaf_error_model"]
    em = ErrorModel()
    for i, r in enumerate(k["rows"]):
        em.set_probabilities(i, r)
    root, _ = oracle.prune(ta, [k["count"]], mats, 22, k["S"], k["S"], err_rows=em.table())
    assert root.tolist() == k["expected"][1:k["S"] + 1]
    kk = KAT["leaf_one_hot"]
    root, _ = oracle.prune(ta, [kk["B"]], mats, 22, kk["S"], kk["S"])
    assert root.tolist() == [1.0 if j + 1 == kk["B"] else 0.0 for j in range(kk["S"])]


def test_base_total_kat():
    k = KAT["base_total"]
    t = parse_newick(k["newick"])
    ta = oracle.TreeArrays.from_tree(t)
    prior = RootPrior.uniform(k["prior_uniform"]).vector()
    tot, fam, _ = oracle.score(ta, np.asarray(k["counts"]), [k["lambda"]], prior=prior, S=k["S"], R=k["R"])
    assert approx5(tot, k["neg_lnl"])


def test_gamma_kats():
    k = KAT["gamma_prune"]
    t = parse_newick(k["newick"])
    ta = oracle.TreeArrays.from_tree(t)
    prior = RootPrior.from_rootdist({int(a): b for a, b in k["rootdist"].items()}).vector()
    tot, fam, cat = oracle.score(ta, np.asarray(k["counts"]), [k["lambda"]], model=1,
                                 multipliers=k["multipliers"], cat_probs=k["cat_probs"], prior=prior, S=k["S"],
                                 R=k["R"])
    assert approx5(cat[0, 0], k["log_cat"][0]) and approx5(cat[0, 1], k["log_cat"][1])
    k = KAT["gamma_saturated"]
    tot, _, _ = oracle.score(ta, np.asarray(k["counts"]), [k["lambda"]], model=1, multipliers=k["multipliers"],
                             cat_probs=k["cat_probs"], prior=RootPrior.uniform(100).vector(), S=k["S"], R=k["R"])
    assert tot == math.inf


def test_reference_matrices_bit_exact():
    d = load_json("ref_matrices.json")
    for m in d["matrices"]:
        ours = oracle.fill_matrix(m["lambda"], m["t"], m["size"])
        ref = np.array([[float.fromhex(x) for x in row] for row in m["hex"]])
        assert np.array_equal(ours, ref), (m["lambda"], m["t"])


def test_discrete_gamma_matches_reference():
    """Bit-exact: the library restates AS 91 / AS 32 / AS 70 as get_gamma does."""
    d = load_json("ref_matrices.json")
    for g in d["gamma"]:
        probs, mult = discrete_gamma(g["alpha"], g["K"])
        ref = [float.fromhex(x) for x in g["multipliers"]]
        assert list(mult) == ref, (g["K"], g["alpha"])
        assert probs == [float.fromhex(x) for x in g["probs"]]


def test_oracle_discrete_gamma_bits_match_reference():
    """The oracle's own AS 91 / AS 32 / AS 70 restatement (used where the
    library must not be loaded, e.g. the timed reference arm) carries the
    reference's bits, and agrees with the library's over a sweep of shapes
    that reaches every branch of AS 91 (small v, v <= 0.32, Wilson-Hilferty)
    and both branches of AS 32."""
    for g in load_json("ref_matrices.json")["gamma"]:
        probs, mult = oracle.discrete_gamma(g["alpha"], g["K"])
        assert [m.hex() for m in mult] == [float.fromhex(x).hex() for x in g["multipliers"]], (g["K"], g["alpha"])
        assert probs == [float.fromhex(x) for x in g["probs"]]
    for a in (0.02, 0.1, 0.16, 0.37, 0.5, 0.51, 1.0, 1.7, 3.3, 12.0, 80.0):
        for K in (2, 3, 4, 5, 8, 16):
            assert oracle.discrete_gamma(a, K) == discrete_gamma(a, K), (a, K)
    with pytest.raises(ValueError):
        oracle.discrete_gamma(0.0, 4)


@pytest.mark.parametrize("case", CASES + CONFIG_CASES, ids=[c.name for c in CASES + CONFIG_CASES])
def test_oracle_matches_reference_end_to_end(case):
    ta = oracle.TreeArrays.from_tree(case.tree, case.lambda_of_node)
    tot, fam, cat = oracle.score(ta, case.counts, case.lambdas, lambda_kind=case.lambda_kind, model=case.model,
                                 multipliers=case.multipliers, cat_probs=case.cat_probs, prior=case.prior,
                                 err_rows=case.err_rows, S=case.S, R=case.R)
    if math.isinf(case.total):
        assert tot == case.total
        return
    assert tot == case.total, (tot, case.total)          # bit-exact
    if case.model == 0:
        for a, b in zip(fam, case.fam_lnl):
            assert a == b
    else:
        for f, cats in enumerate(case.cat):
            lh = sum(float.fromhex(c["cat_lh"]) for c in cats)
            assert math.log(float.fromhex(cats[0]["fam_lh"])) == fam[f]
            for k, c in enumerate(cats):
                assert cat[f, k] == math.log(float.fromhex(c["cat_lh"]))


@pytest.mark.parametrize("case", [c for c in CASES if not math.isinf(c.total)][:6], ids=lambda c: c.name)
def test_scaled_oracle_agrees_where_reference_is_finite(case):
    ta = oracle.TreeArrays.from_tree(case.tree, case.lambda_of_node)
    tot, fam, _ = oracle.score(ta, case.counts, case.lambdas, lambda_kind=case.lambda_kind, model=case.model,
                               multipliers=case.multipliers, cat_probs=case.cat_probs, prior=case.prior,
                               err_rows=case.err_rows, S=case.S, R=case.R, scaled=True)
    assert abs(tot - case.total) <= 1e-12 * abs(case.total)


def test_scaled_oracle_is_finite_where_reference_underflows():
    case = [c for c in CASES if c.name == "syn_base_underflow"][0]
    assert math.isinf(case.total) and math.isinf(case.fam_lnl[0]) and math.isfinite(case.fam_lnl[1])
    ta = oracle.TreeArrays.from_tree(case.tree, case.lambda_of_node)
    tot, fam, _ = oracle.score(ta, case.counts, case.lambdas, prior=case.prior, S=case.S, R=case.R, scaled=True)
    assert math.isfinite(tot) and np.all(np.isfinite(fam))
    assert fam[1] == case.fam_lnl[1]


def test_saturated_category_is_rejected_by_both():
    """K=8 at lambda 0.003: the largest category saturates on the longest
    branch, so the reference returns +inf (gamma_core.cpp:151-152, 216-225)
    and so does the rescaled oracle."""
    case = [c for c in CASES if c.name == "syn_gamma_24taxa_k8_small_cat"][0]
    assert math.isinf(case.total)
    ta = oracle.TreeArrays.from_tree(case.tree, case.lambda_of_node)
    tot, _, _ = oracle.score(ta, case.counts, case.lambdas, model=1, multipliers=case.multipliers,
                             cat_probs=case.cat_probs, prior=case.prior, S=case.S, R=case.R, scaled=True)
    assert tot == math.inf


RECON = [c for c in CASES if c.recon is not None]


@pytest.mark.parametrize("case", RECON, ids=[c.name for c in RECON])
def test_oracle_reconstruction_matches_reference(case):
    """Pupko joint reconstruction and branch probabilities, bit for bit
    against model::reconstruct_ancestral_states and compute_viterbi_sum of
    the compiled reference: node counts, per-category states and weighted
    means (gamma), and every branch probability."""
    ta = oracle.TreeArrays.from_tree(case.tree, case.lambda_of_node)
    gamma = case.model == 1
    state, mean, cnt, rmax = oracle.reconstruct(ta, case.counts, case.lambdas, prior=case.prior, S=case.S,
                                                R=case.R, multipliers=case.multipliers if gamma else None,
                                                cat_probs=case.cat_probs if gamma else None)
    ref = case.recon
    assert np.array_equal(cnt, ref["node_count"])
    if gamma:
        internal = ref["cat_state"][0, 0] >= 0
        assert np.array_equal(state[:, :, internal], ref["cat_state"][:, :, internal])
        assert np.array_equal(mean[:, internal], ref["mean"][:, internal])
    bp = oracle.branch_probabilities(ta, case.lambdas, ref["node_count"], case.S, case.R)
    assert np.array_equal(bp, ref["branch_prob"], equal_nan=True)


def test_reconstruction_edge_cases_present():
    """The fixtures cover a family whose likelihood underflows (root L = 0
    -> the reference's failed reconstruction), a polytomy, two lambdas and
    gamma categories whose root L underflows."""
    names = {c.name for c in RECON}
    assert {"syn_base_underflow", "syn_polytomy", "syn_multilambda_error_32taxa",
            "syn_gamma_24taxa_k8_small_cat"} <= names
    case = [c for c in RECON if c.name == "syn_base_underflow"][0]
    ta = oracle.TreeArrays.from_tree(case.tree, case.lambda_of_node)
    _, _, _, rmax = oracle.reconstruct(ta, case.counts, case.lambdas, prior=case.prior, S=case.S, R=case.R)
    assert rmax[0, 0] == 0 and rmax[0, 1] > 0


PVALUE_CASES = __import__("golden_cases").load_pvalue_cases()


@pytest.mark.parametrize("case", PVALUE_CASES, ids=[c.name for c in PVALUE_CASES])
def test_oracle_pvalues_match_reference(case):
    """compute_pvalues with the same seed: every conditional distribution
    (sorted simulated likelihoods per root size) and every p-value equal
    the compiled reference's bit for bit."""
    ta = oracle.TreeArrays.from_tree(case.tree, case.lambda_of_node)
    pv, cd, _ = oracle.pvalues(ta, case.counts, case.lambdas, S=case.S, R=case.R, n_sim=case.n_sim,
                               seed=case.seed)
    assert np.array_equal(cd, case.conditional)
    assert np.array_equal(pv, case.pvalues)


SIM_CASES = __import__("golden_cases").load_simulation_cases()


@pytest.mark.parametrize("case", SIM_CASES, ids=[c.name for c in SIM_CASES])
def test_oracle_simulation_matches_reference(case):
    """The simulator action with the same seed and root sizes: every
    simulated node size and the lambda of every family equal the compiled
    reference's (simulator::simulate_processes)."""
    ta = oracle.TreeArrays.from_tree(case.tree, case.lambda_of_node)
    kw = {}
    if case.K:
        probs, mult = discrete_gamma(case.alpha, case.K)
        kw = dict(multipliers=mult, cat_probs=probs)
    if case.err is not None:
        kw.update(err_rows=case.err.table(), err_max_count=len(case.err.rows))
    sizes, lam = oracle.simulate(ta, case.lambdas, case.roots, S=case.S, R=case.R, seed=case.seed, **kw)
    assert np.array_equal(sizes, case.sizes)
    assert np.array_equal(lam, case.lambda_used)
