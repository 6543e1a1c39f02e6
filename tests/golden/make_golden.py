"""Regenerate the reference golden fixtures in this folder.

Runs the CAFE5 reference itself -- compiled from its own sources by
oracle/Makefile into oracle/_ref/cafe_ref_harness -- on small seeded
synthetic cases and on the inputs of the reference's own known-answer
tests, and stores inputs plus hex-float outputs:

  ref_cases.json     end-to-end infer_family_likelihoods cases, with the
                     Pupko reconstruction and branch probabilities of each
                     valid case (reconstruct_ancestral_states,
                     compute_viterbi_sum)
  ref_matrices.json  transition matrices from matrix_cache
  ref_optimizer.json Nelder-Mead searches (fminsearch_min) over analytic
                     objectives and over the likelihood scorers
  ref_pvalues.json   compute_pvalues with the random engine seeded:
                     conditional distributions and per-family p-values
  ref_simulations.json  the simulator action with the engine seeded: root
                     sizes and every simulated node size

Only this script reads the reference (the checkout named by the
CAFE_REFERENCE environment variable, and the harness built from it); the
tests read the committed JSON. Usage:
    CAFE_REFERENCE=<checkout> make -C oracle ref && python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from cafe5_gb300.families import FamilySet, global_bounds, write_families  # noqa: E402
from cafe5_gb300.inputs import RootPrior, discrete_gamma  # noqa: E402
from cafe5_gb300.synth import simulate_families, workload  # noqa: E402
from cafe5_gb300.tree import parse_newick  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "cafe_ref_harness")


def run(args):
    out = subprocess.run([HARNESS] + args, check=True, capture_output=True, text=True).stdout
    return out


def parse_output(out: str):
    res = {"fam": {}, "cat": {}}
    for ln in out.splitlines():
        tok = ln.split()
        if tok[0] == "total":
            res["total_hex"] = tok[2]
        elif tok[0] == "bounds":
            res["S"], res["R"] = int(tok[1]), int(tok[2])
        elif tok[0] == "fam":
            res["fam"][tok[1]] = tok[2]
        elif tok[0] == "cat":
            res["cat"].setdefault(tok[1], []).append({"mult": tok[2], "cat_lh": tok[3], "fam_lh": tok[4]})
    return res


def lambda_tree_newick(tree, lam_idx):
    def rec(v):
        lab = tree.name[v] if tree.is_leaf(v) else "(" + ",".join(rec(c) for c in tree.children[v]) + ")"
        if tree.parent[v] >= 0:
            lab += f":{lam_idx[v] + 1}"
        return lab
    return rec(tree.root) + ";"


def parse_search(out: str):
    res = {}
    for ln in out.splitlines():
        tok = ln.split()
        if tok[0] == "best":
            res["best_hex"] = tok[1:]
        elif tok[0] in ("score", "first"):
            res[tok[0] + "_hex"] = tok[1]
        elif tok[0] in ("iters", "evals"):
            res[tok[0]] = int(tok[1])
    return res


def parse_recon(out: str, ids, n_nodes):
    """`rec` / `bp` / `rcat` / `rmean` lines of the harness's --reconstruct."""
    rec, bp, rcat, rmean = {}, {}, {}, {}
    for ln in out.splitlines():
        tok = ln.split()
        if tok[0] == "rec":
            rec[tok[1]] = [int(x) for x in tok[2:]]
        elif tok[0] == "bp":
            bp[tok[1]] = [None if x == "NA" else x for x in tok[2:]]
        elif tok[0] == "rcat":
            rcat.setdefault(tok[1], []).append([int(x) for x in tok[3:]])
        elif tok[0] == "rmean":
            rmean[tok[1]] = [None if x == "NA" else x for x in tok[2:]]
    for d in (rec, bp):
        assert all(len(d[i]) == n_nodes for i in ids)
    # one space-separated string per family (per category for cat_state)
    # keeps the fixture small
    j = lambda v: " ".join("NA" if x is None else str(x) for x in v)
    return {"node_count": [j(rec[i]) for i in ids], "bp_hex": [j(bp[i]) for i in ids],
            "cat_state": [[j(r) for r in rcat[i]] for i in ids] if rcat else None,
            "mean_hex": [j(rmean[i]) for i in ids] if rmean else None}


def make_case(name, tree, fams, lambdas, *, lam_idx=None, model="base", mult=None, probs=None,
              err=None, S=None, R=None, prior="uniform", note="", alpha=None, K=None, optimize=None,
              initial=None, recon=False, estimate_bounds=False):
    with tempfile.TemporaryDirectory() as d:
        tp, fp = os.path.join(d, "t.nwk"), os.path.join(d, "f.tab")
        nwk = tree.to_newick()
        open(tp, "w").write(nwk)
        write_families(fp, fams, tree)
        args = ["--tree", tp, "--families", fp, "--lambdas", ",".join(repr(x) for x in lambdas),
                "--prior", prior]
        lnwk = None
        if lam_idx is not None:
            lp = os.path.join(d, "l.nwk")
            lnwk = lambda_tree_newick(tree, lam_idx)
            open(lp, "w").write(lnwk)
            args += ["--lambda-tree", lp]
        err_text = None
        if err is not None:
            ep = os.path.join(d, "e.txt")
            err_text = err
            open(ep, "w").write(err)
            args += ["--error", ep]
        if model == "gamma" and alpha is not None:
            args += ["--gamma-alpha", repr(alpha), "--gamma-k", str(K)]
        elif model == "gamma":
            args += ["--gamma-mult", ",".join(repr(x) for x in mult), "--gamma-prob", ",".join(repr(x) for x in probs)]
        if S is not None:
            args += ["--max-family", str(S), "--max-root", str(R)]
        if estimate_bounds:
            args += ["--estimate-bounds"]
        if optimize is not None:
            search = parse_search(run(args + ["--optimize", optimize, "--initial",
                                              ",".join(repr(x) for x in initial)]))
        out = parse_output(run(args))
        rec = parse_recon(run(args + ["--reconstruct", "--quiet"]), fams.ids, tree.n_nodes) if recon else None
    case = {
        "name": name, "note": note, "newick": nwk, "lambda_newick": lnwk, "taxa": tree.leaf_names,
        "ids": fams.ids, "counts": fams.counts.tolist(), "lambdas": [float(x).hex() for x in lambdas],
        "model": model, "multipliers": None if mult is None else [float(x).hex() for x in mult],
        "cat_probs": None if probs is None else [float(x).hex() for x in probs],
        "error_model": err_text, "prior": prior, "S": out["S"], "R": out["R"],
        "alpha": alpha, "K": K,
        "expected": {"total_hex": out["total_hex"], "fam_lnl_hex": [out["fam"].get(i) for i in fams.ids],
                     "cat": [out["cat"].get(i) for i in fams.ids] if model == "gamma" else None},
    }
    if rec is not None:
        case["recon"] = rec
    if optimize is not None:
        case["optimize"] = optimize
        case["initial"] = [float(x).hex() for x in initial]
        case["search"] = search
    return case


def make_pvalue_case(name, tree, fams, lambdas, *, n_sim, seed, lam_idx=None, S=None, R=None, note=""):
    """compute_pvalues of the compiled reference with its random engine
    seeded: the sorted conditional distribution of every root size and the
    p-value of every family."""
    with tempfile.TemporaryDirectory() as d:
        tp, fp = os.path.join(d, "t.nwk"), os.path.join(d, "f.tab")
        nwk = tree.to_newick()
        open(tp, "w").write(nwk)
        write_families(fp, fams, tree)
        args = ["--tree", tp, "--families", fp, "--lambdas", ",".join(repr(x) for x in lambdas),
                "--pvalues", str(n_sim), "--seed", str(seed), "--quiet"]
        lnwk = None
        if lam_idx is not None:
            lp = os.path.join(d, "l.nwk")
            lnwk = lambda_tree_newick(tree, lam_idx)
            open(lp, "w").write(lnwk)
            args += ["--lambda-tree", lp]
        if S is not None:
            args += ["--max-family", str(S), "--max-root", str(R)]
        out = run(args).splitlines()
    bounds = [ln for ln in out if ln.startswith("bounds")][0].split()
    cd = [" ".join(ln.split()[2:]) for ln in out if ln.startswith("cd ")]
    pv = {ln.split()[1]: ln.split()[2] for ln in out if ln.startswith("pv ")}
    return {"name": name, "note": note, "newick": nwk, "lambda_newick": lnwk, "taxa": tree.leaf_names,
            "ids": fams.ids, "counts": fams.counts.tolist(), "lambdas": [float(x).hex() for x in lambdas],
            "S": int(bounds[1]), "R": int(bounds[2]), "n_sim": n_sim, "seed": seed,
            "conditional_hex": cd, "pvalue_hex": [pv[i] for i in fams.ids]}


def make_sim_case(name, tree, fams, lambdas, *, n, seed, prior, lam_idx=None, err=None, alpha=None, K=None,
                  note=""):
    """The simulator action of the compiled reference: the prior resized to
    n families (engine seeded with seed + 1), then simulate_processes with
    the engine seeded with `seed`."""
    with tempfile.TemporaryDirectory() as d:
        tp, fp = os.path.join(d, "t.nwk"), os.path.join(d, "f.tab")
        nwk = tree.to_newick()
        open(tp, "w").write(nwk)
        write_families(fp, fams, tree)
        args = ["--tree", tp, "--families", fp, "--lambdas", ",".join(repr(x) for x in lambdas),
                "--prior", prior, "--simulate", str(n), "--seed", str(seed), "--quiet"]
        lnwk = None
        if lam_idx is not None:
            lp = os.path.join(d, "l.nwk")
            lnwk = lambda_tree_newick(tree, lam_idx)
            open(lp, "w").write(lnwk)
            args += ["--lambda-tree", lp]
        if err is not None:
            ep = os.path.join(d, "e.txt")
            open(ep, "w").write(err)
            args += ["--error", ep]
        if alpha is not None:
            args += ["--gamma-alpha", repr(alpha), "--gamma-k", str(K)]
        out = run(args).splitlines()
    bounds = [ln for ln in out if ln.startswith("bounds")][0].split()
    roots = [int(x) for x in [ln for ln in out if ln.startswith("roots")][0].split()[1:]]
    sims = [ln.split()[1:] for ln in out if ln.startswith("sim ")]
    return {"name": name, "note": note, "newick": nwk, "lambda_newick": lnwk, "taxa": tree.leaf_names,
            "ids": fams.ids, "counts": fams.counts.tolist(), "lambdas": [float(x).hex() for x in lambdas],
            "S": int(bounds[1]), "R": int(bounds[2]), "n": n, "seed": seed, "prior": prior, "error_model": err,
            "alpha": alpha, "K": K, "roots": roots, "lambda_hex": [r[0] for r in sims],
            "sizes": [" ".join(r[1:]) for r in sims]}


def make_case_r(*a, **kw):
    kw.setdefault("recon", True)
    return make_case(*a, **kw)


def main():
    if not os.path.exists(HARNESS):
        raise SystemExit("build the harness first: make -C oracle ref")
    cases = []
    # -- the reference's own known-answer inputs (test.cpp) --------------
    t = parse_newick("(A:1,B:1);")
    fams = FamilySet(["f1", "f2", "f3", "f4"], np.array([[1, 2], [2, 1], [3, 6], [6, 3]], np.int32))
    cases.append(make_case_r("kat_infer_processes", t, fams, [0.01], S=56, R=8, prior="uniform:100",
                           note="test.cpp:461-488, expected -lnL 46.56632"))
    t = parse_newick("(A:1,B:3):7;")
    fams = FamilySet(["f1"], np.array([[3, 6]], np.int32))
    cases.append(make_case_r("kat_gamma_prune", t, fams, [0.005], model="gamma", mult=[0.1, 0.5], probs=[0.01, 0.05],
                           S=10, R=8, prior="rootdist:1=2,2=2,3=2,4=2,5=1",
                           note="test.cpp:1269-1294, log category likelihoods -23.04433, -16.68005"))
    t = parse_newick("(A:1,B:3):7;")
    cases.append(make_case_r("kat_gamma_saturated", t, fams, [0.9], model="gamma", mult=[0.1, 0.5], probs=[1.0, 1.0],
                           S=10, R=8, prior="uniform:100", note="test.cpp:1296-1311: saturated -> +inf",
                           recon=False))
    # -- seeded synthetic cases ---------------------------------------------
    w0 = workload(0, n_families=150, seed=3)
    cases.append(make_case_r("syn_base_12taxa", w0.tree, w0.families, [0.0025],
                           note="config-0 shape, global S/R, uniform prior"))
    cases.append(make_case_r("syn_base_12taxa_poisson", w0.tree, w0.families, [0.004], prior="poisson:5.5",
                           note="Poisson root prior (float-rounded)"))
    zero = FamilySet(w0.families.ids[:20] + ["zero"], np.vstack([w0.families.counts[:20],
                                                                  np.zeros((1, 12), np.int32)]))
    cases.append(make_case_r("syn_base_zero_family", w0.tree, zero, [0.003], note="an all-zero family row"))
    cases.append(make_case_r("syn_base_invalid_lambda", w0.tree, zero, [0.0], note="lambda <= 0 -> +inf",
                           recon=False))
    w1 = workload(1, n_families=120, seed=4)
    cases.append(make_case_r("syn_gamma_24taxa_k4", w1.tree, w1.families, [0.002], model="gamma",
                           mult=w1.multipliers, probs=w1.cat_probs, note="config-1 shape, K=4 alpha=0.5"))
    probs8, mult8 = discrete_gamma(0.5, 8)
    cases.append(make_case_r("syn_gamma_24taxa_k8_small_cat", w1.tree, FamilySet(w1.families.ids[:40],
                                                                              w1.families.counts[:40]),
                           [0.003], model="gamma", mult=mult8, probs=probs8, note="K=8"))
    w2 = workload(2, n_families=400, seed=5)
    keep = w2.families.max_counts() <= 30
    f2 = FamilySet([i for i, k in zip(w2.families.ids, keep) if k][:80], w2.families.counts[keep][:80])
    err = "maxcnt: 200\ncntdiff: -1 0 1\n0 0 0.95 0.05\n1 0.05 0.9 0.05\n"
    cases.append(make_case_r("syn_multilambda_error_32taxa", w2.tree, f2, [0.0015, 0.006], lam_idx=w2.lambda_of_node,
                           err=err, note="config-2 shape (counts<=30), two lambdas + error model"))
    # a family whose likelihood underflows FP64 (alternating 0 / 50 counts)
    uf = FamilySet(["alt", "flat"], np.array([[0 if i % 2 else 50 for i in range(24)], [1] * 24], np.int32))
    cases.append(make_case_r("syn_base_underflow", w1.tree, uf, [0.001], S=110, R=75,
                           note="first family underflows to L = 0 in FP64 -> -lnL = +inf"))
    # non-binary tree (a polytomy)
    tp = parse_newick("((A:2,B:2,C:2):3,(D:4,E:4):1);")
    rng = np.random.default_rng(7)
    cnt = simulate_families(tp, 30, np.full(30, 0.01), rng.integers(1, 6, 30), seed=8)
    cases.append(make_case_r("syn_polytomy", tp, FamilySet([f"p{i}" for i in range(30)], cnt), [0.01],
                           note="three children at one node"))
    json.dump({"generator": "tests/golden/make_golden.py", "cases": cases},
              open(os.path.join(HERE, "ref_cases.json"), "w"), indent=1)

    mats = []
    for lam, tt, size in [(0.05, 5.0, 5), (0.006335, 68.7105, 12), (0.002, 13.4, 40), (0.0125, 3.333, 30),
                          (0.05, 25.0, 6), (0.0005, 150.0, 64)]:
        out = run(["matrix", repr(lam), repr(tt), str(size)])
        mats.append({"lambda": lam, "t": tt, "size": size, "hex": [ln.split() for ln in out.splitlines()]})
    gam = []
    for k, a in [(4, 0.5), (8, 0.5), (4, 1.7), (6, 0.37)]:
        rows = [ln.split() for ln in run(["gamma", str(k), repr(a)]).splitlines()]
        gam.append({"K": k, "alpha": a, "probs": [r[0] for r in rows], "multipliers": [r[1] for r in rows]})
    json.dump({"generator": "tests/golden/make_golden.py", "matrices": mats, "gamma": gam},
              open(os.path.join(HERE, "ref_matrices.json"), "w"))

    # -- p-values (compute_pvalues, seeded) -----------------------------------
    pvs = []
    w0p = workload(0, n_families=30, seed=3)
    pvs.append(make_pvalue_case("pv_base_12taxa", w0p.tree, w0p.families, [0.0025], n_sim=50, seed=7,
                                note="config-0 shape, global bounds, 50 simulations per root size"))
    pvs.append(make_pvalue_case("pv_two_lambdas_32taxa", w2.tree, FamilySet(f2.ids[:25], f2.counts[:25]),
                                [0.0015, 0.006], lam_idx=w2.lambda_of_node, n_sim=30, seed=11,
                                note="two lambdas (lambda tree), 30 simulations"))
    pvs.append(make_pvalue_case("pv_polytomy", tp, FamilySet([f"p{i}" for i in range(30)], cnt), [0.01],
                                n_sim=40, seed=5, note="a three-child node"))
    pvs.append(make_pvalue_case("pv_kat_small_bounds", parse_newick("(A:1,B:3):7;"),
                                FamilySet(["f1", "f2"], np.array([[3, 6], [1, 2]], np.int32)), [0.005],
                                n_sim=25, seed=3, S=10, R=8, note="explicit small bounds"))
    json.dump({"generator": "tests/golden/make_golden.py", "cases": pvs},
              open(os.path.join(HERE, "ref_pvalues.json"), "w"))

    # -- the simulator action (seeded) ------------------------------------------
    sims = []
    sims.append(make_sim_case("sim_base_12taxa_rootdist", w0p.tree, w0p.families, [0.0025], n=40, seed=5,
                              prior="rootdist:1=3,2=5,4=4,7=2", note="base model, root sizes from a rootdist"))
    sims.append(make_sim_case("sim_base_12taxa_uniform", w0p.tree, w0p.families, [0.004], n=20, seed=2,
                              prior="uniform:10", note="uniform prior: root size 0 included (50 failed attempts)"))
    sims.append(make_sim_case("sim_gamma_24taxa_k4", w1.tree, FamilySet(w1.families.ids[:30], w1.families.counts[:30]),
                              [0.002], n=30, seed=9, prior="rootdist:2=10,5=10,9=10", alpha=0.5, K=4,
                              note="gamma: one category drawn per family"))
    # the simulator refuses leaf sizes beyond the error model's rows
    # (error_model::get_max_family_size is the row count), so give it 61
    err_sim = "maxcnt: 60\ncntdiff: -1 0 1\n0 0 0.95 0.05\n" + "".join(
        f"{i} 0.05 0.9 0.05\n" for i in range(1, 61))
    sims.append(make_sim_case("sim_two_lambdas_error_32taxa", w2.tree, f2, [0.0015, 0.006], lam_idx=w2.lambda_of_node,
                              n=30, seed=13, prior="rootdist:1=10,3=10,6=10", err=err_sim,
                              note="two lambdas, error model at the leaves"))
    json.dump({"generator": "tests/golden/make_golden.py", "cases": sims},
              open(os.path.join(HERE, "ref_simulations.json"), "w"))

    # -- Nelder-Mead: analytic objectives and likelihood searches ------------
    analytic = []
    for fn, it, x0 in [("rosen", 300, [-1.2, 1.0]), ("wall", 300, [0.99, 0.5]), ("bowl", 300, [0.0, 0.0, 0.0]),
                       ("product", 5, [5.0, 3.0]), ("rosen", 40, [0.5, 0.5, 0.5, 0.5])]:
        r = parse_search(run(["nm", fn, str(it), ",".join(repr(x) for x in x0)]))
        analytic.append({"objective": fn, "max_iterations": it, "initial": x0, **r})
    searches = []
    searches.append(make_case("opt_lambda_base_12taxa", w0.tree, w0.families, [0.003], optimize="lambda",
                              initial=[0.003], note="lambda_optimizer, config-0 shape"))
    searches.append(make_case("opt_two_lambdas_base_32taxa", w2.tree, f2, [0.0015, 0.006], lam_idx=w2.lambda_of_node,
                              optimize="lambda", initial=[0.002, 0.004], note="two lambdas"))
    searches.append(make_case("opt_lambda_epsilon_32taxa", w2.tree, f2, [0.0015, 0.006], lam_idx=w2.lambda_of_node,
                              err=err, optimize="lambda_epsilon", initial=[0.0015, 0.006, 0.05],
                              note="lambda_epsilon_optimizer, one epsilon"))
    f1 = FamilySet(w1.families.ids[:60], w1.families.counts[:60])
    searches.append(make_case("opt_lambda_alpha_gamma_24taxa", w1.tree, f1, [0.002], model="gamma", alpha=0.5, K=4,
                              optimize="lambda_alpha", initial=[0.002, 0.5], note="gamma_lambda_optimizer, K=4"))
    searches.append(make_case("opt_alpha_gamma_24taxa", w1.tree, f1, [0.0025], model="gamma", alpha=0.5, K=4,
                              optimize="alpha", initial=[0.8], note="gamma_optimizer, lambda fixed"))
    json.dump({"generator": "tests/golden/make_golden.py", "analytic": analytic, "searches": searches},
              open(os.path.join(HERE, "ref_optimizer.json"), "w"), indent=1)


# -- the reference's own example inputs --------------------------------------
# Paths are relative to the reference checkout; tests/golden/stage_examples.py
# copies the same files into tests/golden/_refdata/ (git-ignored) for the GPU
# tests, which compare against the values written here.
EXAMPLES = [
    dict(name="mammals_base", tree="examples/mammals_tree.txt", families="examples/mammal_gene_families.txt",
         lambdas=[0.01], note="the mammals example at lambda 0.01: -lnL 210925.6422469711"),
    dict(name="primates_base", tree="Test_data/Primate_data/12Primates.tree",
         families="Test_data/Primate_data/12Primate_genefamilies.tab", lambdas=[0.00453],
         note="the Primates test data at lambda 0.00453: -lnL 159140.7143496017"),
    dict(name="mammals_error_model", tree="examples/mammals_tree.txt",
         families="examples/mammal_gene_families.txt", error="examples/errormodel_0.1.txt", lambdas=[0.01],
         note="the mammals example with its error-model file"),
    dict(name="mammals_two_lambdas", tree="examples/mammals_tree.txt",
         families="examples/mammal_gene_families.txt", lambda_tree="examples/chimphuman_separate_lambda.txt",
         lambdas=[0.01, 0.02], note="the chimp/human lambda tree"),
    dict(name="primates_rootdist", tree="Test_data/Primate_data/12Primates.tree",
         families="Test_data/Primate_data/12Primate_genefamilies.tab", rootdist="Test_data/Primate_data/Root_dist.txt",
         lambdas=[0.00453], note="the Primates root-size distribution as the prior"),
    dict(name="mammals_gamma_k4", tree="examples/mammals_tree.txt", families="examples/mammal_gene_families.txt",
         lambdas=[0.01], gamma=(4, 0.5), note="gamma K=4 alpha=0.5: a family underflows -> +inf"),
]


def reference_checkout():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    d = oracle.reference_dir()
    if d is None:
        raise SystemExit("set CAFE_REFERENCE to the reference checkout")
    return d


def rootdist_spec(path):
    pairs = []
    for ln in open(path):
        tok = ln.split()
        if len(tok) >= 2:
            pairs.append(f"{int(tok[0])}={int(tok[1])}")
    return "rootdist:" + ",".join(pairs)


def canonical_dump(text: str) -> str:
    """The harness's --dump-input lines with every hex float re-printed by
    Python (C's %a and float.hex differ in trailing zeros)."""
    out = []
    for ln in text.splitlines():
        tok = ln.split()
        if tok[0] == "node":
            tok[4] = float.fromhex(tok[4]).hex()
        elif tok[0] == "erow":
            tok[2:] = [float.fromhex(x).hex() for x in tok[2:]]
        out.append(" ".join(tok))
    return "\n".join(out) + "\n"


def examples_main():
    import hashlib
    ref = reference_checkout()
    meta, arrays = [], {}
    for ex in EXAMPLES:
        args = ["--tree", os.path.join(ref, ex["tree"]), "--families", os.path.join(ref, ex["families"]),
                "--lambdas", ",".join(repr(x) for x in ex["lambdas"]), "--exclude-zero-root", "--estimate-bounds"]
        if ex.get("error"):
            args += ["--error", os.path.join(ref, ex["error"])]
        if ex.get("lambda_tree"):
            args += ["--lambda-tree", os.path.join(ref, ex["lambda_tree"])]
        prior = rootdist_spec(os.path.join(ref, ex["rootdist"])) if ex.get("rootdist") else "uniform"
        args += ["--prior", prior]
        if ex.get("gamma"):
            args += ["--gamma-k", str(ex["gamma"][0]), "--gamma-alpha", repr(ex["gamma"][1])]
        dump = canonical_dump(run(args + ["--dump-input"]))
        out = parse_output(run(args))
        fam_ids = [ln.split()[1] for ln in dump.splitlines() if ln.startswith("gf ")]
        m = {k: v for k, v in ex.items()}
        m.update({"prior": prior, "S": out["S"], "R": out["R"], "total_hex": out["total_hex"],
                  "n_families": len(fam_ids), "parse_sha256": hashlib.sha256(dump.encode()).hexdigest()})
        if ex.get("gamma"):
            # per-family lnL of the gamma model: log of family_likelihood
            cats = out["cat"]
            fam = [np.log(float.fromhex(cats[i][0]["fam_lh"])) if i in cats else np.nan for i in fam_ids]
        else:
            fam = [float.fromhex(out["fam"][i]) for i in fam_ids]
        arrays[ex["name"] + "_fam_lnl"] = np.asarray(fam, dtype=np.float64)
        meta.append(m)
        print(ex["name"], m["n_families"], m["S"], m["R"], float.fromhex(m["total_hex"]))
    json.dump({"generator": "tests/golden/make_golden.py --examples", "cases": meta},
              open(os.path.join(HERE, "ref_examples.json"), "w"), indent=1)
    np.savez_compressed(os.path.join(HERE, "ref_examples.npz"), **arrays)


def configs_main():
    """Subsets of the larger benchmark shapes scored by the reference at its
    own global bounds: the two-lambda + error-model shape at S ~ 600 and
    the 48-taxon K = 8 gamma shape."""
    cases = []
    w2 = workload(2, n_families=50000, seed=0)
    mx = w2.families.max_counts()
    order = np.argsort(-mx, kind="stable")
    rng = np.random.default_rng(21)
    pick = np.concatenate([order[:6], rng.choice(order[6:], 34, replace=False)])
    pick.sort()
    f2 = FamilySet([w2.families.ids[i] for i in pick], np.ascontiguousarray(w2.families.counts[pick]))
    err = "maxcnt: 700\ncntdiff: -1 0 1\n0 0 0.95 0.05\n1 0.05 0.9 0.05\n"
    cases.append(make_case("cfg2_two_lambdas_error_S600", w2.tree, f2, [0.0015, 0.006], lam_idx=w2.lambda_of_node,
                           err=err, estimate_bounds=True,
                           note="config-2 shape at the reference's global bound: the 6 largest families of the "
                                "50,000 and 34 others"))
    w3 = workload(3, n_families=20000, seed=0)
    f3 = FamilySet(w3.families.ids[:300], np.ascontiguousarray(w3.families.counts[:300]))
    cases.append(make_case("cfg3_gamma_k8_48taxa_underflow", w3.tree, f3, [0.002], model="gamma",
                           mult=w3.multipliers, probs=w3.cat_probs, estimate_bounds=True,
                           note="config-3 shape: 48 taxa, K=8, alpha=0.5, the first 300 families; some "
                                "families underflow in the smallest category, so the reference returns +inf"))
    # 300 families whose every category is finite in the reference's
    # arithmetic (selected with the oracle, which is bit-exact with it)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from cafe5_gb300.families import global_bounds as gb
    S3, R3 = gb(w3.families)
    cand = np.ascontiguousarray(w3.families.counts[:4000])
    _, fam3, _ = oracle.score(oracle.TreeArrays.from_tree(w3.tree), cand, [0.002], model=1,
                              multipliers=w3.multipliers, cat_probs=w3.cat_probs,
                              prior=RootPrior.uniform(R3).vector(), S=S3, R=R3, dedupe=False)
    ok = np.nonzero(np.isfinite(fam3))[0]      # a failed family's lnL is NaN
    # the 300 finite families with the largest counts, in their input order
    ok = np.sort(ok[np.argsort(-cand[ok].max(axis=1), kind="stable")[:300]])
    f3f = FamilySet([w3.families.ids[i] for i in ok], np.ascontiguousarray(cand[ok]))
    cases.append(make_case("cfg3_gamma_k8_48taxa_finite", w3.tree, f3f, [0.002], model="gamma",
                           mult=w3.multipliers, probs=w3.cat_probs, estimate_bounds=True,
                           note="config-3 shape: 48 taxa, K=8, alpha=0.5 (get_gamma's multipliers); of the first "
                                "4,000 families, the 300 with the largest counts among those whose every category "
                                "is finite in FP64 (only 5 are: the smallest category underflows the others)"))
    for c in cases:
        print(c["name"], c["S"], c["R"], float.fromhex(c["expected"]["total_hex"]))
    json.dump({"generator": "tests/golden/make_golden.py --configs", "cases": cases},
              open(os.path.join(HERE, "ref_configs.json"), "w"))


if __name__ == "__main__":
    if "--examples" in sys.argv:
        examples_main()
    elif "--configs" in sys.argv:
        configs_main()
    else:
        main()
