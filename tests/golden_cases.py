"""Loads the committed golden fixtures into ready-to-score inputs (test helper)."""
from __future__ import annotations

import json
import os
from dataclasses import dataclass
from typing import List, Optional

import numpy as np

from cafe5_gb300.inputs import ErrorModel, RootPrior
from cafe5_gb300.tree import Tree, lambda_index_of_nodes, parse_newick

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def load_json(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def hexf(x):
    return float.fromhex(x) if x not in (None, "inf", "-inf", "nan") else float(x) if x else None


@dataclass
class Case:
    name: str
    tree: Tree
    lambda_of_node: List[int]
    lambda_kind: int
    counts: np.ndarray
    lambdas: List[float]
    model: int
    multipliers: List[float]
    cat_probs: List[float]
    prior: np.ndarray
    err_rows: Optional[np.ndarray]
    S: int
    R: int
    total: float
    fam_lnl: List[Optional[float]]
    cat: Optional[list]
    recon: Optional[dict] = None


def _ints(rows):
    return np.array([[int(x) for x in r.split()] for r in rows], dtype=np.int32)


def _hexes(rows):
    return np.array([[np.nan if x == "NA" else float.fromhex(x) for x in r.split()] for r in rows])


def recon_from_json(r) -> Optional[dict]:
    """The reference's reconstruction of a case: node_count[F][n],
    branch_prob[F][n] (NaN at the root), and for the gamma model
    cat_state[K][F][n] (-1 at leaves) and mean[F][n] (NaN at leaves)."""
    if r is None:
        return None
    out = {"node_count": _ints(r["node_count"]), "branch_prob": _hexes(r["bp_hex"]),
           "cat_state": None, "mean": None}
    if r["cat_state"] is not None:
        out["cat_state"] = np.stack([_ints(per_fam) for per_fam in r["cat_state"]]).transpose(1, 0, 2).copy()
        out["mean"] = _hexes(r["mean_hex"])
    return out


def prior_from_spec(spec: str, R: int) -> RootPrior:
    if spec == "uniform":
        return RootPrior.uniform(R)
    if spec.startswith("uniform:"):
        return RootPrior.uniform(int(spec[8:]))
    if spec.startswith("poisson:"):
        return RootPrior.poisson(float(spec[8:]), R)
    if spec.startswith("rootdist:"):
        rd = {}
        for tok in spec[9:].split(","):
            a, b = tok.split("=")
            rd[int(a)] = int(b)
        return RootPrior.from_rootdist(rd)
    raise ValueError(spec)


def case_from_json(c) -> Case:
    tree = parse_newick(c["newick"])
    assert tree.leaf_names == c["taxa"]
    lam_idx = [0] * tree.n_nodes
    kind = 0
    if c["lambda_newick"]:
        lam_idx = lambda_index_of_nodes(tree, parse_newick(c["lambda_newick"], lambda_tree=True))
        kind = 1
    err = None
    if c["error_model"]:
        err = ErrorModel.parse(c["error_model"]).table()
    prior = prior_from_spec(c["prior"], c["R"]).vector()
    model = 1 if c["model"] == "gamma" else 0
    cat = None
    if c["expected"]["cat"] is not None:
        cat = c["expected"]["cat"]
    return Case(
        name=c["name"], tree=tree, lambda_of_node=lam_idx, lambda_kind=kind,
        counts=np.asarray(c["counts"], dtype=np.int32).reshape(len(c["ids"]), len(c["taxa"])),
        lambdas=[hexf(x) for x in c["lambdas"]], model=model,
        multipliers=[hexf(x) for x in c["multipliers"]] if c["multipliers"] else [1.0],
        cat_probs=[hexf(x) for x in c["cat_probs"]] if c["cat_probs"] else [1.0],
        prior=prior, err_rows=err, S=c["S"], R=c["R"],
        total=float.fromhex(c["expected"]["total_hex"]) if "x" in c["expected"]["total_hex"]
        else float(c["expected"]["total_hex"]),
        fam_lnl=[hexf(x) if x is not None else None for x in c["expected"]["fam_lnl_hex"]],
        cat=cat, recon=recon_from_json(c.get("recon")))


def load_cases(name: str = "ref_cases.json") -> List[Case]:
    """ref_cases.json: the known-answer and small synthetic cases;
    ref_configs.json: subsets of the larger benchmark shapes."""
    return [case_from_json(c) for c in load_json(name)["cases"]]


def load_searches():
    """(raw json, Case) per likelihood search of ref_optimizer.json."""
    return [(c, case_from_json(c)) for c in load_json("ref_optimizer.json")["searches"]]


@dataclass
class PvalueCase:
    name: str
    tree: Tree
    lambda_of_node: List[int]
    lambda_kind: int
    counts: np.ndarray
    lambdas: List[float]
    S: int
    R: int
    n_sim: int
    seed: int
    conditional: np.ndarray    # [R][n_sim], sorted
    pvalues: np.ndarray        # [F]


def load_pvalue_cases() -> List[PvalueCase]:
    out = []
    for c in load_json("ref_pvalues.json")["cases"]:
        tree = parse_newick(c["newick"])
        lam_idx, kind = [0] * tree.n_nodes, 0
        if c["lambda_newick"]:
            lam_idx = lambda_index_of_nodes(tree, parse_newick(c["lambda_newick"], lambda_tree=True))
            kind = 1
        out.append(PvalueCase(
            name=c["name"], tree=tree, lambda_of_node=lam_idx, lambda_kind=kind,
            counts=np.asarray(c["counts"], dtype=np.int32).reshape(len(c["ids"]), len(c["taxa"])),
            lambdas=[hexf(x) for x in c["lambdas"]], S=c["S"], R=c["R"], n_sim=c["n_sim"], seed=c["seed"],
            conditional=_hexes(c["conditional_hex"]), pvalues=np.array([hexf(x) for x in c["pvalue_hex"]])))
    return out


@dataclass
class SimulationCase:
    name: str
    tree: Tree
    lambda_of_node: List[int]
    lambda_kind: int
    lambdas: List[float]
    S: int
    R: int
    seed: int
    roots: np.ndarray          # [n]
    err: Optional["ErrorModel"]
    alpha: Optional[float]
    K: Optional[int]
    lambda_used: np.ndarray    # [n]
    sizes: np.ndarray          # [n][n_nodes], prefix order


def load_simulation_cases() -> List[SimulationCase]:
    out = []
    for c in load_json("ref_simulations.json")["cases"]:
        tree = parse_newick(c["newick"])
        lam_idx, kind = [0] * tree.n_nodes, 0
        if c["lambda_newick"]:
            lam_idx = lambda_index_of_nodes(tree, parse_newick(c["lambda_newick"], lambda_tree=True))
            kind = 1
        out.append(SimulationCase(
            name=c["name"], tree=tree, lambda_of_node=lam_idx, lambda_kind=kind,
            lambdas=[hexf(x) for x in c["lambdas"]], S=c["S"], R=c["R"], seed=c["seed"],
            roots=np.asarray(c["roots"], dtype=np.int32),
            err=ErrorModel.parse(c["error_model"]) if c["error_model"] else None, alpha=c["alpha"], K=c["K"],
            lambda_used=np.array([hexf(x) for x in c["lambda_hex"]]), sizes=_ints(c["sizes"])))
    return out


# ---- the reference's example data (tests/golden/ref_examples.json) ----------

REFDATA = os.path.join(GOLDEN, "_refdata")


def example_cases():
    return load_json("ref_examples.json")["cases"]


def example_path(rel: str) -> Optional[str]:
    """A staged example input (tests/golden/stage_examples.py), else the file
    in the reference checkout named by CAFE_REFERENCE; None if neither."""
    p = os.path.join(REFDATA, rel)
    if os.path.exists(p):
        return p
    ref = os.environ.get("CAFE_REFERENCE")
    if ref and os.path.exists(os.path.join(ref, rel)):
        return os.path.join(ref, rel)
    return None


def example_available(c) -> bool:
    return all(example_path(c[k]) for k in ("tree", "families", "error", "lambda_tree", "rootdist") if c.get(k))


def read_example(c):
    """(tree, all families read, families after the zero-root filter, lambda
    tree or None, ErrorModel or None, RootPrior) through this package's
    readers, as the estimate action reads them."""
    from cafe5_gb300.families import exclude_zero_root_families, global_bounds, read_families
    tree = parse_newick(open(example_path(c["tree"])).read())
    fams = read_families(example_path(c["families"]), tree)
    kept = exclude_zero_root_families(fams, tree)
    ltree = parse_newick(open(example_path(c["lambda_tree"])).read(), lambda_tree=True) if c.get("lambda_tree") else None
    em = ErrorModel.parse(open(example_path(c["error"])).read()) if c.get("error") else None
    S, R = global_bounds(fams)
    if c.get("rootdist"):
        rd = {}
        for ln in open(example_path(c["rootdist"])):
            tok = ln.split()
            if len(tok) >= 2:
                rd[int(tok[0])] = int(tok[1])
        prior = RootPrior.from_rootdist(rd)
    else:
        prior = RootPrior.uniform(R)
    return tree, fams, kept, ltree, em, prior, S, R


def canonical_input_text(tree: Tree, kept, S: int, R: int, ltree=None, em=None) -> str:
    """The same lines the reference harness's --dump-input prints (nodes in
    prefix order with parent and branch length, every kept family's leaf
    counts in that order, the lambda index of every node, the error model's
    rows, the bounds), floats as Python hex."""
    out = []
    for v in range(tree.n_nodes):
        out.append(f"node {v} {tree.name[v]} {tree.parent[v]} {float(tree.branch_length[v]).hex()}")
    out.append(f"families {kept.n_families}")
    for fid, row in zip(kept.ids, kept.counts):
        out.append("gf " + fid + "".join(f" {int(x)}" for x in row))
    if ltree is not None:
        by_name = {ltree.name[v]: ltree.lambda_index[v] - 1 for v in range(ltree.n_nodes)}
        for v in range(tree.n_nodes):
            out.append(f"lambda_index {tree.name[v]} {by_name.get(tree.name[v], 0)}")
    if em is not None:
        for n, row in enumerate(em.rows):
            out.append(f"erow {n}" + "".join(" " + float(x).hex() for x in row))
    out.append(f"bounds {S} {R}")
    return "\n".join(out) + "\n"
