"""Seeded synthetic inputs with the shapes of the benchmark workloads.

No public dataset is named for this path, so every workload is generated:

* `yule_tree(n_taxa, root_age, seed)`: pure-birth (Yule, rate 1) tree grown
  until it has n_taxa lineages, tips extended by one more waiting time, then
  rescaled so the root-to-tip distance is `root_age`; ultrametric, branch
  lengths rounded to 1e-6.
* `simulate_families(...)`: the linear birth-death process with
  lambda = mu along every branch. One lineage over time t leaves 0 copies
  with probability a = lambda t / (1 + lambda t) and c >= 1 copies with
  probability (1-a)^2 a^(c-1); s lineages are s independent copies, so the
  child count is Binomial(s, 1-a) survivors each carrying 1 + Geometric
  extra copies (the same single-lineage law as the reference's matrix row 1,
  src/probability.cpp:104-148 at s = 1).
* `workload(k)`: the five benchmark configurations.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from .families import FamilySet
from .inputs import ErrorModel, discrete_gamma
from .tree import Tree, parse_newick


def yule_tree(n_taxa: int, root_age: float, seed: int = 0) -> Tree:
    rng = np.random.default_rng(seed)
    t = Tree()
    root = t._new(-1)
    active = [t._new(root), t._new(root)]
    birth = {root: 0.0, active[0]: 0.0, active[1]: 0.0}
    now = 0.0
    while len(active) < n_taxa:
        now += rng.exponential(1.0 / len(active))
        i = int(rng.integers(len(active)))
        v = active.pop(i)
        t.branch_length[v] = now - birth[v]
        a, b = t._new(v), t._new(v)
        birth[a] = birth[b] = now
        active[i:i] = [a, b]
    now += rng.exponential(1.0 / len(active))
    for v in active:
        t.branch_length[v] = now - birth[v]
    scale = root_age / now
    for v in range(t.n_nodes):
        t.branch_length[v] = round(t.branch_length[v] * scale, 6) if t.parent[v] >= 0 else 0.0
    # make it exactly ultrametric after rounding: fix tip lengths
    for k, v in enumerate(active):
        t.name[v] = f"T{k:03d}"
    for v in active:
        d = t.depth(v) - t.branch_length[v]
        t.branch_length[v] = round(root_age - d, 6)
    # re-parse so numbering and interior names follow Newick order
    return parse_newick(t.to_newick())


def _bd_step(rng, s: np.ndarray, lam: np.ndarray, t: float) -> np.ndarray:
    a = lam * t / (1.0 + lam * t)
    surv = rng.binomial(s, 1.0 - a)
    extra = np.zeros_like(surv)
    m = surv > 0
    if np.any(m):
        # sum of `surv` Geometric(1-a) (support >= 1) = surv + NegBin(surv, 1-a)
        extra[m] = rng.negative_binomial(surv[m], 1.0 - a[m])
    return surv + extra


def simulate_families(tree: Tree, n_families: int, lam_per_family: np.ndarray, root_sizes: np.ndarray,
                      seed: int = 1, lambda_of_node: Optional[List[float]] = None) -> np.ndarray:
    """Counts [F, n_leaves] (int32) at the leaves; lambda_of_node scales a
    branch's rate (for multi-lambda trees) as a per-node factor."""
    rng = np.random.default_rng(seed)
    F = n_families
    size = np.zeros((tree.n_nodes, F), dtype=np.int64)
    size[tree.root] = root_sizes
    order = list(reversed(tree.reverse_level_order()))  # parents first
    for v in order:
        if v == tree.root:
            continue
        p = tree.parent[v]
        lam = lam_per_family if lambda_of_node is None else lam_per_family * lambda_of_node[v]
        size[v] = _bd_step(rng, size[p], np.broadcast_to(lam, (F,)).astype(np.float64), tree.branch_length[v])
    return np.ascontiguousarray(size[tree.leaves].T.astype(np.int32))


def _poisson_ge1(rng, mean: float, n: int) -> np.ndarray:
    out = rng.poisson(mean, n)
    bad = out < 1
    while np.any(bad):
        out[bad] = rng.poisson(mean, int(bad.sum()))
        bad = out < 1
    return out


@dataclass
class Workload:
    name: str
    tree: Tree
    families: FamilySet
    lambdas: List[float]
    lambda_of_node: List[int]
    K: int = 1
    alpha: float = 0.0
    cat_probs: List[float] = field(default_factory=lambda: [1.0])
    multipliers: List[float] = field(default_factory=lambda: [1.0])
    error: Optional[ErrorModel] = None
    true_lambda: float = 0.0
    description: str = ""


def _keep_nonzero(counts: np.ndarray) -> np.ndarray:
    return counts[counts.max(axis=1) > 0]


def workload(config: int, n_families: Optional[int] = None, seed: int = 0, gamma=None) -> Workload:
    """Synthetic stand-ins for the five benchmark configurations. `gamma(alpha,
    K)` -> (probabilities, multipliers) is get_gamma (the library's by
    default); a caller that must not load the library passes its own."""
    gamma = gamma or discrete_gamma
    if config == 0:
        tree = yule_tree(12, 100.0, seed)
        F = n_families or 1000
        rng = np.random.default_rng(seed + 1)
        root = _poisson_ge1(rng, 5.0, int(F * 1.3))
        c = simulate_families(tree, len(root), np.full(len(root), 0.0025), root, seed + 1)
        c = _keep_nonzero(c)[:F]
        fams = FamilySet([f"F{i:06d}" for i in range(len(c))], c)
        return Workload("config0_base_12taxa_1k", tree, fams, [0.0025], [0] * tree.n_nodes,
                        true_lambda=0.0025,
                        description="12-taxon Yule (root age 100), 1,000 families, root~Poisson(5)>=1, "
                                    "lambda=mu=0.0025, base model")
    if config == 1:
        tree = yule_tree(24, 150.0, seed)
        F = n_families or 10000
        probs, mult = gamma(0.5, 4)
        rng = np.random.default_rng(seed + 1)
        k = rng.integers(0, 4, F)
        lam = 0.002 * np.asarray(mult)[k]
        root = _poisson_ge1(rng, 8.0, F)
        c = simulate_families(tree, F, lam, root, seed + 2)
        fams = FamilySet([f"F{i:06d}" for i in range(F)], c)
        return Workload("config1_gamma_k4_24taxa_10k", tree, fams, [0.002], [0] * tree.n_nodes, K=4, alpha=0.5,
                        cat_probs=probs, multipliers=mult, true_lambda=0.002,
                        description="24-taxon Yule (root age 150), 10,000 families, per-family lambda = "
                                    "0.002 x gamma(alpha=0.5,K=4) multiplier, root~Poisson(8)>=1, gamma K=4")
    if config == 2:
        tree = yule_tree(32, 150.0, seed)
        F = n_families or 50000
        # one clade of 10 taxa gets lambda2: pick the internal node whose
        # leaf count is closest to 10
        lam_idx = [0] * tree.n_nodes
        best, best_d = None, 1 << 30
        for v in range(tree.n_nodes):
            if tree.is_leaf(v) or v == tree.root:
                continue
            n = len(tree._leaf_names_under(v))
            if abs(n - 10) < best_d:
                best, best_d = v, abs(n - 10)
        stack = [best]
        while stack:
            v = stack.pop()
            lam_idx[v] = 1
            stack.extend(tree.children[v])
        rng = np.random.default_rng(seed + 1)
        heavy = rng.random(F) < 0.05
        root = np.where(heavy, rng.geometric(0.02, F), rng.poisson(4.0, F))
        root = np.maximum(root, 1)
        factor = [4.0 if lam_idx[v] == 1 else 1.0 for v in range(tree.n_nodes)]
        c = simulate_families(tree, F, np.full(F, 0.0015), root, seed + 2, lambda_of_node=factor)
        # leaf errors: -1 / +1 each with probability eps
        eps = 0.05
        u = rng.random(c.shape)
        c = np.where(u < eps, c - 1, np.where(u > 1 - eps, c + 1, c))
        c = np.maximum(c, 0).astype(np.int32)
        fams = FamilySet([f"F{i:06d}" for i in range(F)], c)
        em = ErrorModel.symmetric(eps, int(c.max()))
        return Workload("config2_twolambda_err_32taxa_50k", tree, fams, [0.0015, 0.006], lam_idx, error=em,
                        true_lambda=0.0015,
                        description="32-taxon Yule, 10-taxon clade lambda2=0.006, rest lambda1=0.0015, "
                                    "error model eps=0.05, 50,000 families, root 95% Poisson(4) / 5% Geom(0.02)")
    if config == 3:
        tree = yule_tree(48, 200.0, seed)
        F = n_families or 20000
        probs, mult = gamma(0.5, 8)
        rng = np.random.default_rng(seed + 1)
        k = rng.integers(0, 8, F)
        lam = 0.002 * np.asarray(mult)[k]
        root = _poisson_ge1(rng, 5.0, F)
        c = simulate_families(tree, F, lam, root, seed + 2)
        fams = FamilySet([f"F{i:06d}" for i in range(F)], c)
        return Workload("config3_batched_k8_48taxa_20k", tree, fams, [0.002], [0] * tree.n_nodes, K=8, alpha=0.5,
                        cat_probs=probs, multipliers=mult, true_lambda=0.002,
                        description="48-taxon Yule (root age 200), 20,000 families, gamma K=8, "
                                    "64 candidate (lambda, alpha) vectors per round")
    raise ValueError(f"unknown config {config}")
