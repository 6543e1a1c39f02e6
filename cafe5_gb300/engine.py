"""Python mirror of the reference's likelihood API over the C ABI.

Same names and argument meaning as the CAFE5 classes on the hot path:

* `MatrixCache`      matrix_cache (src/matrix_cache.h:70-96)
* `SingleLambda`, `MultipleLambda`  lambda (src/lambda.h:21-100)
* `BaseModel`        base_model::infer_family_likelihoods (src/base_model.cpp:53-100)
* `GammaModel`       gamma_model (src/gamma_core.h, src/gamma_core.cpp:168-237)
* `LambdaOptimizerScorer`, `GammaLambdaOptimizerScorer`, `LambdaEpsilonOptimizerScorer`
                     inference_optimizer_scorer and subclasses
                     (src/optimizer_scorer.cpp:22-180): NaN scores become +inf.

All arithmetic runs in libcafe_gb300.so on the GPU; this module only moves
arguments and results.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from . import _lib
from .families import FamilySet
from .inputs import ErrorModel, RootPrior, discrete_gamma
from .tree import Tree, lambda_index_of_nodes

PREC = {"fp64_ref": _lib.PREC_FP64_REF, "fp64_binned": _lib.PREC_FP64_BINNED,
        "mixed_tf32x3": _lib.PREC_MIXED_TF32X3}


def _p(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data


@dataclass
class Reconstruction:
    """cafe_reconstruct output. node_count[F][n] is what
    reconstruction::get_node_count reports (leaves: observed counts);
    category_state[K][F][n] the Pupko state of each category; root_max[K][F]
    the largest root likelihood (0 = the reference's failed reconstruction)."""
    node_count: np.ndarray
    node_mean: np.ndarray
    category_state: np.ndarray
    root_max: np.ndarray
    n_failed: int
    device_ms: float


@dataclass
class ScoreResult:
    total: float
    family_lnl: np.ndarray
    category_lnl: Optional[np.ndarray]
    status: int
    n_failed: int
    n_fallback: int
    device_ms: float


class Context:
    """One device context: trees, family sets, prior, error model and the
    device-resident matrix cache."""

    def __init__(self, device: int = 0, n_streams: int = 4, matrix_cache_bytes: int = 0):
        self.lib = _lib.load()
        cfg = _lib.Config(device, matrix_cache_bytes, n_streams, 0)
        h = C.c_void_p()
        rc = self.lib.cafe_ctx_create(C.byref(cfg), C.byref(h))
        if rc:
            raise _lib.CafeError(rc, "cafe_ctx_create failed (is a CUDA GPU visible?)")
        self.h = h
        self._tree_leaves = {}
        self._tree_nodes = {}
        self._set_shape = {}

    def close(self):
        if self.h:
            self.lib.cafe_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc:
            raise _lib.CafeError(rc, self.lib.cafe_last_error(self.h).decode())

    # ---- inputs -----------------------------------------------------------
    def upload_tree(self, tree: Tree, lambda_of_node: Optional[Sequence[int]] = None) -> int:
        a = tree.arrays(list(lambda_of_node) if lambda_of_node is not None else None)
        tid = C.c_int()
        self._check(self.lib.cafe_tree_upload(self.h, tree.n_nodes, _p(a["parent"]), _p(a["branch_length"]),
                                              _p(a["lambda_index"]), C.byref(tid)))
        self._tree_leaves[tid.value] = len(tree.leaves)
        self._tree_nodes[tid.value] = tree.n_nodes
        return tid.value

    def upload_families(self, tree_id: int, counts: np.ndarray) -> int:
        counts = np.ascontiguousarray(counts, dtype=np.int32)
        sid = C.c_int()
        self._check(self.lib.cafe_families_upload(self.h, tree_id, _p(counts), counts.shape[0], counts.shape[1],
                                                  C.byref(sid)))
        self._set_shape[sid.value] = counts.shape
        return sid.value

    def update_families(self, set_id: int, counts: np.ndarray):
        counts = np.ascontiguousarray(counts, dtype=np.int32)
        assert counts.shape == self._set_shape[set_id]
        self._check(self.lib.cafe_families_update(self.h, set_id, _p(counts)))

    def free_families(self, set_id: int):
        self._check(self.lib.cafe_families_free(self.h, set_id))
        self._set_shape.pop(set_id, None)

    def set_prior(self, prior: np.ndarray):
        prior = np.ascontiguousarray(prior, dtype=np.float64)
        self._check(self.lib.cafe_prior_set(self.h, _p(prior), len(prior)))

    def set_error_model(self, table: Optional[np.ndarray]):
        if table is None:
            self._check(self.lib.cafe_error_model_set(self.h, None, 0, 0))
            return
        t = np.ascontiguousarray(table, dtype=np.float64)
        self._check(self.lib.cafe_error_model_set(self.h, _p(t), t.shape[0], t.shape[1]))

    # ---- matrix cache -------------------------------------------------------
    def matrices_build(self, lambdas, branch_lengths, size: int):
        l = np.ascontiguousarray(lambdas, dtype=np.float64)
        t = np.ascontiguousarray(branch_lengths, dtype=np.float64)
        self._check(self.lib.cafe_matrices_build(self.h, _p(l), len(l), _p(t), len(t), size))

    def matrix_get(self, lam: float, t: float, size: int) -> np.ndarray:
        out = np.zeros((size, size))
        self._check(self.lib.cafe_matrix_get(self.h, lam, t, size, _p(out)))
        return out

    def cache_size(self) -> int:
        n = C.c_int64()
        self._check(self.lib.cafe_matrix_cache_size(self.h, C.byref(n)))
        return n.value

    def cache_clear(self):
        self._check(self.lib.cafe_matrix_cache_clear(self.h))

    # ---- scoring ------------------------------------------------------------
    def make_request(self, tree_id, set_id, lambdas, *, model=0, lambda_kind=0, multipliers=(1.0,),
                     cat_probs=(1.0,), use_error_model=False, S=0, R=0, precision="fp64_ref", dedupe=False):
        keep = {"lam": np.ascontiguousarray(lambdas, dtype=np.float64),
                "mult": np.ascontiguousarray(multipliers, dtype=np.float64),
                "prob": np.ascontiguousarray(cat_probs, dtype=np.float64)}
        req = _lib.Request(tree_id, set_id, model, lambda_kind, len(keep["lam"]), _p(keep["lam"]),
                           len(keep["mult"]) if model == _lib.MODEL_GAMMA else 1, _p(keep["mult"]), _p(keep["prob"]),
                           1 if use_error_model else 0, int(S), int(R),
                           PREC[precision] if isinstance(precision, str) else int(precision), 1 if dedupe else 0)
        return req, keep

    def score(self, tree_id, set_id, lambdas, *, want_categories=False, **kw) -> ScoreResult:
        req, keep = self.make_request(tree_id, set_id, lambdas, **kw)
        F = self._set_shape.get(set_id, (0,))[0]     # unknown ids are reported by the library
        K = req.n_categories
        fam = np.zeros(F)
        cat = np.zeros((F, K)) if want_categories else None
        res = _lib.Result(_p(fam), _p(cat), 0.0, 0, 0, 0, 0.0)
        self._check(self.lib.cafe_score(self.h, C.byref(req), C.byref(res)))
        return ScoreResult(res.total_neg_lnl, fam, cat, res.status, res.n_failed, res.n_fallback, res.device_ms)

    def score_batch(self, tree_id, set_id, candidates, *, want_categories=False, **kw) -> List[ScoreResult]:
        """cafe_score_batch: candidates is a sequence of dicts with `lambdas`
        (and for the gamma model `multipliers`, `cat_probs`); every other
        request field is shared (keyword arguments as for score())."""
        arr, keep = self._batch_requests(tree_id, set_id, candidates, kw)
        reqs = list(arr)
        n = len(reqs)
        F = self._set_shape.get(set_id, (0,))[0]
        fams = [np.zeros(F) for _ in range(n)]
        cats = [np.zeros((F, r.n_categories)) if want_categories else None for r in reqs]
        res = (_lib.Result * n)(*[_lib.Result(_p(fams[i]), _p(cats[i]), 0.0, 0, 0, 0, 0.0) for i in range(n)])
        self._check(self.lib.cafe_score_batch(self.h, C.cast(arr, C.c_void_p), n, C.cast(res, C.c_void_p)))
        return [ScoreResult(res[i].total_neg_lnl, fams[i], cats[i], res[i].status, res[i].n_failed, res[i].n_fallback,
                            res[i].device_ms) for i in range(n)]

    def _batch_requests(self, tree_id, set_id, candidates, kw):
        reqs, keep = [], []
        for cand in candidates:
            ck = dict(kw)
            for key in ("multipliers", "cat_probs"):
                if key in cand:
                    ck[key] = cand[key]
            r, k = self.make_request(tree_id, set_id, cand["lambdas"], **ck)
            reqs.append(r)
            keep.append(k)
        return (_lib.Request * len(reqs))(*reqs), keep

    def autotune(self, tree_id, set_id, candidates, reps: int = 3, **kw) -> List[dict]:
        """cafe_autotune: pick the tensor-core launch shape of every S-bin by
        timing this batch (precision mixed_tf32x3)."""
        kw.setdefault("precision", "mixed_tf32x3")
        arr, keep = self._batch_requests(tree_id, set_id, candidates, kw)
        out = (_lib.TuneResult * 16)()
        n = C.c_int()
        self._check(self.lib.cafe_autotune(self.h, C.cast(arr, C.c_void_p), len(arr), reps, C.cast(out, C.c_void_p),
                                           16, C.byref(n)))
        return [{"width": out[i].width, "ctas_per_sm": out[i].ctas_per_sm, "stages": out[i].stages, "ms": out[i].ms}
                for i in range(n.value)]

    def score_batch_device(self, tree_id, set_id, candidates, d_family_lnl=0, d_total=0, stream=0, **kw):
        """cafe_score_batch_device: d_family_lnl [n][F], d_total [n] (device pointers)."""
        arr, keep = self._batch_requests(tree_id, set_id, candidates, kw)
        self._check(self.lib.cafe_score_batch_device(self.h, C.cast(arr, C.c_void_p), len(arr), d_family_lnl or None,
                                                     d_total or None, stream or None))

    def score_device(self, tree_id, set_id, lambdas, d_family_lnl=0, d_total=0, stream=0, **kw):
        req, keep = self.make_request(tree_id, set_id, lambdas, **kw)
        self._check(self.lib.cafe_score_device(self.h, C.byref(req), d_family_lnl or None, d_total or None,
                                               stream or None))

    def submit(self, tree_id, set_id, lambdas, **kw):
        """Queue a request for the serving loop; returns a handle for poll()."""
        want_cat = kw.pop("want_categories", False)
        req, keep = self.make_request(tree_id, set_id, lambdas, **kw)
        F = self._set_shape[set_id][0]
        fam = np.zeros(F)
        cat = np.zeros((F, req.n_categories)) if want_cat else None
        res = _lib.Result(_p(fam), _p(cat), 0.0, 0, 0, 0, 0.0)
        t = C.c_uint64()
        self._check(self.lib.cafe_submit(self.h, C.byref(req), C.byref(res), C.byref(t)))
        return {"ticket": t.value, "res": res, "fam": fam, "cat": cat, "keep": keep}

    def poll(self, handle, wait_ms: int = -1) -> Optional[ScoreResult]:
        rc = self.lib.cafe_poll(self.h, handle["ticket"], wait_ms)
        if rc == 8:
            return None
        self._check(rc)
        r = handle["res"]
        return ScoreResult(r.total_neg_lnl, handle["fam"], handle["cat"], r.status, r.n_failed, r.n_fallback,
                           r.device_ms)

    # ---- ancestral reconstruction -------------------------------------------
    def reconstruct(self, tree_id, set_id, lambdas, *, S: int, R: int, model=0, lambda_kind=0,
                    multipliers=(1.0,), cat_probs=(1.0,), exhaustive: bool = False) -> Reconstruction:
        """cafe_reconstruct: Pupko joint reconstruction of every family
        (one pass per gamma category) with states 0..S and root sizes
        1..min(S, R)."""
        req, keep = self.make_request(tree_id, set_id, lambdas, model=model, lambda_kind=lambda_kind,
                                      multipliers=multipliers, cat_probs=cat_probs, S=S, R=R)
        F, _ = self._set_shape.get(set_id, (0, 0))
        n = self._tree_nodes.get(tree_id, 0)
        K = req.n_categories
        cnt = np.zeros((F, n), np.int32)
        mean = np.zeros((F, n))
        st = np.zeros((K, F, n), np.int32)
        rmax = np.zeros((K, F))
        out = _lib.Reconstruction(_p(cnt), _p(mean), _p(st), _p(rmax), 1 if exhaustive else 0, 0, 0.0)
        self._check(self.lib.cafe_reconstruct(self.h, C.byref(req), C.byref(out)))
        return Reconstruction(cnt, mean, st, rmax, out.n_failed, out.device_ms)

    def branch_probabilities(self, tree_id, set_id, lambdas, node_count: np.ndarray, *, S: int, R: int,
                             lambda_kind=0) -> np.ndarray:
        """cafe_branch_probabilities: compute_viterbi_sum of every family and
        node ([F][n], NaN at the root)."""
        req, keep = self.make_request(tree_id, set_id, lambdas, lambda_kind=lambda_kind, S=S, R=R)
        nc = np.ascontiguousarray(node_count, dtype=np.int32)
        out = np.zeros(nc.shape)
        self._check(self.lib.cafe_branch_probabilities(self.h, C.byref(req), _p(nc), _p(out)))
        return out

    def pvalues(self, tree_id, set_id, lambdas, *, S: int, R: int, n_simulations: int = 1000, seed: int = 10,
                lambda_kind=0, device_sampling: bool = False) -> dict:
        """cafe_pvalues (compute_pvalues): per-family p-values, the sorted
        conditional distributions [R][n_simulations] and the observed root
        vectors [F][R]. device_sampling draws the simulated families on the
        GPU (not the reference's random stream: equal in distribution)."""
        req, keep = self.make_request(tree_id, set_id, lambdas, lambda_kind=lambda_kind, S=S, R=R)
        F, _ = self._set_shape.get(set_id, (0, 0))
        pv = np.zeros(F)
        cd = np.zeros((R, n_simulations))
        rl = np.zeros((F, R))
        out = _lib.PvaluesOut(n_simulations, seed & 0xFFFFFFFF, _p(pv), _p(cd), _p(rl), 0.0, 0.0,
                              1 if device_sampling else 0)
        self._check(self.lib.cafe_pvalues(self.h, C.byref(req), C.byref(out)))
        return {"pvalues": pv, "conditional": cd, "root_likelihood": rl, "device_ms": out.device_ms,
                "host_ms": out.host_ms}

    def simulate(self, tree_id, set_id, lambdas, root_sizes, *, S: int, R: int, seed: int = 10, model=0,
                 lambda_kind=0, multipliers=(1.0,), cat_probs=(1.0,), use_error_model=False):
        """cafe_simulate (the simulator action): (sizes[n][n_nodes], lambda[n])."""
        req, keep = self.make_request(tree_id, set_id, lambdas, model=model, lambda_kind=lambda_kind,
                                      multipliers=multipliers, cat_probs=cat_probs, use_error_model=use_error_model,
                                      S=S, R=R)
        roots = np.ascontiguousarray(root_sizes, dtype=np.int32)
        n_nodes = self._tree_nodes.get(tree_id, 0)
        sizes = np.zeros((len(roots), n_nodes), np.int32)
        lam = np.zeros(len(roots))
        io = _lib.Simulation(len(roots), _p(roots), seed & 0xFFFFFFFF, _p(sizes), _p(lam))
        self._check(self.lib.cafe_simulate(self.h, C.byref(req), C.byref(io)))
        return sizes, lam

    def debug_set(self, knob: int, value: int):
        """Test hooks (cafe_debug_set); see include/cafe_gb300.h."""
        self._check(self.lib.cafe_debug_set(self.h, int(knob), int(value)))

    def profile(self, enable: bool = True):
        self._check(self.lib.cafe_profile_enable(self.h, 1 if enable else 0))

    def profile_read(self) -> dict:
        t = _lib.Timings()
        self._check(self.lib.cafe_profile_read(self.h, C.byref(t)))
        return {k: getattr(t, k) for k, _ in _lib.Timings._fields_}

    def serving_stats(self):
        n = C.c_int64()
        p50 = C.c_double()
        p99 = C.c_double()
        inf = C.c_int()
        self._check(self.lib.cafe_serving_stats(self.h, C.byref(n), C.byref(p50), C.byref(p99), C.byref(inf)))
        si = _lib.ServingInfo()
        self._check(self.lib.cafe_serving_counters(self.h, C.byref(si)))
        return {"completed": n.value, "p50_ms": p50.value, "p99_ms": p99.value, "in_flight": inf.value,
                "batches": si.batches, "merged": si.merged, "retried": si.retried, "enqueue_ms": si.enqueue_ms,
                "wait_ms": si.wait_ms, "device_ms": si.device_ms, "overlap_ms": si.overlap_ms}


_default_ctx: Optional[Context] = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context()
    return _default_ctx


# ---------------------------------------------------------------- reference mirror

class MatrixCache:
    """matrix_cache: precalculate_matrices / get_matrix / get_cache_size /
    is_saturated, backed by the device-resident cache."""

    def __init__(self, matrix_size: int, ctx: Optional[Context] = None):
        self.ctx = ctx or default_context()
        self.size = matrix_size
        self._keys = set()

    def precalculate_matrices(self, lambdas: Sequence[float], branch_lengths: Sequence[float]):
        self.ctx.matrices_build(list(lambdas), list(branch_lengths), self.size)
        for l in lambdas:
            for t in branch_lengths:
                self._keys.add((int(l * 1000000000), int(t * 1000)))

    def get_matrix(self, branch_length: float, lam: float) -> np.ndarray:
        return self.ctx.matrix_get(lam, branch_length, self.size)

    def get_cache_size(self) -> int:
        return len(self._keys)

    def get_matrix_size(self) -> int:
        return self.size

    @staticmethod
    def is_saturated(branch_length: float, lam: float) -> bool:
        return bool(_lib.load().cafe_is_saturated(branch_length, lam))


class SingleLambda:
    def __init__(self, lam: float):
        self.values = [float(lam)]
        self.kind = _lib.LAMBDA_SINGLE

    def multiply(self, factor):
        return SingleLambda(self.values[0] * factor)

    def update(self, values):
        self.values = [float(values[0])]

    def count(self):
        return 1

    def is_valid(self):
        return self.values[0] > 0


class MultipleLambda:
    def __init__(self, lambda_tree: Tree, lambdas: Sequence[float]):
        self.lambda_tree = lambda_tree
        self.values = [float(x) for x in lambdas]
        self.kind = _lib.LAMBDA_MULTIPLE

    def multiply(self, factor):
        return MultipleLambda(self.lambda_tree, [v * factor for v in self.values])

    def update(self, values):
        self.values = [float(v) for v in values[:len(self.values)]]

    def count(self):
        return len(self.values)

    def is_valid(self):
        return all(v >= 0 for v in self.values)


class BaseModel:
    """base_model over the GPU path. `precision` selects fp64_ref (the
    reference's global bounds, unscaled), fp64_binned or mixed_tf32x3."""

    def __init__(self, lam, tree: Tree, families: FamilySet, max_family_size: int, max_root_family_size: int,
                 error_model: Optional[ErrorModel] = None, precision: str = "fp64_ref", dedupe: bool = True,
                 ctx: Optional[Context] = None):
        self.ctx = ctx or default_context()
        self.lam = lam
        self.tree = tree
        self.families = families
        self.max_family_size = max_family_size
        self.max_root_family_size = max_root_family_size
        self.error_model = error_model
        self.precision = precision
        self.dedupe = dedupe
        lam_idx = lambda_index_of_nodes(tree, lam.lambda_tree) if isinstance(lam, MultipleLambda) else None
        self.tree_id = self.ctx.upload_tree(tree, lam_idx)
        self.set_id = self.ctx.upload_families(self.tree_id, families.counts)
        self.results: Optional[np.ndarray] = None
        self.category_results: Optional[np.ndarray] = None
        self.last: Optional[ScoreResult] = None

    def _common(self, prior: RootPrior):
        n = max(self.max_root_family_size, 1) + 8
        self.ctx.set_prior(prior.vector(max(n, len(prior.vector()))))
        self.ctx.set_error_model(self.error_model.table() if self.error_model else None)

    def _kw(self):
        ref = self.precision == "fp64_ref"
        return dict(use_error_model=self.error_model is not None, S=self.max_family_size if ref else 0,
                    R=self.max_root_family_size if ref else 0, precision=self.precision)

    def _score_kw(self, lam):
        return dict(model=_lib.MODEL_BASE, lambda_kind=lam.kind, dedupe=self.dedupe, **self._kw())

    def reconstruct_ancestral_states(self, prior: RootPrior, lam=None, exhaustive: bool = False) -> Reconstruction:
        """base_model::reconstruct_ancestral_states (src/base_model.cpp:133-170)."""
        lam = lam or self.lam
        self._common(prior)
        return self.ctx.reconstruct(self.tree_id, self.set_id, lam.values, S=self.max_family_size,
                                    R=self.max_root_family_size, lambda_kind=lam.kind, **self._recon_kw())

    def _recon_kw(self):
        return dict(model=_lib.MODEL_BASE)

    def branch_probabilities(self, rec: Reconstruction, lam=None) -> np.ndarray:
        """compute_viterbi_sum for every family and node (the estimate action
        applies it to families below the p-value threshold,
        src/execute.cpp:177-185); uses the model's own lambdas."""
        lam = lam or self.lam
        return self.ctx.branch_probabilities(self.tree_id, self.set_id, lam.values, rec.node_count,
                                             S=self.max_family_size, R=self.max_root_family_size,
                                             lambda_kind=lam.kind)

    def compute_pvalues(self, n_simulations: int = 1000, seed: int = 10, lam=None) -> np.ndarray:
        """compute_pvalues (src/probability.cpp:530-570) at the model's own
        lambdas, as the estimate action calls it (src/execute.cpp:166-171);
        `seed` seeds the simulation stream (the reference's randomizer_engine)."""
        lam = lam or self.lam
        return self.ctx.pvalues(self.tree_id, self.set_id, lam.values, S=self.max_family_size,
                                R=self.max_root_family_size, n_simulations=n_simulations, seed=seed,
                                lambda_kind=lam.kind)["pvalues"]

    def infer_family_likelihoods(self, prior: RootPrior, lam=None) -> float:
        lam = lam or self.lam
        self._common(prior)
        r = self.ctx.score(self.tree_id, self.set_id, lam.values, **self._score_kw(lam))
        self.last = r
        self.results = r.family_lnl
        return r.total


class GammaModel(BaseModel):
    def __init__(self, lam, tree, families, max_family_size, max_root_family_size, n_gamma_cats: int = 0,
                 fixed_alpha: float = -1.0, error_model=None, cat_probs=None, multipliers=None, **kw):
        super().__init__(lam, tree, families, max_family_size, max_root_family_size, error_model, **kw)
        if multipliers is not None:
            self.cat_probs, self.multipliers = list(cat_probs), list(multipliers)
            self.alpha = fixed_alpha
        else:
            self.cat_probs, self.multipliers = [1.0] * n_gamma_cats, [1.0] * n_gamma_cats
            self.set_alpha(fixed_alpha)

    def set_alpha(self, alpha: float):
        """gamma_model::set_alpha (src/gamma_core.cpp:61-67). An alpha <= 0
        leaves unit multipliers; can_infer then rejects it (score +inf)."""
        self.alpha = alpha
        K = len(self.cat_probs)
        if K > 1:
            if alpha > 0:
                self.cat_probs, self.multipliers = discrete_gamma(alpha, K)
            else:
                self.cat_probs, self.multipliers = [1.0 / K] * K, [1.0] * K

    def _score_kw(self, lam):
        return dict(model=_lib.MODEL_GAMMA, lambda_kind=lam.kind, multipliers=self.multipliers,
                    cat_probs=self.cat_probs, **self._kw())

    def _recon_kw(self):
        """gamma_model::reconstruct_ancestral_states (src/gamma_core.cpp:290-339):
        one pass per category at lambda * m_k, node counts from the
        probability-weighted category states."""
        return dict(model=_lib.MODEL_GAMMA, multipliers=self.multipliers, cat_probs=self.cat_probs)

    def infer_family_likelihoods(self, prior: RootPrior, lam=None) -> float:
        lam = lam or self.lam
        if self.alpha is not None and self.alpha <= 0 and len(self.cat_probs) > 1 and self.multipliers == [1.0] * len(self.cat_probs):
            return math.inf
        self._common(prior)
        r = self.ctx.score(self.tree_id, self.set_id, lam.values, want_categories=True, **self._score_kw(lam))
        self.last = r
        self.results = r.family_lnl
        self.category_results = r.category_lnl
        return r.total


class InferenceOptimizerScorer:
    """inference_optimizer_scorer::calculate_score: prepare, infer, NaN -> inf."""

    def __init__(self, lam, model: BaseModel, prior: RootPrior):
        self.lam, self.model, self.prior = lam, model, prior

    def prepare_calculation(self, values):
        raise NotImplementedError

    def calculate_score(self, values) -> float:
        self.prepare_calculation(values)
        score = self.model.infer_family_likelihoods(self.prior, self.lam)
        return math.inf if math.isnan(score) else score


class LambdaOptimizerScorer(InferenceOptimizerScorer):
    def __init__(self, lam, model, prior, longest_branch: float):
        super().__init__(lam, model, prior)
        self.longest_branch = longest_branch

    def initial_guesses(self, rng: np.random.Generator) -> List[float]:
        """lambda_optimizer::initial_guesses (src/optimizer_scorer.cpp:40-55)."""
        distmean = 0.002 / (1.0 / self.longest_branch)
        out = []
        for _ in range(self.lam.count()):
            x = -1.0
            while x < 0:
                x = 1.0 / self.longest_branch * rng.normal(distmean, 0.2)
            out.append(x)
        return out

    def prepare_calculation(self, values):
        self.lam.update(values)

    def finalize(self, values):
        self.lam.update(values)


class GammaLambdaOptimizerScorer(LambdaOptimizerScorer):
    """gamma_lambda_optimizer: lambdas then alpha."""

    def initial_guesses(self, rng):
        return super().initial_guesses(rng) + [float(rng.gamma(4.0, 0.25))]

    def prepare_calculation(self, values):
        n = self.lam.count()
        self.lam.update(values[:n])
        self.model.set_alpha(float(values[n]))

    def finalize(self, values):
        self.prepare_calculation(values)


class LambdaEpsilonOptimizerScorer(LambdaOptimizerScorer):
    """lambda_epsilon_optimizer: lambdas then epsilons, replaced in the error
    model (src/optimizer_scorer.cpp:72-109)."""

    def __init__(self, lam, model, prior, longest_branch, error_model: ErrorModel):
        super().__init__(lam, model, prior, longest_branch)
        self.error_model = error_model
        self.current = error_model.get_epsilons()

    def initial_guesses(self, rng):
        return super().initial_guesses(rng) + list(self.current)

    def prepare_calculation(self, values):
        n = self.lam.count()
        self.lam.update(values[:n])
        repl = {}
        for i, old in enumerate(self.current):
            repl[old] = float(values[n + i])
            self.current[i] = float(values[n + i])
        self.error_model.replace_epsilons(repl)

    def finalize(self, values):
        """lambda_epsilon_optimizer::finalize: lambdas, then the first epsilon
        through error_model::update_single_epsilon."""
        n = self.lam.count()
        self.lam.update(values[:n])
        self.error_model.replace_epsilons({self.current[0]: float(values[n])})
        self.current = self.error_model.get_epsilons()


class GammaOptimizerScorer(InferenceOptimizerScorer):
    """gamma_optimizer: alpha only, lambdas fixed (src/optimizer_scorer.cpp:112-150)."""

    def initial_guesses(self, rng):
        return [float(rng.gamma(4.0, 0.25))]

    def prepare_calculation(self, values):
        self.model.set_alpha(float(values[0]))

    def finalize(self, values):
        self.model.set_alpha(float(values[0]))


@dataclass
class OptimizerResult:
    values: List[float]
    score: float
    num_iterations: int
    evaluations: int
    converged: bool


class Optimizer:
    """optimizer (src/optimizer.h, src/optimizer.cpp:537-560) with the
    Standard Nelder-Mead strategy. The simplex search runs natively in the
    library (cafe_optimize): the host C++ loop proposes points and each
    objective evaluation is one GPU score of the scorer's model, exactly as
    the scorer's calculate_score would compute it."""

    def __init__(self, scorer: InferenceOptimizerScorer):
        self.scorer = scorer

    def _kind(self):
        sc = self.scorer
        if isinstance(sc, LambdaEpsilonOptimizerScorer):
            return _lib.OPT_LAMBDA_EPSILON
        if isinstance(sc, GammaLambdaOptimizerScorer):
            return _lib.OPT_LAMBDA_ALPHA
        if isinstance(sc, GammaOptimizerScorer):
            return _lib.OPT_ALPHA
        if isinstance(sc, LambdaOptimizerScorer):
            return _lib.OPT_LAMBDA
        raise TypeError(f"no native search for {type(sc).__name__}")

    def optimize(self, initial: Optional[Sequence[float]] = None, rng: Optional[np.random.Generator] = None,
                 max_iterations: int = 300, expansion: float = 2.0, reflection: float = 1.0) -> OptimizerResult:
        sc = self.scorer
        model = sc.model
        if initial is None:
            initial = sc.initial_guesses(rng or np.random.default_rng())
        x0 = np.ascontiguousarray(initial, dtype=np.float64)
        kind = self._kind()
        model._common(sc.prior)
        if kind == _lib.OPT_LAMBDA_EPSILON:
            model.ctx.set_error_model(sc.error_model.table())
        req, keep = model.ctx.make_request(model.tree_id, model.set_id, sc.lam.values, **model._score_kw(sc.lam))
        cfg = _lib.OptConfig(kind, len(x0), _p(x0), int(max_iterations), float(reflection), float(expansion))
        best = np.zeros(len(x0))
        res = _lib.OptResult(_p(best), 0.0, 0, 0, 0)
        model.ctx._check(model.ctx.lib.cafe_optimize(model.ctx.h, C.byref(req), C.byref(cfg), C.byref(res)))
        return OptimizerResult(best.tolist(), res.score, res.iterations, res.evaluations, bool(res.converged))
