"""ctypes binding of the CPU oracle (cafe_oracle.c) -- TEST INFRASTRUCTURE.

Imported only by tests/, __graft_entry__.smoke() and bench.py's
cpu_baseline / reference legs, as the checker. `build()` compiles
_build/libcafe_oracle.so with the committed Makefile.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libcafe_oracle.so")
REF_HARNESS = os.path.join(HERE, "_ref", "cafe_ref_harness")
_lib = None


class _Tree(C.Structure):
    _fields_ = [("n_nodes", C.c_int), ("parent", C.c_void_p), ("branch_length", C.c_void_p),
                ("lambda_index", C.c_void_p), ("leaf_col", C.c_void_p)]


def reference_dir() -> Optional[str]:
    """The CAFE5 reference checkout the `ref` recipe compiles: the directory
    named by the CAFE_REFERENCE environment variable, else the checkout this
    build's fixtures came from when it exists; None when neither is there
    (then only the restatement is built)."""
    d = os.environ.get("CAFE_REFERENCE") or "/root/reference"
    return d if os.path.isdir(os.path.join(d, "src")) else None


def build(ref: bool = False) -> None:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    d = reference_dir()
    if ref and d:
        subprocess.run(["make", "-s", "-j8", "-C", HERE, "ref", f"REF={d}"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = C.CDLL(LIB_PATH)
        d, i, p = C.c_double, C.c_int, C.c_void_p
        _lib.oracle_bd_rate.restype = d
        _lib.oracle_bd_rate.argtypes = [i, i, d, d]
        _lib.oracle_transition.restype = d
        _lib.oracle_transition.argtypes = [d, d, i, i]
        _lib.oracle_chooseln.restype = d
        _lib.oracle_chooseln.argtypes = [d, d]
        _lib.oracle_is_saturated.restype = i
        _lib.oracle_is_saturated.argtypes = [d, d]
        _lib.oracle_fill_matrix.argtypes = [d, d, i, p]
        _lib.oracle_quantize.argtypes = [d, d, p, p]
        _lib.oracle_multiply.argtypes = [p, i, p, i, i, i, i, p]
        _lib.oracle_discrete_gamma.restype = i
        _lib.oracle_discrete_gamma.argtypes = [i, d, p, p]
        _lib.oracle_prune.restype = i
        _lib.oracle_prune.argtypes = [C.POINTER(_Tree), p, p, i, p, i, i, i, i, i, p, p]
        _lib.oracle_score.restype = i
        _lib.oracle_score.argtypes = [C.POINTER(_Tree), p, C.c_int64, i, p, i, i, i, p, p, p, i, p, i, i,
                                      i, i, p, p, i, i, i, i, p, p, p]
        _lib.oracle_reconstruct.restype = i
        _lib.oracle_reconstruct.argtypes = [C.POINTER(_Tree), p, C.c_int64, i, p, i, i, p, p, p, i, i, i, i,
                                            p, p, p, p]
        _lib.oracle_branch_probabilities.restype = i
        _lib.oracle_branch_probabilities.argtypes = [C.POINTER(_Tree), p, i, p, C.c_int64, i, i, p]
        _lib.oracle_pvalues.restype = i
        _lib.oracle_pvalues.argtypes = [C.POINTER(_Tree), p, C.c_int64, i, p, i, i, i, i, C.c_uint32, p, p, p]
        _lib.oracle_simulate.restype = i
        _lib.oracle_simulate.argtypes = [C.POINTER(_Tree), p, i, i, p, p, p, i, i, i, i, i, i, p, C.c_uint32, p, p]
    return _lib


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data


def discrete_gamma(alpha: float, K: int):
    """(category probabilities, rate multipliers) of get_gamma for K median
    categories -- the oracle's own restatement, bit for bit the reference's."""
    if K <= 1:
        return [1.0], [1.0]
    probs = np.zeros(K)
    mult = np.zeros(K)
    if lib().oracle_discrete_gamma(K, float(alpha), probs.ctypes.data, mult.ctypes.data):
        raise ValueError(f"discrete gamma needs alpha > 0 (got {alpha})")
    return probs.tolist(), mult.tolist()


def bd_rate(s, c, log_alpha, coeff):
    return lib().oracle_bd_rate(s, c, log_alpha, coeff)


def transition(lam, t, s, c):
    return lib().oracle_transition(lam, t, s, c)


def quantize(lam, t):
    a = np.zeros(1)
    b = np.zeros(1)
    lib().oracle_quantize(lam, t, a.ctypes.data, b.ctypes.data)
    return float(a[0]), float(b[0])


def fill_matrix(lam, t, size, quantized: bool = True) -> np.ndarray:
    if quantized:
        lam, t = quantize(lam, t)
    out = np.zeros((size, size))
    lib().oracle_fill_matrix(lam, t, size, out.ctypes.data)
    return out


class TreeArrays:
    def __init__(self, parent, branch_length, lambda_index, leaf_col):
        self.parent = np.ascontiguousarray(parent, dtype=np.int32)
        self.branch_length = np.ascontiguousarray(branch_length, dtype=np.float64)
        self.lambda_index = np.ascontiguousarray(lambda_index, dtype=np.int32)
        self.leaf_col = np.ascontiguousarray(leaf_col, dtype=np.int32)
        self.c = _Tree(len(self.parent), self.parent.ctypes.data, self.branch_length.ctypes.data,
                       self.lambda_index.ctypes.data, self.leaf_col.ctypes.data)

    @classmethod
    def from_tree(cls, tree, lambda_of_node=None):
        a = tree.arrays(lambda_of_node)
        return cls(a["parent"], a["branch_length"], a["lambda_index"], a["leaf_col"])


def prune(tree: TreeArrays, counts_row, node_matrices: Sequence[Optional[np.ndarray]], size: int,
          S: int, R: int, err_rows=None, scaled=False):
    counts_row = np.ascontiguousarray(counts_row, dtype=np.int32)
    keep = [None if m is None else np.ascontiguousarray(m, dtype=np.float64) for m in node_matrices]
    ptrs = (C.c_void_p * len(keep))(*[None if m is None else m.ctypes.data for m in keep])
    out = np.zeros(R)
    ls = np.zeros(1)
    er = None if err_rows is None else np.ascontiguousarray(err_rows, dtype=np.float64)
    rc = lib().oracle_prune(C.byref(tree.c), counts_row.ctypes.data, C.cast(ptrs, C.c_void_p), size, _ptr(er),
                            0 if er is None else er.shape[0], 0 if er is None else er.shape[1], S, R,
                            1 if scaled else 0, out.ctypes.data, ls.ctypes.data)
    if rc:
        raise RuntimeError(f"oracle_prune failed: {rc}")
    return out, float(ls[0])


def score(tree: TreeArrays, counts: np.ndarray, lambdas: Sequence[float], *, lambda_kind: int = 0,
          model: int = 0, multipliers: Sequence[float] = (1.0,), cat_probs: Sequence[float] = (1.0,),
          prior: np.ndarray, err_rows: Optional[np.ndarray] = None, S: int = 0, R: int = 0,
          fam_S: Optional[np.ndarray] = None, fam_R: Optional[np.ndarray] = None, dedupe: bool = True,
          scaled: bool = False, n_threads: int = 0):
    """One infer_family_likelihoods: returns (total, fam_lnl[F], cat_log[F, K])."""
    counts = np.ascontiguousarray(counts, dtype=np.int32)
    F, n_leaves = counts.shape
    lam = np.ascontiguousarray(lambdas, dtype=np.float64)
    mult = np.ascontiguousarray(multipliers, dtype=np.float64)
    cp = np.ascontiguousarray(cat_probs, dtype=np.float64)
    K = len(mult) if model == 1 else 1
    pr = np.ascontiguousarray(prior, dtype=np.float64)
    er = None if err_rows is None else np.ascontiguousarray(err_rows, dtype=np.float64)
    fS = None if fam_S is None else np.ascontiguousarray(fam_S, dtype=np.int32)
    fR = None if fam_R is None else np.ascontiguousarray(fam_R, dtype=np.int32)
    fam = np.zeros(F)
    cat = np.zeros((F, K))
    tot = np.zeros(1)
    rc = lib().oracle_score(C.byref(tree.c), counts.ctypes.data, F, n_leaves, lam.ctypes.data, len(lam),
                            lambda_kind, K, mult.ctypes.data, cp.ctypes.data, pr.ctypes.data, len(pr), _ptr(er),
                            0 if er is None else er.shape[0], 0 if er is None else er.shape[1], S, R, _ptr(fS),
                            _ptr(fR), model, 1 if dedupe else 0, 1 if scaled else 0, n_threads, fam.ctypes.data,
                            cat.ctypes.data, tot.ctypes.data)
    if rc:
        raise RuntimeError(f"oracle_score failed: {rc}")
    return float(tot[0]), fam, cat


def reconstruct(tree: TreeArrays, counts: np.ndarray, lambdas: Sequence[float], *, prior: np.ndarray,
                S: int, R: int, multipliers: Optional[Sequence[float]] = None,
                cat_probs: Optional[Sequence[float]] = None, n_threads: int = 0):
    """Pupko reconstruction: (state[K][F][n], mean[F][n], node_count[F][n],
    root_max[K][F]); K = 1 for the base model (multipliers None)."""
    counts = np.ascontiguousarray(counts, dtype=np.int32)
    F, n_leaves = counts.shape
    n = len(tree.parent)
    lam = np.ascontiguousarray(lambdas, dtype=np.float64)
    gamma = multipliers is not None
    mult = np.ascontiguousarray(multipliers if gamma else [1.0], dtype=np.float64)
    cp = np.ascontiguousarray(cat_probs if gamma else [1.0], dtype=np.float64)
    K = len(mult)
    pr = np.ascontiguousarray(prior, dtype=np.float64)
    state = np.zeros((K, F, n), np.int32)
    mean = np.zeros((F, n))
    cnt = np.zeros((F, n), np.int32)
    rmax = np.zeros((K, F))
    rc = lib().oracle_reconstruct(C.byref(tree.c), counts.ctypes.data, F, n_leaves, lam.ctypes.data, len(lam),
                                  K if gamma else 0, mult.ctypes.data, cp.ctypes.data, pr.ctypes.data, len(pr),
                                  S, R, n_threads, state.ctypes.data, mean.ctypes.data, cnt.ctypes.data,
                                  rmax.ctypes.data)
    if rc:
        raise RuntimeError(f"oracle_reconstruct failed: {rc}")
    return state, mean, cnt, rmax


def branch_probabilities(tree: TreeArrays, lambdas: Sequence[float], node_count: np.ndarray, S: int, R: int):
    """compute_viterbi_sum for every family and node: [F][n], NaN at the root."""
    nc = np.ascontiguousarray(node_count, dtype=np.int32)
    lam = np.ascontiguousarray(lambdas, dtype=np.float64)
    out = np.zeros(nc.shape)
    rc = lib().oracle_branch_probabilities(C.byref(tree.c), lam.ctypes.data, len(lam), nc.ctypes.data,
                                           nc.shape[0], S, R, out.ctypes.data)
    if rc:
        raise RuntimeError(f"oracle_branch_probabilities failed: {rc}")
    return out


def pvalues(tree: TreeArrays, counts: np.ndarray, lambdas: Sequence[float], *, S: int, R: int, n_sim: int,
            seed: int):
    """compute_pvalues: (pvalues[F], conditional[R][n_sim], root_vectors[F][R])."""
    counts = np.ascontiguousarray(counts, dtype=np.int32)
    F, n_leaves = counts.shape
    lam = np.ascontiguousarray(lambdas, dtype=np.float64)
    pv = np.zeros(F)
    cd = np.zeros((R, n_sim))
    rv = np.zeros((F, R))
    rc = lib().oracle_pvalues(C.byref(tree.c), counts.ctypes.data, F, n_leaves, lam.ctypes.data, len(lam), S, R,
                              n_sim, seed, pv.ctypes.data, cd.ctypes.data, rv.ctypes.data)
    if rc:
        raise RuntimeError(f"oracle_pvalues failed: {rc}")
    return pv, cd, rv


def simulate(tree: TreeArrays, lambdas: Sequence[float], root_sizes: Sequence[int], *, S: int, R: int, seed: int,
             multipliers: Optional[Sequence[float]] = None, cat_probs: Optional[Sequence[float]] = None,
             err_rows: Optional[np.ndarray] = None, err_max_count: int = 0):
    """The simulator action: (sizes[n][n_nodes], lambda[n])."""
    lam = np.ascontiguousarray(lambdas, dtype=np.float64)
    roots = np.ascontiguousarray(root_sizes, dtype=np.int32)
    gamma = multipliers is not None
    mult = np.ascontiguousarray(multipliers if gamma else [1.0], dtype=np.float64)
    cp = np.ascontiguousarray(cat_probs if gamma else [1.0], dtype=np.float64)
    er = None if err_rows is None else np.ascontiguousarray(err_rows, dtype=np.float64)
    n = len(tree.parent)
    sizes = np.zeros((len(roots), n), np.int32)
    lout = np.zeros(len(roots))
    rc = lib().oracle_simulate(C.byref(tree.c), lam.ctypes.data, len(lam), len(mult) if gamma else 0,
                               mult.ctypes.data, cp.ctypes.data, _ptr(er), 0 if er is None else er.shape[0],
                               0 if er is None else er.shape[1], err_max_count, S, R, len(roots),
                               roots.ctypes.data, seed, sizes.ctypes.data, lout.ctypes.data)
    if rc:
        raise RuntimeError(f"oracle_simulate failed: {rc}")
    return sizes, lout
