"""Gene-family count tables, bounds and S-binning.

* `read_families` / `write_families`: the CAFE tab-separated format read by
  the reference's `read_gene_families` (src/io.cpp:134-217): a header line
  `Desc<TAB>Family ID<TAB>taxon...` then one row per family.
* `global_bounds`: the reference's single global state bound and root bound,
  `max_root = max(30, rint(1.25 * max))`, `max_family = max + max(50, max/5)`
  (src/user_data.cpp:39-48).
* `bin_families`: the GB300 path's per-family bound. A family whose largest
  count is m needs states up to ceil(1.2 m) + 20; it is placed in the
  smallest bin width W (states 0..W-1) that holds that, and uses the whole
  bin (S_f = W - 1), which only adds states. Its root bound is
  R_f = min(S_f, max(30, rint(1.25 m))).
* `dedupe`: identical count rows are pruned once, as `build_reference_list`
  does (src/base_model.cpp:27-51).
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import List, Optional, Sequence, Tuple

import numpy as np

from .tree import Tree

# bin widths shared with the library (kDefaultBins in csrc/cafe_abi.cu)
DEFAULT_BINS = (32, 64, 96, 128, 192, 256, 384, 512, 768, 1024)


@dataclass
class FamilySet:
    ids: List[str]
    counts: np.ndarray          # int32 [F, n_leaves], columns in tree leaf order

    @property
    def n_families(self) -> int:
        return int(self.counts.shape[0])

    def max_counts(self) -> np.ndarray:
        return self.counts.max(axis=1) if self.counts.size else np.zeros(0, np.int32)


def read_families(path_or_text: str, tree: Tree, is_text: bool = False) -> FamilySet:
    text = path_or_text if is_text else open(path_or_text).read()
    lines = [ln for ln in text.splitlines() if ln.strip()]
    header = lines[0].rstrip("\r").split("\t")
    taxa = header[2:]
    # species names match case-insensitively (src/gene_family.h:12-20)
    leaf_pos = {nm.lower(): i for i, nm in enumerate(tree.leaf_names)}
    cols = []
    for nm in taxa:
        if nm.lower() not in leaf_pos:
            raise ValueError(f"{nm} not located in tree")
        cols.append(leaf_pos[nm.lower()])
    ids, rows = [], []
    for ln in lines[1:]:
        tok = ln.rstrip("\r").split("\t")
        ids.append(tok[1])
        row = np.zeros(len(tree.leaf_names), dtype=np.int32)
        for c, v in zip(cols, tok[2:]):
            row[c] = int(v)
        rows.append(row)
    return FamilySet(ids, np.asarray(rows, dtype=np.int32).reshape(len(rows), len(tree.leaf_names)))


def write_families(path: str, fams: FamilySet, tree: Tree) -> None:
    with open(path, "w") as f:
        f.write("Desc\tFamily ID\t" + "\t".join(tree.leaf_names) + "\n")
        for fid, row in zip(fams.ids, fams.counts):
            f.write("(null)\t" + fid + "\t" + "\t".join(str(int(x)) for x in row) + "\n")


def global_bounds(fams: FamilySet) -> Tuple[int, int]:
    """(max_family_size S, max_root_family_size R) as the reference sets them."""
    mx = int(fams.counts.max()) if fams.counts.size else 0
    max_root = max(30, int(np.rint(mx * 1.25)))
    max_family = mx + max(50, mx // 5)
    return max_family, max_root


def bin_families(fams: FamilySet, bins: Sequence[int] = DEFAULT_BINS,
                 cap: Optional[int] = None) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Per-family (bin width W_f, S_f, R_f). Families needing more than the
    largest bin are capped to it (their state space is truncated there)."""
    mx = fams.max_counts().astype(np.int64)
    need = np.ceil(1.2 * mx).astype(np.int64) + 20 + 1          # states 0..S
    bins = np.asarray(sorted(bins), dtype=np.int64)
    idx = np.searchsorted(bins, need, side="left")
    idx = np.minimum(idx, len(bins) - 1)
    W = bins[idx]
    if cap is not None:
        W = np.minimum(W, cap)
    S = W - 1
    R = np.minimum(S, np.maximum(30, np.rint(mx * 1.25).astype(np.int64)))
    return W.astype(np.int32), S.astype(np.int32), R.astype(np.int32)


def dedupe(counts: np.ndarray) -> Tuple[np.ndarray, np.ndarray]:
    """(unique_rows_index, ref) where ref[f] is the first family with the
    same counts row, as in build_reference_list."""
    if counts.shape[0] == 0:
        return np.zeros(0, np.int64), np.zeros(0, np.int64)
    _, first, inv = np.unique(counts, axis=0, return_index=True, return_inverse=True)
    ref = first[inv.reshape(-1)]
    return np.unique(ref), ref.astype(np.int64)
