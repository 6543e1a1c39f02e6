"""Gene-family count tables, bounds and S-binning.

* `read_families` / `write_families`: the CAFE tab-separated format read by
  the reference's `read_gene_families` (src/io.cpp:134-217): a header line
  `Desc<TAB>Family ID<TAB>taxon...` then one row per family.
* `global_bounds`: the reference's single global state bound and root bound,
  `max_root = max(30, rint(1.25 * m))`, `max_family = m + max(50, m/5)` with
  m = max(120, largest count) (src/user_data.cpp:39-48; the 120 is
  user_data's default, src/user_data.h:26).
* `bin_families`: the GB300 path's per-family bound. A family whose largest
  count is m needs states up to ceil(1.2 m) + 20; it is placed in the
  smallest bin width W (states 0..W-1) that holds that, and uses the whole
  bin (S_f = W - 1), which only adds states. Its root bound is
  R_f = min(S_f, max(30, rint(1.25 m))).
* `dedupe`: identical count rows are pruned once, as `build_reference_list`
  does (src/base_model.cpp:27-51).
"""
from __future__ import annotations

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
    """A family table in either format `read_gene_families` accepts
    (src/io.cpp:134-217):

    * CAFE: one header line `Desc<TAB>Family ID<TAB>taxon...`, then rows
      `desc<TAB>id<TAB>count...`. Header columns that name no leaf of the
      tree are read and ignored.
    * CAFExp: header lines `#taxon`, one per column, each naming a node of
      the tree (internal nodes too; only leaf columns carry counts); the
      first line without `#` ends the header; the last column is the id.

    Species names match case-insensitively (the reference's map compares
    with `ci_less`, src/gene_family.h:10-25). Every leaf of the tree must
    have a count in every family (`get_species_size` throws otherwise);
    counts are parsed like `atoi` (leading digits, else 0). Blank lines are
    skipped; an empty table raises."""
    text = path_or_text if is_text else open(path_or_text).read()
    leaf_pos = {nm.lower(): i for i, nm in enumerate(tree.leaf_names)}
    node_names = {tree.name[v].lower() for v in range(tree.n_nodes)}
    n_leaves = len(tree.leaf_names)
    col_leaf = {}           # column -> leaf position
    cafexp = False
    header = True
    ids, rows = [], []
    index = 0
    for ln in text.split("\n"):
        if not ln:
            continue
        tok = ln.split("\t")
        if col_leaf and cafexp and ln[0] != "#":
            header = False
        if header:
            if ln[0] == "#":
                cafexp = True
                name = ln[1:].rstrip("\r")
                if name.lower() not in node_names:
                    raise ValueError(f"{name} not located in tree")
                if name.lower() in leaf_pos:
                    col_leaf[index] = leaf_pos[name.lower()]
                index += 1
                continue
            header = False
            if not cafexp:
                for i, nm in enumerate(tok):
                    if i >= 2 and nm.rstrip("\r").lower() in leaf_pos:
                        col_leaf[i] = leaf_pos[nm.rstrip("\r").lower()]
                continue
        row = np.zeros(n_leaves, dtype=np.int32)
        seen = np.zeros(n_leaves, dtype=bool)
        fid = ""
        for i, v in enumerate(tok):
            if not cafexp and i == 1:
                fid = v
            if i in col_leaf and (cafexp or i >= 2):
                row[col_leaf[i]] = _atoi(v)
                seen[col_leaf[i]] = True
            elif cafexp and i not in col_leaf and i == len(tok) - 1:
                fid = v
        if not seen.all():
            missing = tree.leaf_names[int(np.argmin(seen))]
            raise ValueError(f"{missing} was not found in gene family {fid}")
        ids.append(fid)
        rows.append(row)
    if not rows:
        raise ValueError("No families found")
    return FamilySet(ids, np.asarray(rows, dtype=np.int32).reshape(len(rows), n_leaves))


def _atoi(v: str) -> int:
    """C atoi: optional blanks and sign, then leading digits; 0 if none."""
    v = v.lstrip(" \t\r\n\f\v")
    sign, i = 1, 0
    if v[:1] in "+-" and v[:1]:
        sign = -1 if v[0] == "-" else 1
        i = 1
    j = i
    while j < len(v) and v[j].isdigit():
        j += 1
    return sign * int(v[i:j]) if j > i else 0


def exclude_zero_root_families(fams: FamilySet, tree: Tree) -> FamilySet:
    """The estimate action's default filter (exclude_zero_root_families,
    src/core.cpp:190-205): keep a family iff its parsimony reconstruction
    has the gene at the root, i.e. every child of the root has a leaf with a
    nonzero count below it (gene_family::exists_at_root,
    src/gene_family.cpp:62-91)."""
    col = tree.leaf_col()
    keep = np.ones(fams.n_families, dtype=bool)
    for c in tree.children[tree.root]:
        stack, leaves = [c], []
        while stack:
            v = stack.pop()
            if tree.is_leaf(v):
                leaves.append(int(col[v]))
            stack.extend(tree.children[v])
        keep &= (fams.counts[:, leaves] > 0).any(axis=1)
    idx = np.nonzero(keep)[0]
    return FamilySet([fams.ids[i] for i in idx], np.ascontiguousarray(fams.counts[idx]))


def write_families(path: str, fams: FamilySet, tree: Tree) -> None:
    with open(path, "w") as f:
        f.write("Desc\tFamily ID\t" + "\t".join(tree.leaf_names) + "\n")
        for fid, row in zip(fams.ids, fams.counts):
            f.write("(null)\t" + fid + "\t" + "\t".join(str(int(x)) for x in row) + "\n")


def global_bounds(fams: FamilySet, floor: int = 120) -> Tuple[int, int]:
    """(max_family_size S, max_root_family_size R) as the reference sets them
    (user_data::read_gene_family_data, src/user_data.cpp:24-48): the largest
    count m is taken over every family read and starts from user_data's
    default max_family_size of 120 (src/user_data.h:26), so m = max(120,
    largest count); then R = max(30, rint(1.25 m)) and S = m + max(50, m/5).
    `floor=0` gives the bounds of the counts alone."""
    mx = max(int(floor), int(fams.counts.max()) if fams.counts.size else 0)
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
