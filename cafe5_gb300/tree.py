"""Species tree as flat arrays, parsed from Newick the way CAFE5 parses it.

Mirrors the reference's `clade` (src/clade.h:25-121) for what the
likelihood path needs: the tokenizer and parse rules of `parse_newick`
(src/clade.cpp:293-419), interior names from sorted leaf names
(`_name_interior_clade`), the reverse-level order used by `inference_prune`
(src/clade.cpp:69-100) and the distinct positive branch-length set of
`get_branch_lengths` (src/clade.cpp:236-245), root branch included.

Nodes are numbered in Newick (pre-)order, so the children of a node appear
in increasing index, which is the reference's descendant order.
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

# Same token classes as src/clade.cpp:295: '(' ')' names ':number' ',' ';'
_TOKEN = re.compile(r"\(|\)|[^\s\(\)\:\;\,]+|\:[+-]?[0-9]*\.?[0-9]+(?:[eE][+-]?[0-9]+)?|\,|\;")


@dataclass
class Tree:
    parent: List[int] = field(default_factory=list)
    branch_length: List[float] = field(default_factory=list)
    name: List[str] = field(default_factory=list)
    lambda_index: List[int] = field(default_factory=list)   # 1-based as in a lambda tree; 0 = unset
    children: List[List[int]] = field(default_factory=list)

    # ---- construction -------------------------------------------------
    def _new(self, parent: int) -> int:
        self.parent.append(parent)
        self.branch_length.append(0.0)
        self.name.append("")
        self.lambda_index.append(0)
        self.children.append([])
        if parent >= 0:
            self.children[parent].append(len(self.parent) - 1)
        return len(self.parent) - 1

    @property
    def n_nodes(self) -> int:
        return len(self.parent)

    @property
    def root(self) -> int:
        return self.parent.index(-1)

    def is_leaf(self, v: int) -> bool:
        return not self.children[v]

    @property
    def leaves(self) -> List[int]:
        return [v for v in range(self.n_nodes) if self.is_leaf(v)]

    @property
    def leaf_names(self) -> List[str]:
        return [self.name[v] for v in self.leaves]

    def leaf_col(self) -> np.ndarray:
        """Counts-matrix column of every node (-1 for internal nodes)."""
        col = np.full(self.n_nodes, -1, dtype=np.int32)
        for i, v in enumerate(self.leaves):
            col[v] = i
        return col

    def reverse_level_order(self) -> List[int]:
        """Breadth-first from the root, reversed (src/clade.cpp:69-100)."""
        q = [self.root]
        i = 0
        while i < len(q):
            q.extend(self.children[q[i]])
            i += 1
        return q[::-1]

    def postorder(self) -> List[int]:
        return self.reverse_level_order()

    def branch_lengths(self) -> List[float]:
        """Distinct positive branch lengths, sorted (a std::set<double>)."""
        return sorted({t for t in self.branch_length if t > 0.0})

    def longest_branch(self) -> float:
        b = self.branch_lengths()
        return max(b) if b else 0.0

    def find(self, name: str) -> int:
        for v, nm in enumerate(self.name):
            if nm == name:
                return v
        raise KeyError(name)

    def depth(self, v: int) -> float:
        d = 0.0
        while self.parent[v] >= 0:
            d += self.branch_length[v]
            v = self.parent[v]
        return d

    # ---- naming ---------------------------------------------------------
    def _leaf_names_under(self, v: int) -> List[str]:
        if self.is_leaf(v):
            return [self.name[v]]
        out: List[str] = []
        for c in self.children[v]:
            out.extend(self._leaf_names_under(c))
        return out

    def name_interior(self) -> None:
        """Unlabelled interior clades are named by their sorted leaf names
        joined (CAFE5's `_name_interior_clade`), e.g. ((A,B),C) -> AB, ABC;
        an explicit Newick label after ')' wins, as in the reference."""
        for v in range(self.n_nodes):
            if not self.is_leaf(v) and not self.name[v]:
                self.name[v] = "".join(sorted(self._leaf_names_under(v)))

    # ---- Newick ---------------------------------------------------------
    def to_newick(self, fmt: str = "{:.6f}") -> str:
        def rec(v: int) -> str:
            lab = self.name[v] if self.is_leaf(v) else ""
            if self.children[v]:
                lab = "(" + ",".join(rec(c) for c in self.children[v]) + ")"
            if self.parent[v] >= 0:
                lab += ":" + fmt.format(self.branch_length[v])
            return lab
        return rec(self.root) + ";"

    def arrays(self, lambda_of_node: Optional[List[int]] = None) -> Dict[str, np.ndarray]:
        """Flat arrays for the C-ABI / oracle: parent, branch_length,
        lambda_index (0-based), leaf_col."""
        lam = lambda_of_node if lambda_of_node is not None else [0] * self.n_nodes
        return {
            "parent": np.asarray(self.parent, dtype=np.int32),
            "branch_length": np.asarray(self.branch_length, dtype=np.float64),
            "lambda_index": np.asarray(lam, dtype=np.int32),
            "leaf_col": self.leaf_col(),
        }


def parse_newick(text: str, lambda_tree: bool = False) -> Tree:
    """Parse Newick with the token rules of src/clade.cpp:293-419.

    With lambda_tree=True the ':x' fields are integer lambda indices (the
    `-y` lambda tree), else branch lengths. Branch lengths must be positive
    on every non-root node (src/clade.cpp:411-414)."""
    t = Tree()
    root = t._new(-1)
    cur = root
    for tok in _TOKEN.findall(text):
        if tok == "(":
            cur = t._new(cur)
        elif tok == ",":
            if cur == root:
                # missing outer parentheses: a new root above the current one
                new_root = len(t.parent)
                t.parent.append(-1)
                t.branch_length.append(0.0)
                t.name.append("")
                t.lambda_index.append(0)
                t.children.append([cur])
                t.parent[cur] = new_root
                root = new_root
            cur = t._new(t.parent[cur])
        elif tok == ")":
            cur = t.parent[cur]
        elif tok == ";":
            break
        elif tok.startswith(":"):
            if lambda_tree:
                t.lambda_index[cur] = int(float(tok[1:]))
            else:
                t.branch_length[cur] = float(tok[1:])
        else:
            t.name[cur] = tok
    t = _renumber_preorder(t)
    t.name_interior()
    if lambda_tree:
        r = t.root
        if t.lambda_index[r] == 0:
            t.lambda_index[r] = 1
        for v in range(t.n_nodes):
            if t.lambda_index[v] < 1:
                raise ValueError("Invalid lambda index set for " + t.name[v])
    else:
        for v in range(t.n_nodes):
            if t.parent[v] >= 0 and not t.branch_length[v] > 0:
                raise ValueError("Invalid branch length set for " + t.name[v])
    return t


def _renumber_preorder(t: Tree) -> Tree:
    order: List[int] = []
    stack = [t.root]
    while stack:
        v = stack.pop()
        order.append(v)
        stack.extend(reversed(t.children[v]))
    new_id = {v: i for i, v in enumerate(order)}
    out = Tree()
    for v in order:
        out.parent.append(new_id[t.parent[v]] if t.parent[v] >= 0 else -1)
        out.branch_length.append(t.branch_length[v])
        out.name.append(t.name[v])
        out.lambda_index.append(t.lambda_index[v])
        out.children.append([new_id[c] for c in t.children[v]])
    return out


def lambda_index_of_nodes(tree: Tree, lambda_tree: Optional[Tree]) -> List[int]:
    """0-based lambda index of the branch above every node of `tree`, from a
    lambda tree matched by node name (multiple_lambda::calculate_child_factor,
    src/lambda.cpp:32-40; get_lambda_index_map, src/clade.cpp:194-204)."""
    if lambda_tree is None:
        return [0] * tree.n_nodes
    by_name = {lambda_tree.name[v]: lambda_tree.lambda_index[v] - 1 for v in range(lambda_tree.n_nodes)}
    return [by_name[tree.name[v]] for v in range(tree.n_nodes)]
