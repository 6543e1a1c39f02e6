"""The readers against the reference's own parse of its example data.

For each input set of tests/golden/ref_examples.json -- the mammals and
Primates trees and family tables, the error-model file, the chimp/human
lambda tree -- the compiled reference (read_gene_families,
src/io.cpp:134-217; read_error_model_file, :228-274; parse_newick,
src/clade.cpp:293-419; exists_at_root, src/gene_family.cpp:62-91;
read_gene_family_data's bounds, src/user_data.cpp:24-48) printed what it
read; its SHA-256 is committed. This package's readers must print the same
text. The inputs come from tests/golden/_refdata/ (staged by
tests/golden/stage_examples.py) or the checkout in CAFE_REFERENCE; without
either the tests skip.
"""
import hashlib

import numpy as np
import pytest

import oracle
from cafe5_gb300.families import FamilySet, exclude_zero_root_families, read_families
from cafe5_gb300.tree import parse_newick
from golden_cases import canonical_input_text, example_available, example_cases, read_example

CASES = example_cases()


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_readers_match_reference_parse(case):
    if not example_available(case):
        pytest.skip("example inputs not staged (tests/golden/stage_examples.py)")
    tree, fams, kept, ltree, em, prior, S, R = read_example(case)
    assert (S, R) == (case["S"], case["R"])
    assert kept.n_families == case["n_families"]
    text = canonical_input_text(tree, kept, S, R, ltree, em)
    assert hashlib.sha256(text.encode()).hexdigest() == case["parse_sha256"]


def test_oracle_matches_reference_on_mammals():
    """The oracle restatement reproduces the reference's per-family lnL on
    its mammals example bit for bit (global S = 170, R = 150, dedupe)."""
    case = next(c for c in CASES if c["name"] == "mammals_base")
    if not example_available(case):
        pytest.skip("example inputs not staged (tests/golden/stage_examples.py)")
    from golden_cases import GOLDEN
    import os
    tree, fams, kept, ltree, em, prior, S, R = read_example(case)
    ta = oracle.TreeArrays.from_tree(tree)
    tot, fam, _ = oracle.score(ta, kept.counts, case["lambdas"], prior=prior.vector(), S=S, R=R, dedupe=True)
    exp = np.load(os.path.join(GOLDEN, "ref_examples.npz"))["mammals_base_fam_lnl"]
    assert np.array_equal(fam, exp)
    assert tot.hex() == float.fromhex(case["total_hex"]).hex()


def test_cafexp_header_format_reads_like_cafe_format():
    """read_gene_families' second format (`#taxon` header lines naming tree
    nodes, counts in leaf columns, the id last) gives the same table."""
    tree = parse_newick("((A:1,B:1):2,C:3);")
    cafe = "Desc\tFamily ID\tA\tB\tC\tZ\n(null)\tf1\t1\t2\t3\t9\n(null)\tf2\t0\t5\t1\t9\n"
    a = read_families(cafe, tree, is_text=True)
    cafexp = "#A\n#B\n#AB\n#C\n1\t2\t7\t3\tf1\n0\t5\t7\t1\tf2\n"
    b = read_families(cafexp, tree, is_text=True)
    assert a.ids == b.ids == ["f1", "f2"]
    assert np.array_equal(a.counts, b.counts) and a.counts.tolist() == [[1, 2, 3], [0, 5, 1]]
    with pytest.raises(ValueError):
        read_families("Desc\tFamily ID\tA\tB\n(null)\tf1\t1\t2\n", tree, is_text=True)   # C missing
    with pytest.raises(ValueError):
        read_families("#A\n#Q\n1\t2\tf1\n", tree, is_text=True)                          # Q not in tree


def test_zero_root_filter():
    tree = parse_newick("((A:1,B:1):2,C:3);")
    fams = FamilySet(["keep", "left_only", "right_only", "zero"],
                     np.array([[1, 0, 2], [3, 1, 0], [0, 0, 4], [0, 0, 0]], np.int32))
    kept = exclude_zero_root_families(fams, tree)
    assert kept.ids == ["keep"]
