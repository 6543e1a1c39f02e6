"""The reference's own example data on the GPU, through the C ABI.

Inputs: the mammals and Primates trees and family tables, the mammals
error-model file, the chimp/human lambda tree and the Primates root-size
distribution, read by this package's readers (pinned against the
reference's parse in tests/test_inputs_cpu.py) and filtered like the
estimate action (families absent at the root dropped). Expected values:
the compiled reference's total and per-family lnL at its own global bounds
(S = 170, R = 150 on both data sets), tests/golden/ref_examples.json/.npz.

Tolerances: FP64_REF (the reference's bounds) 1e-10 relative per family
and in total; FP64_BINNED (per-family S-bins, the same prior) 1e-10 --
the bins truncate the state space where the reference's values are below
FP64 resolution; MIXED_TF32X3 1e-6 relative per family. The gamma case
underflows in FP64 in the reference (+inf); the FP64 paths must return +inf
as well.
"""
import math
import os

import numpy as np
import pytest

from golden_cases import GOLDEN, example_available, example_cases, read_example

pytestmark = pytest.mark.gpu

CASES = example_cases()
FAM = np.load(os.path.join(GOLDEN, "ref_examples.npz"))


@pytest.fixture(scope="module")
def ctx():
    from cafe5_gb300.engine import Context
    c = Context()
    yield c
    c.close()


def _prepare(ctx, case):
    if not example_available(case):
        pytest.skip("example inputs not staged (tests/golden/stage_examples.py)")
    from cafe5_gb300.families import bin_families
    from cafe5_gb300.inputs import discrete_gamma
    from cafe5_gb300.tree import lambda_index_of_nodes
    tree, fams, kept, ltree, em, prior, S, R = read_example(case)
    lam_idx = lambda_index_of_nodes(tree, ltree)
    tid = ctx.upload_tree(tree, lam_idx)
    sid = ctx.upload_families(tid, kept.counts)
    W, _, _ = bin_families(kept)
    ctx.set_prior(prior.vector(max(R, int(W.max()) + 8)))
    ctx.set_error_model(None if em is None else em.table())
    kw = dict(lambda_kind=1 if ltree is not None else 0, use_error_model=em is not None)
    if case.get("gamma"):
        probs, mult = discrete_gamma(case["gamma"][1], case["gamma"][0])
        kw.update(model=1, multipliers=mult, cat_probs=probs)
    return tid, sid, kept, S, R, kw


def _rel(a, b):
    return np.abs(a - b) / np.abs(b)


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_fp64_ref_matches_reference_examples(ctx, case):
    tid, sid, kept, S, R, kw = _prepare(ctx, case)
    try:
        exp_total = float.fromhex(case["total_hex"])
        for dedupe in (True, False):
            r = ctx.score(tid, sid, case["lambdas"], S=S, R=R, precision="fp64_ref", dedupe=dedupe, **kw)
            if math.isinf(exp_total):
                assert r.total == math.inf
                continue
            assert abs(r.total - exp_total) <= 1e-10 * abs(exp_total), (r.total, exp_total)
            exp = FAM[case["name"] + "_fam_lnl"]
            assert np.all(_rel(r.family_lnl, exp) <= 1e-10)
    finally:
        ctx.free_families(sid)


@pytest.mark.parametrize("case", [c for c in CASES if not c.get("gamma")], ids=lambda c: c["name"])
def test_binned_and_mixed_paths_match_reference_examples(ctx, case):
    """The GPU's binned paths compute the reference's objective: with the
    reference's prior the per-family S-bins change nothing above FP64
    resolution, so FP64_BINNED is held to 1e-10 and the tensor-core path to
    1e-6 against the reference's own per-family lnL."""
    tid, sid, kept, S, R, kw = _prepare(ctx, case)
    try:
        exp = FAM[case["name"] + "_fam_lnl"]
        b = ctx.score(tid, sid, case["lambdas"], precision="fp64_binned", **kw)
        assert np.all(_rel(b.family_lnl, exp) <= 1e-10), float(np.max(_rel(b.family_lnl, exp)))
        m = ctx.score(tid, sid, case["lambdas"], precision="mixed_tf32x3", **kw)
        assert np.all(_rel(m.family_lnl, exp) <= 1e-6), float(np.max(_rel(m.family_lnl, exp)))
    finally:
        ctx.free_families(sid)
