"""The no-allocation entry point, cafe_prune_fp64_noalloc.

Some callers cannot call cudaMalloc (a host framework whose own pool owns
every device allocation, a serving loop that must not allocate per request);
this entry point runs the FP64 pruning kernel with its working space in a
static device array and only the caller's buffers for inputs and outputs.

Each case calls it through the C ABI twice in a row and checks both results
at the parity tolerance of the FP64 path, 1e-10 relative per family:
  * 700 families: against the existing entry point (cafe_score, FP64_REF);
  * 20,000 families: more 32-family tiles than the static array holds CTAs
    for, so every CTA walks several tiles through the shared array --
    against cafe_score, and with scaled = 1 (per-node power-of-two rescale)
    against the rescaled CPU oracle.
Sizes past the stated maximum are refused. This file is collected last.
"""
import ctypes

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

REL = 1e-10


@pytest.fixture(scope="module")
def ctx():
    from cafe5_gb300.engine import Context
    c = Context()
    yield c
    c.close()


def _run(ctx, n_families, seed, scaled):
    import torch
    from cafe5_gb300 import _lib
    from cafe5_gb300.families import global_bounds
    from cafe5_gb300.inputs import RootPrior
    from cafe5_gb300.synth import workload

    w = workload(0, n_families=n_families, seed=seed)
    S, R = global_bounds(w.families)
    prior = RootPrior.uniform(R).vector()
    lam = 0.0031
    tid = ctx.upload_tree(w.tree)
    sid = ctx.upload_families(tid, w.families.counts)
    ctx.set_prior(prior)
    ctx.set_error_model(None)
    if scaled:
        ta = oracle.TreeArrays.from_tree(w.tree)
        _, expect, _ = oracle.score(ta, w.families.counts, [lam], prior=prior, S=S, R=R, dedupe=False, scaled=True)
    else:
        expect = ctx.score(tid, sid, [lam], S=S, R=R, precision="fp64_ref", dedupe=False).family_lnl
    ctx.free_families(sid)

    # the same matrices, in caller-owned device memory
    msize = max(R, S) + 1
    ctx.matrices_build([lam], [w.tree.branch_length[v] for v in range(w.tree.n_nodes) if w.tree.parent[v] >= 0],
                       msize)
    dev = torch.device("cuda", 0)
    keep = []
    ptrs = (ctypes.c_void_p * w.tree.n_nodes)()
    for v in range(w.tree.n_nodes):
        if w.tree.parent[v] < 0:
            ptrs[v] = None
            continue
        m = torch.from_numpy(ctx.matrix_get(lam, w.tree.branch_length[v], msize)).to(dev)
        keep.append(m)
        ptrs[v] = m.data_ptr()
    parent = np.ascontiguousarray(w.tree.parent, dtype=np.int32)
    d_counts = torch.from_numpy(np.ascontiguousarray(w.families.counts, dtype=np.int32)).to(dev)
    d_prior = torch.from_numpy(prior).to(dev)
    F, nl = w.families.counts.shape
    d_out = torch.empty(F, dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(dev)
    lib = _lib.load()
    args = (w.tree.n_nodes, parent.ctypes.data, ctypes.cast(ptrs, ctypes.c_void_p), msize, d_counts.data_ptr())
    for call in range(2):
        d_out.fill_(float("nan"))
        torch.cuda.synchronize()
        rc = lib.cafe_prune_fp64_noalloc(*args, F, nl, S, R, d_prior.data_ptr(), len(prior), scaled,
                                         d_out.data_ptr(), stream.cuda_stream)
        assert rc == 0, f"call {call}: status {rc}"
        stream.synchronize()
        got = d_out.cpu().numpy()
        assert np.all(np.isfinite(got)), f"call {call}"
        rel = np.abs(got - expect) / np.abs(expect)
        assert rel.max() <= REL, f"call {call}: max rel err {rel.max():.3e}"
    return lib, args, nl, S, R, d_prior, prior, d_out, stream


def test_noalloc_matches_cafe_score_on_two_calls(ctx):
    lib, args, nl, S, R, d_prior, prior, d_out, stream = _run(ctx, 700, 13, 0)
    # sizes past the stated maximum are refused before any launch
    rc = lib.cafe_prune_fp64_noalloc(*args, (1 << 18) + 1, nl, S, R, d_prior.data_ptr(), len(prior), 0,
                                     d_out.data_ptr(), stream.cuda_stream)
    assert rc == 6


def test_noalloc_ctas_walk_several_tiles(ctx):
    """20,000 families = 625 tiles; the static array's node-vector region
    holds fewer CTAs than that at S = 170, so CTAs reuse their slice of the
    shared array tile after tile."""
    _run(ctx, 20000, 14, 0)


def test_noalloc_scaled_matches_scaled_oracle(ctx):
    _run(ctx, 20000, 15, 1)
