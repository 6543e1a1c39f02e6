"""The no-allocation entry point, cafe_prune_fp64_noalloc.

Some callers cannot call cudaMalloc (a host framework whose own pool owns
every device allocation, a serving loop that must not allocate per request);
this entry point runs the FP64 pruning kernel with its working space in a
static device array and only the caller's buffers for inputs and outputs.

The test calls it through the C ABI twice in a row and checks both results
against the existing entry point (cafe_score, FP64_REF, base model) at the
parity tolerance of the FP64 path, 1e-10 relative per family. It lives in a
file of its own, collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL = 1e-10


def test_noalloc_matches_cafe_score_on_two_calls():
    import torch
    from cafe5_gb300 import _lib
    from cafe5_gb300.engine import Context
    from cafe5_gb300.families import global_bounds
    from cafe5_gb300.inputs import RootPrior
    from cafe5_gb300.synth import workload

    w = workload(0, n_families=700, seed=13)
    S, R = global_bounds(w.families)
    prior = RootPrior.uniform(R).vector()
    lam = 0.0031
    ctx = Context()
    try:
        tid = ctx.upload_tree(w.tree)
        sid = ctx.upload_families(tid, w.families.counts)
        ctx.set_prior(prior)
        ctx.set_error_model(None)
        expect = ctx.score(tid, sid, [lam], S=S, R=R, precision="fp64_ref", dedupe=False).family_lnl

        # the same matrices, in caller-owned device memory
        msize = max(R, S) + 1
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
        for call in range(2):
            d_out.fill_(float("nan"))
            torch.cuda.synchronize()
            rc = lib.cafe_prune_fp64_noalloc(w.tree.n_nodes, parent.ctypes.data, ctypes.cast(ptrs, ctypes.c_void_p),
                                             msize, d_counts.data_ptr(), F, nl, S, R, d_prior.data_ptr(), len(prior),
                                             0, d_out.data_ptr(), stream.cuda_stream)
            assert rc == 0, f"call {call}: status {rc}"
            stream.synchronize()
            got = d_out.cpu().numpy()
            rel = np.abs(got - expect) / np.abs(expect)
            assert np.all(np.isfinite(got)), f"call {call}"
            assert rel.max() <= REL, f"call {call}: max rel err {rel.max():.3e}"

        # sizes past the stated maximum are refused before any launch
        rc = lib.cafe_prune_fp64_noalloc(w.tree.n_nodes, parent.ctypes.data, ctypes.cast(ptrs, ctypes.c_void_p),
                                         msize, d_counts.data_ptr(), (1 << 18) + 1, nl, S, R, d_prior.data_ptr(),
                                         len(prior), 0, d_out.data_ptr(), stream.cuda_stream)
        assert rc == 6
    finally:
        ctx.close()
