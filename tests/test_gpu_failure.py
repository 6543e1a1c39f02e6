"""Failure detection without a GPU fault: a bounded wait of the tensor-core
kernel made to run out on purpose (cafe_debug_set, CAFE_DEBUG_TC_WAIT_LIMIT
= 1: the wait for a node's GEMMs gives up at once). The kernel must record
the time-out, drain its own copies and MMAs (those waits keep their full
bound), free TMEM and return; the call reports CAFE_ERR_TIMEOUT; the next
call on the same context succeeds with the same results as before."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_tensor_core_wait_time_out_is_reported_and_the_context_recovers():
    from cafe5_gb300 import _lib
    from cafe5_gb300.engine import Context
    from cafe5_gb300.inputs import RootPrior
    from cafe5_gb300.synth import workload
    w = workload(1, n_families=3000, seed=31)
    ctx = Context()
    try:
        tid = ctx.upload_tree(w.tree)
        sid = ctx.upload_families(tid, w.families.counts)
        ctx.set_prior(RootPrior.uniform(150).vector(264))
        ctx.set_error_model(None)
        kw = dict(model=1, multipliers=w.multipliers, cat_probs=w.cat_probs, precision="mixed_tf32x3")
        before = ctx.score(tid, sid, [0.002], **kw)
        ctx.debug_set(_lib.DEBUG_TC_WAIT_LIMIT, 1)
        with pytest.raises(_lib.CafeError) as e:
            ctx.score(tid, sid, [0.002], **kw)
        assert e.value.code == 5          # CAFE_ERR_TIMEOUT
        ctx.debug_set(_lib.DEBUG_TC_WAIT_LIMIT, 0)
        after = ctx.score(tid, sid, [0.002], **kw)
        assert after.total == before.total
        assert np.array_equal(after.family_lnl, before.family_lnl)
        # the FP64 path on the same context is untouched as well
        r = ctx.score(tid, sid, [0.002], model=1, multipliers=w.multipliers, cat_probs=w.cat_probs,
                      precision="fp64_binned")
        assert np.isfinite(r.total)
    finally:
        ctx.close()
