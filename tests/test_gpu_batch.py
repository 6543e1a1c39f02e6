"""Batched candidate scoring (cafe_score_batch): B candidate parameter
vectors over one tree and family set in the same launches.

Bars (stated per test):
  * FP64_REF and FP64_BINNED: each batched result is bit-identical to the
    same request scored alone, and the reference's golden -lnL is met to
    1e-10 relative;
  * MIXED_TF32X3: each batched result is within 1e-6 relative per family of
    the FP64_BINNED value; a candidate's results equal its results alone
    except for families that another candidate flagged for the FP64
    recompute (then within 1e-6);
  * a candidate the reference rejects (lambda <= 0, saturation) scores +inf
    and leaves the others unchanged."""
import math

import numpy as np
import pytest

from golden_cases import load_cases

pytestmark = pytest.mark.gpu

CASES = {c.name: c for c in load_cases()}


@pytest.fixture(scope="module")
def ctx():
    from cafe5_gb300.engine import Context
    c = Context()
    yield c
    c.close()


def _setup(ctx, tree, counts, lam_idx=None, prior=None, err=None):
    tid = ctx.upload_tree(tree, lam_idx)
    sid = ctx.upload_families(tid, counts)
    if prior is not None:
        ctx.set_prior(prior)
    ctx.set_error_model(err)
    return tid, sid


def _alone(ctx, tid, sid, cand, **kw):
    ck = dict(kw)
    for key in ("multipliers", "cat_probs"):
        if key in cand:
            ck[key] = cand[key]
    return ctx.score(tid, sid, cand["lambdas"], **ck)


@pytest.mark.parametrize("name,dedupe", [("syn_gamma_24taxa_k4", False), ("syn_base_12taxa", True),
                                         ("syn_multilambda_error_32taxa", False)])
@pytest.mark.parametrize("precision", ["fp64_ref", "fp64_binned"])
def test_fp64_batch_is_bit_identical_to_alone(ctx, name, dedupe, precision):
    case = CASES[name]
    gamma = case.model == 1
    prior = np.zeros(max(len(case.prior), 700))
    prior[:len(case.prior)] = case.prior
    tid, sid = _setup(ctx, case.tree, case.counts, case.lambda_of_node, prior, case.err_rows)
    kw = dict(model=case.model, lambda_kind=case.lambda_kind, use_error_model=case.err_rows is not None,
              precision=precision, dedupe=dedupe)
    if precision == "fp64_ref":
        kw.update(S=case.S, R=case.R)
    base = dict(lambdas=case.lambdas)
    if gamma:
        base.update(multipliers=case.multipliers, cat_probs=case.cat_probs)
    cands = [base]
    for f in (0.7, 1.3, -1.0, 1.05):
        c = dict(base)
        c["lambdas"] = [x * f for x in case.lambdas]
        cands.append(c)
    if gamma:
        c = dict(base)
        c["multipliers"] = [m * 1.1 for m in case.multipliers]
        cands.append(c)
    got = ctx.score_batch(tid, sid, cands, want_categories=True, **kw)
    for i, cand in enumerate(cands):
        one = _alone(ctx, tid, sid, cand, want_categories=True, **kw)
        if cand["lambdas"][0] < 0:
            assert got[i].total == math.inf and one.total == math.inf
            continue
        assert got[i].total == one.total or (math.isnan(got[i].total) and math.isnan(one.total)), i
        assert np.array_equal(got[i].family_lnl, one.family_lnl, equal_nan=True), i
        assert np.array_equal(got[i].category_lnl, one.category_lnl, equal_nan=True), i
        assert got[i].status == one.status
    if precision == "fp64_ref" and not math.isinf(case.total):
        assert abs(got[0].total - case.total) <= 1e-10 * abs(case.total)
    ctx.free_families(sid)


def test_mixed_batch_config3_shape(ctx):
    """16 candidate (lambda, alpha) vectors x K=8 x 1,500 families on the
    48-taxon tree (the config-3 shape at test size)."""
    from cafe5_gb300.inputs import RootPrior, discrete_gamma
    from cafe5_gb300.synth import workload
    w = workload(3, n_families=1500, seed=31)
    prior = RootPrior.uniform(400).vector()
    tid, sid = _setup(ctx, w.tree, w.families.counts, prior=prior)
    rng = np.random.default_rng(5)
    cands = []
    # lambda x (largest multiplier) x (longest branch, ~157) stays below 1:
    # a saturated category would make every family fail (+inf)
    for _ in range(16):
        lam = float(0.0008 * np.exp(rng.normal(0, 0.2)))
        alpha = float(0.8 * np.exp(rng.normal(0, 0.2)))
        p, m = discrete_gamma(alpha, 8)
        cands.append(dict(lambdas=[lam], multipliers=m, cat_probs=p))
    kw = dict(model=1)
    mixed = ctx.score_batch(tid, sid, cands, precision="mixed_tf32x3", **kw)
    fp64 = ctx.score_batch(tid, sid, cands, precision="fp64_binned", **kw)
    for i, cand in enumerate(cands):
        a, b = fp64[i], mixed[i]
        fin = np.isfinite(a.family_lnl)
        rel = np.abs(b.family_lnl[fin] - a.family_lnl[fin]) / np.abs(a.family_lnl[fin])
        assert rel.max() <= 1e-6, (i, rel.max())
        assert abs(b.total - a.total) <= 1e-6 * abs(a.total)
        alone = _alone(ctx, tid, sid, cand, precision="mixed_tf32x3", **kw)
        d = np.abs(alone.family_lnl - b.family_lnl) / np.abs(a.family_lnl)
        assert d.max() <= 1e-6
        same = alone.family_lnl == b.family_lnl
        assert same.mean() >= 0.99
    ctx.free_families(sid)


def test_mixed_batch_with_a_rejected_candidate(ctx):
    from cafe5_gb300.inputs import RootPrior
    from cafe5_gb300.synth import workload
    w = workload(1, n_families=800, seed=32)
    tid, sid = _setup(ctx, w.tree, w.families.counts, prior=RootPrior.uniform(400).vector())
    good = dict(lambdas=[0.002], multipliers=w.multipliers, cat_probs=w.cat_probs)
    sat = dict(lambdas=[0.5], multipliers=w.multipliers, cat_probs=w.cat_probs)      # lambda * t > 1
    neg = dict(lambdas=[-0.001], multipliers=w.multipliers, cat_probs=w.cat_probs)
    got = ctx.score_batch(tid, sid, [sat, good, neg], model=1, precision="mixed_tf32x3")
    one = _alone(ctx, tid, sid, good, model=1, precision="mixed_tf32x3")
    assert got[0].total == math.inf and got[0].status == 3
    assert got[2].total == math.inf
    assert np.array_equal(got[1].family_lnl, one.family_lnl)
    assert got[1].total == one.total
    ctx.free_families(sid)


def test_batch_rejects_mismatched_requests(ctx):
    from cafe5_gb300._lib import CafeError
    from cafe5_gb300.inputs import RootPrior
    from cafe5_gb300.synth import workload
    w = workload(0, n_families=100, seed=33)
    tid, sid = _setup(ctx, w.tree, w.families.counts, prior=RootPrior.uniform(100).vector())
    reqs = [dict(lambdas=[0.002]), dict(lambdas=[0.003])]
    with pytest.raises(CafeError):
        # FP64_REF bounds differ between the two requests
        from cafe5_gb300 import _lib
        import ctypes as C
        r0, k0 = ctx.make_request(tid, sid, [0.002], S=80, R=40)
        r1, k1 = ctx.make_request(tid, sid, [0.003], S=90, R=40)
        arr = (_lib.Request * 2)(r0, r1)
        res = (_lib.Result * 2)()
        ctx._check(ctx.lib.cafe_score_batch(ctx.h, C.cast(arr, C.c_void_p), 2, C.cast(res, C.c_void_p)))
    ctx.free_families(sid)


def test_serving_merges_requests_and_matches_alone(ctx):
    """Continuous batching: requests from many optimizers queued together on
    two family sets (mixed precision and FP64) are merged into batched
    launches where compatible; every result equals the request scored alone
    (bit for bit in FP64, within 1e-6 relative per family in mixed
    precision)."""
    from cafe5_gb300.inputs import RootPrior
    from cafe5_gb300.synth import workload
    w = workload(1, n_families=1500, seed=34)
    w0 = workload(0, n_families=400, seed=35)
    ctx.set_prior(RootPrior.uniform(400).vector())
    ctx.set_error_model(None)
    t1 = ctx.upload_tree(w.tree)
    s1 = ctx.upload_families(t1, w.families.counts)
    t0 = ctx.upload_tree(w0.tree)
    s0 = ctx.upload_families(t0, w0.families.counts)
    jobs = []
    for i in range(24):
        if i % 3 == 2:
            jobs.append((t0, s0, dict(lambdas=[0.002 * (1 + 0.03 * i)], model=0, precision="fp64_binned")))
        else:
            jobs.append((t1, s1, dict(lambdas=[0.002 * (1 + 0.01 * i)], model=1, multipliers=w.multipliers,
                                      cat_probs=w.cat_probs, precision="mixed_tf32x3")))
    handles = []
    for t, s, kw in jobs:
        kw = dict(kw)
        lam = kw.pop("lambdas")
        handles.append(ctx.submit(t, s, lam, **kw))
    got = [ctx.poll(h, -1) for h in handles]
    for (t, s, kw), g in zip(jobs, got):
        kw = dict(kw)
        lam = kw.pop("lambdas")
        one = ctx.score(t, s, lam, **kw)
        if kw["precision"] == "fp64_binned":
            assert np.array_equal(g.family_lnl, one.family_lnl) and g.total == one.total
        else:
            rel = np.abs(g.family_lnl - one.family_lnl) / np.abs(one.family_lnl)
            assert rel.max() <= 1e-6
    ctx.free_families(s1)
    ctx.free_families(s0)


def test_serving_large_requests_overlap_on_device(ctx):
    """Requests that each fill the device (10,000 families x K = 4 = 40,000
    family-categories, more than one 128-family tile per SM) on two family
    sets, so no two share a launch: the serving loop keeps two batches in
    flight on its streams and their device work overlaps (overlap_ms, the
    summed intersections of the batches' event intervals, grows), and every
    result equals the request scored alone (within 1e-6 relative per
    family)."""
    from cafe5_gb300.inputs import RootPrior
    from cafe5_gb300.synth import workload
    w = workload(1, n_families=10000, seed=36)
    ctx.set_prior(RootPrior.uniform(400).vector())
    ctx.set_error_model(None)
    tid = ctx.upload_tree(w.tree)
    sets = [ctx.upload_families(tid, w.families.counts),
            ctx.upload_families(tid, np.ascontiguousarray(w.families.counts[::-1]))]
    kw = dict(model=1, multipliers=w.multipliers, cat_probs=w.cat_probs, precision="mixed_tf32x3")
    jobs = [(sets[i % 2], [0.002 * (1 + 0.01 * i)]) for i in range(8)]
    before = ctx.serving_stats()["overlap_ms"]
    handles = [ctx.submit(tid, s, lam, **kw) for s, lam in jobs]
    got = [ctx.poll(h, -1) for h in handles]
    st = ctx.serving_stats()
    assert st["overlap_ms"] > before, st
    for (s, lam), g in zip(jobs, got):
        one = ctx.score(tid, s, lam, **kw)
        rel = np.abs(g.family_lnl - one.family_lnl) / np.abs(one.family_lnl)
        assert rel.max() <= 1e-6
    for s in sets:
        ctx.free_families(s)


def test_autotune_picks_shapes_and_keeps_results(ctx):
    """cafe_autotune times the candidate launch shapes of every tensor-core
    S-bin and keeps the fastest; the scores do not depend on the shape (bit
    for bit)."""
    from cafe5_gb300.inputs import RootPrior
    from cafe5_gb300.families import bin_families
    from cafe5_gb300.synth import workload
    w = workload(1, n_families=3000, seed=36)
    tid, sid = _setup(ctx, w.tree, w.families.counts, prior=RootPrior.uniform(400).vector())
    cands = [dict(lambdas=[0.002], multipliers=w.multipliers, cat_probs=w.cat_probs),
             dict(lambdas=[0.0021], multipliers=w.multipliers, cat_probs=w.cat_probs)]
    before = ctx.score_batch(tid, sid, cands, model=1, precision="mixed_tf32x3")
    tuned = ctx.autotune(tid, sid, cands, reps=2, model=1)
    Wb, _, _ = bin_families(w.families)
    assert sorted(t["width"] for t in tuned) == sorted(set(int(x) for x in Wb if x <= 256))
    for t in tuned:
        assert 1 <= t["ctas_per_sm"] <= 16 and 1 <= t["stages"] <= 4 and t["ms"] > 0
    after = ctx.score_batch(tid, sid, cands, model=1, precision="mixed_tf32x3")
    for a, b in zip(before, after):
        assert np.array_equal(a.family_lnl, b.family_lnl) and a.total == b.total
    ctx.free_families(sid)


def test_graph_replay_matches_direct_launches(ctx):
    """The pruning phase replayed from a captured CUDA graph gives the same
    bits as direct launches (profiling forces direct launches), across many
    steps at new lambdas that reuse the graph."""
    from cafe5_gb300.inputs import RootPrior
    from cafe5_gb300.synth import workload
    w = workload(1, n_families=2500, seed=37)
    tid, sid = _setup(ctx, w.tree, w.families.counts, prior=RootPrior.uniform(400).vector())
    kw = dict(model=1, precision="mixed_tf32x3")
    for i in range(5):
        cands = [dict(lambdas=[0.002 * (1 + 1e-4 * i + 0.01 * b)], multipliers=w.multipliers, cat_probs=w.cat_probs)
                 for b in range(3)]
        graph = ctx.score_batch(tid, sid, cands, **kw)        # graph path (captured once, then replayed)
        ctx.profile(True)
        direct = ctx.score_batch(tid, sid, cands, **kw)       # direct launches
        ctx.profile_read()
        ctx.profile(False)
        for g, d in zip(graph, direct):
            assert np.array_equal(g.family_lnl, d.family_lnl) and g.total == d.total
    ctx.free_families(sid)


def test_families_update_rebuilds_derived_tables(ctx):
    """cafe_families_update: new counts (a larger maximum moves families
    into wider S-bins) score like a fresh upload; re-sending unchanged
    counts leaves the results unchanged."""
    from cafe5_gb300.families import global_bounds
    from cafe5_gb300.inputs import RootPrior
    from cafe5_gb300.synth import workload
    w = workload(1, n_families=500, seed=31)
    counts = w.families.counts.copy()
    tid = ctx.upload_tree(w.tree)
    sid = ctx.upload_families(tid, counts)
    ctx.set_prior(RootPrior.uniform(400).vector())
    ctx.set_error_model(None)
    kw = dict(model=1, multipliers=w.multipliers, cat_probs=w.cat_probs, precision="fp64_binned")
    a = ctx.score(tid, sid, [0.002], **kw)
    ctx.update_families(sid, counts)                 # unchanged
    b = ctx.score(tid, sid, [0.002], **kw)
    assert np.array_equal(a.family_lnl, b.family_lnl)
    bigger = counts.copy()
    bigger[::7, 0] += 60                             # wider bins for every 7th family
    ctx.update_families(sid, bigger)
    c = ctx.score(tid, sid, [0.002], **kw)
    sid2 = ctx.upload_families(tid, bigger)
    d = ctx.score(tid, sid2, [0.002], **kw)
    assert np.array_equal(c.family_lnl, d.family_lnl)
    assert not np.array_equal(c.family_lnl, a.family_lnl)
    for pr in ("fp64_ref",):
        S, R = global_bounds(type(w.families)(w.families.ids, bigger))
        e = ctx.score(tid, sid, [0.002], model=1, multipliers=w.multipliers, cat_probs=w.cat_probs,
                      precision=pr, S=S, R=R)
        f = ctx.score(tid, sid2, [0.002], model=1, multipliers=w.multipliers, cat_probs=w.cat_probs,
                      precision=pr, S=S, R=R)
        assert np.array_equal(e.family_lnl, f.family_lnl)


def test_matrix_cache_recycling_keeps_results():
    """A context whose matrix cache is capped below one call's matrices
    starts the cache over in the same device memory at every call, while the
    device-pointer calls issued before it may still be reading theirs (no
    synchronisation: its builds wait for those calls). Every call's results
    equal the same request scored in a context with the default cache, bit
    for bit, in both precisions, and the cache never holds more than one
    call's matrices."""
    import torch
    from cafe5_gb300.engine import Context
    from cafe5_gb300.inputs import RootPrior
    from cafe5_gb300.synth import workload
    w = workload(1, n_families=2000, seed=44)
    small, ref = Context(matrix_cache_bytes=16 << 20), Context()
    try:
        prior = RootPrior.uniform(400).vector()
        t1, s1 = _setup(small, w.tree, w.families.counts, prior=prior)
        t2, s2 = _setup(ref, w.tree, w.families.counts, prior=prior)
        F = w.families.n_families
        B, steps = 4, 6
        dev = torch.device("cuda", 0)
        stream = torch.cuda.Stream(dev)
        for precision in ("mixed_tf32x3", "fp64_binned"):
            kw = dict(model=1, precision=precision)
            cands = [[dict(lambdas=[0.002 * (1 + 0.01 * b) * (1 + 1e-5 * (s + 1))], multipliers=w.multipliers,
                           cat_probs=w.cat_probs) for b in range(B)] for s in range(steps)]
            fam = [torch.empty(B * F, dtype=torch.float64, device=dev) for _ in range(steps)]
            tot = [torch.empty(B, dtype=torch.float64, device=dev) for _ in range(steps)]
            with torch.cuda.stream(stream):
                for s in range(steps):
                    small.score_batch_device(t1, s1, cands[s], fam[s].data_ptr(), tot[s].data_ptr(),
                                             stream.cuda_stream, **kw)
            stream.synchronize()
            assert 0 < small.cache_size() <= B * len(w.multipliers) * len(w.tree.parent)
            for s in range(steps):
                want = ref.score_batch(t2, s2, cands[s], **kw)
                got = fam[s].view(B, F).cpu().numpy()
                got_tot = tot[s].cpu().numpy()
                for b in range(B):
                    assert np.array_equal(got[b], want[b].family_lnl), (precision, s, b)
                    assert got_tot[b] == want[b].total, (precision, s, b)
    finally:
        small.close()
        ref.close()


def test_back_to_back_device_calls_match_synchronous_calls(ctx):
    """Device-pointer calls issued back to back build each call's matrices on
    a build stream while the previous call still prunes, and alternate
    between two workspaces; every call's per-family lnL and total equal the
    same request scored synchronously (matrices built in line), bit for bit,
    in both precisions."""
    import torch
    from cafe5_gb300.inputs import RootPrior
    from cafe5_gb300.synth import workload
    w = workload(1, n_families=3000, seed=38)
    tid, sid = _setup(ctx, w.tree, w.families.counts, prior=RootPrior.uniform(400).vector())
    F = w.families.n_families
    B, steps = 4, 6
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)
    for precision in ("mixed_tf32x3", "fp64_binned"):
        kw = dict(model=1, precision=precision)
        cands = [[dict(lambdas=[0.002 * (1 + 0.01 * b) * (1 + 1e-5 * (s + 1) + (0.1 if precision == "fp64_binned" else 0))],
                       multipliers=w.multipliers, cat_probs=w.cat_probs) for b in range(B)] for s in range(steps)]
        fam = [torch.empty(B * F, dtype=torch.float64, device=dev) for _ in range(steps)]
        tot = [torch.empty(B, dtype=torch.float64, device=dev) for _ in range(steps)]
        with torch.cuda.stream(stream):
            for s in range(steps):
                ctx.score_batch_device(tid, sid, cands[s], fam[s].data_ptr(), tot[s].data_ptr(), stream.cuda_stream,
                                       **kw)
        stream.synchronize()
        for s in range(steps):
            ref = ctx.score_batch(tid, sid, cands[s], **kw)
            got = fam[s].view(B, F).cpu().numpy()
            got_tot = tot[s].cpu().numpy()
            for b in range(B):
                assert np.array_equal(got[b], ref[b].family_lnl), (precision, s, b)
                assert got_tot[b] == ref[b].total, (precision, s, b)
    ctx.free_families(sid)
