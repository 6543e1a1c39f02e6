"""Benchmark of the CAFE5 likelihood hot path on GB300.

Workload: 24-taxon Yule tree (root age 150), 10,000 families per GPU, gamma
model with K = 4 categories (alpha = 0.5): the gamma configuration the
headline metric is quoted on. Synthetic and seeded (no public dataset exists
for this path). A "step" is one batched score of B candidate parameter
vectors (lambda and alpha of B concurrent optimizer steps) over every
family: the transition matrices of the step's new lambdas are built, every
family is pruned in every category of every candidate, and each candidate's
-lnL is reduced. One family-lnL evaluation is one family's lnL for one
candidate with all K categories, so a step is B x F evaluations.

  value        mixed-precision (TF32x3 tensor-core) evals/s with inputs
               resident in HBM (cafe_score_batch_device), CUDA events on the
               launching stream, L2 flushed between steps (256 MB write)
  fp64_paths   the plain FP64 GPU paths on the same steps: FP64_BINNED (same
               per-family state bins) and FP64_REF (the reference's global
               bounds); `mixed_over_fp64` is value / FP64_BINNED
  e2e          the same metric through the public API with host buffers:
               cafe_families_update from pinned host memory, cafe_score_batch
               copying every candidate's per-family lnL back; host clock
  serving      closed-loop clients (one optimizer each) submitting
               single-candidate requests to the continuous-batching loop
               (cafe_submit / cafe_poll): throughput, p50 and p99 latency
  accuracy     max relative |dlnL| per family of the mixed path vs FP64_BINNED

Under torchrun each rank scores its own shard of world x 10,000 families
(weak scaling; the candidates' totals are combined across ranks).

`--impl reference` times the reference algorithm on the host cores instead
(the CPU oracle that restates it; the compiled reference does not exist on
the GPU machine).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "family-lnL evals/s, batched mixed-prec vs plain FP64 GPU (dLnL<=1e-6); p99 ms"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default=os.environ.get("CAFE_BENCH_PRECISION", "mixed_tf32x3"))
    ap.add_argument("--families", type=int, default=10000, help="families per GPU")
    ap.add_argument("--candidates", type=int, default=16, help="candidate parameter vectors per step")
    ap.add_argument("--cpu-seconds", type=float, default=8.0)
    ap.add_argument("--fp64-steps", type=int, default=3)
    ap.add_argument("--serving-clients", type=int, default=8)
    ap.add_argument("--serving-requests", type=int, default=12, help="requests per client")
    ap.add_argument("--serving-optimizers", type=int, default=256,
                    help="clients of the config-4 request stream (0: skip)")
    ap.add_argument("--no-reconstruct", dest="reconstruct", action="store_false",
                    help="skip the ancestral-reconstruction measurement")
    ap.add_argument("--no-pvalues", dest="pvalues", action="store_false",
                    help="skip the p-value measurement")
    ap.add_argument("--no-config3", dest="config3", action="store_false",
                    help="skip the config-3 batched-candidates measurement")
    ap.add_argument("--no-config0", dest="config0", action="store_false",
                    help="skip the config-0 (plain FP64 base model, dedupe, Nelder-Mead fit) measurement")
    ap.add_argument("--no-config2", dest="config2", action="store_false",
                    help="skip the config-2 (two lambdas, error model, S-bins to 512) measurement")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default tensor-core launch shapes (no cafe_autotune before the warm-up)")
    ap.add_argument("--profile-config2", action="store_true",
                    help="two batched scores of the config-2 workload and nothing else (a small case for ncu)")
    ap.add_argument("--profile-only", action="store_true",
                    help="two batched scores of the workload and nothing else (a small case for ncu captures)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload(n_families: int):
    from cafe5_gb300.synth import workload as wl
    return wl(1, n_families=n_families, seed=0)


def workload_cfg(config: int, n_families=None):
    from cafe5_gb300.synth import workload as wl
    return wl(config, n_families=n_families, seed=0)


def global_bounds(fams):
    from cafe5_gb300.families import global_bounds as gb
    return gb(fams)


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            import tempfile
            fd, self.path = tempfile.mkstemp(prefix="cafe_bench_clocks_", suffix=".csv")
            self.f = os.fdopen(fd, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in open(self.path):
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        try:
            os.unlink(self.path)
        except OSError:
            pass
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def fp64_peak_tflops(torch, dev):
    """FP64 denominator measured here: cuBLAS DGEMM 4096^3, best of 5."""
    a = torch.randn(4096, 4096, dtype=torch.float64, device=dev)
    b = torch.randn(4096, 4096, dtype=torch.float64, device=dev)
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return 2 * 4096 ** 3 / (best / 1e3) / 1e12


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def cpu_baseline(w, S, R, seconds: float, threads: int):
    """The reference algorithm on the host cores: the compiled reference is
    not available on this machine's architecture, so the CPU oracle (a
    line-by-line restatement: the reference's lgamma tables and per-term
    exp/pow matrices, dense products, OpenMP over families) is timed on a
    bounded family sample of one candidate."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    ta = oracle.TreeArrays.from_tree(w.tree)
    prior = uniform_prior(R)
    counts = w.families.counts
    n = 250
    lam = w.true_lambda
    done_fam, t_total, reps = 0, 0.0, 0
    while True:
        sample = counts[:n]
        t0 = time.perf_counter()
        oracle.score(ta, sample, [lam * (1 + 1e-4 * reps)], model=1, multipliers=w.multipliers,
                     cat_probs=w.cat_probs, prior=prior, S=S, R=R, dedupe=False, n_threads=threads)
        dt = time.perf_counter() - t0
        reps += 1
        if dt < seconds / 4 and n < len(counts):
            n = min(len(counts), n * 4)
            continue
        done_fam += len(sample)
        t_total += dt
        if t_total >= seconds or reps > 50:
            break
    return {"value": done_fam / t_total, "unit": "family-lnL evals/s", "cores": threads, "kind": "port",
            "sample": f"{len(sample)} of {len(counts)} families x K={len(w.multipliers)}, global S={S} R={R}, "
                      f"{done_fam // len(sample)} evaluations, matrices rebuilt each evaluation"}


def uniform_prior(R: int, n: int = 0) -> np.ndarray:
    """The uniform root prior over sizes 1..R, float-rounded as
    root_equilibrium_distribution::compute returns it, zero past R (the same
    vector as inputs.RootPrior.uniform(R).vector(n), built without the
    library so the reference arm loads nothing of the product)."""
    v = np.zeros(max(n, R))
    v[:R] = float(np.float32(1.0) / np.float32(R))
    return v


def candidates(w, B: int, step: int, gamma=None):
    """B candidate (lambda, alpha) vectors around the simulating values, as B
    concurrent optimizer steps would propose them; new lambdas every step.
    `gamma(alpha, K)` gives (probabilities, multipliers): the library's
    get_gamma by default, the oracle's in the reference arm."""
    if gamma is None:
        from cafe5_gb300.inputs import discrete_gamma as gamma
    out = []
    for b in range(B):
        alpha = w.alpha * (1.0 + 0.02 * b)
        probs, mult = gamma(alpha, len(w.multipliers))
        # every step's lambdas are new (new matrices) but stay within 1 % of
        # the simulating value: far from the saturation bound lambda*m*t < 1
        out.append(dict(lambdas=[w.true_lambda * (1.0 + 0.01 * b) * (1.0 + 1e-6 * (step % 10000))],
                        multipliers=mult, cat_probs=probs))
    return out


def shared_config(w, families_per_gpu: int, B: int, world: int):
    """The `config` object both arms print: the workload, not the way an arm
    computes it (precision, bins and launch shapes are reported beside it)."""
    return {"workload": w.name, "families_per_gpu": families_per_gpu, "taxa": len(w.tree.leaves), "K": len(w.multipliers),
            "alpha": w.alpha, "candidates_per_step": B,
            "step": f"{B} candidate (lambda, alpha) vectors x every family x K categories; new lambdas each "
                    "step (transition matrices rebuilt)",
            "inputs": "GPU arm: counts resident in HBM, L2 flushed between timed steps (256 MB write on the "
                      "stream, inside the timed region); CPU arm: counts in host memory",
            "parallelism": f"families sharded x{world}"}


def profiled_traffic(kernel: str, workload_name: str):
    """DRAM bytes per launch of `kernel` from the committed ncu summary of
    this workload (profiles/), or None when no capture covers it."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        d = json.load(open(path))
        e = d.get(kernel, {})
        if e.get("workload") == workload_name:
            return e.get("bytes_per_launch"), e.get("source")
    except Exception:
        pass
    return None, None


def run_reference(args):
    """The reference algorithm timed on the host cores, on the GPU arm's
    workload and step: the same families, the same B candidates per step
    with new lambdas each step, K = 4 gamma categories, at the reference's
    global bounds S and R (what it computes; the GPU arm bins S per family).
    Only the oracle is loaded -- the product library is never mapped."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from cafe5_gb300.families import global_bounds as gb
    from cafe5_gb300.synth import workload as wl
    w = wl(1, n_families=args.families, seed=0, gamma=oracle.discrete_gamma)
    S, R = gb(w.families)
    threads = os.cpu_count() or 1
    B = max(1, args.candidates)
    ta = oracle.TreeArrays.from_tree(w.tree)
    prior = uniform_prior(R)
    counts = np.ascontiguousarray(w.families.counts)
    F = counts.shape[0]

    def step(i, n, off):
        rows = counts[off:off + n] if off + n <= F else np.concatenate([counts[off:], counts[:off + n - F]])
        tot = []
        for c in candidates(w, B, i, gamma=oracle.discrete_gamma):
            t, _, _ = oracle.score(ta, rows, c["lambdas"], model=1, multipliers=c["multipliers"],
                                   cat_probs=c["cat_probs"], prior=prior, S=S, R=R, dedupe=False, n_threads=threads)
            tot.append(t)
        return tot

    # full steps unless K + W of them would take more than ~4 minutes: then
    # each step scores every candidate on a rotating window of families
    n = F
    budget = 240.0
    for i in range(max(0, args.warmup)):
        t0 = time.perf_counter()
        step(-1 - i, n, 0)
        dt = time.perf_counter() - t0
        if i == 0 and dt * (args.steps + args.warmup) > budget:
            n = max(100, min(F, int(F * budget / (dt * (args.steps + args.warmup)))))
    steps = max(1, args.steps)
    t0 = time.perf_counter()
    for i in range(steps):
        totals = step(i, n, (i * n) % F)
        if i == 0:
            first = totals[0]
    total_s = time.perf_counter() - t0
    value = B * n * steps / total_s
    sample = (f"every step: {B} candidates x {n} of {F} families x K=4 at global S={S} R={R}, matrices rebuilt "
              f"per candidate, no dedupe (the gamma model has none)" +
              ("" if n == F else "; families in rotating windows to bound the run"))
    line = {"metric": METRIC, "value": value, "unit": "family-lnL evals/s", "n_gpus": args.gpus,
            "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * total_s / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": shared_config(w, args.families, B, 1),
            "bounds": {"S": S, "R": R, "kind": "global (the reference's max_family_size / max_root_family_size)"},
            "cpu_baseline": {"value": value, "unit": "family-lnL evals/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "family-lnL evals/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "neg_lnl_check": {"step": 0, "candidate": 0, "value": first,
                              "families": "all" if n == F else f"the first {n}"}}
    print(json.dumps(line))
    return 0


def time_steps(ctx, torch, stream, flush, tid, sid, w, B, steps, warmup, d_fam, d_tot, kw, step0=0, make=None):
    """Device time (ms) of `steps` batched scores issued back to back after
    `warmup` untimed ones: the host prepares step i + 1 while the device
    runs step i, as a deployment's loop does. Between steps a 256 MB write
    on the same stream evicts L2; its time is inside the timed region."""
    make = make or candidates
    for i in range(warmup):
        ctx.score_batch_device(tid, sid, make(w, B, step0 - 1 - i), d_fam.data_ptr(), d_tot.data_ptr(),
                               stream.cuda_stream, **kw)
    torch.cuda.synchronize()
    if steps <= 0:
        return 0.0
    cands = [make(w, B, step0 + i) for i in range(steps)]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    flush.fill_(-1.0)
    e0.record(stream)
    for i in range(steps):
        if i:
            flush.fill_(float(i))                  # evict L2 between steps
        ctx.score_batch_device(tid, sid, cands[i], d_fam.data_ptr(), d_tot.data_ptr(), stream.cuda_stream, **kw)
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1)


def serving_phase(ctx, tid, sid, w, clients: int, per_client: int, kw):
    """Closed-loop optimizer clients on the continuous-batching loop."""
    lat = []
    lock = threading.Lock()

    def client(c):
        for r in range(per_client):
            cand = candidates(w, 1, 5000 + 100 * c + r)[0]
            t0 = time.perf_counter()
            h = ctx.submit(tid, sid, cand["lambdas"], multipliers=cand["multipliers"], cat_probs=cand["cat_probs"],
                           **kw)
            ctx.poll(h, -1)
            with lock:
                lat.append((time.perf_counter() - t0) * 1e3)

    t0 = time.perf_counter()
    ths = [threading.Thread(target=client, args=(c,)) for c in range(clients)]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    wall = time.perf_counter() - t0
    lat.sort()
    pct = lambda q: lat[min(len(lat) - 1, int(round(q * (len(lat) - 1))))]
    return {"clients": clients, "requests": len(lat), "evals_per_s": len(lat) * w.families.n_families / wall,
            "p50_ms": pct(0.5), "p99_ms": pct(0.99), "unit": "family-lnL evals/s",
            "note": "single-candidate requests from concurrent closed-loop optimizer clients, merged by the continuous-batching loop; latency submit -> done"}


def serving_stream(ctx, n_optimizers: int = 256, requests_each: int = 4, think_ms: float = 1.0, seed: int = 4):
    """The served request stream of the config-4 shape: n_optimizers
    independent Nelder-Mead clients, each on its own data set (Yule tree of
    8/16/32/64 taxa, root age 50-250; 100-100,000 families, log-uniform,
    simulated as in config 0; lambda log-uniform in [5e-4, 1e-2]; K in
    {1, 4, 8}), each submitting its next request an exponential think time
    after its previous result (Poisson arrivals). Mixed precision; one event
    loop drives every client through cafe_submit / cafe_poll. Reports
    throughput, p50/p99 latency and dlnL against FP64 on a sample."""
    from cafe5_gb300.families import FamilySet
    from cafe5_gb300.inputs import RootPrior, discrete_gamma
    from cafe5_gb300.synth import _keep_nonzero, _poisson_ge1, simulate_families, yule_tree
    rng = np.random.default_rng(seed)
    sizes = [100, 316, 1000, 3162, 10000, 31623, 100000]
    trees = {}
    for taxa in (8, 16, 32, 64):
        tree = yule_tree(taxa, float(rng.uniform(50, 250)), seed + taxa)
        root = _poisson_ge1(rng, 5.0, 130000)
        c = _keep_nonzero(simulate_families(tree, len(root), np.full(len(root), 0.0025), root, seed + 7 * taxa))
        tid = ctx.upload_tree(tree)
        sets = {n: ctx.upload_families(tid, np.ascontiguousarray(c[:n])) for n in sizes}
        trees[taxa] = (tid, sets, tree)
    ctx.set_prior(RootPrior.uniform(1100).vector())
    ctx.set_error_model(None)
    opts = []
    for i in range(n_optimizers):
        taxa = int(rng.choice([8, 16, 32, 64]))
        F = int(np.exp(rng.uniform(np.log(100), np.log(100000))))
        n = min(sizes, key=lambda x: abs(np.log(x) - np.log(F)))
        K = int(rng.choice([1, 4, 8]))
        lam = float(np.exp(rng.uniform(np.log(5e-4), np.log(1e-2))))
        kw = dict(precision="mixed_tf32x3")
        if K > 1:
            probs, mult = discrete_gamma(0.5, K)
            kw.update(model=1, multipliers=mult, cat_probs=probs)
        opts.append({"tid": trees[taxa][0], "sid": trees[taxa][1][n], "F": n, "lam": lam, "kw": kw, "left": requests_each,
                     "step": 0, "h": None, "t_sub": 0.0, "next": 0.0})
    lat, done_fam = [], 0
    t0 = time.perf_counter()
    for o in opts:
        o["next"] = t0 + rng.exponential(think_ms) / 1e3
    active = len(opts)
    while active:
        now = time.perf_counter()
        for o in opts:
            if o["h"] is None:
                if o["left"] and now >= o["next"]:
                    lam = o["lam"] * (1.0 + 1e-3 * o["step"])   # the optimizer's next candidate
                    o["h"] = ctx.submit(o["tid"], o["sid"], [lam], **o["kw"])
                    o["t_sub"] = now
            else:
                r = ctx.poll(o["h"], 0)
                if r is not None:
                    t = time.perf_counter()
                    lat.append((t - o["t_sub"]) * 1e3)
                    done_fam += o["F"]
                    o["h"] = None
                    o["left"] -= 1
                    o["step"] += 1
                    o["next"] = t + rng.exponential(think_ms) / 1e3
                    if not o["left"]:
                        active -= 1
    wall = time.perf_counter() - t0
    lat.sort()
    pct = lambda q, v=lat: v[min(len(v) - 1, int(round(q * (len(v) - 1))))]
    # open loop: requests of the same clients arriving as a Poisson process
    # at 60 % of the closed loop's request rate; latency under that load
    rate = 0.6 * len(lat) / wall
    n_open = min(600, 4 * len(opts))
    gaps = rng.exponential(1.0 / rate, n_open)
    pend, lat_open = [], []
    t1 = time.perf_counter()
    due = t1 + np.cumsum(gaps)
    i = 0
    while i < n_open or pend:
        now = time.perf_counter()
        while i < n_open and now >= due[i]:
            o = opts[int(rng.integers(len(opts)))]
            pend.append((ctx.submit(o["tid"], o["sid"], [o["lam"] * (1.0 + 1e-3 * (100 + i))], **o["kw"]), now))
            i += 1
        keep = []
        for h, ts in pend:
            if ctx.poll(h, 0) is not None:
                lat_open.append((time.perf_counter() - ts) * 1e3)
            else:
                keep.append((h, ts))
        pend = keep
    lat_open.sort()
    # accuracy on a sample of the clients' data sets: mixed vs FP64 at the same bins
    dl = 0.0
    for o in opts[:: max(1, len(opts) // 16)]:
        kw64 = dict(o["kw"], precision="fp64_binned")
        a = ctx.score(o["tid"], o["sid"], [o["lam"]], **kw64)
        b = ctx.score(o["tid"], o["sid"], [o["lam"]], **o["kw"])
        fin = np.isfinite(a.family_lnl)
        if fin.any():
            dl = max(dl, float(np.max(np.abs(b.family_lnl[fin] - a.family_lnl[fin]) / np.abs(a.family_lnl[fin]))))
    return {"optimizers": n_optimizers, "requests": len(lat), "evals_per_s": done_fam / wall,
            "p50_ms": pct(0.5), "p99_ms": pct(0.99), "unit": "family-lnL evals/s", "max_rel_dlnl_vs_fp64": dl,
            "open_loop": {"requests": len(lat_open), "arrivals_per_s": rate, "p50_ms": pct(0.5, lat_open),
                          "p99_ms": pct(0.99, lat_open)},
            "note": "config-4 shape: trees of 8/16/32/64 taxa, 100-100,000 families per request (log-uniform), "
                    "lambda log-uniform [5e-4, 1e-2], K in {1, 4, 8}. Closed loop: every client waits for its "
                    f"result, then an exponential think time ({think_ms} ms), so latency includes the queue of "
                    "all clients; open loop: Poisson arrivals at 60 % of the closed loop's rate. Latency "
                    "submit -> result"}


def config3_phase(ctx, torch, stream, flush, steps: int = 2, B: int = 64):
    """Batched optimizer scoring at the config-3 shape: 64 candidate
    (lambda, alpha) vectors x K = 8 x 20,000 families on a 48-taxon tree
    (about 64 x 8 x 94 FP64 matrices built per round). Device time of the
    batched mixed-precision call per round, and each candidate's dlnL
    against FP64 at the same bins."""
    from cafe5_gb300.inputs import RootPrior
    w = workload_cfg(3)
    F = w.families.n_families
    tid = ctx.upload_tree(w.tree)
    sid = ctx.upload_families(tid, w.families.counts)
    ctx.set_prior(RootPrior.uniform(1100).vector())
    kw = dict(model=1, precision="mixed_tf32x3")
    dev = torch.device("cuda", torch.cuda.current_device())
    d_fam = torch.empty(B * F, dtype=torch.float64, device=dev)
    d_tot = torch.empty(B, dtype=torch.float64, device=dev)
    # the tree's longest branch is 180: the largest category (m = 3.76)
    # saturates above lambda = 0.00148, where the gamma model fails almost
    # every family (+inf), so the candidates sit around lambda = 0.001
    w.true_lambda = 0.001
    ms = time_steps(ctx, torch, stream, flush, tid, sid, w, B, steps, 1, d_fam, d_tot, kw, step0=30000)
    ms64 = time_steps(ctx, torch, stream, flush, tid, sid, w, B, 1, 1, d_fam, d_tot,
                      dict(kw, precision="fp64_binned"), step0=32000)
    cands = candidates(w, B, 31000)
    cur = ctx.score_batch(tid, sid, cands, **kw)
    ref = ctx.score_batch(tid, sid, cands, model=1, precision="fp64_binned")
    per = []
    for c, r in zip(cur, ref):
        fin = np.isfinite(r.family_lnl)
        per.append(float(np.max(np.abs(c.family_lnl[fin] - r.family_lnl[fin]) / np.abs(r.family_lnl[fin])))
                   if fin.any() else 0.0)
    # one direct call on new candidates (matrices built) with per-launch events
    ctx.profile(True)
    ctx.profile_read()
    ctx.score_batch(tid, sid, candidates(w, B, 33000), **kw)
    prof = ctx.profile_read()
    ctx.profile(False)
    ctx.free_families(sid)
    return {"workload": w.name, "candidates": B, "K": 8, "families": F, "taxa": 48, "steps": steps,
            "profiled_call_ms": {k: round(v, 3) for k, v in prof.items()
                                 if k in ("matrix_ms", "prune_ms", "other_ms", "finish_ms", "host_keys_ms",
                                          "host_build_ms", "host_plan_ms", "host_total_ms")},
            "ms_per_round": ms / steps, "value": B * F * steps / (ms / 1e3), "unit": "family-lnL evals/s",
            "fp64_binned_ms_per_round": ms64, "fp64_binned_value": B * F / (ms64 / 1e3),
            "max_rel_dlnl_vs_fp64": max(per), "median_rel_dlnl_vs_fp64": float(np.median(per)),
            "finite_families": int(min(np.isfinite(r.family_lnl).sum() for r in ref)),
            "n_fallback": int(max(c.n_fallback for c in cur)),
            "note": "64 new (lambda, alpha) candidates per round around lambda = 0.001 (below the largest "
                    "category's saturation bound 0.00148 on this tree), all 512 candidate-categories in one "
                    "batched call"}


def config2_phase(ctx, torch, stream, flush, steps: int = 4, B: int = 4):
    """The two-lambda local model with the error model: a 32-taxon tree whose
    10-taxon clade runs at lambda2, epsilon 0.05, 50,000 families from a
    heavy-tailed root (95 % Poisson(4), 5 % geometric(0.02); S-bins 32 to
    512). Every bin goes into one request on the tensor cores (bins of 384
    and 512 states in CTA pairs), replayed as one CUDA graph. B candidate
    (lambda1, lambda2) vectors per step; device
    time per step, the FP64 path at the same bins, and the largest
    per-family dlnL against it."""
    from cafe5_gb300.families import bin_families
    from cafe5_gb300.inputs import ErrorModel, RootPrior
    w = workload_cfg(2)
    F = w.families.n_families
    Wb, _, _ = bin_families(w.families)
    tid = ctx.upload_tree(w.tree, w.lambda_of_node)
    sid = ctx.upload_families(tid, w.families.counts)
    ctx.set_prior(RootPrior.uniform(1100).vector())
    ctx.set_error_model(ErrorModel.symmetric(0.05, 1100).table())
    base = dict(model=0, lambda_kind=1, use_error_model=True)

    def make(w, B, step):
        f = 1.0 + 1e-6 * (step % 10000)
        return [dict(lambdas=[w.lambdas[0] * (1.0 + 0.01 * b) * f, w.lambdas[1] * (1.0 + 0.01 * b) * f])
                for b in range(B)]

    dev = torch.device("cuda", torch.cuda.current_device())
    d_fam = torch.empty(B * F, dtype=torch.float64, device=dev)
    d_tot = torch.empty(B, dtype=torch.float64, device=dev)
    kw = dict(base, precision="mixed_tf32x3")
    ms = time_steps(ctx, torch, stream, flush, tid, sid, w, B, steps, 3, d_fam, d_tot, kw, step0=20000, make=make)
    kw64 = dict(base, precision="fp64_binned")
    ms64 = time_steps(ctx, torch, stream, flush, tid, sid, w, B, 2, 1, d_fam, d_tot, kw64, step0=21000, make=make)
    cands = make(w, B, 22000)
    cur = ctx.score_batch(tid, sid, cands, **kw)
    ref = ctx.score_batch(tid, sid, cands, **kw64)
    per = []
    for c, r in zip(cur, ref):
        fin = np.isfinite(r.family_lnl)
        per.append(float(np.max(np.abs(c.family_lnl[fin] - r.family_lnl[fin]) / np.abs(r.family_lnl[fin]))))
    ctx.profile(True)
    ctx.profile_read()
    ctx.score_batch(tid, sid, make(w, B, 23000), **kw)     # new candidates: matrices built
    prof = ctx.profile_read()
    ctx.profile(False)
    ctx.free_families(sid)
    ctx.set_error_model(None)
    bins = {int(b): int((Wb == b).sum()) for b in sorted(set(int(x) for x in Wb))}
    return {"workload": w.name, "candidates": B, "families": F, "taxa": 32, "bins": bins, "steps": steps,
            "ms_per_step": ms / steps, "value": B * F * steps / (ms / 1e3), "unit": "family-lnL evals/s",
            "fp64_binned_ms_per_step": ms64 / 2, "fp64_binned_value": B * F * 2 / (ms64 / 1e3),
            "max_rel_dlnl_vs_fp64": max(per), "n_fallback": int(max(c.n_fallback for c in cur)),
            "profiled_call_ms": {k: round(v, 3) for k, v in prof.items()
                                 if k in ("matrix_ms", "prune_ms", "other_ms", "finish_ms", "host_total_ms")},
            "note": "profiled_call_ms: one direct (unreplayed) call on new candidates with per-launch events: prune_ms = "
                    "tensor-core bins (384 and 512 in CTA pairs), other_ms = TF32 conversion"}


def config0_phase(ctx, cpu_seconds: float, reps: int = 10):
    """The plain base model in FP64: 12-taxon tree (root age 100), 1,000
    families, single lambda, the reference's global S and R, uniform prior.
    Latency of one score through the public API (host counts resident,
    per-family lnL back to the host) for FP64_REF with and without the
    reference's dedupe and for MIXED_TF32X3; the Nelder-Mead fit of lambda
    (cafe_optimize: the host search, each evaluation one FP64_REF score on
    the GPU) and, as the CPU baseline, the same search (cafe_nelder_mead)
    over the oracle port's score on all host cores."""
    from cafe5_gb300 import _lib, engine
    from cafe5_gb300.inputs import RootPrior
    import ctypes
    w = workload_cfg(0)
    F = w.families.n_families
    S, R = global_bounds(w.families)
    root_prior = RootPrior.uniform(R)
    prior = root_prior.vector()
    tid = ctx.upload_tree(w.tree)
    sid = ctx.upload_families(tid, w.families.counts)
    ctx.set_prior(prior)
    ctx.set_error_model(None)
    out = {"workload": w.name, "families": F, "taxa": 12, "S": S, "R": R}
    for name, kw in (("fp64_ref", dict(precision="fp64_ref", S=S, R=R, dedupe=False)),
                     ("fp64_ref_dedupe", dict(precision="fp64_ref", S=S, R=R, dedupe=True)),
                     ("mixed_tf32x3", dict(precision="mixed_tf32x3"))):
        ctx.score(tid, sid, [0.0025], **kw)
        ts = []
        for i in range(reps):
            t0 = time.perf_counter()
            r = ctx.score(tid, sid, [0.0025 * (1.0 + 1e-4 * (i + 1))], **kw)
            ts.append((time.perf_counter() - t0) * 1e3)
        med = float(np.median(ts))
        out[name] = {"ms_per_score": med, "evals_per_s": F / (med / 1e3), "neg_lnl": r.total}
    ctx.free_families(sid)
    longest = max(w.tree.branch_length[v] for v in range(w.tree.n_nodes) if w.tree.parent[v] >= 0)
    lam = engine.SingleLambda(0.01)
    model = engine.BaseModel(lam, w.tree, w.families, S, R, ctx=ctx)
    scorer = engine.LambdaOptimizerScorer(lam, model, root_prior, longest)
    t0 = time.perf_counter()
    res = engine.Optimizer(scorer).optimize(initial=[0.01])
    fit = {"lambda": res.values[0], "neg_lnl": res.score, "iterations": res.num_iterations,
           "evaluations": res.evaluations, "wall_ms": (time.perf_counter() - t0) * 1e3}
    out["nm_fit_gpu"] = fit
    if cpu_seconds > 0:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        ta = oracle.TreeArrays.from_tree(w.tree)
        counts = np.ascontiguousarray(w.families.counts)
        threads = os.cpu_count() or 1

        def objective(xp, n, user):
            x = xp[0]
            if not x > 0:
                return float("inf")
            tot, _, _ = oracle.score(ta, counts, [x], prior=prior, S=S, R=R, dedupe=True, n_threads=threads)
            return float("inf") if math.isnan(tot) else float(tot)

        lib = _lib.load()
        x0 = np.array([0.01])
        best = np.zeros(1)
        cfg = _lib.OptConfig(_lib.OPT_LAMBDA, 1, x0.ctypes.data, 300, 1.0, 2.0)
        r = _lib.OptResult(best.ctypes.data, 0.0, 0, 0, 0)
        cb = _lib.OBJECTIVE(objective)
        t0 = time.perf_counter()
        first = objective(x0.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 1, None)
        rc = lib.cafe_nelder_mead(ctypes.byref(cfg), cb, None, ctypes.byref(r))
        wall = (time.perf_counter() - t0) * 1e3
        out["nm_fit_cpu_port"] = {"lambda": float(best[0]), "neg_lnl": r.score, "iterations": r.iterations,
                                  "evaluations": r.evaluations + 1, "wall_ms": wall, "status": rc,
                                  "cores": threads, "kind": "port", "initial_score": first}
        out["fit_speedup_vs_cpu_port"] = wall / fit["wall_ms"]
        out["same_fit"] = bool(float(best[0]) == fit["lambda"])
    return out


def reconstruction_phase(ctx, tid, sid, w, fams, S, R, cpu_seconds: float, reps: int = 3):
    """Pupko joint reconstruction of every family x gamma category at the
    reference's global bounds (cafe_reconstruct): the log2-filtered kernel,
    the exhaustive FP64 scan, and the CPU oracle on a bounded sample."""
    from cafe5_gb300.inputs import RootPrior
    prior = RootPrior.uniform(R).vector(R + 8)
    ctx.set_prior(prior)
    kw = dict(S=S, R=R, model=1, multipliers=w.multipliers, cat_probs=w.cat_probs)
    lam = [w.true_lambda]
    ctx.reconstruct(tid, sid, lam, **kw)                     # matrices built, buffers sized
    ms = min(ctx.reconstruct(tid, sid, lam, **kw).device_ms for _ in range(reps))
    ex = ctx.reconstruct(tid, sid, lam, exhaustive=True, **kw)
    rec = ctx.reconstruct(tid, sid, lam, **kw)
    F, K = fams.n_families, len(w.multipliers)
    out = {"unit": "family-category reconstructions/s", "value": F * K / (ms / 1e3), "device_ms": ms,
           "exhaustive_fp64_device_ms": ex.device_ms, "filter_speedup": ex.device_ms / ms,
           "identical_to_exhaustive": bool(np.array_equal(ex.category_state, rec.category_state)),
           "families": F, "K": K, "S": S, "R": R, "n_failed": int(rec.n_failed),
           "note": "device time of cafe_reconstruct (matrices cached); states 0..S per node"}
    if cpu_seconds > 0:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        ta = oracle.TreeArrays.from_tree(w.tree)

        def timed(n):
            t0 = time.perf_counter()
            oracle.reconstruct(ta, fams.counts[:n], lam, prior=prior, S=S, R=R, multipliers=w.multipliers,
                               cat_probs=w.cat_probs, n_threads=os.cpu_count() or 1)
            return time.perf_counter() - t0

        # the oracle builds its matrices inside each call: the difference of
        # two sample sizes leaves the per-family work
        t0 = timed(16)
        n = 64
        while True:
            dt = timed(n)
            if dt - t0 >= cpu_seconds / 2 or n >= F:
                break
            n = min(F, n * 4)
        out["cpu_port"] = {"value": (n - 16) * K / max(dt - t0, 1e-9), "cores": os.cpu_count() or 1,
                           "kind": "port",
                           "sample": f"{n} minus 16 of {F} families x K={K} (matrix build cancelled out)"}
    return out


def pvalue_phase(ctx, tid, sid, w, fams, S, R, cpu_seconds: float, n_sim: int = 1000):
    """compute_pvalues at the reference's defaults (1,000 simulated families
    per root size 1..R, global bounds): wall time of cafe_pvalues, split into
    host (simulation with the reference's random stream, sorting, ranks) and
    device (pruning every simulated and observed family)."""
    lam = [w.true_lambda]
    ctx.pvalues(tid, sid, lam, S=S, R=R, n_simulations=50, seed=1)      # buffers, matrices
    t0 = time.perf_counter()
    r = ctx.pvalues(tid, sid, lam, S=S, R=R, n_simulations=n_sim, seed=10)
    wall = (time.perf_counter() - t0) * 1e3
    F = fams.n_families
    pruned = R * n_sim + F
    out = {"unit": "families pruned/s (simulated + observed)", "value": pruned / (wall / 1e3), "wall_ms": wall,
           "device_ms": r["device_ms"], "host_ms": r["host_ms"], "n_simulations": n_sim, "root_sizes": R,
           "simulated_families": R * n_sim, "observed_families": F, "S": S,
           "note": "whole cafe_pvalues call; the simulation is sequential on the host (the reference's "
                   "mt19937 stream), both prunings on the GPU"}
    # the opt-in device-sampled mode: every step on the GPU, the same
    # distributions but not the reference's random stream
    ctx.pvalues(tid, sid, lam, S=S, R=R, n_simulations=50, seed=1, device_sampling=True)
    t0 = time.perf_counter()
    rd = ctx.pvalues(tid, sid, lam, S=S, R=R, n_simulations=n_sim, seed=10, device_sampling=True)
    wall_d = (time.perf_counter() - t0) * 1e3
    out["device_sampled"] = {"value": pruned / (wall_d / 1e3), "wall_ms": wall_d, "device_ms": rd["device_ms"],
                             "host_ms": rd["host_ms"],
                             "mean_abs_dp_vs_reference_stream": float(np.mean(np.abs(rd["pvalues"] - r["pvalues"]))),
                             "note": "device_sampling = 1: draws, grouping, pruning, sort and ranks on the GPU "
                                     "(counter-based generator; equal in distribution, not the reference's stream)"}
    if cpu_seconds > 0:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        ta = oracle.TreeArrays.from_tree(w.tree)

        def timed(ns, nf):
            t = time.perf_counter()
            oracle.pvalues(ta, fams.counts[:nf], lam, S=S, R=R, n_sim=ns, seed=10)
            return time.perf_counter() - t

        # the oracle builds its matrices inside each call: the difference of
        # two sample sizes leaves the per-family work
        base = timed(10, 50)
        ns, nf = 40, 200
        while True:
            dt = timed(ns, nf)
            if dt - base >= cpu_seconds / 2 or ns >= n_sim:
                break
            ns, nf = ns * 2, min(F, nf * 2)
        fam = (ns * R + nf) - (10 * R + 50)
        out["cpu_port"] = {"value": fam / max(dt - base, 1e-9), "cores": os.cpu_count() or 1, "kind": "port",
                           "sample": f"{ns} simulations x {R} root sizes + {nf} observed families, minus a "
                                     f"10 x {R} + 50 run (matrix build cancelled out)"}
    return out


def run_ours(args):
    import torch
    from cafe5_gb300.engine import Context
    from cafe5_gb300.families import FamilySet, bin_families
    from cafe5_gb300.inputs import RootPrior
    from cafe5_gb300.shard import allgather_totals, shard_range

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)

    # weak scaling: world x F families, this rank's contiguous shard
    wall_fams = workload(args.families * world)
    lo, hi = shard_range(wall_fams.families.n_families, rank, world)
    w = wall_fams
    fams = FamilySet(w.families.ids[lo:hi], np.ascontiguousarray(w.families.counts[lo:hi]))
    F = fams.n_families
    B = max(1, args.candidates)
    S, R = global_bounds(fams)
    prec = args.precision
    Wb, Sb, Rb = bin_families(fams)
    # the reference's prior: uniform over root sizes 1..R (R_f <= R for every
    # family), zero past R up to the widest bin -- with it the per-family
    # bins and the reference's global bounds give the same objective
    prior = RootPrior.uniform(R).vector(max(R, int(Wb.max()) + 8))

    ctx = Context(device=local)
    tid = ctx.upload_tree(w.tree)
    sid = ctx.upload_families(tid, fams.counts)
    ctx.set_prior(prior)
    ctx.set_error_model(None)

    def kw_for(p):
        return dict(model=1, precision=p, S=S if p == "fp64_ref" else 0, R=R if p == "fp64_ref" else 0)

    kw = kw_for(prec)
    # a dedicated stream: the legacy default stream has handle 0, which the
    # C ABI reads as "the context's own stream"
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    d_fam = torch.empty(B * F, dtype=torch.float64, device=dev)
    d_tot = torch.empty(B, dtype=torch.float64, device=dev)
    if args.profile_config2:
        # two batched mixed-precision scores of the config-2 workload (a small
        # case for ncu captures of the FP64 cluster walk and the wide bins)
        from cafe5_gb300.inputs import ErrorModel
        w2 = workload_cfg(2)
        tid2 = ctx.upload_tree(w2.tree, w2.lambda_of_node)
        sid2 = ctx.upload_families(tid2, w2.families.counts)
        ctx.set_prior(RootPrior.uniform(1100).vector())
        ctx.set_error_model(ErrorModel.symmetric(0.05, 1100).table())
        for i in range(2):
            c = [dict(lambdas=[w2.lambdas[0] * (1.0 + 0.01 * b) * (1.0 + 1e-6 * i),
                               w2.lambdas[1] * (1.0 + 0.01 * b) * (1.0 + 1e-6 * i)]) for b in range(B)]
            r = ctx.score_batch(tid2, sid2, c, model=0, lambda_kind=1, use_error_model=True, precision=prec)
        if rank == 0:
            print(json.dumps({"profile_config2": True, "candidates": B, "families": w2.families.n_families,
                              "neg_lnl": r[0].total}))
        ctx.close()
        return 0
    if args.profile_only:
        for i in range(2):
            ctx.score_batch_device(tid, sid, candidates(w, B, i), d_fam.data_ptr(), d_tot.data_ptr(),
                                   stream.cuda_stream, **kw)
        torch.cuda.synchronize()
        if rank == 0:
            print(json.dumps({"profile_only": True, "candidates": B, "families": F, "neg_lnl": float(d_tot[0].item())}))
        ctx.close()
        return 0
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)   # > 129 MB L2

    # launch shapes tuned once per workload (untimed), as a deployment would
    tuned = None
    if prec.startswith("mixed") and not args.no_autotune:
        tuned = ctx.autotune(tid, sid, candidates(w, B, 9000), reps=2, **kw)
    # warm-up, then the timed steps (barrier + synchronize on both sides)
    time_steps(ctx, torch, stream, flush, tid, sid, w, B, 0, args.warmup, d_fam, d_tot, kw)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    total_ms = time_steps(ctx, torch, stream, flush, tid, sid, w, B, args.steps, 0, d_fam, d_tot, kw)
    torch.cuda.synchronize()
    clk = clocks.stop()
    # kernel breakdown from separate, untimed profiled steps (profiling records
    # events around every launch, so profiled calls bypass the CUDA graphs)
    prof_steps = 3
    ctx.profile(True)
    ctx.profile_read()
    time_steps(ctx, torch, stream, flush, tid, sid, w, B, prof_steps, 0, d_fam, d_tot, kw, step0=7000)
    torch.cuda.synchronize()
    prof = ctx.profile_read()
    ctx.profile(False)
    if world > 1:
        torch.distributed.barrier()
        t = torch.tensor([total_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    value = B * F * world * args.steps / (total_ms / 1e3)
    step_totals = allgather_totals(d_tot.cpu().numpy().tolist()) if world > 1 else d_tot.cpu().numpy().tolist()

    # the plain FP64 GPU paths on the same kind of steps
    fp64 = {}
    for p in ("fp64_binned", "fp64_ref"):
        if p == prec:
            continue
        ms = time_steps(ctx, torch, stream, flush, tid, sid, w, B, max(1, args.fp64_steps), 1, d_fam, d_tot,
                        kw_for(p), step0=20000)
        fp64[p] = {"value": B * F * world * max(1, args.fp64_steps) / (ms / 1e3), "ms_per_step":
                   ms / max(1, args.fp64_steps)}

    # end to end through the public API, host buffers
    pinned = torch.empty((F, fams.counts.shape[1]), dtype=torch.int32, pin_memory=True)
    pinned.numpy()[:] = fams.counts
    host_counts = pinned.numpy()
    e2e_ms = 0.0
    n_e2e = max(3, min(args.steps, 10))
    for i in range(n_e2e + 1):
        flush.fill_(float(i))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.update_families(sid, host_counts)
        res = ctx.score_batch(tid, sid, candidates(w, B, 1000 + i), **kw)
        dt = (time.perf_counter() - t0) * 1e3
        if i > 0:
            e2e_ms += dt
    e2e_value = B * F * world * n_e2e / (e2e_ms / 1e3)

    # accuracy of this path vs FP64 at the same bins (dLnL per family, per candidate)
    cands = candidates(w, B, 0)
    ref64 = ctx.score_batch(tid, sid, cands, **kw_for("fp64_binned"))
    cur = ctx.score_batch(tid, sid, cands, **kw)
    dl = max(float(np.max(np.abs(c.family_lnl - r.family_lnl) / np.maximum(np.abs(r.family_lnl), 1e-300)))
             for c, r in zip(cur, ref64))
    n_fb = int(max(c.n_fallback for c in cur))

    serving = None
    if rank == 0 and args.serving_clients > 0:
        serving = serving_phase(ctx, tid, sid, w, args.serving_clients, args.serving_requests, kw)

    cfg3 = None
    if rank == 0 and args.config3:
        cfg3 = config3_phase(ctx, torch, stream, flush)
        ctx.set_prior(prior)

    cfg2 = None
    if rank == 0 and args.config2:
        cfg2 = config2_phase(ctx, torch, stream, flush)
        ctx.set_prior(prior)

    cfg0 = None
    if rank == 0 and args.config0:
        cfg0 = config0_phase(ctx, args.cpu_seconds)
        ctx.set_prior(prior)
        ctx.set_error_model(None)

    stream4 = None
    if rank == 0 and args.serving_optimizers > 0:
        stream4 = serving_stream(ctx, args.serving_optimizers)
        ctx.set_prior(prior)

    recon = None
    if rank == 0 and args.reconstruct:
        recon = reconstruction_phase(ctx, tid, sid, w, fams, S, R, args.cpu_seconds / 2)
    pvals = None
    if rank == 0 and args.pvalues:
        pvals = pvalue_phase(ctx, tid, sid, w, fams, S, R, args.cpu_seconds / 2)

    peaks = measured_peaks()
    fp64_peak = fp64_peak_tflops(torch, dev)
    nl = max(prof["prune_launches"], 1)
    achieved = prof["prune_flops"] / nl / (prof["prune_ms"] / nl / 1e3) / 1e12 if prof["prune_ms"] > 0 else 0.0
    if prec.startswith("mixed"):
        roof = {"bound": "tensor", "achieved": achieved, "peak": peaks.get("bf16_tflops", 1900.0),
                "unit": "TFLOP/s",
                "peak_source": "MEASURED_PEAKS.json bf16_tflops (of measured)" if "bf16_tflops" in peaks
                else "fallback 1.9 PFLOP/s bf16 (of fallback)"}
    else:
        roof = {"bound": "fp64", "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                "peak_source": "cuBLAS DGEMM 4096^3 measured in this run (FP64 pipe)"}
    roof["frac"] = roof["achieved"] / roof["peak"] if roof["peak"] else None
    kernel = "k_prune64" if not prec.startswith("mixed") else "k_prune_tc"
    traffic, tsrc = profiled_traffic(kernel, w.name + f"_B{B}")
    roof["traffic"] = traffic
    roof["traffic_source"] = tsrc
    roof["kernel"] = kernel
    roof["achieved_basis"] = ("algorithmic flops of the pruning launches (2 x rows x states per child "
                              "contraction + child products) / their CUDA-event time")
    roof["breakdown_basis"] = f"{prof_steps} profiled steps (direct launches, per-launch events)"
    roof["prune_ms_per_step"] = prof["prune_ms"] / prof_steps
    roof["matrix_ms_per_step"] = prof["matrix_ms"] / prof_steps
    roof["other_ms_per_step"] = prof["other_ms"] / prof_steps
    roof["finish_ms_per_step"] = prof["finish_ms"] / prof_steps
    roof["host_enqueue_ms_per_step"] = prof["host_total_ms"] / prof_steps
    roof["host_ms_per_step"] = {k: prof[k] / prof_steps for k in ("host_keys_ms", "host_build_ms", "host_plan_ms")}

    base = None
    if rank == 0 and world == 1 and args.cpu_seconds > 0:
        base = cpu_baseline(w, S, R, args.cpu_seconds, os.cpu_count() or 1)

    if rank == 0:
        fb = fp64.get("fp64_binned", {}).get("value")
        ratio = lambda a, b: (a / b) if (a and b) else None
        per_config = {"config1": {"value": value, "fp64_binned_value": fb, "mixed_over_fp64": ratio(value, fb),
                                  "fp64_ref_value": fp64.get("fp64_ref", {}).get("value")}}
        if cfg0:
            m0, r0 = cfg0["mixed_tf32x3"]["evals_per_s"], cfg0["fp64_ref"]["evals_per_s"]
            per_config["config0"] = {"value": m0, "fp64_ref_value": r0, "mixed_over_fp64": ratio(m0, r0),
                                     "basis": "one score through the public API (latency-bound: 1,000 families)"}
        if cfg2:
            per_config["config2"] = {"value": cfg2["value"], "fp64_binned_value": cfg2["fp64_binned_value"],
                                     "mixed_over_fp64": ratio(cfg2["value"], cfg2["fp64_binned_value"])}
        if cfg3:
            per_config["config3"] = {"value": cfg3["value"], "fp64_binned_value": cfg3["fp64_binned_value"],
                                     "mixed_over_fp64": ratio(cfg3["value"], cfg3["fp64_binned_value"])}
        if stream4:
            per_config["config4"] = {"value": stream4["evals_per_s"], "p50_ms": stream4["open_loop"]["p50_ms"],
                                     "p99_ms": stream4["open_loop"]["p99_ms"],
                                     "max_rel_dlnl_vs_fp64": stream4["max_rel_dlnl_vs_fp64"]}
        line = {"metric": METRIC, "value": value, "unit": "family-lnL evals/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64" if "fp64" in prec else "tf32x3",
                "data": "synthetic",
                "config": shared_config(w, F, B, world),
                "precision": prec,
                "bins": sorted(set(int(x) for x in Wb)),
                "tc_shapes": tuned,
                "timing": "steps issued back to back (host preparation of a step overlaps the previous one); "
                          "CUDA events on the launching stream",
                "roofline": roof,
                "fp64_paths": fp64,
                "cpu_baseline": base,
                "e2e": {"value": e2e_value, "unit": "family-lnL evals/s",
                        "h2d_bytes_per_step": int(fams.counts.nbytes), "d2h_bytes_per_step": int(B * (F * 8 + 8))},
                "serving": serving,
                "serving_stream": stream4,
                "config3_batched": cfg3,
                "config2_local_lambdas_error_model": cfg2,
                "config0_base_fp64_fit": cfg0,
                "reconstruction": recon,
                "pvalues": pvals,
                "cuda_graphs": "pruning phase (conversion, tensor-core bins, fallback, finish) replayed as a CUDA "
                               "graph per launch signature; matrix builds launched directly",
                "accuracy": {"max_rel_dlnl_vs_fp64": dl, "n_fallback": n_fb},
                "neg_lnl": step_totals[0],
                "neg_lnl_check": {"step": 0, "candidate": 0, "value": cur[0].total,
                                  "fp64_binned": ref64[0].total},
                # the metric's own numbers last, where a truncated tail keeps them
                "per_config": per_config,
                "fp64_binned_value": fb,
                "mixed_over_fp64": ratio(value, fb),
                "p50_ms": stream4["open_loop"]["p50_ms"] if stream4 else None,
                "p99_ms": stream4["open_loop"]["p99_ms"] if stream4 else None,
                "latency_basis": "config-4 served stream, open loop (Poisson arrivals from 256 Nelder-Mead "
                                 "clients), submit -> result",
                "gpu_launches": int(round(prof["launches"] / prof_steps * args.steps)),
                "clocks": clk}
        print(json.dumps(line))
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
