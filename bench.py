"""Benchmark of the CAFE5 likelihood hot path on one GB300.

Workload: 24-taxon Yule tree (root age 150), 10,000 families, gamma model
with K = 4 categories (alpha = 0.5): the gamma configuration the headline
metric is quoted on. Synthetic, seeded (no public dataset exists for this
path). A "step" is one infer_family_likelihoods evaluation over all
families at a new lambda (as one optimizer step: matrices are rebuilt for
the new lambda every step). One family-lnL evaluation is one family's lnL
with all K categories.

  value   family-lnL evals/s with inputs resident in HBM (cafe_score_device),
          CUDA events on the launching stream, L2 flushed between steps
  e2e     the same through the public API (cafe_families_update from pinned
          host memory + cafe_score copying per-family lnL back), host clock

`--impl reference` times the reference algorithm on the host cores instead
(the compiled reference when it exists on this machine, else the CPU
oracle that restates it).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "family-lnL evals/s (gamma K=4, 24 taxa, 10k families; batched, dLnL<=1e-6 vs FP64)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default=os.environ.get("CAFE_BENCH_PRECISION", "auto"))
    ap.add_argument("--families", type=int, default=10000)
    ap.add_argument("--cpu-seconds", type=float, default=8.0)
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload(n_families: int):
    from cafe5_gb300.synth import workload as wl
    return wl(1, n_families=n_families, seed=0)


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
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_{os.getpid()}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
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
    line-by-line restatement: per-term exp/pow matrices, dense products,
    OpenMP over families) is timed on a bounded family sample."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from cafe5_gb300.inputs import RootPrior
    ta = oracle.TreeArrays.from_tree(w.tree)
    prior = RootPrior.uniform(R).vector()
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


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    w = workload(args.families)
    S, R = global_bounds(w.families)
    threads = os.cpu_count() or 1
    steps = max(1, args.steps)
    per_step = max(1.0, min(8.0, 120.0 / (steps + args.warmup)))
    base = cpu_baseline(w, S, R, per_step * steps, threads)
    line = {"metric": METRIC, "value": base["value"], "unit": "family-lnL evals/s", "n_gpus": args.gpus,
            "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * args.families / base["value"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": w.name, "families": args.families, "taxa": 24, "K": 4, "alpha": 0.5,
                       "S": S, "R": R},
            "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": "family-lnL evals/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_ours(args):
    import torch
    from cafe5_gb300.engine import Context
    from cafe5_gb300.families import bin_families
    from cafe5_gb300.inputs import RootPrior

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)

    w = workload(args.families)
    F = w.families.n_families
    S, R = global_bounds(w.families)
    prec = args.precision
    if prec == "auto":
        prec = "mixed_tf32x3"
    Wb, Sb, Rb = bin_families(w.families)
    prior = RootPrior.uniform(max(R, int(Wb.max()) + 8)).vector()

    ctx = Context(device=local)
    tid = ctx.upload_tree(w.tree)
    sid = ctx.upload_families(tid, w.families.counts)
    ctx.set_prior(prior)
    ctx.set_error_model(None)
    kw = dict(model=1, multipliers=w.multipliers, cat_probs=w.cat_probs, precision=prec,
              S=S if prec == "fp64_ref" else 0, R=R if prec == "fp64_ref" else 0)
    # a dedicated stream: the legacy default stream has handle 0, which the
    # C ABI reads as "the context's own stream"
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    d_fam = torch.empty(F, dtype=torch.float64, device=dev)
    d_tot = torch.empty(1, dtype=torch.float64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)   # > 129 MB L2

    def lam_of(step):
        return [w.true_lambda * (1.0 + 1e-4 * step)]

    # warm-up
    for i in range(args.warmup):
        ctx.score_device(tid, sid, lam_of(-1 - i), d_fam.data_ptr(), d_tot.data_ptr(), stream.cuda_stream, **kw)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()

    clocks = ClockSampler(local)
    clocks.start()
    ctx.profile(True)
    ctx.profile_read()
    total_ms = 0.0
    for i in range(args.steps):
        flush.fill_(float(i))                       # evict L2 between steps (untimed)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.score_device(tid, sid, lam_of(i), d_fam.data_ptr(), d_tot.data_ptr(), stream.cuda_stream, **kw)
        e1.record(stream)
        e1.synchronize()
        total_ms += e0.elapsed_time(e1)
    torch.cuda.synchronize()
    prof = ctx.profile_read()
    ctx.profile(False)
    clk = clocks.stop()
    if world > 1:
        t = torch.tensor([total_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    value = F * world * args.steps / (total_ms / 1e3)

    # end to end through the public API, host buffers
    pinned = torch.empty((F, w.families.counts.shape[1]), dtype=torch.int32, pin_memory=True)
    pinned.numpy()[:] = w.families.counts
    host_counts = pinned.numpy()
    e2e_ms = 0.0
    n_e2e = max(3, min(args.steps, 10))
    last = None
    for i in range(n_e2e + 1):
        flush.fill_(float(i))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.update_families(sid, host_counts)
        last = ctx.score(tid, sid, lam_of(1000 + i), **kw)
        dt = (time.perf_counter() - t0) * 1e3
        if i > 0:
            e2e_ms += dt
    e2e_value = F * world * n_e2e / (e2e_ms / 1e3)

    # accuracy of this path vs FP64 at the same bins (dLnL per family)
    ref64 = ctx.score(tid, sid, lam_of(0), **dict(kw, precision="fp64_binned"))
    cur = ctx.score(tid, sid, lam_of(0), **kw)
    dl = np.abs(cur.family_lnl - ref64.family_lnl) / np.maximum(np.abs(ref64.family_lnl), 1e-300)

    peaks = measured_peaks()
    fp64_peak = fp64_peak_tflops(torch, dev)
    achieved = prof["prune_flops"] / max(prof["prune_launches"], 1) / (prof["prune_ms"] / max(prof["prune_launches"], 1) / 1e3) / 1e12 if prof["prune_ms"] > 0 else 0.0
    if prec.startswith("mixed"):
        roof = {"bound": "tensor", "achieved": achieved, "peak": peaks.get("bf16_tflops", 1900.0),
                "unit": "TFLOP/s", "peak_source": "MEASURED_PEAKS.json bf16_tflops (of measured)"}
    else:
        roof = {"bound": "fp64", "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                "peak_source": "cuBLAS DGEMM 4096^3 measured in this run (FP64 pipe)"}
    roof["frac"] = roof["achieved"] / roof["peak"] if roof["peak"] else None
    roof["traffic"] = None
    roof["kernel"] = "k_prune64" if not prec.startswith("mixed") else "k_prune_tc"
    roof["other_ms_per_step"] = prof["other_ms"] / args.steps
    roof["prune_ms_per_step"] = prof["prune_ms"] / args.steps
    roof["matrix_ms_per_step"] = prof["matrix_ms"] / args.steps
    roof["finish_ms_per_step"] = prof["finish_ms"] / args.steps

    base = None
    if rank == 0 and world == 1 and args.cpu_seconds > 0:
        base = cpu_baseline(w, S, R, args.cpu_seconds, os.cpu_count() or 1)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "family-lnL evals/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64" if "fp64" in prec else "tf32x3",
                "data": "synthetic",
                "config": {"workload": w.name, "families": F, "taxa": 24, "K": 4, "alpha": 0.5,
                           "precision": prec, "bins": sorted(set(int(x) for x in Wb)),
                           "l2": "flushed between timed steps (256 MB write)", "lambda": "new each step"},
                "roofline": roof,
                "cpu_baseline": base,
                "e2e": {"value": e2e_value, "unit": "family-lnL evals/s",
                        "h2d_bytes_per_step": int(w.families.counts.nbytes), "d2h_bytes_per_step": int(F * 8 + 8)},
                "gpu_launches": int(prof["launches"]),
                "clocks": clk,
                "accuracy": {"max_rel_dlnl_vs_fp64": float(np.max(dl)), "n_fallback": int(cur.n_fallback)},
                "neg_lnl": cur.total}
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
