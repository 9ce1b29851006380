#!/usr/bin/env python3
"""Benchmark: time-to-exact reset length per random DFA on one GB300.

Workload (default, `--workload n200`): 16 random binary DFAs, n = 200 states,
k = 2 letters, transitions uniform from SplitMix64 seeds, solved with the
reference's plain Exact plan (`{"algorithms": [{"name": "Exact"}]}`, default
upper bound n^3/6).  One step = solving all 16 DFAs through the public API.
The reference has no public benchmark suite; these seeded synthetic automata
stand in with the shapes its configs name.

Printed JSON line (rank 0):
  value     ms per DFA: the step's time between device-wide synchronisations
            (the step runs on several device streams and the batched
            launches' stream, so no single stream's events cover it); max
            over ranks
  e2e       ms per DFA by wall clock around the public call (host automaton in,
            bounds + word out)
  roofline  the kernel class with the most device time in one profiled step:
            algorithmic bytes / event-timed duration vs measured HBM peak
  cpu_baseline  the oracle (CPU restatement of the reference, oracle/) on a
            bounded sample of the same DFAs, all host threads

`--impl reference` times that CPU restatement alone (rank 0; other ranks exit).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

PLAN_EXACT = json.dumps({"algorithms": [{"name": "Exact", "config": {}}]})

# configs/exact.json of the reference without its Brute / Eppstein entries
PLAN_BEAM_EXACT = json.dumps({
    "upper_bound": "1ULL * (AUT_N - 1) * (AUT_N - 1) + 1",
    "algorithms": [
        {"name": "Beam", "config": {"presort": "indeg", "dynamic": True,
                                    "min_beam_size": "AUT_N * std::log2(AUT_N)",
                                    "max_beam_size": "AUT_N * AUT_N * std::log2(AUT_N)",
                                    "beam_exact_ratio": 0.01}},
        {"name": "Exact", "config": {"dfs_min_list_size": "8192", "bfs_small_list_size": "AUT_N * AUT_K",
                                     "dfs": True, "dfs_shortcut": True, "max_memory_mb": "12 * 1024"}}]})

# the same Exact entry, its upper bound from the learned forward beam instead
PLAN_LEARNED_EXACT = json.dumps({
    "upper_bound": "1ULL * (AUT_N - 1) * (AUT_N - 1) + 1",
    "algorithms": [
        {"name": "LearnedBeam", "config": {"beam_size": "4096", "order": "model"}},
        {"name": "Exact", "config": {"dfs_min_list_size": "8192", "bfs_small_list_size": "AUT_N * AUT_K",
                                     "dfs": True, "dfs_shortcut": True, "max_memory_mb": "12 * 1024"}}]})

# the same Exact entry with no beam before it: the plain bidirectional search
PLAN_PLAIN_EXACT = json.dumps({
    "upper_bound": "1ULL * (AUT_N - 1) * (AUT_N - 1) + 1",
    "algorithms": [
        {"name": "Exact", "config": {"dfs_min_list_size": "8192", "bfs_small_list_size": "AUT_N * AUT_K",
                                     "dfs": True, "dfs_shortcut": True, "max_memory_mb": "12 * 1024"}}]})

WORKLOADS = {
    # name: (n, k, count, plan, description); n = 0 marks the uneven batch
    "n200": (200, 2, 16, PLAN_EXACT, "plain exact, 16 random binary DFAs, n=200 (256-bit sets)"),
    "n48": (48, 2, 64, PLAN_EXACT, "plain exact, 64 random binary DFAs, n=48 (64-bit sets)"),
    "batch4096": (0, 0, 4096, PLAN_EXACT,
                  "plain exact, 4096 random DFAs, n ~ U[32,160], k ~ U{2,3} (64/128/192-bit sets)"),
    "n320": (320, 2, 8, PLAN_BEAM_EXACT, "Beam(dynamic)+Exact (configs/exact.json), 8 random binary DFAs, n=320"),
    "n384": (384, 2, 8, PLAN_BEAM_EXACT, "Beam(dynamic)+Exact (configs/exact.json), 8 random binary DFAs, n=384"),
    "n384_plain": (384, 2, 8, PLAN_PLAIN_EXACT,
                   "plain Exact (the configs/exact.json Exact entry, no beam), 8 random binary DFAs, n=384"),
    "n384_learned": (384, 2, 8, PLAN_LEARNED_EXACT,
                     "LearnedBeam(4096, distance model)+Exact, 8 random binary DFAs, n=384"),
}


def plan_name(plan: str) -> str:
    return {PLAN_EXACT: "Exact (defaults)", PLAN_BEAM_EXACT: "Beam(dynamic)+Exact",
            PLAN_PLAIN_EXACT: "Exact (configs/exact.json entry)", PLAN_LEARNED_EXACT: "LearnedBeam+Exact"}[plan]


def workload_dfas(name: str, rank: int, held_out: int = 0):
    """The workload's automata for this rank; with held_out > 0, that many
    other automata of the same shape (seeds no rank's workload uses)."""
    from synchrowords_gb300.generate import batch, random_dfa
    n, k, count, _, _ = WORKLOADS[name]
    if held_out:
        if n == 0:
            return batch(held_out, 90210 + rank)
        return [(n, k, random_dfa(n, k, 50000 + rank * 100000 + i)) for i in range(held_out)]
    if n == 0:
        return batch(count, 2026 + rank)
    base = 1 + rank * 100000
    return [(n, k, random_dfa(n, k, base + i)) for i in range(count)]


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic():
    p = ROOT / "profiles" / "traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except Exception:
            return {}
    return {}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.samples = []
        if self.proc is None:
            return
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out, _ = self.proc.communicate()
        for line in out.splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.samples.append(parts)

    def summary(self):
        if not getattr(self, "samples", None):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def barrier_max(value: float, world: int) -> float:
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def cpu_baseline(dfas, sample: int, threads: int, plan: str = PLAN_EXACT):
    """Oracle (CPU restatement of the reference) running `plan` on the first `sample` DFAs."""
    import math
    import oracle
    oracle.build()
    t0 = time.perf_counter()
    lengths = []
    for n, k, d in dfas[:sample]:
        if plan in (PLAN_BEAM_EXACT, PLAN_PLAIN_EXACT, PLAN_LEARNED_EXACT):  # at n >= 320: the reference's own plan
            lg = math.log2(n)
            b = oracle.beam(d, n, k, oracle.BeamParams(dynamic=True, presort_indeg=True, min_beam_size=int(n * lg),
                                                       max_beam_size=int(n * n * lg)), upper=(n - 1) ** 2 + 1)
            r = oracle.exact(d, n, k, oracle.ExactParams(dfs_min_list_size=8192, bfs_small_list_size=n * k,
                                                         max_memory_mb=12 * 1024, threads=threads),
                             upper=b.upper)
        else:
            r = oracle.exact(d, n, k, oracle.ExactParams(threads=threads))
        lengths.append(r.upper)
    dt = time.perf_counter() - t0
    return dt * 1000.0 / sample, lengths


def run_reference(args, world, rank):
    if rank != 0:
        return
    dfas = workload_dfas(args.workload, 0)
    threads = max(1, min(64, os.cpu_count() or 1))
    per_step = max(1, min(len(dfas), args.ref_sample))
    n, k, count, plan, desc = WORKLOADS[args.workload]
    for w in range(args.warmup):
        cpu_baseline(dfas[w % len(dfas):] + dfas, 1, threads, plan)
    times = []
    for s in range(args.steps):
        sub = [dfas[(s * per_step + i) % len(dfas)] for i in range(per_step)]
        ms, _ = cpu_baseline(sub, per_step, threads, plan)
        times.append(ms)
    value = sum(times) / len(times)
    line = {
        "impl": "reference", "metric": "time-to-exact reset length per random DFA", "value": round(value, 4),
        "unit": "ms", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(value * per_step, 3), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "config": {"workload": desc, "n": n, "k": k, "dfas_per_step": per_step,
                   "plan": plan_name(plan), "l2": "host-only run"},
        "cpu_baseline": {"value": round(value, 4), "unit": "ms", "cores": threads, "kind": "port",
                         "sample": f"{per_step} DFAs per step out of {count}, rotating"},
        "e2e": {"value": round(value, 4), "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def learned_vs_plain(ctx, count: int) -> dict:
    """The learned-bound comparison on the first `count` n = 384 bench automata,
    one at a time, wall seconds per automaton: the plain GPU bidirectional
    search (the configs/exact.json Exact entry, no beam) at the reference's
    12 GB budget and at a budget sized to the GPU (200 GB), and
    LearnedBeam(4096)+Exact at 12 GB.  Every run must reach the exact length."""
    import synchrowords_gb300 as sw
    from synchrowords_gb300.generate import random_dfa
    big = PLAN_PLAIN_EXACT.replace('"12 * 1024"', '"200 * 1024"')
    out = {"n": 384, "automata": [], "plans": {"plain_12gb": "Exact (configs/exact.json entry, 12 GB)",
                                               "plain_gpu_budget": "Exact, max_memory_mb 200 GB",
                                               "learned": "LearnedBeam(4096)+Exact (12 GB)"}}
    for seed in range(1, count + 1):
        d = random_dfa(384, 2, seed)
        rec = {"seed": seed}
        for name, plan in (("plain_12gb", PLAN_PLAIN_EXACT), ("plain_gpu_budget", big), ("learned", PLAN_LEARNED_EXACT)):
            t0 = time.perf_counter()
            r = ctx.solve(d, 384, 2, plan)
            dt = time.perf_counter() - t0
            if r.lower != r.upper or r.word is None:
                raise RuntimeError(f"{name}: bounds [{r.lower}, {r.upper}] are not an exact length")
            rec[name] = {"s": round(dt, 3), "length": r.upper}
        if len({rec[k]["length"] for k in out["plans"]}) != 1:
            raise RuntimeError(f"lengths differ between plans: {rec}")
        rec["speedup_vs_plain_12gb"] = round(rec["plain_12gb"]["s"] / rec["learned"]["s"], 2)
        rec["speedup_vs_plain_gpu_budget"] = round(rec["plain_gpu_budget"]["s"] / rec["learned"]["s"], 2)
        out["automata"].append(rec)
    return out


def run_ours(args, world, rank, local):
    import torch
    import synchrowords_gb300 as sw
    from synchrowords_gb300 import build as nb
    nb.build()
    torch.cuda.set_device(local)
    dfas = workload_dfas(args.workload, rank)
    n, k, count, plan, desc = WORKLOADS[args.workload]
    if args.instances:
        dfas = dfas[:args.instances]
        count = len(dfas)
    ctx = sw.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")  # > 129 MB L2

    tuned = tuned_c = tuned_scan = None
    if args.scan_tune < 0:  # default: tune where a held-out pass takes seconds, not minutes
        args.scan_tune = 8 if n <= 256 else (2 if n <= 320 else 0)
    if args.scan_tune:
        # untimed: the subset check's launch shape tuned on held-out automata of the same shape
        tuned_scan = ctx.autotune_scan(workload_dfas(args.workload, rank, args.scan_tune), plan)
    if args.autotune:
        tuned = ctx.autotune_batch(dfas, plan)  # untimed; keeps the fastest tuning on ctx
        tuned_c = ctx.autotune_cluster(dfas, plan)
    step_workers = 0 if args.autotune else args.streams

    def one_step():
        launches = 0
        lengths = []
        for r in ctx.solve_batch(dfas, plan, workers=step_workers):
            launches += r.stats["kernel_launches"]
            if r.non_synchro:
                lengths.append(None)  # no reset word exists (uneven batch has a few)
                continue
            lengths.append(r.upper)
            if r.lower != r.upper:
                raise RuntimeError(f"solve ended with bounds [{r.lower}, {r.upper}], not an exact length")
            if r.word is None or len(r.word) != r.upper:
                raise RuntimeError("solve returned no verified word")
        return launches, lengths

    for _ in range(args.warmup):
        one_step()
    torch.cuda.synchronize()
    dev_ms, wall_ms, launches, batched_ms = [], [], 0, 0.0
    lengths = None
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            barrier(world)
            t0 = time.perf_counter()
            l, lengths = one_step()
            t1 = time.perf_counter()
            torch.cuda.synchronize()
            t2 = time.perf_counter()
            launches += l
            batched_ms += ctx.last_batch_profile()["device_ms"]
            dev_ms.append((t2 - t0) * 1000.0)
            wall_ms.append((t1 - t0) * 1000.0)
    barrier(world)
    dev_total = barrier_max(sum(dev_ms), world)
    wall_total = barrier_max(sum(wall_ms), world)
    total_dfas = args.steps * count * world
    value = dev_total / (args.steps * count)  # per-rank DFAs run concurrently on separate GPUs
    value_job = dev_total / total_dfas
    e2e = wall_total / total_dfas

    # one extra, untimed step with per-kernel-class CUDA-event profiling
    flush.zero_()
    torch.cuda.synchronize()
    ctx.profile_begin()
    pairs = 0
    for (nn, kk, d) in dfas:
        r = ctx.solve(d, nn, kk, plan)
        pairs += r.stats["logical_pairs"]
    prof = ctx.profile_end()
    peak, peak_kind = load_peaks()
    top = max(prof, key=lambda c: prof[c]["ms"])
    p = prof[top]
    achieved = (p["bytes"] / 1e9) / (p["ms"] / 1e3) if p["ms"] > 0 else 0.0
    traffic = load_traffic().get(f"{args.workload}:{top}")
    roofline = {"bound": "hbm", "kernel": top, "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 5), "peak_kind": peak_kind,
                "algorithmic_bytes_per_launch": round(p["bytes"] / max(1, p["launches"]), 1),
                "avg_launch_us": round(1000.0 * p["ms"] / max(1, p["launches"]), 3),
                "traffic": traffic,
                "classes": {c: {"launches": v["launches"], "ms": round(v["ms"], 3),
                                "GB/s": round((v["bytes"] / 1e9) / (v["ms"] / 1e3), 2) if v["ms"] > 0 else 0.0}
                            for c, v in prof.items()}}
    if rank != 0:
        return
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        threads = max(1, min(64, os.cpu_count() or 1))
        sample = min(args.cpu_sample, count)
        cpu_ms, cpu_len = cpu_baseline(dfas, sample, threads, plan)
        for got, want in zip(lengths[:sample], cpu_len):
            if got is not None and got != want:
                raise RuntimeError(f"length mismatch vs oracle: {lengths[:sample]} != {cpu_len}")
        cpu = {"value": round(cpu_ms, 3), "unit": "ms", "cores": threads, "kind": "port",
               "sample": f"first {sample} of the {count} DFAs, oracle Exact with {threads} threads"}
    h2d = sum(4 * nn * kk for nn, kk, _ in dfas)
    d2h = sum(4 * ((L or 0) + 8) for L in lengths)
    line = {
        "metric": "time-to-exact reset length per random DFA", "value": round(value_job, 4), "unit": "ms",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(dev_total / args.steps, 3), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "config": {"workload": desc, "n": n, "k": k, "dfas_per_step_per_gpu": count, "plan": plan_name(plan),
                   "streams": args.streams if not args.autotune else ctx.get_batch_tuning()["workers"],
                   "batch_tuning": dict(ctx.get_batch_tuning(), autotune_ms=tuned["ms"] if tuned else None,
                                        cluster_autotune_ms=tuned_c["ms"] if tuned_c else None),
                   "scan_shapes": ({"tuned_on": f"{args.scan_tune} held-out automata of the same shape",
                                    "keys": tuned_scan} if tuned_scan is not None else
                                   {"tuned_on": None, "default": sw.DEFAULT_SCAN_SHAPE}),
                   "routes": {k: v for k, v in ctx.last_batch_profile().items()
                              if k in ("small_solved", "cluster_solved", "streamed")},
                   "batched_launch_ms_per_step": round(batched_ms / args.steps, 3),
                   "value_timing": "wall clock between device-wide synchronisations around each step",
                   "l2": "flushed (256 MB write) before every timed step", "per_gpu_ms_per_dfa": round(value, 4)},
        "e2e": {"value": round(e2e, 4), "unit": "ms", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": roofline,
        "subset_check_pairs_per_s": round(pairs / (sum(v["ms"] for v in prof.values()) / 1e3), 1) if prof else None,
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "lengths": lengths if len(lengths) <= 64 else {
            "count": len(lengths), "non_synchronizing": sum(L is None for L in lengths),
            "sum": sum(L for L in lengths if L is not None)},
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if args.learned_vs_plain:
        line["learned_vs_plain"] = learned_vs_plain(ctx, args.learned_vs_plain)
    print(json.dumps(line), flush=True)
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="n200")
    ap.add_argument("--cpu-sample", type=int, default=4)
    ap.add_argument("--ref-sample", type=int, default=4)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--streams", type=int, default=16, help="concurrent device streams (host threads)")
    ap.add_argument("--autotune", action="store_true",
                    help="before the warm-up, tune the batch's worker count and batched-launch limit on the workload")
    ap.add_argument("--scan-tune", type=int, default=-1, metavar="N",
                    help="before the warm-up, tune the subset check's launch shape on N held-out automata of the "
                         "workload's shape (0 = the default shape; default: 8 up to n = 256, 2 at n = 320, "
                         "0 above)")
    ap.add_argument("--learned-vs-plain", type=int, default=0, metavar="N",
                    help="also solve the first N n=384 automata plainly (12 GB and GPU-sized budgets) and with the "
                         "learned bound, and report their wall times (minutes per automaton; off by default)")
    ap.add_argument("--instances", type=int, default=0,
                    help="solve only the first N DFAs of the workload (profiling runs; 0 = all)")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if world > 1:
        import torch.distributed as dist
        import torch
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
