"""Throughput benchmark of the KGMT planning loop on one node.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (one "step"): the batched homogeneous configuration -- 256
independent 3-D double-integrator queries, each with its own seeded scene of
50 axis-aligned boxes and its own start / goal pair, tree capacity 50k nodes,
4 samples per expanded node, at most 200 iterations -- planned to completion
in one device-resident launch chain.  The metric is planning queries per
second over the whole job (all ranks); p50 / p99 solve latency and the success
rate of the step are reported beside it, together with the plain form (one
query per launch chain, same queries, same Philox seeds, same results).

Under torchrun every rank plans its own 256-query shard (weak scaling, no
collective on the data path); the step time is the max over ranks.

``--impl reference`` times the CPU restatement of the reference planner (the
reference's own CPU planner needs OMPL, which is not installed) on all host
threads, on the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_QUERIES = 256
N_OBSTACLES = 50
CAPACITY = 50_000
WORKLOAD = (f"batched homogeneous: {N_QUERIES} double-integrator queries per GPU, {N_OBSTACLES} seeded AABBs each "
            f"(edges U[0.05,0.15]), own start/goal, T={CAPACITY} nodes, S=4 samples/node, <=200 iterations, "
            f"8^3/2^3 region grid")
L2_FLUSH_BYTES = 256 << 20
L2_NOTE = ("trees, frontiers and samples of a step are ~1.4 GB, larger than L2; the GPU arm also flushes L2 "
           "(256 MiB write) between timed steps")
# configs 4 and 5 measured beside the headline: the mixed batch and a served
# Poisson stream drawn from it
N_MIXED = 1024
MIXED_PLAIN_SAMPLE = 32
# (offered queries/s, queries): the last stream offers about twice what one
# GPU serves, for long enough that its rate is the saturated one rather than
# the drain of the last queries' plans
SERVED_STREAMS = ((1000.0, 2000), (4000.0, 2000), (8000.0, 8000))


def config_of(world: int) -> dict:
    """The same `config` in both arms: what is planned per step."""
    return {"workload": WORKLOAD, "queries_per_step": N_QUERIES * world, "l2": L2_NOTE}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def make_workload(rank: int, n_queries: int = N_QUERIES):
    """The 256-query shard of one rank: every rank draws its own scenes
    (seed 1 + rank), so ranks never share a query (weak scaling)."""
    from kgmt_gb300 import workloads as W
    return W.double_integrator_batch(n_queries, n_obstacles=N_OBSTACLES, seed=1 + rank, tree_capacity=CAPACITY)


def whole_job_rate(local_ms: float, queries_per_rank: int, steps: int, world: int, device=None):
    """Max over ranks of the timed region and the whole-job queries/s
    (queries of all ranks / slowest rank's time).  No data-path collective:
    only this one reduction of a scalar."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([local_ms], dtype=torch.float64, device=device)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    slowest = float(t.item())
    return slowest, queries_per_rank * world * steps / (slowest * 1e-3)


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self._t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "25"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self._t = threading.Thread(target=self._read, daemon=True)
        self._t.start()
        # the timed region is tens of milliseconds: start it only once samples flow
        t0 = time.time()
        while not self.lines and time.time() - t0 < 3.0 and self.proc.poll() is None:
            time.sleep(0.005)
        self.lines.clear()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self._t:
            self._t.join(timeout=2)
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None, "samples": len(sm), "reasons": sorted(reasons)}


# DRAM traffic of k_propagate comes from an ncu capture of the current kernel
# sources (three launches of this workload, one-pass metrics), summarised
# under profiles/ with the hash of the sources it was taken on; a summary of
# other sources is stale and gives no traffic figure (null).
TRAFFIC_PROFILE = ROOT / "profiles" / "k_propagate_dram_batched_di256.md"
KERNEL_SOURCES = ["kgmt_kernels.cu", "kgmt_iter.cuh", "kgmt_device.cuh", "kgmt_types.h"]


def kernel_source_hash() -> str:
    import hashlib
    h = hashlib.sha256()
    for name in KERNEL_SOURCES:
        h.update((ROOT / "kgmt_gb300" / "csrc" / name).read_bytes())
    return h.hexdigest()[:16]


def propagate_traffic(samples_per_launch: float) -> dict:
    """DRAM bytes per k_propagate launch of this workload: the captured
    bytes per propagated sample times this run's samples per launch (traffic
    grows with the samples: each reads its parent row and writes its region
    word, the accepted ones their rows)."""
    import re
    if not TRAFFIC_PROFILE.exists():
        return {"traffic": None, "traffic_note": f"{TRAFFIC_PROFILE.name} missing"}
    text = TRAFFIC_PROFILE.read_text()
    sha = re.search(r"kernel_source_hash:\s*(\w+)", text)
    per = re.search(r"dram_bytes_per_sample:\s*([0-9.eE+]+)", text)
    if not sha or not per:
        return {"traffic": None, "traffic_note": f"{TRAFFIC_PROFILE.name} has no figures"}
    if sha.group(1) != kernel_source_hash():
        return {"traffic": None, "traffic_note": f"{TRAFFIC_PROFILE.name} was captured on other kernel sources"}
    b = float(per.group(1))
    return {"traffic": b * samples_per_launch, "traffic_bytes_per_sample": b,
            "traffic_note": f"ncu dram__bytes_read.sum + dram__bytes_write.sum per sample on three main-phase launches of this "
                            f"workload ({TRAFFIC_PROFILE.name}, sources {sha.group(1)}), times this run's samples per launch"}


# algorithmic bytes of the double-integrator propagate: per sample the
# frontier index and the parent's row (10 floats) read and the region-and-
# accept word written; per sample that joins the tree also its row and parent
PROPAGATE_BYTES_PER_SAMPLE = 4 + 10 * 4 + 4
PROPAGATE_BYTES_PER_ACCEPTED = 10 * 4 + 4


# ---------------------------------------------------------------------------
# FP32 denominator of the propagate roofline
# ---------------------------------------------------------------------------
def measured_fp32_lane_ops(torch) -> float:
    """FP32 lane operations per second: cuBLAS SGEMM (TF32 off) FLOP/s / 2.

    SGEMM issues fused multiply-adds (2 FLOP per lane-op); the propagate
    kernel is built without contraction, so one multiply or add is one lane
    operation."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    n = 8192
    a = torch.randn(n, n, device="cuda", dtype=torch.float32)
    b = torch.randn(n, n, device="cuda", dtype=torch.float32)
    for _ in range(2):
        torch.mm(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.mm(a, b)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1) * 1e-3)
    torch.backends.cuda.matmul.allow_tf32 = prev
    del a, b
    return 2.0 * n ** 3 / best / 2.0


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except ValueError:
            pass
    return {"hbm_gbs": 6800.0, "fallback": True}


# ---------------------------------------------------------------------------
# CPU baseline (oracle on the host cores)
# ---------------------------------------------------------------------------
def cpu_baseline(queries, min_seconds: float = 8.0, max_queries: int = 512) -> dict:
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    done, t_total, succ, i = 0, 0.0, 0, 0
    while t_total < min_seconds and done < max_queries:
        chunk = [queries[(i + j) % len(queries)] for j in range(64)]
        i += 64
        t0 = time.perf_counter()
        res = O.plan_batch(chunk, threads=threads)
        t_total += time.perf_counter() - t0
        done += len(chunk)
        succ += sum(r["status"] == 1 for r in res)
    return {"value": done / t_total, "unit": "queries/s", "cores": threads, "kind": "port",
            "sample": f"{done} queries of the same workload (64 per OpenMP batch, one query per thread), "
                      f"{t_total:.1f} s wall on {threads} threads; success {succ / done:.3f}",
            "success_rate": succ / done}


# ---------------------------------------------------------------------------
# reference arm
# ---------------------------------------------------------------------------
def run_reference(args) -> None:
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O
    queries = make_workload(0)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        O.plan_batch(queries[:16], threads=threads)
    t_total, succ = 0.0, 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        res = O.plan_batch(queries, threads=threads)
        t_total += time.perf_counter() - t0
        succ += sum(r["status"] == 1 for r in res)
    value = N_QUERIES * args.steps / t_total
    line = {
        "impl": "reference", "metric": "planning queries/sec", "value": value, "unit": "queries/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded Philox scenes, no dataset)",
        "config": config_of(1), "parallelism": f"OpenMP over queries, {threads} threads",
        "success_rate": succ / (N_QUERIES * args.steps),
        "cpu_baseline": {"value": value, "unit": "queries/s", "cores": threads, "kind": "port",
                         "sample": f"the full {N_QUERIES}-query batch per step; CPU restatement of the reference planner "
                                   f"(the reference's src/cpu planner needs OMPL, unavailable)"},
        "e2e": {"value": value, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def run_ours(args) -> None:
    import torch
    import torch.distributed as dist

    from kgmt_gb300 import workloads as W
    from kgmt_gb300.planner import KGMT, BatchPlanner, pack_configs
    from kgmt_gb300._abi import KgmtResult

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local)
    queries = make_workload(rank)
    cfgs = [q.config for q in queries]
    inits, goals, obs, offs, cnts = W.pack_queries(queries)
    stream = torch.cuda.Stream(device=dev)
    h = stream.cuda_stream

    planner = BatchPlanner(N_QUERIES, iters_per_graph=4, stream=h)
    d_inits = torch.from_numpy(inits).to(dev)
    d_goals = torch.from_numpy(goals).to(dev)
    d_obs = torch.from_numpy(obs).to(dev)
    carr = pack_configs(cfgs)
    res = (KgmtResult * N_QUERIES)()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()

    for _ in range(args.warmup):
        planner.plan_device(cfgs, d_inits, d_goals, d_obs, offs, cnts, carr=carr, res=res)

    clocks = ClockSampler(local)
    clocks.start()
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    total_ms = 0.0
    launches = 0
    step_results = []
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        planner.plan_device(cfgs, d_inits, d_goals, d_obs, offs, cnts, carr=carr, res=res)
        e1.record(stream)
        e1.synchronize()
        total_ms += e0.elapsed_time(e1)
        launches += planner.stats()["kernel_launches"]
        step_results.append([res[i].as_dict() for i in range(N_QUERIES)])
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    clk = clocks.stop()
    total_ms, value = whole_job_rate(total_ms, N_QUERIES, args.steps, ws, device=dev)

    last = step_results[-1]
    solve = sorted(r["solve_ms"] for r in last)
    success = sum(r["status"] == 1 for r in last) / N_QUERIES

    # ---- end to end through the public API with host buffers ----
    # (configs packed and the result array made once, as a caller that plans
    # repeatedly would; every step still copies configs, starts, goals and
    # boxes to the device and the results back)
    pin = lambda a: torch.from_numpy(a).pin_memory().numpy()  # noqa: E731
    h_inits, h_goals, h_obs = pin(inits), pin(goals), pin(obs)
    e2e_res = (KgmtResult * N_QUERIES)()
    planner.plan(cfgs, h_inits, h_goals, h_obs, offs, cnts, carr=carr, res=e2e_res)
    torch.cuda.synchronize()
    e2e_ms = 0.0
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        stream.synchronize()
        t0 = time.perf_counter()
        out = planner.plan(cfgs, h_inits, h_goals, h_obs, offs, cnts, carr=carr, res=e2e_res)
        e2e_ms += (time.perf_counter() - t0) * 1e3
    e2e_ms, e2e_value = whole_job_rate(e2e_ms, N_QUERIES, args.steps, ws, device=dev)
    h2d = inits.nbytes + goals.nbytes + obs.nbytes + len(cfgs) * C_SIZEOF_CONFIG
    d2h = N_QUERIES * C_SIZEOF_RESULT

    line = None
    if rank == 0:
        # ---- per-kernel CUDA-event times (separate profiled pass, direct launches) ----
        prof = BatchPlanner(N_QUERIES, stream=h, profile_kernels=True)
        prof.plan_device(cfgs, d_inits, d_goals, d_obs, offs, cnts)
        st = prof.stats()
        prof.close()
        fp32_peak = measured_fp32_lane_ops(torch)
        prop_ms_avg = st["ms_propagate"] / max(1, st["launches_propagate"])
        # the k_propagate launches' own work (the persistent tail launch propagates too)
        achieved = (st["fp32_ops"] - st["fp32_ops_tail"]) / max(1e-9, st["ms_propagate"] * 1e-3)
        # ---- plain form: the same queries one at a time ----
        n_plain = 32
        plain_times, plain_res = [], []
        p = KGMT(cfgs[0], stream=h)
        for q in queries[:n_plain]:
            d_o = torch.from_numpy(q.obstacles).to(dev)
            if p.config != q.config:
                p.close()
                p = KGMT(q.config, stream=h)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r = p.plan(q.init, q.goal, d_o, q.obstacles.shape[0])
            plain_times.append((time.perf_counter() - t0) * 1e3)
            plain_res.append(r)
        p.close()
        plain_ms = sum(plain_times)
        same = all(plain_res[i]["tree_size"] == last[i]["tree_size"] and plain_res[i]["goal_index"] == last[i]["goal_index"]
                   for i in range(n_plain))
        plain_qps = n_plain / (plain_ms * 1e-3)
        plain_succ = sum(r["status"] == 1 for r in plain_res) / n_plain
        cpu = cpu_baseline(queries)
        peaks = measured_peaks()
        # ---- configs 4 and 5: the mixed batch, and a served stream from it ----
        from kgmt_gb300 import measure as M
        mixed_qs = W.mixed_batch(N_MIXED, seed=1)
        mixed = M.mixed_line(mixed_qs, reps=3, plain_sample=MIXED_PLAIN_SAMPLE)
        served = []
        for rate, n_served in SERVED_STREAMS:
            sv = M.served_line(mixed_qs, rate, n_served)
            sv["served_over_plain"] = sv["queries_per_s"] / mixed["plain"]["queries_per_s"]
            served.append(sv)
        total_kernel_ms = st["ms_propagate"] + st["ms_tail"] + st["ms_append"]
        line = {
            "metric": "planning queries/sec", "value": value, "unit": "queries/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded Philox scenes, no dataset)",
            "config": config_of(ws), "parallelism": "query-sharded (one 256-query shard per GPU)",
            "settings": {"propagate_block": 256, "iters_per_graph": 4},
            "p50_solve_ms": float(np.percentile(solve, 50)), "p99_solve_ms": float(np.percentile(solve, 99)),
            "success_rate": success,
            "plain": {"value": plain_qps, "unit": "queries/s", "queries": n_plain, "success_rate": plain_succ,
                      "p50_solve_ms": float(np.percentile(plain_times, 50)),
                      "p99_solve_ms": float(np.percentile(plain_times, 99)), "results_identical_to_batched": same},
            "batched_over_plain": value / ws / plain_qps,
            "e2e": {"value": e2e_value, "unit": "queries/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "roofline": {"kernel": "k_propagate", "bound": "fp32", "achieved": achieved * 1e-12, "peak": fp32_peak * 1e-12,
                         "unit": "T FP32 lane-ops/s", "frac": achieved / fp32_peak,
                         **propagate_traffic((st["samples"] - st["samples_tail"]) / max(1, st["launches_propagate"])),
                         "traffic_unit": "DRAM bytes per launch",
                         # the k_propagate launches' samples; their accepted ones in the
                         # batch's proportion (the tail launch propagates the rest)
                         "algorithmic_bytes_per_launch": ((st["samples"] - st["samples_tail"]) * PROPAGATE_BYTES_PER_SAMPLE
                                                          + sum(r["tree_size"] - 1 for r in last) * PROPAGATE_BYTES_PER_ACCEPTED
                                                          * (st["samples"] - st["samples_tail"]) / max(1, st["samples"]))
                         / max(1, st["launches_propagate"]),
                         "peak_source": "measured: cuBLAS SGEMM 8192^3 (TF32 off) FLOP/s / 2",
                         "avg_launch_ms": prop_ms_avg, "launches": st["launches_propagate"],
                         "share_of_kernel_time": st["ms_propagate"] / max(1e-9, total_kernel_ms)},
            "kernel_ms": {"propagate": st["ms_propagate"], "tail": st["ms_tail"], "append": st["ms_append"],
                          "tail_iterations": st["iterations_tail"],
                          "iterations": st["iterations_launched"], "samples": st["samples"],
                          "steps": st["steps_executed"], "obstacle_tests": st["obstacle_tests"]},
            "mixed": mixed,
            "served": {"plain_queries_per_s": mixed["plain"]["queries_per_s"],
                       "plain_note": "the plain form serves one query per launch chain: its rate is the mixed batch's plain rate",
                       "streams": served},
            "hbm_peak_gbs": peaks.get("hbm_gbs"),
            "cpu_baseline": cpu,
            "clocks": clk,
            "gpu_launches": launches,
        }
        print(json.dumps(line), flush=True)
    planner.close()
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()


def _c_sizes():
    import ctypes

    from kgmt_gb300._abi import KgmtConfig, KgmtResult
    return ctypes.sizeof(KgmtConfig), ctypes.sizeof(KgmtResult)


C_SIZEOF_CONFIG, C_SIZEOF_RESULT = _c_sizes()


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    args = ap.parse_args(argv)
    if args.warmup < 3:
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)
    return 0


if __name__ == "__main__":
    sys.exit(main())
