"""Runs a batched planning workload a few times through the C ABI (host
buffers, no torch), for kernel profiling:

    python -m kgmt_gb300.profile_workload [--queries 256] [--steps 2] [--no-graph]
                                          [--model di|quad|mixed] [--profile-kernels]

Prints one line per step with the wall time and the success rate.  The
workloads: the seeded double-integrator batch (50 boxes per query, T=50k),
quadrotor queries (200 boxes, T=capacity), or the mixed batch (half double
integrator, half quadrotor; 5..1000 boxes; 8^3..32^3 grids; T 10k..500k).
--profile-kernels times every kernel with CUDA events (direct launches) and
prints the per-kernel totals of the last step.
"""
from __future__ import annotations

import argparse
import sys
import time

import numpy as np

from . import workloads as W
from .planner import BatchPlanner


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--queries", type=int, default=256)
    ap.add_argument("--obstacles", type=int, default=50)
    ap.add_argument("--capacity", type=int, default=50_000)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--block", type=int, default=256)
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--model", choices=["di", "quad", "mixed"], default="di")
    ap.add_argument("--profile-kernels", action="store_true")
    a = ap.parse_args(argv)
    if a.model == "di":
        qs = W.double_integrator_batch(a.queries, n_obstacles=a.obstacles, seed=1, tree_capacity=a.capacity)
    elif a.model == "mixed":
        qs = W.mixed_batch(a.queries, seed=1)
    else:
        qs = [W.quadrotor_query(seed=1 + i, n_obstacles=a.obstacles, tree_capacity=a.capacity) for i in range(a.queries)]
    inits, goals, obs, offs, cnts = W.pack_queries(qs)
    b = BatchPlanner(a.queries, propagate_block=a.block, use_graph=not a.no_graph, profile_kernels=a.profile_kernels)
    for s in range(a.steps):
        t0 = time.perf_counter()
        res = b.plan([q.config for q in qs], inits, goals, obs, offs, cnts)
        dt = time.perf_counter() - t0
        succ = np.mean([r["status"] == 1 for r in res])
        st = b.stats()
        print(f"step {s}: {dt * 1e3:.2f} ms, {a.queries / dt:.0f} queries/s, success {succ:.3f}, "
              f"iterations {st['iterations_launched']} (+{st['iterations_tail']} in tail launches), "
              f"launches {st['kernel_launches']}, samples {st['samples']}")
    if a.profile_kernels:
        print(f"kernels (CUDA events, last step): propagate {st['ms_propagate']:.3f} ms in {st['launches_propagate']} launches, "
              f"append {st['ms_append']:.3f} ms in {st['launches_append']}, tail {st['ms_tail']:.3f} ms in {st['launches_tail']}")
    b.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
