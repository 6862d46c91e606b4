"""Measurements of the five planning workloads (one JSON line each):

    python -m kgmt_gb300.measure single     # 1: one double-integrator query, T=100k, plain form
    python -m kgmt_gb300.measure quad       # 2: one quadrotor query, T=2M, 200 boxes, plain form
    python -m kgmt_gb300.measure batch      # 3: 256 double-integrator queries, batched
    python -m kgmt_gb300.measure mixed      # 4: 1024 mixed queries, batched, checked against plain
    python -m kgmt_gb300.measure served     # 5: Poisson stream from the mixed set, continuous batching
    python -m kgmt_gb300.measure dubins     # Dubins airplane: plain single queries, then 256 batched
    python -m kgmt_gb300.measure unicycle   # planar unicycle: plain single queries, then 256 batched

Queries/s, p50/p99 solve latency, success rate; the plain form (one query per
launch chain) is measured beside the batched and served forms on the same
queries.  Inputs are seeded synthetic scenes (kgmt_gb300/workloads.py).
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np

from . import workloads as W
from .planner import KGMT, BatchPlanner, Server


def _pct(x, p):
    return float(np.percentile(np.asarray(x, dtype=np.float64), p)) if len(x) else None


def _device_obstacles(q):
    # the single-query plan takes the model's own rows (4 floats for the planar unicycle)
    import torch
    return torch.from_numpy(np.ascontiguousarray(W.boxes_for_plan(q), np.float32)).to("cuda")


def plain_run(queries, repeat: int = 1):
    """One query per launch chain, sequentially; wall time per query."""
    times, res = [], []
    planner, cur = None, None
    for q in queries:
        if cur != q.config:
            if planner:
                planner.close()
            planner, cur = KGMT(q.config), q.config
        d = _device_obstacles(q)
        for _ in range(repeat):
            t0 = time.perf_counter()
            r = planner.plan(q.init, q.goal, d, q.obstacles.shape[0])
            times.append((time.perf_counter() - t0) * 1e3)
        res.append(r)
    if planner:
        planner.close()
    return times, res


def summarise(name, times_ms, results, extra=None):
    line = {"workload": name, "queries": len(results), "queries_per_s": len(times_ms) / (sum(times_ms) * 1e-3),
            "p50_solve_ms": _pct(times_ms, 50), "p99_solve_ms": _pct(times_ms, 99),
            "success_rate": float(np.mean([r["status"] == 1 for r in results])),
            "mean_iterations": float(np.mean([r["iterations"] for r in results])),
            "mean_tree_size": float(np.mean([r["tree_size"] for r in results]))}
    if extra:
        line.update(extra)
    return line


def m_single(args):
    qs = [W.double_integrator_query(seed=s) for s in range(1, args.n + 1)]
    times, res = plain_run(qs, repeat=1)
    times2, _ = plain_run(qs, repeat=1)  # warm second pass
    return summarise("single double integrator, T=100k, 10 boxes, plain", times2, res)


def _model_workload(name, make, args):
    """Plain single queries of one model, then 256 of them batched."""
    qs = [make(seed=s) for s in range(1, args.n + 1)]
    plain_run(qs[:1])
    times, res = plain_run(qs)
    line = summarise(name + ", plain", times, res)
    batch = [make(seed=1000 + s) for s in range(256)]
    walls, bres, _ = _batched(batch, args.reps)
    wall = float(np.median(walls))
    line.update({"batched_256_queries_per_s": len(batch) / wall, "batched_ms": wall * 1e3,
                 "batched_success_rate": float(np.mean([r["status"] == 1 for r in bres]))})
    return line


def m_dubins(args):
    return _model_workload("Dubins airplane, T=200k, 10 boxes", W.dubins_query, args)


def m_unicycle(args):
    return _model_workload("planar unicycle, T=100k, 10 boxes", W.unicycle_query, args)


def m_quad(args):
    qs = [W.quadrotor_query(seed=s) for s in range(1, args.n + 1)]
    plain_run(qs[:1])
    times, res = plain_run(qs)
    return summarise("single quadrotor, T=2M, 200 boxes, dt=0.02, plain", times, res,
                     {"samples_per_query": float(np.mean([r["samples_drawn"] for r in res]))})


def _batched(qs, reps: int, profile: bool = False):
    inits, goals, obs, offs, cnts = W.pack_queries(qs)
    b = BatchPlanner(len(qs), profile_kernels=profile)
    cfgs = [q.config for q in qs]
    b.plan(cfgs, inits, goals, obs, offs, cnts)  # warm-up
    walls, res = [], None
    for _ in range(reps):
        t0 = time.perf_counter()
        res = b.plan(cfgs, inits, goals, obs, offs, cnts)
        walls.append(time.perf_counter() - t0)
    st = b.stats()
    b.close()
    return walls, res, st


def m_batch(args):
    qs = W.double_integrator_batch(256, n_obstacles=50, seed=1)
    walls, res, st = _batched(qs, args.reps)
    wall = min(walls)
    solve = [r["solve_ms"] for r in res]
    return {"workload": "batched 256 double-integrator queries, 50 boxes, T=50k", "queries": len(qs),
            "queries_per_s": len(qs) / wall, "batch_ms": wall * 1e3, "p50_solve_ms": _pct(solve, 50),
            "p99_solve_ms": _pct(solve, 99), "success_rate": float(np.mean([r["status"] == 1 for r in res])),
            "iterations_launched": st["iterations_launched"], "kernel_launches": st["kernel_launches"]}


def mixed_line(qs, reps: int, plain_sample: int) -> dict:
    """The heterogeneous batch planned in one launch chain (best of `reps`
    host-clocked runs after a warm-up), and the plain form -- one query per
    launch chain -- on `plain_sample` of the same queries spread over the
    batch, with their results compared."""
    walls, res, st = _batched(qs, reps)
    wall = min(walls)
    solve = [r["solve_ms"] for r in res]
    idx = list(range(0, len(qs), max(1, len(qs) // plain_sample)))[:plain_sample]
    ptimes, pres = plain_run([qs[i] for i in idx])
    same = all(pres[k]["tree_size"] == res[i]["tree_size"] and pres[k]["goal_index"] == res[i]["goal_index"]
               and pres[k]["iterations"] == res[i]["iterations"] for k, i in enumerate(idx))
    by_model = {}
    for q, r in zip(qs, res):
        m = "quad" if q.config.model == 3 else "di"
        by_model.setdefault(m, []).append(r["status"] == 1)
    plain_qps = len(ptimes) / (sum(ptimes) * 1e-3)
    return {"workload": f"batched heterogeneous {len(qs)} queries (half DI, half quad; 5..1000 boxes; grids 8^3..32^3; "
                        f"T 10k..500k)", "queries": len(qs), "queries_per_s": len(qs) / wall, "batch_ms": wall * 1e3,
            "p50_solve_ms": _pct(solve, 50), "p99_solve_ms": _pct(solve, 99),
            "success_rate": float(np.mean([r["status"] == 1 for r in res])),
            "success_by_model": {k: float(np.mean(v)) for k, v in by_model.items()},
            "iterations_launched": st["iterations_launched"],
            "plain": {"queries": len(idx), "sample": f"every {max(1, len(qs) // plain_sample)}-th query of the batch",
                      "queries_per_s": plain_qps, "p50_solve_ms": _pct(ptimes, 50), "p99_solve_ms": _pct(ptimes, 99),
                      "success_rate": float(np.mean([r["status"] == 1 for r in pres])),
                      "results_identical_to_batched": same},
            "batched_over_plain": (len(qs) / wall) / plain_qps}


def served_line(pool, rate: float, n: int, slots: int = 1024, budget_gb: float = 150.0, iters_per_step: int = 2,
                seed: int | None = None) -> dict:
    """A Poisson stream of n queries drawn in order from `pool`, offered at
    `rate` queries/s to a server (continuous batching, admission by device
    memory); latency is submit -> result, host clock."""
    arrivals = W.poisson_arrivals(n, rate, seed=int(rate) if seed is None else seed)
    srv = Server(max_slots=slots, memory_budget=int(budget_gb * (1 << 30)), iters_per_step=iters_per_step)
    t0 = time.perf_counter()
    nxt, done, lat, solve, succ = 0, 0, [], [], []
    steps = 0
    while done < n:
        now = time.perf_counter() - t0
        while nxt < n and arrivals[nxt] <= now:
            q = pool[nxt % len(pool)]
            srv.submit(q.config, q.init, q.goal, q.obstacles)
            nxt += 1
        running, queued = srv.step()
        steps += 1
        for r in srv.poll():
            done += 1
            lat.append(r["latency_ms"])
            solve.append(r["solve_ms"])
            succ.append(r["status"] == 1)
        if running == 0 and queued == 0 and nxt < n:
            time.sleep(max(0.0, min(0.001, arrivals[nxt] - (time.perf_counter() - t0))))
    wall = time.perf_counter() - t0
    srv.close()
    return {"workload": f"served Poisson stream at {rate:.0f} queries/s from the mixed set", "offered_qps": rate,
            "queries": n, "queries_per_s": n / wall, "p50_latency_ms": _pct(lat, 50), "p99_latency_ms": _pct(lat, 99),
            "p50_solve_ms": _pct(solve, 50), "p99_solve_ms": _pct(solve, 99),
            "success_rate": float(np.mean(succ)), "server_steps": steps, "slots": slots, "memory_budget_gb": budget_gb}


def m_mixed(args):
    return mixed_line(W.mixed_batch(args.n_mixed, seed=1), args.reps, args.plain_sample)


def m_served(args):
    pool = W.mixed_batch(args.n_mixed, seed=2)
    return [served_line(pool, float(r), args.n_served, args.slots, args.budget_gb, args.iters_per_step)
            for r in args.rates.split(",")]


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["single", "quad", "batch", "mixed", "served", "dubins", "unicycle"])
    ap.add_argument("--n", type=int, default=16, help="queries for the plain single-query workloads")
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--n-mixed", type=int, default=1024)
    ap.add_argument("--plain-sample", type=int, default=32)
    ap.add_argument("--rates", default="500,2000,5000")
    ap.add_argument("--n-served", type=int, default=2000)
    ap.add_argument("--slots", type=int, default=1024)
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--iters-per-step", type=int, default=2)
    a = ap.parse_args(argv)
    fn = {"single": m_single, "quad": m_quad, "batch": m_batch, "mixed": m_mixed, "served": m_served, "dubins": m_dubins,
          "unicycle": m_unicycle}[a.what]
    out = fn(a)
    for line in out if isinstance(out, list) else [out]:
        print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
