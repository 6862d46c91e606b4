"""Seeded synthetic planning workloads (no public dataset is involved).

Obstacles are axis-aligned boxes stored as rows ``min x, min y, min z, max x,
max y, max z`` -- the layout of the reference's obstacle CSVs
(include/config/obstacles/*/obstacles.csv, read by src/helper/helper.cu:13-39).
Boxes that would contain the start or touch the goal ball are redrawn.
All randomness comes from numpy's counter-based Philox generator, so a seed
gives the same scene on every machine.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .config import (MAX_SAMPLE_DIM, MODEL_DOUBLE_INTEGRATOR, MODEL_QUADROTOR, PlannerConfig,
                     double_integrator_batched, double_integrator_single, dubins_airplane, quadrotor_large, sample_dim,
                     unicycle)


@dataclass
class Query:
    config: PlannerConfig
    init: np.ndarray  # float32 [sample_dim]
    goal: np.ndarray  # float32 [sample_dim]
    obstacles: np.ndarray  # float32 [n, 6]


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.Philox(key=seed & 0xFFFFFFFFFFFFFFFF))


def _blocked(box: np.ndarray, start: np.ndarray, goal: np.ndarray, goal_r: float, margin: float) -> bool:
    lo, hi = box[:3], box[3:]
    if np.all(start >= lo - margin) and np.all(start <= hi + margin):
        return True
    nearest = np.clip(goal, lo, hi)
    return float(np.linalg.norm(nearest - goal)) <= goal_r + margin


def random_boxes(rng: np.random.Generator, n: int, edge_lo: float, edge_hi: float, start: np.ndarray, goal: np.ndarray,
                 goal_r: float, centre_lo: float = 0.1, centre_hi: float = 0.9, margin: float = 0.01) -> np.ndarray:
    """n boxes with centres U[centre_lo, centre_hi]^3 and edges U[edge_lo, edge_hi]."""
    out = np.zeros((n, 6), np.float32)
    i = 0
    while i < n:
        c = rng.uniform(centre_lo, centre_hi, 3)
        e = rng.uniform(edge_lo, edge_hi, 3)
        box = np.concatenate([c - e / 2, c + e / 2]).astype(np.float32)
        if _blocked(box, start, goal, goal_r, margin):
            continue
        out[i] = box
        i += 1
    return out


def _state(model: int, pos) -> np.ndarray:
    x = np.zeros(sample_dim(model), np.float32)
    x[:3] = pos
    return x


def double_integrator_query(seed: int = 1, n_obstacles: int = 10) -> Query:
    """Single double-integrator query: 10 boxes, edges U[0.05,0.15], start
    (0.05,0.05,0.05) at rest, goal ball r=0.05 at (0.95,0.95,0.95)."""
    cfg = double_integrator_single(seed)
    start = np.float32([0.05, 0.05, 0.05])
    goal = np.float32([0.95, 0.95, 0.95])
    obs = random_boxes(_rng(seed * 7919 + 11), n_obstacles, 0.05, 0.15, start, goal, cfg.goal_radius)
    return Query(cfg, _state(cfg.model, start), _state(cfg.model, goal), obs)


def quadrotor_query(seed: int = 1, n_obstacles: int = 200, **overrides) -> Query:
    """Single quadrotor query: 200 boxes with edges U[0.02, 0.1]."""
    cfg = quadrotor_large(seed).replace(**overrides)
    start = np.float32([0.05, 0.05, 0.05])
    goal = np.float32([0.95, 0.95, 0.95])
    obs = random_boxes(_rng(seed * 7919 + 13), n_obstacles, 0.02, 0.1, start, goal, cfg.goal_radius)
    return Query(cfg, _state(cfg.model, start), _state(cfg.model, goal), obs)


def dubins_query(seed: int = 1, n_obstacles: int = 10, **overrides) -> Query:
    """Single Dubins-airplane query: 10 boxes with edges U[0.05, 0.15], start
    (0.05, 0.05, 0.05) heading yaw pi/4, pitch 0.4, speed 0.15; goal ball
    r=0.05 at (0.95, 0.95, 0.95)."""
    cfg = dubins_airplane(seed).replace(**overrides)
    start = np.float32([0.05, 0.05, 0.05])
    goal = np.float32([0.95, 0.95, 0.95])
    obs = random_boxes(_rng(seed * 7919 + 17), n_obstacles, 0.05, 0.15, start, goal, cfg.goal_radius)
    init = np.zeros(cfg.sample_dim, np.float32)
    init[:6] = [start[0], start[1], start[2], math.pi / 4, 0.4, 0.15]
    return Query(cfg, init, _state(cfg.model, goal), obs)


def planar_boxes(rng: np.random.Generator, n: int, edge_lo: float, edge_hi: float, start: np.ndarray, goal: np.ndarray,
                 goal_r: float, margin: float = 0.01) -> np.ndarray:
    """n boxes in the plane, centres U[0.1, 0.9]^2, edges U[edge_lo, edge_hi],
    stored as rows of 6 with z extents [0, 1] (a planar query ignores them)."""
    out = np.zeros((n, 6), np.float32)
    i = 0
    while i < n:
        c = rng.uniform(0.1, 0.9, 2)
        e = rng.uniform(edge_lo, edge_hi, 2)
        lo, hi = c - e / 2, c + e / 2
        if np.all(start >= lo - margin) and np.all(start <= hi + margin):
            continue
        if float(np.linalg.norm(np.clip(goal, lo, hi) - goal)) <= goal_r + margin:
            continue
        out[i] = [lo[0], lo[1], 0.0, hi[0], hi[1], 1.0]
        i += 1
    return out


def unicycle_query(seed: int = 1, n_obstacles: int = 10, **overrides) -> Query:
    """Single planar unicycle query: 10 boxes with edges U[0.05, 0.15], start
    (0.05, 0.05) heading pi/4 at speed 0.1; goal disc r=0.05 at (0.95, 0.95)."""
    cfg = unicycle(seed).replace(**overrides)
    start = np.float32([0.05, 0.05])
    goal = np.float32([0.95, 0.95])
    obs = planar_boxes(_rng(seed * 7919 + 19), n_obstacles, 0.05, 0.15, start, goal, cfg.goal_radius)
    init = np.zeros(cfg.sample_dim, np.float32)
    init[:4] = [start[0], start[1], math.pi / 4, 0.1]
    goal_row = np.zeros(cfg.sample_dim, np.float32)
    goal_row[:2] = goal
    return Query(cfg, init, goal_row, obs)


def boxes_for_plan(q: Query) -> np.ndarray:
    """The query's boxes in its model's own layout: rows of 4 (x, y extents)
    for the planar unicycle, rows of 6 otherwise -- what the single-query
    plan takes, like the reference's [n][2 * W_DIM] array."""
    if q.config.ws_dims == 2:
        return np.ascontiguousarray(q.obstacles[:, [0, 1, 3, 4]])
    return q.obstacles


def all_models_batch(n_queries: int = 64, seed: int = 1, tree_capacity: int = 20_000) -> list[Query]:
    """Heterogeneous batch cycling through the four models (unicycle, double
    integrator, Dubins airplane, quadrotor), each query with its own seed and
    scene."""
    out = []
    for q in range(n_queries):
        s = seed * 1_000_003 + q
        m = q % 4
        if m == 0:
            out.append(unicycle_query(seed=s, tree_capacity=tree_capacity))
        elif m == 1:
            qq = double_integrator_query(seed=s)
            qq.config = qq.config.replace(tree_capacity=tree_capacity)
            out.append(qq)
        elif m == 2:
            out.append(dubins_query(seed=s, tree_capacity=tree_capacity))
        else:
            out.append(quadrotor_query(seed=s, n_obstacles=50, tree_capacity=tree_capacity, coarse_len=8, fine_len=2))
    return out


def double_integrator_batch(n_queries: int = 256, n_obstacles: int = 50, seed: int = 1, **overrides) -> list[Query]:
    """Homogeneous batch: each query has its own 50 boxes and its own start
    (U[0.03,0.2]^3) / goal (U[0.8,0.97]^3) pair; T = 50k nodes each."""
    rng = _rng(seed * 104729 + 3)
    out = []
    for q in range(n_queries):
        cfg = double_integrator_batched(seed=seed * 1_000_003 + q).replace(**overrides)
        start = rng.uniform(0.03, 0.2, 3).astype(np.float32)
        goal = rng.uniform(0.8, 0.97, 3).astype(np.float32)
        obs = random_boxes(rng, n_obstacles, 0.05, 0.15, start, goal, cfg.goal_radius)
        out.append(Query(cfg, _state(cfg.model, start), _state(cfg.model, goal), obs))
    return out


def mixed_batch(n_queries: int = 1024, seed: int = 1, capacity_scale: float = 1.0) -> list[Query]:
    """Heterogeneous batch: half double integrator, half quadrotor; obstacle
    counts log-uniform in [5, 1000] with edges shrinking as counts grow, grids
    8^3..32^3 coarse, tree capacities 10k..500k (log-uniform)."""
    rng = _rng(seed * 15485863 + 5)
    out = []
    for q in range(n_queries):
        quad = (q % 2) == 1
        n_obs = int(round(math.exp(rng.uniform(math.log(5), math.log(1000)))))
        coarse = int(rng.choice([8, 16, 32]))
        fine = 2 if coarse == 32 else int(rng.choice([2, 4]))
        cap = int(round(math.exp(rng.uniform(math.log(10_000), math.log(500_000)))) * capacity_scale)
        cap = max(cap, 1000)
        qseed = seed * 1_000_003 + q
        if quad:
            cfg = quadrotor_large(qseed).replace(tree_capacity=cap, coarse_len=coarse, fine_len=fine)
        else:
            cfg = double_integrator_single(qseed).replace(tree_capacity=cap, coarse_len=coarse, fine_len=fine)
        start = rng.uniform(0.03, 0.2, 3).astype(np.float32)
        goal = rng.uniform(0.8, 0.97, 3).astype(np.float32)
        # keep the filled volume near 5%: edge ~ (0.05 / n)^(1/3)
        e_mid = min(0.15, (0.05 / n_obs) ** (1.0 / 3.0))
        obs = random_boxes(rng, n_obs, 0.5 * e_mid, 1.5 * e_mid, start, goal, cfg.goal_radius)
        out.append(Query(cfg, _state(cfg.model, start), _state(cfg.model, goal), obs))
    return out


def poisson_arrivals(n: int, rate_qps: float, seed: int = 1) -> np.ndarray:
    """Arrival times (s) of a Poisson stream."""
    rng = _rng(seed * 32452843 + 7)
    return np.cumsum(rng.exponential(1.0 / rate_qps, n))


def pack_queries(queries: list[Query]):
    """Flatten queries into the arrays the batch entry points take."""
    n = len(queries)
    inits = np.zeros((n, MAX_SAMPLE_DIM), np.float32)
    goals = np.zeros((n, MAX_SAMPLE_DIM), np.float32)
    counts = np.zeros(n, np.uint32)
    offs = np.zeros(n, np.uint32)
    tot = 0
    for i, q in enumerate(queries):
        inits[i, : q.init.size] = q.init
        goals[i, : q.goal.size] = q.goal
        counts[i] = q.obstacles.shape[0]
        offs[i] = tot
        tot += q.obstacles.shape[0]
    obs = np.zeros((max(tot, 1), 6), np.float32)
    for i, q in enumerate(queries):
        if counts[i]:
            obs[offs[i]: offs[i] + counts[i]] = q.obstacles
    return inits, goals, obs, offs, counts
