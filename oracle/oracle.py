"""ctypes binding of the CPU oracle (test infrastructure only).

Only the tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg load this module; the product never does.  ``load()`` builds
``oracle/_build/libkgmt_oracle.so`` with ``make`` when it is missing.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libkgmt_oracle.so"
MAX_SAMPLE_DIM = 17


class KoConfig(C.Structure):
    _fields_ = [
        ("model", C.c_int32), ("di_rule", C.c_int32), ("tree_capacity", C.c_uint32), ("samples_per_node", C.c_uint32),
        ("max_iterations", C.c_uint32), ("min_steps", C.c_uint32), ("max_steps", C.c_uint32), ("step_size", C.c_float),
        ("goal_radius", C.c_float), ("epsilon", C.c_float), ("ws_min", C.c_float), ("ws_max", C.c_float),
        ("coarse_len", C.c_uint32), ("fine_len", C.c_uint32), ("v_min", C.c_float), ("v_max", C.c_float),
        ("u_min", C.c_float * 4), ("u_max", C.c_float * 4), ("nu", C.c_float), ("mu", C.c_float), ("ix", C.c_float),
        ("iy", C.c_float), ("iz", C.c_float), ("gravity", C.c_float), ("mass_inv", C.c_float), ("seed", C.c_uint64),
        ("pitch_min", C.c_float), ("pitch_max", C.c_float), ("wheelbase", C.c_float), ("reserved", C.c_uint32),
    ]


class KoResult(C.Structure):
    _fields_ = [("status", C.c_int32), ("iterations", C.c_uint32), ("tree_size", C.c_uint32), ("goal_index", C.c_int32),
                ("path_len", C.c_uint32), ("samples_drawn", C.c_uint32)]


class KoIterView(C.Structure):
    _fields_ = [("itr", C.c_uint32), ("tree_size", C.c_uint32), ("frontier_size", C.c_uint32), ("expanded", C.c_uint32),
                ("n_react", C.c_uint32), ("n_rep_new", C.c_uint32), ("goal_index", C.c_int32), ("regions", C.c_uint32),
                ("rep_old", C.POINTER(C.c_uint32)), ("rep_new", C.POINTER(C.c_uint32)), ("counter", C.POINTER(C.c_int32)),
                ("valid", C.POINTER(C.c_int32)), ("score", C.POINTER(C.c_float))]


KO_ITER_HOOK = C.CFUNCTYPE(None, C.POINTER(KoIterView), C.c_void_p)


class KoTrace(C.Structure):
    _fields_ = [("itr", C.c_uint32), ("tree_size_before", C.c_uint32), ("n_samples", C.c_uint32),
                ("samples_per_entry", C.c_uint32), ("n_next", C.c_uint32), ("n_react", C.c_uint32),
                ("repeat_total", C.c_uint32), ("f_accept", C.c_float), ("score_total", C.c_float)]


def to_ko(cfg) -> KoConfig:
    k = KoConfig()
    for name, _ in KoConfig._fields_:
        v = getattr(cfg, name)
        if name in ("u_min", "u_max"):
            arr = (C.c_float * 4)(*[float(x) for x in v])
            setattr(k, name, arr)
        else:
            setattr(k, name, v)
    return k


def _ptr(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


_lib = None


def build(force: bool = False) -> Path:
    if force or not LIB_PATH.exists():
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


def load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB_PATH))
        f = C.c_float
        fp, u8p, i32p, u32p = C.POINTER(C.c_float), C.POINTER(C.c_uint8), C.POINTER(C.c_int32), C.POINTER(C.c_uint32)
        cfgp = C.POINTER(KoConfig)
        lib.ko_u01.restype = f
        lib.ko_react_uniform.restype = f
        lib.ko_react_uniform.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32]
        lib.ko_sample_uniforms.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, fp]
        lib.ko_sincosf.argtypes = [f, fp, fp]
        lib.ko_region.argtypes = [cfgp, fp]
        lib.ko_subregion.argtypes = [cfgp, fp, C.c_int]
        lib.ko_segment_valid.argtypes = [fp, fp, fp, C.c_uint32]
        lib.ko_distance.restype = f
        lib.ko_distance.argtypes = [fp, fp]
        lib.ko_propagate_f32.argtypes = [cfgp, fp, fp, fp, C.c_uint32, C.c_uint32, fp, u8p, i32p, i32p]
        lib.ko_propagate_f64.argtypes = [cfgp, fp, fp, fp, C.c_uint32, C.c_uint32, C.POINTER(C.c_double), u8p]
        lib.ko_verdict_margin_f64.restype = C.c_double
        lib.ko_verdict_margin_f64.argtypes = [cfgp, fp, fp, fp, C.c_uint32]
        lib.ko_score_update.argtypes = [cfgp, i32p, i32p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), fp, fp]
        lib.ko_f_accept.restype = f
        lib.ko_f_accept.argtypes = [C.c_uint32, f, C.c_uint32, C.c_uint32, C.c_uint32]
        lib.ko_plan.argtypes = [cfgp, fp, fp, fp, C.c_uint32, C.POINTER(KoResult), fp, i32p, fp, fp, C.POINTER(KoTrace)]
        lib.ko_plan_hooked.argtypes = [cfgp, fp, fp, fp, C.c_uint32, C.POINTER(KoResult), fp, i32p, fp, fp, C.POINTER(KoTrace),
                                       KO_ITER_HOOK, C.c_void_p]
        lib.ko_plan_batch.argtypes = [C.c_uint32, cfgp, fp, fp, fp, u32p, u32p, C.POINTER(KoResult), C.c_int]
        _lib = lib
    return _lib


def philox(ctr, key):
    lib = load()
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib.ko_philox4x32_10(c, k, o)
    return list(o)


def sample_uniforms(seed: int, slot: int, itr: int) -> np.ndarray:
    u = np.zeros(8, np.float32)
    load().ko_sample_uniforms(seed, slot, itr, _ptr(u, C.c_float))
    return u


def react_uniform(seed: int, node: int, itr: int) -> float:
    return float(load().ko_react_uniform(seed, node, itr))


def sincos(x: float):
    s, c = C.c_float(), C.c_float()
    load().ko_sincosf(C.c_float(x), C.byref(s), C.byref(c))
    return s.value, c.value


def _f32(a, shape=None):
    a = np.ascontiguousarray(a, np.float32)
    return a if shape is None else a.reshape(shape)


def region(cfg, x) -> int:
    k = to_ko(cfg)
    return int(load().ko_region(C.byref(k), _ptr(_f32(x), C.c_float)))


def subregion(cfg, x, r1) -> int:
    k = to_ko(cfg)
    return int(load().ko_subregion(C.byref(k), _ptr(_f32(x), C.c_float), int(r1)))


def segment_valid(p0, p1, obstacles) -> int:
    obs = _f32(obstacles).reshape(-1, 6)  # 3-D
    return int(load().ko_segment_valid(_ptr(_f32(p0), C.c_float), _ptr(_f32(p1), C.c_float), _ptr(obs, C.c_float),
                                       obs.shape[0]))


def distance(a, b) -> float:
    return float(load().ko_distance(_ptr(_f32(a), C.c_float), _ptr(_f32(b), C.c_float)))


def ws_dims(model: int) -> int:
    return 2 if model == 0 else 3


def boxes(cfg, obstacles) -> np.ndarray:
    """Boxes in the model's layout, rows of 2W floats (min corner, max
    corner).  A [m, 6] array given for a planar model keeps its x and y
    extents; a flat array is taken as rows of 2W already."""
    w = ws_dims(cfg.model)
    a = _f32(obstacles)
    if a.size == 0:
        return np.zeros((0, 2 * w), np.float32)
    if w == 2 and a.ndim == 2 and a.shape[1] == 6:
        a = a[:, [0, 1, 3, 4]]
    return np.ascontiguousarray(a.reshape(-1, 2 * w))


def propagate_f32(cfg, x0, u, obstacles):
    """x0 [n, D], u [n, 8], obstacles [m, 6] or [m, 2W] -> (x1 [n, D], valid [n], r1, r2)."""
    k = to_ko(cfg)
    x0 = _f32(x0)
    u = _f32(u)
    obs = boxes(cfg, obstacles)
    n = x0.shape[0]
    x1 = np.zeros_like(x0)
    valid = np.zeros(n, np.uint8)
    r1 = np.zeros(n, np.int32)
    r2 = np.zeros(n, np.int32)
    load().ko_propagate_f32(C.byref(k), _ptr(x0, C.c_float), _ptr(u, C.c_float), _ptr(obs, C.c_float), obs.shape[0], n,
                            _ptr(x1, C.c_float), _ptr(valid, C.c_uint8), _ptr(r1, C.c_int32), _ptr(r2, C.c_int32))
    return x1, valid, r1, r2


def propagate_f64(cfg, x0, u, obstacles):
    k = to_ko(cfg)
    x0 = _f32(x0)
    u = _f32(u)
    obs = boxes(cfg, obstacles)
    n = x0.shape[0]
    x1 = np.zeros(x0.shape, np.float64)
    valid = np.zeros(n, np.uint8)
    load().ko_propagate_f64(C.byref(k), _ptr(x0, C.c_float), _ptr(u, C.c_float), _ptr(obs, C.c_float), obs.shape[0], n,
                            _ptr(x1, C.c_double), _ptr(valid, C.c_uint8))
    return x1, valid


def verdict_margin_f64(cfg, x0, u, obstacles) -> float:
    k = to_ko(cfg)
    obs = boxes(cfg, obstacles)
    return float(load().ko_verdict_margin_f64(C.byref(k), _ptr(_f32(x0), C.c_float), _ptr(_f32(u), C.c_float),
                                           _ptr(obs, C.c_float), obs.shape[0]))


def score_update(cfg, counter, valid, marks, newmarks):
    k = to_ko(cfg)
    counter = np.ascontiguousarray(counter, np.int32)
    valid = np.ascontiguousarray(valid, np.int32)
    marks = np.array(marks, np.uint64)
    newmarks = np.array(newmarks, np.uint64)
    score = np.zeros(counter.size, np.float32)
    tot = C.c_float()
    load().ko_score_update(C.byref(k), _ptr(counter, C.c_int32), _ptr(valid, C.c_int32), _ptr(marks, C.c_uint64),
                           _ptr(newmarks, C.c_uint64), _ptr(score, C.c_float), C.byref(tot))
    return score, tot.value, marks


def f_accept(itr, eps, tree_size, n_next, capacity) -> float:
    return float(load().ko_f_accept(itr, eps, tree_size, n_next, capacity))


def plan(query, trace: bool = False, tables: bool = False):
    """Run one query; returns dict with result fields, tree and path.  With
    ``tables`` also ``out["tables"]``: per iteration the sizes, the region
    counters, valid counts and scores after it, and the next frontier as
    per-node flags and repeat counts (what the reference's planBench dumps,
    KGMT.cu:405-488)."""
    cfg = query.config
    k = to_ko(cfg)
    D = cfg.sample_dim
    T = cfg.tree_capacity
    samples = np.zeros((T, D), np.float32)
    parents = np.zeros(T, np.int32)
    costs = np.zeros(T, np.float32)
    path = np.zeros((cfg.max_iterations + 2, D), np.float32)
    tr = (KoTrace * cfg.max_iterations)() if trace else None
    res = KoResult()
    init = _f32(query.init)
    goal = _f32(query.goal)
    obs = boxes(cfg, query.obstacles)
    snaps = []

    def on_iteration(v_p, _user):
        v = v_p.contents
        arr = lambda p, n: np.ctypeslib.as_array(p, shape=(n,)).copy() if n else np.zeros(0)  # noqa: E731
        frontier = np.zeros(T, np.uint8)
        repeat = np.zeros(T, np.uint32)
        old = arr(v.rep_old, v.n_react).astype(np.int64)
        new = arr(v.rep_new, v.n_rep_new).astype(np.int64)
        frontier[old] = 1
        frontier[new] = 1
        np.add.at(repeat, old, 1)
        np.add.at(repeat, new, 1)
        snaps.append(dict(itr=v.itr, tree_size=v.tree_size, frontier_size=v.frontier_size, expanded=v.expanded,
                          goal_index=v.goal_index, next_frontier_size=int(frontier.sum()), counter=arr(v.counter, v.regions),
                          valid=arr(v.valid, v.regions), score=arr(v.score, v.regions), frontier=frontier, repeat=repeat))

    hook = KO_ITER_HOOK(on_iteration) if tables else KO_ITER_HOOK()
    rc = load().ko_plan_hooked(C.byref(k), _ptr(init, C.c_float), _ptr(goal, C.c_float), _ptr(obs, C.c_float), obs.shape[0],
                               C.byref(res), _ptr(samples, C.c_float), _ptr(parents, C.c_int32), _ptr(costs, C.c_float),
                               _ptr(path, C.c_float), tr, hook, None)
    if rc != 0:
        raise RuntimeError(f"ko_plan failed: {rc}")
    out = dict(status=res.status, iterations=res.iterations, tree_size=res.tree_size, goal_index=res.goal_index,
               path_len=res.path_len, samples_drawn=res.samples_drawn)
    n = res.tree_size
    out["samples"] = samples[:n]
    out["parents"] = parents[:n]
    out["costs"] = costs[:n]
    out["path"] = path[: res.path_len]
    if tables:
        out["tables"] = snaps
    if trace:
        out["trace"] = [dict((f, getattr(tr[i], f)) for f, _ in KoTrace._fields_) for i in range(res.iterations)]
    return out


def plan_batch(queries, threads: int = 0):
    """Independent queries, OpenMP over queries.  Returns list of result dicts."""
    n = len(queries)
    cfgs = (KoConfig * n)(*[to_ko(q.config) for q in queries])
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
        obs[offs[i]: offs[i] + counts[i]] = q.obstacles
    res = (KoResult * n)()
    rc = load().ko_plan_batch(n, cfgs, _ptr(inits, C.c_float), _ptr(goals, C.c_float), _ptr(obs, C.c_float),
                              _ptr(offs, C.c_uint32), _ptr(counts, C.c_uint32), res, threads)
    if rc != 0:
        raise RuntimeError("ko_plan_batch failed")
    return [dict(status=r.status, iterations=r.iterations, tree_size=r.tree_size, goal_index=r.goal_index,
                 path_len=r.path_len, samples_drawn=r.samples_drawn) for r in res]


def max_threads() -> int:
    return int(load().ko_max_threads())
