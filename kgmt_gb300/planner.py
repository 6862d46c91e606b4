"""Python host API over the C ABI.

``KGMT`` keeps the reference planner's surface (include/planners/Planner.cuh:
19-44, include/planners/KGMT.cuh:5-36): ``plan(h_initial, h_goal,
d_obstacles_ptr, h_obstaclesCount)`` with a caller-owned device obstacle array,
and the readout fields ``h_treeSize_``, ``h_itr_``, ``h_pathToGoal_``,
``h_controlPathToGoal_``, ``d_treeSamples_ptr_``,
``d_treeSamplesParentIdxs_ptr_``, ``d_treeSampleCosts_ptr_``.  The reference
configures at compile time; here the constructor takes a ``PlannerConfig``.

``BatchPlanner`` and ``Server`` are the batched and served forms.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from ._abi import KgmtBatchOptions, KgmtResult, KgmtServerOptions, check, load, ptr, to_c
from .config import PlannerConfig


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


class KGMT:
    """Single-query planner (drop-in for the reference ``KGMT`` class)."""

    def __init__(self, config: PlannerConfig | None = None, stream: int | None = None):
        self.config = config or PlannerConfig()
        self._lib = load()
        self._cfg = to_c(self.config)
        h = C.c_void_p()
        check(self._lib.kgmt_create(C.byref(self._cfg), stream, C.byref(h)))
        self._h = h
        self.h_treeSize_ = 0
        self.h_itr_ = 0
        self.h_pathToGoal_ = 0
        self.h_controlPathToGoal_ = np.zeros((0, self.config.sample_dim), np.float32)
        self.result: dict | None = None

    def close(self):
        if getattr(self, "_h", None):
            self._lib.kgmt_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def plan(self, h_initial, h_goal, d_obstacles_ptr, h_obstaclesCount: int) -> dict:
        """``KGMT::plan`` (src/planners/KGMT.cu:41-105).  ``d_obstacles_ptr``
        is a device tensor / address of [n][6] floats owned by the caller."""
        D = self.config.sample_dim
        init = np.zeros(D, np.float32)
        goal = np.zeros(D, np.float32)
        a = _f32(h_initial).ravel()
        g = _f32(h_goal).ravel()
        init[: min(D, a.size)] = a[:D]
        goal[: min(D, g.size)] = g[:D]
        check(self._lib.kgmt_plan(self._h, init.ctypes.data, goal.ctypes.data, ptr(d_obstacles_ptr), int(h_obstaclesCount)))
        r = KgmtResult()
        check(self._lib.kgmt_get_result(self._h, C.byref(r)))
        self.result = r.as_dict()
        self.h_treeSize_ = r.tree_size
        self.h_itr_ = r.iterations
        # reference: index of the goal node, 0 while not found (KGMT.cu:72, 345)
        self.h_pathToGoal_ = r.goal_index if r.goal_index > 0 else 0
        self.h_controlPathToGoal_ = self.copy_path()
        return self.result

    def plan_traced(self, h_initial, h_goal, d_obstacles_ptr, h_obstaclesCount: int, hook=None) -> list[dict] | dict:
        """``KGMT::planBench`` (src/planners/KGMT.cu:107-165) without the
        files: the same plan one iteration at a time.  ``hook(it)`` gets a
        dict per iteration (sizes and numpy copies of the tree rows, region
        tables and next frontier); without a hook the dicts are returned."""
        D = self.config.sample_dim
        init = np.zeros(D, np.float32)
        goal = np.zeros(D, np.float32)
        a = _f32(h_initial).ravel()
        g = _f32(h_goal).ravel()
        init[: min(D, a.size)] = a[:D]
        goal[: min(D, g.size)] = g[:D]
        out = []

        def on_iteration(it_p, _user):
            it = it_p.contents
            T, Dd, R = it.capacity, it.sample_dim, it.regions
            arr = lambda p, n: np.ctypeslib.as_array(p, shape=(n,)).copy()  # noqa: E731
            d = {f: getattr(it, f) for f in ("itr", "tree_size", "frontier_size", "expanded", "next_frontier_size",
                                             "goal_index", "path_len")}
            d["samples"] = arr(it.samples, T * Dd).reshape(T, Dd)
            d["parents"] = arr(it.parents, T)
            d["counter"] = arr(it.counter, R)
            d["valid"] = arr(it.valid, R)
            d["score"] = arr(it.score, R)
            d["frontier"] = arr(it.frontier, T)
            d["repeat"] = arr(it.repeat, T)
            d["path"] = arr(it.path, it.path_len * Dd).reshape(it.path_len, Dd) if it.path_len else np.zeros((0, Dd), np.float32)
            if hook is None:
                out.append(d)
            else:
                hook(d)

        cb = _abi.ITERATION_HOOK(on_iteration)
        check(self._lib.kgmt_plan_traced(self._h, init.ctypes.data, goal.ctypes.data, ptr(d_obstacles_ptr), int(h_obstaclesCount),
                                         cb, None))
        r = KgmtResult()
        check(self._lib.kgmt_get_result(self._h, C.byref(r)))
        self.result = r.as_dict()
        self.h_treeSize_ = r.tree_size
        self.h_itr_ = r.iterations
        self.h_pathToGoal_ = r.goal_index if r.goal_index > 0 else 0
        self.h_controlPathToGoal_ = self.copy_path()
        return out if hook is None else self.result

    def copy_tree(self):
        n = self.h_treeSize_
        D = self.config.sample_dim
        samples = np.zeros((n, D), np.float32)
        parents = np.zeros(n, np.int32)
        costs = np.zeros(n, np.float32)
        check(self._lib.kgmt_copy_tree(self._h, samples.ctypes.data, parents.ctypes.data, costs.ctypes.data, n))
        return samples, parents, costs

    def copy_path(self) -> np.ndarray:
        rows = np.zeros((self.config.max_iterations + 2, self.config.sample_dim), np.float32)
        n = C.c_uint32()
        check(self._lib.kgmt_copy_path(self._h, rows.ctypes.data, rows.shape[0], C.byref(n)))
        return rows[: n.value]

    def _device_tree(self):
        s, p, c = C.c_void_p(), C.c_void_p(), C.c_void_p()
        check(self._lib.kgmt_device_tree(self._h, C.byref(s), C.byref(p), C.byref(c)))
        return s.value, p.value, c.value

    @property
    def d_treeSamples_ptr_(self) -> int:
        return self._device_tree()[0]

    @property
    def d_treeSamplesParentIdxs_ptr_(self) -> int:
        return self._device_tree()[1]

    @property
    def d_treeSampleCosts_ptr_(self) -> int:
        return self._device_tree()[2]


def pack_configs(cfgs) -> C.Array:
    arr = (_abi.KgmtConfig * len(cfgs))()
    for i, c in enumerate(cfgs):
        arr[i] = to_c(c)
    return arr


class BatchPlanner:
    """Many independent queries in one device-resident launch chain."""

    def __init__(self, max_queries: int, iters_per_graph: int = 4, propagate_block: int = 256, use_graph: bool = True,
                 stream: int | None = None, profile_kernels: bool = False):
        self._lib = load()
        opt = KgmtBatchOptions(max_queries, iters_per_graph, propagate_block, 1 if use_graph else 0,
                               1 if profile_kernels else 0)
        h = C.c_void_p()
        check(self._lib.kgmt_batch_create(C.byref(opt), stream, C.byref(h)))
        self._h = h
        self.max_queries = max_queries
        self._n = 0

    def close(self):
        if getattr(self, "_h", None):
            self._lib.kgmt_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def plan(self, cfgs, inits, goals, obstacles, obs_offset, obs_count, carr=None, res=None):
        """Host arrays: inits / goals [n][17], obstacles [m][6], offsets and
        counts in boxes.  Returns one result dict per query, or -- when the
        caller passes its own result array `res` (and, to skip repacking,
        the configs packed once with pack_configs as `carr`) -- fills `res`
        and returns it."""
        n = len(cfgs)
        raw = res is not None
        carr = pack_configs(cfgs) if carr is None else carr
        res = (KgmtResult * n)() if res is None else res
        inits, goals, obstacles = _f32(inits), _f32(goals), _f32(obstacles)
        off = np.ascontiguousarray(obs_offset, np.uint32)
        cnt = np.ascontiguousarray(obs_count, np.uint32)
        check(self._lib.kgmt_plan_batch(self._h, n, carr, inits.ctypes.data, goals.ctypes.data, obstacles.ctypes.data,
                                        off.ctypes.data, cnt.ctypes.data, res))
        self._n = n
        self._cfgs = list(cfgs)
        return res if raw else [r.as_dict() for r in res]

    def plan_device(self, cfgs, d_inits, d_goals, d_obstacles, obs_offset, obs_count, carr=None, res=None):
        """Inputs already on the device (torch tensors or addresses)."""
        n = len(cfgs)
        carr = carr if carr is not None else pack_configs(cfgs)
        res = res if res is not None else (KgmtResult * n)()
        off = np.ascontiguousarray(obs_offset, np.uint32)
        cnt = np.ascontiguousarray(obs_count, np.uint32)
        check(self._lib.kgmt_plan_batch_device(self._h, n, carr, ptr(d_inits), ptr(d_goals), ptr(d_obstacles),
                                               off.ctypes.data, cnt.ctypes.data, res))
        self._n = n
        self._cfgs = list(cfgs)
        return res

    def stats(self) -> dict:
        s = _abi.KgmtBatchStats()
        check(self._lib.kgmt_batch_get_stats(self._h, C.byref(s)))
        return s.as_dict()

    def copy_tree(self, i: int):
        r_cfg = self._cfgs[i]
        D = r_cfg.sample_dim
        T = r_cfg.tree_capacity
        samples = np.zeros((T, D), np.float32)
        parents = np.zeros(T, np.int32)
        costs = np.zeros(T, np.float32)
        check(self._lib.kgmt_batch_copy_tree(self._h, i, samples.ctypes.data, parents.ctypes.data, costs.ctypes.data, T))
        return samples, parents, costs

    def copy_path(self, i: int) -> np.ndarray:
        c = self._cfgs[i]
        rows = np.zeros((c.max_iterations + 2, c.sample_dim), np.float32)
        n = C.c_uint32()
        check(self._lib.kgmt_batch_copy_path(self._h, i, rows.ctypes.data, rows.shape[0], C.byref(n)))
        return rows[: n.value]

    def autotune(self, cfgs, inits, goals, obstacles, obs_offset, obs_count) -> int:
        n = len(cfgs)
        carr = pack_configs(cfgs)
        inits, goals, obstacles = _f32(inits), _f32(goals), _f32(obstacles)
        off = np.ascontiguousarray(obs_offset, np.uint32)
        cnt = np.ascontiguousarray(obs_count, np.uint32)
        best = C.c_uint32()
        check(self._lib.kgmt_batch_autotune(self._h, n, carr, inits.ctypes.data, goals.ctypes.data, obstacles.ctypes.data,
                                            off.ctypes.data, cnt.ctypes.data, C.byref(best)))
        return best.value

    def autotune_full(self, cfgs, inits, goals, obstacles, obs_offset, obs_count) -> dict:
        """Block size x samples per node sweep (kgmt_batch_autotune_full): the
        batch keeps the chosen block size; the chosen samples per node is
        returned for the caller to put into its configs."""
        n = len(cfgs)
        carr = pack_configs(cfgs)
        inits, goals, obstacles = _f32(inits), _f32(goals), _f32(obstacles)
        off = np.ascontiguousarray(obs_offset, np.uint32)
        cnt = np.ascontiguousarray(obs_count, np.uint32)
        out = _abi.KgmtAutotuneResult()
        check(self._lib.kgmt_batch_autotune_full(self._h, n, carr, inits.ctypes.data, goals.ctypes.data, obstacles.ctypes.data,
                                                 off.ctypes.data, cnt.ctypes.data, C.byref(out)))
        return out.as_dict()


class Server:
    """Continuous batching with memory-based admission."""

    def __init__(self, max_slots: int, memory_budget: int, iters_per_step: int = 1, propagate_block: int = 256,
                 stream: int | None = None):
        self._lib = load()
        opt = KgmtServerOptions(max_slots, memory_budget, iters_per_step, propagate_block)
        h = C.c_void_p()
        check(self._lib.kgmt_server_create(C.byref(opt), stream, C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.kgmt_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, cfg: PlannerConfig, init, goal, obstacles) -> int:
        c = to_c(cfg)
        init = _f32(init)
        goal = _f32(goal)
        obs = _f32(obstacles).reshape(-1, 6)
        t = C.c_uint64()
        check(self._lib.kgmt_server_submit(self._h, C.byref(c), init.ctypes.data, goal.ctypes.data, obs.ctypes.data,
                                           obs.shape[0], C.byref(t)))
        return t.value

    def step(self):
        r, q = C.c_uint32(), C.c_uint32()
        check(self._lib.kgmt_server_step(self._h, C.byref(r), C.byref(q)))
        return r.value, q.value

    def cancel(self, ticket: int) -> None:
        """Withdraws a queued or running query; poll() returns it with status
        cancelled (KgmtError NOT_READY if it is unknown or already done)."""
        check(self._lib.kgmt_server_cancel(self._h, ticket))

    def poll(self, max_results: int = 4096) -> list[dict]:
        out = (KgmtResult * max_results)()
        n = C.c_uint32()
        check(self._lib.kgmt_server_poll(self._h, out, max_results, C.byref(n)))
        return [out[i].as_dict() for i in range(n.value)]


def propagate_samples(cfg: PlannerConfig, d_x0, d_uniforms, d_obstacles, n_obstacles: int, n: int, d_x1, d_valid, d_r1=None,
                      d_r2=None, stream: int | None = None) -> None:
    """Function-level propagation with explicit uniforms (device buffers)."""
    lib = load()
    c = to_c(cfg)
    check(lib.kgmt_propagate_samples(C.byref(c), ptr(d_x0), ptr(d_uniforms), ptr(d_obstacles), n_obstacles, n, ptr(d_x1),
                                     ptr(d_valid), ptr(d_r1), ptr(d_r2), stream))
