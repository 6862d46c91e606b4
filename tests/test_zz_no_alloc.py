"""kgmt_plan_noalloc: the planning entry point for callers that cannot call
cudaMalloc (memory owned by a fixed pool, real-time loops that must not enter
the allocator).  Its working memory is a static device array; it must give
exactly what kgmt_plan gives -- and what the CPU oracle plans -- call after
call, whatever the previous call left in that array, and it must not change
the device's free memory.  Collected last on purpose (file name), so a
failure here never hides the other tests."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from kgmt_gb300 import _abi
from kgmt_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return _abi.load()


def plan_reference_entry(q):
    """the existing entry point, kgmt_plan, through the C ABI"""
    from kgmt_gb300.planner import KGMT
    d_obs = torch.from_numpy(np.ascontiguousarray(q.obstacles, np.float32)).to(DEV)
    p = KGMT(q.config)
    res = p.plan(q.init, q.goal, d_obs, q.obstacles.shape[0])
    samples, parents, costs = p.copy_tree()
    path = p.copy_path()
    p.close()
    return res, samples, parents, costs, path


def plan_noalloc(lib, q):
    cfg = q.config
    D, T = cfg.sample_dim, cfg.tree_capacity
    d_obs = torch.from_numpy(np.ascontiguousarray(q.obstacles, np.float32)).to(DEV)
    d_samples = torch.full((T, D), -7.0, dtype=torch.float32, device=DEV)
    d_parents = torch.full((T,), -7, dtype=torch.int32, device=DEV)
    d_costs = torch.full((T,), -7.0, dtype=torch.float32, device=DEV)
    rows = cfg.max_iterations + 2
    d_path = torch.zeros((rows, D), dtype=torch.float32, device=DEV)
    torch.cuda.synchronize()
    init = np.ascontiguousarray(q.init, np.float32)
    goal = np.ascontiguousarray(q.goal, np.float32)
    k = _abi.to_c(cfg)
    r = _abi.KgmtResult()
    rc = lib.kgmt_plan_noalloc(C.byref(k), init.ctypes.data, goal.ctypes.data, d_obs.data_ptr(), q.obstacles.shape[0],
                               d_samples.data_ptr(), d_parents.data_ptr(), d_costs.data_ptr(), T, d_path.data_ptr(), rows,
                               C.byref(r), None)
    _abi.check(rc)
    n = r.tree_size
    return (r.as_dict(), d_samples[:n].cpu().numpy(), d_parents[:n].cpu().numpy(), d_costs[:n].cpu().numpy(),
            d_path[: r.path_len].cpu().numpy())


def assert_same(a, b):
    ra, sa, pa, ca, xa = a
    rb, sb, pb, cb, xb = b
    for key in ("status", "iterations", "tree_size", "goal_index", "path_len", "samples_drawn"):
        assert ra[key] == rb[key], key
    # the same bit-exact tolerance as every other parity test
    assert np.array_equal(pa, pb)
    assert np.array_equal(sa.view(np.uint32), sb.view(np.uint32))
    assert np.array_equal(ca.view(np.uint32), cb.view(np.uint32))
    assert np.array_equal(xa.view(np.uint32), xb.view(np.uint32))


def as_oracle(ref):
    return ({k: ref[k] for k in ("status", "iterations", "tree_size", "goal_index", "path_len", "samples_drawn")},
            ref["samples"], ref["parents"], ref["costs"], ref["path"])


def test_noalloc_matches_plan_on_consecutive_calls(lib):
    # two different queries back to back, then the first again: the static
    # array holds the previous call's tree and tables each time
    q1 = W.double_integrator_query(seed=21)
    q2 = W.double_integrator_query(seed=22, n_obstacles=40)
    q2.config = q2.config.replace(tree_capacity=60_000)
    for q in (q1, q2, q1):
        got = plan_noalloc(lib, q)
        assert_same(got, plan_reference_entry(q))
        assert_same(got, as_oracle(O.plan(q)))


def test_noalloc_leaves_device_memory_unchanged(lib):
    """The property the entry point exists for: once the library is loaded
    (its static array placed), a call takes no device memory -- the free
    bytes the driver reports are the same before and after it."""
    q = W.double_integrator_query(seed=23)
    plan_noalloc(lib, q)  # loads the module and its static array
    cfg = q.config
    D, T = cfg.sample_dim, cfg.tree_capacity
    d_obs = torch.from_numpy(np.ascontiguousarray(q.obstacles, np.float32)).to(DEV)
    d_samples = torch.empty((T, D), dtype=torch.float32, device=DEV)
    d_parents = torch.empty((T,), dtype=torch.int32, device=DEV)
    d_costs = torch.empty((T,), dtype=torch.float32, device=DEV)
    d_path = torch.empty((cfg.max_iterations + 2, D), dtype=torch.float32, device=DEV)
    init = np.ascontiguousarray(q.init, np.float32)
    goal = np.ascontiguousarray(q.goal, np.float32)
    k = _abi.to_c(cfg)
    r = _abi.KgmtResult()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    rc = lib.kgmt_plan_noalloc(C.byref(k), init.ctypes.data, goal.ctypes.data, d_obs.data_ptr(), q.obstacles.shape[0],
                               d_samples.data_ptr(), d_parents.data_ptr(), d_costs.data_ptr(), T, d_path.data_ptr(),
                               cfg.max_iterations + 2, C.byref(r), None)
    free1, _ = torch.cuda.mem_get_info()
    _abi.check(rc)
    assert free1 == free0, (free0, free1)
    assert r.tree_size > 1


def test_noalloc_rejects_host_pointers(lib):
    """A host array where device memory is expected is refused before any
    kernel runs (the GPU would otherwise read or write host memory)."""
    q = W.double_integrator_query(seed=24)
    k = _abi.to_c(q.config)
    r = _abi.KgmtResult()
    init = np.ascontiguousarray(q.init, np.float32)
    h_obs = np.ascontiguousarray(q.obstacles, np.float32)
    rc = lib.kgmt_plan_noalloc(C.byref(k), init.ctypes.data, init.ctypes.data, h_obs.ctypes.data, h_obs.shape[0], None, None,
                               None, 0, None, 0, C.byref(r), None)
    assert rc == 1  # KGMT_ERR_INVALID_ARG
    assert "obstacles must be a device pointer" in lib.kgmt_last_error().decode()
    d_obs = torch.from_numpy(h_obs).to(DEV)
    h_out = np.zeros((q.config.tree_capacity, q.config.sample_dim), np.float32)
    rc = lib.kgmt_plan_noalloc(C.byref(k), init.ctypes.data, init.ctypes.data, d_obs.data_ptr(), h_obs.shape[0],
                               h_out.ctypes.data, None, None, q.config.tree_capacity, None, 0, C.byref(r), None)
    assert rc == 1
    assert "d_samples must be a device pointer" in lib.kgmt_last_error().decode()


def test_noalloc_rejects_queries_beyond_the_static_scratch(lib):
    q = W.quadrotor_query(seed=1)  # 2M-node tree: far beyond 32 MiB
    k = _abi.to_c(q.config)
    r = _abi.KgmtResult()
    init = np.ascontiguousarray(q.init, np.float32)
    rc = lib.kgmt_plan_noalloc(C.byref(k), init.ctypes.data, init.ctypes.data, None, 0, None, None, None, 0, None, 0,
                               C.byref(r), None)
    assert rc == 1  # KGMT_ERR_INVALID_ARG
    assert "static scratch" in lib.kgmt_last_error().decode()
    need = lib.kgmt_query_bytes(C.byref(k), 0)
    assert need + 4096 > (32 << 20)


def test_noalloc_limit_is_query_bytes_plus_reserved_head(lib):
    """The documented rule: accepted exactly when kgmt_query_bytes(cfg, n) +
    KGMT_NOALLOC_RESERVED_BYTES <= KGMT_NOALLOC_SCRATCH_BYTES.  Capacities on
    either side of the limit, found by bisection on kgmt_query_bytes."""
    q = W.double_integrator_query(seed=25)
    q.config = q.config.replace(max_iterations=3)
    n = q.obstacles.shape[0]
    limit = (32 << 20) - 4096

    def need(cap):
        return lib.kgmt_query_bytes(C.byref(_abi.to_c(q.config.replace(tree_capacity=cap))), n)

    lo, hi = 1000, 1_000_000
    while hi - lo > 1:
        mid = (lo + hi) // 2
        lo, hi = (mid, hi) if need(mid) <= limit else (lo, mid)
    assert need(lo) <= limit < need(hi)
    d_obs = torch.from_numpy(np.ascontiguousarray(q.obstacles, np.float32)).to(DEV)
    init = np.ascontiguousarray(q.init, np.float32)
    goal = np.ascontiguousarray(q.goal, np.float32)
    for cap, ok in ((lo, True), (hi, False)):
        k = _abi.to_c(q.config.replace(tree_capacity=cap))
        r = _abi.KgmtResult()
        rc = lib.kgmt_plan_noalloc(C.byref(k), init.ctypes.data, goal.ctypes.data, d_obs.data_ptr(), n, None, None, None, 0,
                                   None, 0, C.byref(r), None)
        assert (rc == 0) == ok, (cap, rc, lib.kgmt_last_error())
