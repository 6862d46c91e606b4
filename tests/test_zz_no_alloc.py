"""kgmt_plan_noalloc: the planning entry point for callers that cannot call
cudaMalloc (memory owned by a fixed pool, real-time loops that must not enter
the allocator).  Its working memory is a static device array; it must give
exactly what kgmt_plan gives, call after call, whatever the previous call
left in that array.  Collected last on purpose (file name), so a failure here
never hides the other tests."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from kgmt_gb300 import _abi
from kgmt_gb300 import workloads as W
from kgmt_gb300.config import quadrotor_large

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


def test_noalloc_matches_plan_on_consecutive_calls(lib):
    # two different queries back to back, then the first again: the static
    # array holds the previous call's tree and tables each time
    q1 = W.double_integrator_query(seed=21)
    q2 = W.double_integrator_query(seed=22, n_obstacles=40)
    q2.config = q2.config.replace(tree_capacity=60_000)
    for q in (q1, q2, q1):
        assert_same(plan_noalloc(lib, q), plan_reference_entry(q))


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
    assert need > (32 << 20)
