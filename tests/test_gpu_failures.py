"""Failure detection without a GPU fault.

- A bounded device-side wait that runs out: the planning kernels' look-back
  wait, pointed at a predecessor that never publishes (a word nothing sets)
  with a short poll limit, gives up and reports KGMT_ERR_TIMEOUT; the same
  context then plans a query exactly as the oracle does.
- Admission by device memory: a served query larger than the server's whole
  memory budget is refused with KGMT_ERR_OOM, and the server keeps serving.
Nothing here traps, faults or hangs the GPU."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from kgmt_gb300 import _abi
from kgmt_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

KGMT_ERR_OOM, KGMT_ERR_TIMEOUT = 2, 4


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return _abi.load()


def plan_matches_oracle(q):
    from kgmt_gb300.planner import KGMT
    d_obs = torch.from_numpy(np.ascontiguousarray(W.boxes_for_plan(q), np.float32)).to("cuda:0")
    p = KGMT(q.config)
    res = p.plan(q.init, q.goal, d_obs, q.obstacles.shape[0])
    samples, parents, _ = p.copy_tree()
    p.close()
    ref = O.plan(q)
    for k in ("status", "iterations", "tree_size", "goal_index"):
        assert res[k] == ref[k], (k, res[k], ref[k])
    assert np.array_equal(parents, ref["parents"])
    assert np.array_equal(samples.view(np.uint32), ref["samples"].view(np.uint32))


@pytest.mark.parametrize("polls", [1, 1000, 100_000])
def test_bounded_wait_times_out_and_the_context_survives(lib, polls):
    bits = C.c_uint32(0)
    rc = lib.kgmt_selftest_bounded_wait(polls, C.byref(bits))
    assert rc == KGMT_ERR_TIMEOUT, lib.kgmt_last_error().decode()
    assert bits.value & 1  # look-back timeout
    assert "gave up" in lib.kgmt_last_error().decode()
    plan_matches_oracle(W.double_integrator_query(seed=7))


def test_selftest_rejects_unbounded_polls(lib):
    bits = C.c_uint32(0)
    assert lib.kgmt_selftest_bounded_wait(0, C.byref(bits)) == 1
    assert lib.kgmt_selftest_bounded_wait((1 << 22) + 1, C.byref(bits)) == 1


def test_server_refuses_a_query_over_its_memory_budget_and_keeps_serving(lib):
    from kgmt_gb300.planner import Server
    small = W.double_integrator_batch(3, seed=8, tree_capacity=5_000)
    big = W.double_integrator_query(seed=2)
    big.config = big.config.replace(tree_capacity=400_000)  # tens of MiB, over a 16 MiB budget
    srv = Server(max_slots=2, memory_budget=16 << 20, iters_per_step=2)
    with pytest.raises(_abi.KgmtError) as e:
        srv.submit(big.config, big.init, big.goal, big.obstacles)
    assert e.value.code == KGMT_ERR_OOM
    tickets = {srv.submit(q.config, q.init, q.goal, q.obstacles): i for i, q in enumerate(small)}
    got = {}
    for _ in range(2000):
        srv.step()
        for r in srv.poll():
            got[tickets[r["ticket"]]] = r
        if len(got) == len(small):
            break
    refs = O.plan_batch(small)
    for i, ref in enumerate(refs):
        for k in ("status", "iterations", "tree_size", "goal_index"):
            assert got[i][k] == ref[k], (i, k, got[i][k], ref[k])


CHECKED_SCRIPT = r'''
import numpy as np, torch
from kgmt_gb300 import workloads as W
from kgmt_gb300.planner import KGMT, BatchPlanner
from oracle import oracle as O
qs = [W.double_integrator_query(seed=3), W.quadrotor_query(seed=1, tree_capacity=50_000, max_iterations=8),
      W.dubins_query(seed=2), W.unicycle_query(seed=2)]
for q in qs:
    d_obs = torch.from_numpy(np.ascontiguousarray(W.boxes_for_plan(q), np.float32)).to("cuda:0")
    p = KGMT(q.config)
    res = p.plan(q.init, q.goal, d_obs, q.obstacles.shape[0])
    s, par, c = p.copy_tree()
    p.close()
    ref = O.plan(q)
    assert res["tree_size"] == ref["tree_size"] and np.array_equal(par, ref["parents"]), q.config.model
    assert np.array_equal(s.view(np.uint32), ref["samples"].view(np.uint32)), q.config.model
batch = W.double_integrator_batch(48, n_obstacles=50, seed=5, tree_capacity=20_000)
inits, goals, obs, offs, cnts = W.pack_queries(batch)
b = BatchPlanner(len(batch))
res = b.plan([q.config for q in batch], inits, goals, obs, offs, cnts)
for r, ref in zip(res, O.plan_batch(batch)):
    assert (r["status"], r["iterations"], r["tree_size"]) == (ref["status"], ref["iterations"], ref["tree_size"])
print("checked build ok")
'''


def test_bounds_checked_build_plans_like_the_oracle(lib):
    """libkgmt_checked.so tests every scattered index of the kernels against
    its buffer (a failed test is recorded and reported, the access skipped):
    planning all four models and a batch through it gives the oracle's
    results and no failed test (a failure would raise KGMT_ERR_INTERNAL)."""
    import os
    import subprocess
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    checked = root / "kgmt_gb300" / "_lib" / "libkgmt_checked.so"
    assert checked.exists(), "build() makes the bounds-checked library"
    env = dict(os.environ, KGMT_LIBRARY=str(checked), PYTHONPATH=str(root))
    r = subprocess.run([sys.executable, "-c", CHECKED_SCRIPT], cwd=root, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "checked build ok" in r.stdout


def test_server_cancels_queued_and_running_queries(lib):
    """A cancelled query leaves the server with status cancelled (a queued one
    at iteration 0, a running one where its last step left it) and frees its
    slot; the other queries' results are the oracle's, unaffected; an unknown
    ticket is refused."""
    from kgmt_gb300.planner import Server
    qs = W.double_integrator_batch(5, seed=9, tree_capacity=20_000)
    srv = Server(max_slots=2, memory_budget=1 << 28, iters_per_step=1)
    tickets = [srv.submit(q.config, q.init, q.goal, q.obstacles) for q in qs]
    srv.cancel(tickets[4])  # still queued
    srv.step()              # admits the first two
    srv.cancel(tickets[0])  # running
    with pytest.raises(_abi.KgmtError) as e:
        srv.cancel(10_000)
    assert e.value.code == 7
    got = {}
    for _ in range(5000):
        srv.step()
        for r in srv.poll():
            got[r["ticket"]] = r
        if len(got) == len(qs):
            break
    assert got[tickets[4]]["status"] == 4 and got[tickets[4]]["iterations"] == 0
    assert got[tickets[0]]["status"] == 4 and got[tickets[0]]["iterations"] >= 1
    refs = O.plan_batch(qs[1:4])
    for t, ref in zip(tickets[1:4], refs):
        for k in ("status", "iterations", "tree_size", "goal_index"):
            assert got[t][k] == ref[k], (t, k, got[t][k], ref[k])
    with pytest.raises(_abi.KgmtError):
        srv.cancel(tickets[1])  # finished


FAULT_SCRIPT = r'''
from kgmt_gb300 import _abi, workloads as W
from kgmt_gb300.planner import BatchPlanner
from oracle import oracle as O
qs = W.double_integrator_batch(4, seed=10, tree_capacity=5_000)
inits, goals, obs, offs, cnts = W.pack_queries(qs)
try:
    b = BatchPlanner(len(qs))
    res = b.plan([q.config for q in qs], inits, goals, obs, offs, cnts)
    refs = O.plan_batch(qs)
    same = all((r["status"], r["tree_size"]) == (f["status"], f["tree_size"]) for r, f in zip(res, refs))
    b.close()
    print("planned", same)
except _abi.KgmtError as e:
    print("error", e.code)
'''


@pytest.mark.parametrize("after,expect", [(0, "error 2"), (2, "error 2"), (5, "error 2"), (7, "error 2"), (8, "error 2"),
                                          (1000, "planned True")])
def test_injected_allocation_failure_is_an_error_not_a_crash(lib, after, expect):
    """KGMT_FAULT_ALLOC_AFTER=n makes the library's (n+1)-th device
    allocation fail as out of memory without reaching the driver (a host-side
    injector): creating the batch engine (allocations 0-7: descriptors, tile
    bases, the tail launch's scratch, the admission slot list) or growing its
    arena while planning (8) then raises KGMT_ERR_OOM and the process exits
    cleanly; with no failure in reach the batch plans as the oracle does."""
    import os
    import subprocess
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    env = dict(os.environ, KGMT_FAULT_ALLOC_AFTER=str(after), PYTHONPATH=str(root))
    r = subprocess.run([sys.executable, "-c", FAULT_SCRIPT], cwd=root, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-3000:]
    assert r.stdout.strip().splitlines()[-1] == expect, r.stdout
