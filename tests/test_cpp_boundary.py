"""The C++ boundary run on the GPU: the kgmt_plan driver, compiled against
include/kgmt.hpp like the reference's example mains (examples/gpu/main.cu,
benchMain.cu, executionTimeMain.cu), plans a seeded scene with
KGMT::plan and then twice with KGMT::planBench (src/planners/KGMT.cu:107-165).
Its printed fields, its tree export and every line of the per-iteration
files planBench writes (writeDeviceVectorsToCSV, KGMT.cu:405-488) are
compared with the oracle, formatted the way the reference formats them
(fixed notation, 6 decimals; helper.cuh:56-107).  The traced plan through
the Python binding is compared table for table, bit for bit."""
import re
import subprocess

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from kgmt_gb300 import _abi
from kgmt_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


@pytest.fixture(scope="module", autouse=True)
def _need_cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    _abi.load()


def _query(seed=10, capacity=8000):
    q = W.double_integrator_query(seed=seed)
    q.config = q.config.replace(tree_capacity=capacity)
    return q


def fmt_rows(a) -> list[str]:
    """rows as the reference writes them: std::fixed, setprecision(6) for
    floats, plain integers otherwise"""
    a = np.asarray(a)
    if a.ndim == 1:
        a = a[None, :]
    if a.dtype.kind == "f":
        cells = np.char.mod("%.6f", a.astype(np.float64))
    else:
        cells = a.astype(np.int64).astype(str)
    return [",".join(r) for r in cells]


def read_lines(path) -> list[str]:
    return path.read_text().splitlines()


def test_python_traced_plan_matches_oracle_tables():
    """kgmt_plan_traced (the iteration hook under planBench): per iteration
    the sizes, tree rows, region counters, valid counts, scores and the next
    frontier's flags and repeat counts equal the oracle's, and the plan is
    kgmt_plan's."""
    from kgmt_gb300.planner import KGMT
    for q in (_query(10), _query(7, capacity=60)):  # a success, and a tree that fills
        d_obs = torch.from_numpy(q.obstacles).to(DEV)
        p = KGMT(q.config)
        its = p.plan_traced(q.init, q.goal, d_obs, q.obstacles.shape[0])
        res = dict(p.result)
        samples, parents, costs = p.copy_tree()
        plain = KGMT(q.config)
        assert plain.plan(q.init, q.goal, d_obs, q.obstacles.shape[0])["tree_size"] == res["tree_size"]
        ref = O.plan(q, tables=True)
        assert (res["status"], res["iterations"], res["tree_size"], res["goal_index"]) == \
            (ref["status"], ref["iterations"], ref["tree_size"], ref["goal_index"])
        assert np.array_equal(parents, ref["parents"])
        assert len(its) == len(ref["tables"]) == res["iterations"]
        T = q.config.tree_capacity
        for it, tb in zip(its, ref["tables"]):
            for k in ("itr", "tree_size", "frontier_size", "expanded", "next_frontier_size"):
                assert it[k] == tb[k], (it["itr"], k, it[k], tb[k])
            n = it["tree_size"]
            assert np.array_equal(it["samples"][:n].view(np.uint32), ref["samples"][:n].view(np.uint32))
            assert not it["samples"][n:].any() and (it["parents"][n:] == -1).all()
            assert np.array_equal(it["parents"][:n], ref["parents"][:n])
            assert np.array_equal(it["counter"], tb["counter"]) and np.array_equal(it["valid"], tb["valid"])
            assert np.array_equal(it["score"].view(np.uint32), tb["score"].view(np.uint32))
            assert np.array_equal(it["frontier"], tb["frontier"]) and np.array_equal(it["repeat"], tb["repeat"])
            assert it["frontier"].shape == (T,)
        if res["status"] == 1:
            assert np.array_equal(its[-1]["path"].view(np.uint32), ref["path"].view(np.uint32))
        p.close()
        plain.close()


def test_cpp_plan_and_planbench_match_oracle(tmp_path):
    q = _query()
    cfg = q.config
    scene = tmp_path / "obstacles.csv"
    scene.write_text("\n".join(",".join("%.9g" % v for v in row) for row in q.obstacles) + "\n")
    cli = _abi.LIB_PATH.parent / "kgmt_plan"
    assert cli.exists(), "the C++ driver is built by kgmt_gb300.build"
    vec = lambda v: ",".join("%.9g" % x for x in v[:3])  # noqa: E731
    out_dir = tmp_path / "tree"
    out_dir.mkdir()
    cmd = [str(cli), "--obstacles", str(scene), "--model", "di", "--init", vec(q.init), "--goal", vec(q.goal), "--seed",
           str(cfg.seed), "--capacity", str(cfg.tree_capacity), "--iterations", str(cfg.max_iterations), "--bench", "2",
           "--out", str(out_dir)]
    r = subprocess.run(cmd, cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    ref = O.plan(q, tables=True)
    D = cfg.sample_dim
    # --- KGMT::plan through the wrapper: printed fields ---
    m = re.search(r"Iterations: (\d+)\. Tree Size: (\d+)\. Status: (-?\d+)\. Goal: (-?\d+)\. Path: (\d+)\. Cost to goal: (\S+)",
                  r.stdout)
    assert m, r.stdout
    itr, tree, status, goal, plen = map(int, m.groups()[:5])
    assert (itr, tree, status, goal, plen) == (ref["iterations"], ref["tree_size"], ref["status"], ref["goal_index"],
                                                ref["path_len"])
    assert status == 1, "the scene is chosen to reach the goal"
    assert np.float32(float(m.group(6))) == ref["costs"][goal]  # h_costToGoal_
    # tree export (the CLI's --out) and h_controlPathToGoal_
    n = ref["tree_size"]
    assert read_lines(out_dir / "samples.csv") == fmt_rows(ref["samples"][:n])
    assert read_lines(out_dir / "parents.csv") == fmt_rows(ref["parents"][:n, None])
    assert read_lines(out_dir / "costs.csv") == fmt_rows(ref["costs"][:n, None])
    assert read_lines(out_dir / "controlPathToGoal.csv") == fmt_rows(ref["path"])
    # --- KGMT::planBench, bench runs 0 and 1: the per-iteration files ---
    T = cfg.tree_capacity
    tabs = ref["tables"]
    zero_rows = fmt_rows(np.zeros((1, D), np.float32))[0]
    for b in (0, 1):
        data = tmp_path / "Data"
        for k, tb in enumerate(tabs, start=1):
            rows = read_lines(data / "Samples" / f"Samples{b}" / f"samples{k}.csv")
            assert len(rows) == T
            nk = tb["tree_size"]
            assert rows[:nk] == fmt_rows(ref["samples"][:nk]), (b, k)
            assert all(x == zero_rows for x in rows[nk:])
            prow = read_lines(data / "Parents" / f"Parents{b}" / f"parents{k}.csv")
            want = np.full(T, -1, np.int64)
            want[:nk] = ref["parents"][:nk]
            assert prow == fmt_rows(want[:, None]), (b, k)
        per_itr = {
            "TotalCountPerVertex/TotalCountPerVertex{b}/totalCountPerVertex.csv": [fmt_rows(t["counter"])[0] for t in tabs],
            "ValidCountPerVertex/ValidCountPerVertex{b}/validCountPerVertex.csv": [fmt_rows(t["valid"])[0] for t in tabs],
            "VertexScores/VertexScores{b}/vertexScores.csv": [fmt_rows(t["score"])[0] for t in tabs],
            "Frontier/Frontier{b}/frontier.csv": [fmt_rows(t["frontier"])[0] for t in tabs],
            "FrontierRepeatCount/FrontierRepeatCount{b}/frontierRepeatCount.csv": [fmt_rows(t["repeat"])[0] for t in tabs],
            "FrontierSize/FrontierSize{b}/frontierSize.csv": [str(t["frontier_size"]) for t in tabs],
            "TreeSize/TreeSize{b}/treeSize.csv": [str(t["tree_size"]) for t in tabs],
            "ExpandedNodes/ExpandedNodes{b}/expandedNodes.csv": [str(t["expanded"]) for t in tabs],
            "ControlPathToGoal/ControlPathToGoal{b}/controlPathToGoal.csv": fmt_rows(ref["path"]),
        }
        for rel, want in per_itr.items():
            assert read_lines(data / rel.format(b=b)) == want, (b, rel)
    assert r.stdout.count("KGMT bench") == 2
