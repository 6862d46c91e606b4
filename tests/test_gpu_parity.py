"""CUDA planner vs the CPU oracle and the reference-made golden vectors.

Integer results (region ids, verdicts, tree parents, node counts, iteration
counts, goal indices) must be bit-exact; with the same float operation order
the samples themselves are bit-exact too.  Propagated states are checked
against the FP64 RK4 oracle with |delta| <= 1e-5 * max(|ref|, scale)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from kgmt_gb300 import workloads as W
from kgmt_gb300.config import (DI_RULE_REFERENCE, MODEL_DUBINS_AIRPLANE, MODEL_UNICYCLE, double_integrator_single,
                               dubins_airplane, quadrotor_large, unicycle)
from oracle import oracle as O

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5
DEV = "cuda:0"


@pytest.fixture(scope="module", autouse=True)
def _need_cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from kgmt_gb300._abi import load
    load()


def state_scales(cfg):
    D = cfg.sample_dim
    s = np.ones(D)
    s[:3] = cfg.ws_max - cfg.ws_min
    if cfg.model == MODEL_UNICYCLE:  # x y theta v | a steering dt
        s[2] = np.pi
        s[3] = 0.3
    elif cfg.model == MODEL_DUBINS_AIRPLANE:  # x y z yaw pitch v | yr pr a | k h
        s[3:5] = np.pi
        s[5] = cfg.v_max
        s[9] = cfg.step_size
    elif D == 10:
        s[3:6] = cfg.v_max
        s[9] = cfg.step_size
    else:
        s[3:6] = np.pi
        s[6:9] = cfg.v_max
        s[16] = cfg.step_size
    return s


def gpu_propagate(cfg, x0, u, obs):
    from kgmt_gb300.planner import propagate_samples
    n, D = x0.shape
    d_x0 = torch.from_numpy(np.ascontiguousarray(x0, np.float32)).to(DEV)
    d_u = torch.from_numpy(np.ascontiguousarray(u, np.float32)).to(DEV)
    d_obs = torch.from_numpy(O.boxes(cfg, obs)).to(DEV)  # rows of 2W floats, the model's layout
    d_x1 = torch.zeros((n, D), dtype=torch.float32, device=DEV)
    d_valid = torch.zeros(n, dtype=torch.uint8, device=DEV)
    d_r1 = torch.zeros(n, dtype=torch.int32, device=DEV)
    d_r2 = torch.zeros(n, dtype=torch.int32, device=DEV)
    propagate_samples(cfg, d_x0, d_u, d_obs, d_obs.shape[0], n, d_x1, d_valid, d_r1, d_r2)
    torch.cuda.synchronize()
    return d_x1.cpu().numpy(), d_valid.cpu().numpy(), d_r1.cpu().numpy(), d_r2.cpu().numpy()


def random_inputs(cfg, n, seed):
    rng = np.random.Generator(np.random.Philox(key=seed))
    D = cfg.sample_dim
    x0 = np.zeros((n, D), np.float32)
    x0[:, :3] = rng.uniform(0.05, 0.95, (n, 3))
    if cfg.model == MODEL_UNICYCLE:
        x0[:, 2] = rng.uniform(-np.pi, np.pi, n)
        x0[:, 3] = rng.uniform(0.0, 0.3, n)
    elif cfg.model == MODEL_DUBINS_AIRPLANE:
        x0[:, 3] = rng.uniform(-np.pi, np.pi, n)
        x0[:, 4] = rng.uniform(-1.0, 1.0, n)
        x0[:, 5] = rng.uniform(0.0, 0.3, n)
    elif D == 10:
        x0[:, 3:6] = rng.uniform(-0.3, 0.3, (n, 3))
    else:
        x0[:, 3:6] = rng.uniform(-0.6, 0.6, (n, 3))
        x0[:, 6:9] = rng.uniform(-0.25, 0.25, (n, 3))
        x0[:, 9:12] = rng.uniform(-1.5, 1.5, (n, 3))
    u = np.stack([O.sample_uniforms(seed, i, 3) for i in range(n)])
    return x0, u


# ---------------------------------------------------------------------------
# function level
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("rule", [0, 1])
def test_propagate_di_bit_exact_vs_oracle(rule):
    q = W.double_integrator_query(seed=2)
    cfg = q.config.replace(di_rule=rule)
    x0, u = random_inputs(cfg, 4096, 11)
    gx, gv, g1, g2 = gpu_propagate(cfg, x0, u, q.obstacles)
    ox, ov, o1, o2 = O.propagate_f32(cfg, x0, u, q.obstacles)
    assert np.array_equal(gv, ov)
    assert np.array_equal(gx.view(np.uint32), ox.view(np.uint32))
    assert np.array_equal(g1, o1) and np.array_equal(g2, o2)


@pytest.mark.parametrize("rule", [0, 1])
def test_propagate_di_exact_division_fallback(rule):
    """Samples whose RK4 increments are zero or below 2^-98 in magnitude take
    the true-division branch of the step (the fused multiply-add form of x / 6
    is exact only above that): zero acceleration (u = 0.5 on [-1, 1]) with zero
    or tiny velocities, and signed zeros."""
    q = W.double_integrator_query(seed=2)
    cfg = q.config.replace(di_rule=rule)
    x0, u = random_inputs(cfg, 256, 17)
    u[:, 0:3] = 0.5
    x0[:64, 3:6] = 0.0
    x0[64:96, 3:6] = -0.0
    x0[96:160, 3:6] = np.float32(1e-33) * np.sign(x0[96:160, 3:6] + 1e-30)
    x0[160:192, 3:6] = np.float32(2.0 ** -140)  # subnormal velocities
    gx, gv, g1, g2 = gpu_propagate(cfg, x0, u, q.obstacles)
    ox, ov, o1, o2 = O.propagate_f32(cfg, x0, u, q.obstacles)
    assert np.array_equal(gv, ov)
    assert np.array_equal(gx.view(np.uint32), ox.view(np.uint32))
    assert np.array_equal(g1, o1) and np.array_equal(g2, o2)


def test_propagate_quad_bit_exact_vs_oracle():
    q = W.quadrotor_query(seed=2)
    cfg = q.config
    x0, u = random_inputs(cfg, 2048, 12)
    gx, gv, g1, g2 = gpu_propagate(cfg, x0, u, q.obstacles)
    ox, ov, o1, o2 = O.propagate_f32(cfg, x0, u, q.obstacles)
    assert np.array_equal(gv, ov)
    assert np.array_equal(gx.view(np.uint32), ox.view(np.uint32))
    assert np.array_equal(g1, o1) and np.array_equal(g2, o2)


def _same_bits_or_both_nan(a, b):
    # a NaN's payload is the platform's (the GPU's canonical NaN is not the
    # CPU's); every other value must match bit for bit
    nan = np.isnan(a) | np.isnan(b)
    return np.array_equal(np.isnan(a), np.isnan(b)) and np.array_equal(a[~nan].view(np.uint32), b[~nan].view(np.uint32))


@pytest.mark.parametrize("model", ["quad", "dubins"])
def test_propagate_large_angles_bit_exact_vs_oracle(model):
    """Angles far outside one turn (|x| up to 1e4 rad): the portable
    sine/cosine takes the nearest multiple of pi/2 and its quadrant from one
    1.5 * 2^23 addition on both sides, so every quadrant and sign comes out
    the same on the GPU and in the oracle."""
    if model == "quad":
        q = W.quadrotor_query(seed=3)
        cfg = q.config
        x0, u = random_inputs(cfg, 4096, 21)
        rng = np.random.default_rng(5)
        x0[:, 3:6] = rng.uniform(-100.0, 100.0, (4096, 3))
        x0[:256, 3:6] = rng.uniform(-1e4, 1e4, (256, 3))
    else:
        q = W.dubins_query(seed=3)
        cfg = q.config
        x0, u = random_inputs(cfg, 4096, 22)
        rng = np.random.default_rng(6)
        x0[:, 3] = rng.uniform(-1e3, 1e3, 4096)
        x0[:256, 3] = rng.uniform(-1e4, 1e4, 256)
    gx, gv, g1, g2 = gpu_propagate(cfg, x0, u, q.obstacles)
    ox, ov, o1, o2 = O.propagate_f32(cfg, x0, u, q.obstacles)
    assert np.array_equal(gv, ov)
    assert _same_bits_or_both_nan(gx, ox)
    assert np.array_equal(g1, o1) and np.array_equal(g2, o2)


@pytest.mark.parametrize("make", [W.dubins_query, W.unicycle_query], ids=["dubins", "unicycle"])
def test_propagate_new_models_bit_exact_vs_oracle(make):
    q = make(seed=2, n_obstacles=40)
    cfg = q.config
    x0, u = random_inputs(cfg, 4096, 14)
    gx, gv, g1, g2 = gpu_propagate(cfg, x0, u, q.obstacles)
    ox, ov, o1, o2 = O.propagate_f32(cfg, x0, u, q.obstacles)
    assert 0.05 < ov.mean() < 0.95
    assert np.array_equal(gv, ov)
    assert np.array_equal(gx.view(np.uint32), ox.view(np.uint32))
    assert np.array_equal(g1, o1) and np.array_equal(g2, o2)


QUERIES = {"di": W.double_integrator_query, "quad": W.quadrotor_query, "dubins": W.dubins_query, "unicycle": W.unicycle_query}


@pytest.mark.parametrize("model", ["di", "quad", "dubins", "unicycle"])
def test_propagate_within_tolerance_of_fp64(model):
    q = QUERIES[model](seed=3)
    cfg = q.config
    x0, u = random_inputs(cfg, 4096, 13)
    gx, gv, _, _ = gpu_propagate(cfg, x0, u, q.obstacles)
    dx, dv = O.propagate_f64(cfg, x0, u, q.obstacles)
    same = gv == dv
    mism = np.flatnonzero(~same)
    # a verdict may flip only where the FP64 trajectory passes within 1e-5 of
    # a threshold (obstacle face, velocity or workspace bound); such samples
    # are reported, not failed
    margins = [O.verdict_margin_f64(cfg, x0[i], u[i], q.obstacles) for i in mism]
    print(f"{model}: {len(mism)} / {len(gv)} verdicts differ from FP64, all near a threshold: "
          f"max margin {max(margins) if margins else 0:.2e}")
    assert all(m < 1e-5 for m in margins)
    tol = REL_TOL * np.maximum(np.abs(dx), state_scales(cfg))
    err = np.abs(gx.astype(np.float64) - dx)
    assert np.all(err[same] <= tol[same]), float((err[same] / tol[same]).max())


def test_propagate_matches_reference_golden(golden_dir):
    g = np.load(golden_dir / "ref_di.npz")
    cfg = double_integrator_single().replace(di_rule=DI_RULE_REFERENCE)
    gx, gv, _, _ = gpu_propagate(cfg, g["x0"], g["u"], g["obstacles"])
    assert np.array_equal(gv, g["valid"])
    assert np.array_equal(gx.view(np.uint32), g["x1"].view(np.uint32))
    gq = np.load(golden_dir / "ref_quad.npz")
    cq = quadrotor_large().replace(min_steps=1, max_steps=15)
    qx, qv, _, _ = gpu_propagate(cq, gq["x0"], gq["u"], gq["obstacles"])
    same = qv == gq["valid"]
    # the reference's propagateAndCheckQuadRungeKutta (statePropagator.cu:
    # 246-323): a verdict may differ only within 1e-6 of a bound or a face
    for i in np.flatnonzero(~same):
        assert O.verdict_margin_f64(cq, gq["x0"][i], gq["u"][i], gq["obstacles"]) < 1e-6, ("quad", i)
    tol = REL_TOL * np.maximum(np.abs(gq["x1"]), state_scales(cq))
    assert np.all(np.abs(qx - gq["x1"])[same] <= tol[same])
    # Dubins airplane and unicycle: the reference's own code fed the same
    # uniforms (its unicycle boxes span z in [-1, 1]; ours are planar)
    for name, cfg in (("ref_dubins.npz", dubins_airplane(seed=3)), ("ref_unicycle.npz", unicycle(seed=3))):
        g = np.load(golden_dir / name)
        x, v, _, _ = gpu_propagate(cfg, g["x0"], g["u"], g["obstacles"])
        same = v == g["valid"]
        for i in np.flatnonzero(~same):
            assert O.verdict_margin_f64(cfg, g["x0"][i], g["u"][i], g["obstacles"]) < 1e-6, (name, i)
        tol = REL_TOL * np.maximum(np.abs(g["x1"]), state_scales(cfg))
        assert np.all(np.abs(x - g["x1"])[same] <= tol[same]), name


# ---------------------------------------------------------------------------
# whole plans
# ---------------------------------------------------------------------------
def plan_gpu(q):
    from kgmt_gb300.planner import KGMT
    d_obs = torch.from_numpy(np.ascontiguousarray(W.boxes_for_plan(q), np.float32)).to(DEV)
    p = KGMT(q.config)
    res = p.plan(q.init, q.goal, d_obs, q.obstacles.shape[0])
    samples, parents, costs = p.copy_tree()
    path = p.copy_path()
    p.close()
    return res, samples, parents, costs, path


def assert_same_plan(res, samples, parents, costs, path, ref):
    for k in ("status", "iterations", "tree_size", "goal_index", "path_len", "samples_drawn"):
        assert res[k] == ref[k], (k, res[k], ref[k])
    assert np.array_equal(parents, ref["parents"])
    assert np.array_equal(samples.view(np.uint32), ref["samples"].view(np.uint32))
    assert np.array_equal(costs.view(np.uint32), ref["costs"].view(np.uint32))
    assert np.array_equal(path.view(np.uint32), ref["path"].view(np.uint32))


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_plan_double_integrator_bit_exact(seed):
    q = W.double_integrator_query(seed=seed)
    out = plan_gpu(q)
    assert_same_plan(*out, O.plan(q))


def test_plan_double_integrator_reference_rule_bit_exact():
    q = W.double_integrator_query(seed=4)
    q.config = q.config.replace(di_rule=DI_RULE_REFERENCE)
    assert_same_plan(*plan_gpu(q), O.plan(q))


def test_plan_quadrotor_small_bit_exact():
    q = W.quadrotor_query(seed=1, tree_capacity=30_000, max_iterations=25)
    assert_same_plan(*plan_gpu(q), O.plan(q))


@pytest.mark.parametrize("seed", [1, 2])
def test_plan_dubins_bit_exact(seed):
    q = W.dubins_query(seed=seed, tree_capacity=40_000)
    assert_same_plan(*plan_gpu(q), O.plan(q))


@pytest.mark.parametrize("seed", [1, 2])
def test_plan_unicycle_bit_exact(seed):
    """Planar model: the single-query plan takes the reference's [n][4] box
    rows; regions are 8^2 with 4^2 fine cells."""
    q = W.unicycle_query(seed=seed, tree_capacity=40_000)
    assert_same_plan(*plan_gpu(q), O.plan(q))


def test_batch_all_models_matches_oracle():
    """The four models in one batch (the mixed propagate variant); each query
    as its oracle plan, and as the same query planned alone."""
    qs = W.all_models_batch(16, seed=4, tree_capacity=20_000)
    for q in qs:
        q.config = q.config.replace(max_iterations=40)
    b, res = _batch(qs)
    refs = O.plan_batch(qs)
    for i, (r, ref) in enumerate(zip(res, refs)):
        for k in ("status", "iterations", "tree_size", "goal_index", "path_len", "samples_drawn"):
            assert r[k] == ref[k], (i, k, r[k], ref[k])
    for i in (0, 2):
        alone = plan_gpu(qs[i])
        s, p, c = b.copy_tree(i)
        n = res[i]["tree_size"]
        assert np.array_equal(p[:n], alone[2])
        assert np.array_equal(s[:n].view(np.uint32), alone[1].view(np.uint32))


@pytest.mark.parametrize("kind", ["di2", "di3", "di4", "models4"])
def test_tail_launch_matches_chain_and_oracle(kind, monkeypatch):
    """Batches of 2-4 queries run whole iterations in the persistent tail
    launch from the first iteration on (several running queries, then fewer
    as they finish, then one: both ways of scoring regions); the plans equal
    the oracle's, the trees equal those of the two-kernel chain alone
    (KGMT_TAIL=0), and so do the step, box-test and sample counts."""
    if kind == "models4":
        qs = W.all_models_batch(4, seed=6, tree_capacity=20_000)
        for q in qs:
            q.config = q.config.replace(max_iterations=60)
    else:
        qs = W.double_integrator_batch(int(kind[2:]), n_obstacles=50, seed=11, tree_capacity=20_000)
    b, res = _batch(qs)
    st = b.stats()
    assert st["iterations_tail"] > 0
    monkeypatch.setenv("KGMT_TAIL", "0")
    b0, res0 = _batch(qs)
    st0 = b0.stats()
    assert st0["iterations_tail"] == 0
    refs = O.plan_batch(qs)
    for i, (r, r0, ref) in enumerate(zip(res, res0, refs)):
        for k in ("status", "iterations", "tree_size", "goal_index", "path_len", "samples_drawn"):
            assert r[k] == ref[k] == r0[k], (kind, i, k, r[k], r0[k], ref[k])
        s, p, c = b.copy_tree(i)
        s0, p0, c0 = b0.copy_tree(i)
        n = r["tree_size"]
        assert np.array_equal(p[:n], p0[:n]) and np.array_equal(s[:n].view(np.uint32), s0[:n].view(np.uint32))
        assert np.array_equal(c[:n].view(np.uint32), c0[:n].view(np.uint32))
    for k in ("steps_executed", "obstacle_tests", "samples"):
        assert st[k] == st0[k], (kind, k, st[k], st0[k])
    b.close()
    b0.close()


def test_plan_edge_cases():
    # no obstacles
    q = W.double_integrator_query(seed=6)
    q.obstacles = np.zeros((0, 6), np.float32)
    assert_same_plan(*plan_gpu(q), O.plan(q))
    # tiny tree: capacity exhausted, truncated frontier expansion
    q = W.double_integrator_query(seed=7)
    q.config = q.config.replace(tree_capacity=60, max_iterations=50)
    out = plan_gpu(q)
    ref = O.plan(q)
    assert ref["status"] == 3
    assert_same_plan(*out, ref)
    # one iteration budget
    q = W.double_integrator_query(seed=8)
    q.config = q.config.replace(max_iterations=1)
    assert_same_plan(*plan_gpu(q), O.plan(q))
    # goal ball around the start: found by the first accepted child
    q = W.double_integrator_query(seed=9)
    q.goal = q.init.copy()
    q.config = q.config.replace(goal_radius=0.2)
    assert_same_plan(*plan_gpu(q), O.plan(q))
    # many obstacles (global-memory path past the shared-memory stage)
    q = W.double_integrator_query(seed=10, n_obstacles=1500)
    q.obstacles[:, 3:] = q.obstacles[:, :3] + 0.01
    q.config = q.config.replace(tree_capacity=20_000, max_iterations=15)
    assert_same_plan(*plan_gpu(q), O.plan(q))


def test_plan_obstacle_grid_edge_cases():
    """Boxes the culling grid must still find: large boxes spanning many
    cells, inverted (min > max) boxes, boxes partly outside the workspace,
    boxes whose faces lie exactly on grid-cell boundaries."""
    q = W.double_integrator_query(seed=11)
    extra = np.float32([
        [0.30, 0.30, 0.30, 0.80, 0.55, 0.60],     # spans many cells
        [0.70, 0.20, 0.20, 0.60, 0.10, 0.10],     # inverted
        [-0.2, 0.40, 0.40, 0.05, 0.45, 0.45],     # outside on -x
        [0.9375, 0.5, 0.5, 1.3, 0.5625, 0.5625],  # faces on 1/16 boundaries, outside on +x
        [0.25, 0.25, 0.0, 0.3125, 0.3125, 0.0625],
    ])
    q.obstacles = np.concatenate([q.obstacles, extra]).astype(np.float32)
    q.config = q.config.replace(tree_capacity=30_000, max_iterations=40)
    assert_same_plan(*plan_gpu(q), O.plan(q))
    # function level with the same boxes: verdicts equal brute force
    cfg = q.config
    x0, u = random_inputs(cfg, 4096, 21)
    gx, gv, _, _ = gpu_propagate(cfg, x0, u, q.obstacles)
    ox, ov, _, _ = O.propagate_f32(cfg, x0, u, q.obstacles)
    assert np.array_equal(gv, ov)


# ---------------------------------------------------------------------------
# batched and served forms
# ---------------------------------------------------------------------------
def _batch(queries, block=256, graph=True):
    from kgmt_gb300.planner import BatchPlanner
    inits, goals, obs, offs, cnts = W.pack_queries(queries)
    b = BatchPlanner(len(queries), propagate_block=block, use_graph=graph)
    res = b.plan([q.config for q in queries], inits, goals, obs, offs, cnts)
    return b, res


def test_batch_matches_oracle_and_plain():
    qs = W.double_integrator_batch(24, n_obstacles=50, seed=3, tree_capacity=20_000)
    b, res = _batch(qs)
    refs = O.plan_batch(qs)
    for i, (r, ref) in enumerate(zip(res, refs)):
        for k in ("status", "iterations", "tree_size", "goal_index", "path_len", "samples_drawn"):
            assert r[k] == ref[k], (i, k, r[k], ref[k])
    # the same query alone gives the same tree
    for i in (0, 7, 23):
        alone = plan_gpu(qs[i])
        s, p, c = b.copy_tree(i)
        n = res[i]["tree_size"]
        assert np.array_equal(p[:n], alone[2])
        assert np.array_equal(s[:n].view(np.uint32), alone[1].view(np.uint32))


def test_large_batch_matches_oracle():
    """A batch large enough for the big-iteration paths: two samples per
    thread in the propagate tiles (iterations of more than twice the resident
    threads' samples) and 4096-node re-activation tiles (trees filling more
    large tiles than there are SMs), then the small-tile tail of its last
    queries; every query as the oracle plans it."""
    qs = W.double_integrator_batch(96, n_obstacles=50, seed=21, tree_capacity=50_000)
    b, res = _batch(qs)
    refs = O.plan_batch(qs)
    for i, (r, ref) in enumerate(zip(res, refs)):
        for k in ("status", "iterations", "tree_size", "goal_index", "path_len", "samples_drawn"):
            assert r[k] == ref[k], (i, k, r[k], ref[k])
    for i in (0, 50, 95):
        s, par, c = b.copy_tree(i)
        n = res[i]["tree_size"]
        ref = O.plan(qs[i])
        assert np.array_equal(par[:n], ref["parents"])
        assert np.array_equal(s[:n].view(np.uint32), ref["samples"].view(np.uint32))
    b.close()


def test_batch_heterogeneous_matches_oracle():
    qs = W.mixed_batch(24, seed=2, capacity_scale=0.1)
    for q in qs:
        q.config = q.config.replace(max_iterations=30)
    b, res = _batch(qs)
    refs = O.plan_batch(qs)
    for i, (r, ref) in enumerate(zip(res, refs)):
        for k in ("status", "iterations", "tree_size", "goal_index", "samples_drawn"):
            assert r[k] == ref[k], (i, k, r[k], ref[k])


@pytest.mark.parametrize("block", [128, 512])
def test_block_size_does_not_change_results(block):
    qs = W.double_integrator_batch(8, seed=5, tree_capacity=20_000)
    _, base = _batch(qs, 256)
    _, other = _batch(qs, block, graph=False)
    assert [(r["tree_size"], r["goal_index"], r["iterations"]) for r in base] == \
        [(r["tree_size"], r["goal_index"], r["iterations"]) for r in other]


def test_autotuner_block_and_samples_per_node():
    """kgmt_batch_autotune picks a block size the batch then keeps, and the
    results do not depend on it; kgmt_batch_autotune_full sweeps block size x
    samples per node and keeps the success rate within 95 % of the configs'
    own (its pick, planned again, gives that success rate)."""
    from kgmt_gb300.planner import BatchPlanner
    qs = W.double_integrator_batch(16, seed=12, tree_capacity=20_000)
    cfgs = [q.config for q in qs]
    inits, goals, obs, offs, cnts = W.pack_queries(qs)
    b = BatchPlanner(len(qs))
    base = b.plan(cfgs, inits, goals, obs, offs, cnts)
    blk = b.autotune(cfgs, inits, goals, obs, offs, cnts)
    assert blk in (128, 256, 512)
    again = b.plan(cfgs, inits, goals, obs, offs, cnts)
    assert [(r["tree_size"], r["goal_index"]) for r in again] == [(r["tree_size"], r["goal_index"]) for r in base]
    t = b.autotune_full(cfgs, inits, goals, obs, offs, cnts)
    assert t["propagate_block"] in (128, 256, 512) and t["samples_per_node"] in (2, 4, 8, 16)
    assert t["success_rate"] >= 0.95 * t["base_success_rate"] - 1e-6
    assert t["queries_per_s"] > 0 and t["base_queries_per_s"] > 0
    tuned = [c.replace(samples_per_node=t["samples_per_node"]) for c in cfgs]
    res = b.plan(tuned, inits, goals, obs, offs, cnts)
    assert abs(sum(r["status"] == 1 for r in res) / len(qs) - t["success_rate"]) < 1e-6
    # the tuned batch is still the oracle's
    refs = O.plan_batch([type(q)(c, q.init, q.goal, q.obstacles) for q, c in zip(qs, tuned)])
    for r, ref in zip(res, refs):
        assert (r["status"], r["tree_size"], r["goal_index"]) == (ref["status"], ref["tree_size"], ref["goal_index"])
    b.close()


def test_server_results_same_alone_and_in_mix():
    from kgmt_gb300.planner import Server
    qs = W.double_integrator_batch(12, seed=6, tree_capacity=20_000)
    refs = O.plan_batch(qs)
    srv = Server(max_slots=4, memory_budget=1 << 30, iters_per_step=2)
    tickets = {}
    pending = list(range(len(qs)))
    got = {}
    steps = 0
    while len(got) < len(qs):
        # staggered arrivals: two new queries every step
        for _ in range(2):
            if pending:
                i = pending.pop(0)
                tickets[srv.submit(qs[i].config, qs[i].init, qs[i].goal, qs[i].obstacles)] = i
        srv.step()
        for r in srv.poll():
            got[tickets[r["ticket"]]] = r
        steps += 1
        assert steps < 5000
    for i, ref in enumerate(refs):
        for k in ("status", "iterations", "tree_size", "goal_index", "samples_drawn"):
            assert got[i][k] == ref[k], (i, k, got[i][k], ref[k])


def test_server_lets_small_queries_pass_a_head_that_does_not_fit():
    """Admission by device memory with passing: four small queries fill part
    of a 20 MiB budget, a large one (T = 150k, 15.5 MiB) queued behind them
    does not fit, and four more small ones queued behind it are admitted
    first; the large one runs once memory frees up.  Every result is the
    oracle's (each query alone), whatever order the queries ran in."""
    from kgmt_gb300.planner import Server
    small = W.double_integrator_batch(8, seed=14, tree_capacity=20_000)
    big = W.double_integrator_batch(1, seed=15, tree_capacity=150_000)[0]
    order = small[:4] + [big] + small[4:]
    srv = Server(max_slots=16, memory_budget=20 << 20, iters_per_step=2)
    tickets = [srv.submit(q.config, q.init, q.goal, q.obstacles) for q in order]
    got, finished = {}, []
    for _ in range(5000):
        srv.step()
        for r in srv.poll():
            got[r["ticket"]] = r
            finished.append(r["ticket"])
        if len(got) == len(order):
            break
    refs = O.plan_batch(order)
    for t, ref in zip(tickets, refs):
        for k in ("status", "iterations", "tree_size", "goal_index", "samples_drawn"):
            assert got[t][k] == ref[k], (t, k, got[t][k], ref[k])
    # the small queries queued behind the large one ran first
    later_small = set(tickets[5:])
    assert any(finished.index(t) < finished.index(tickets[4]) for t in later_small)
    srv.close()


def _assert_results_match(res, refs, idx, keys=("status", "iterations", "tree_size", "goal_index", "path_len", "samples_drawn")):
    for i, ref in zip(idx, refs):
        for k in keys:
            assert res[i][k] == ref[k], (i, k, res[i][k], ref[k])


def test_bench_workload_matches_oracle():
    """The workload bench.py measures -- its own 256-query double-integrator
    batch (50 boxes, T = 50k, seed 1) -- planned by the GPU and by the
    oracle: every query's status, iterations, tree size, goal index, path
    length and samples drawn bit-exact, and 16 whole trees (the slowest and
    the largest among them) node for node."""
    import bench
    qs = bench.make_workload(0)
    assert len(qs) == bench.N_QUERIES
    b, res = _batch(qs)
    refs = O.plan_batch(qs)
    _assert_results_match(res, refs, range(len(qs)))
    slowest = int(np.argmax([r["iterations"] for r in res]))
    largest = int(np.argmax([r["tree_size"] for r in res]))
    pick = sorted({slowest, largest, *range(0, 256, 18)})[:16]
    assert len(pick) == 16
    for i in pick:
        s, par, c = b.copy_tree(i)
        n = res[i]["tree_size"]
        ref = O.plan(qs[i])
        assert np.array_equal(par[:n], ref["parents"]), i
        assert np.array_equal(s[:n].view(np.uint32), ref["samples"].view(np.uint32)), i
        assert np.array_equal(c[:n].view(np.uint32), ref["costs"].view(np.uint32)), i
        assert np.array_equal(b.copy_path(i).view(np.uint32), ref["path"].view(np.uint32)), i
    b.close()


def test_mixed_workload_subset_matches_oracle():
    """The 1024-query mixed batch at its real sizes (half double integrator,
    half quadrotor; 5..1000 boxes; 8^3..32^3 grids; T 10k..500k), planned
    once on the GPU; 64 of its queries -- the largest tree, the slowest and
    the most obstacles of each model, the rest spread over the batch -- planned
    by the oracle: results bit-exact, and the four smallest trees node for
    node."""
    qs = W.mixed_batch(1024, seed=1)
    b, res = _batch(qs)
    pick = set()
    for odd in (0, 1):  # even slots double integrator, odd ones quadrotor
        idx = [i for i in range(len(qs)) if i % 2 == odd]
        pick.add(max(idx, key=lambda i: res[i]["tree_size"]))
        pick.add(max(idx, key=lambda i: res[i]["iterations"]))
        pick.add(max(idx, key=lambda i: qs[i].obstacles.shape[0]))
    rest = [i for i in range(0, len(qs), 13) if i not in pick]
    pick = sorted(pick | set(rest[: 64 - len(pick)]))
    assert len(pick) == 64 and {i % 2 for i in pick} == {0, 1}
    refs = O.plan_batch([qs[i] for i in pick])
    _assert_results_match(res, refs, pick)
    for i in sorted(pick, key=lambda i: res[i]["tree_size"])[:4]:
        s, par, c = b.copy_tree(i)
        n = res[i]["tree_size"]
        ref = O.plan(qs[i])
        assert np.array_equal(par[:n], ref["parents"]), i
        assert np.array_equal(s[:n].view(np.uint32), ref["samples"].view(np.uint32)), i
    b.close()


# ---------------------------------------------------------------------------
# The reference's own configurations at full size, too large for the oracle
# to plan in seconds: properties that hold whatever the size.
# ---------------------------------------------------------------------------
def reconstruct_uniforms(cfg, rows):
    """The uniforms that give a tree row's controls and step count: each
    control c = u_min + u * (u_max - u_min) in unfused FP32 (as the kernels
    and the oracle compute it) inverted, then moved by ulps until it gives c
    back exactly; the step draw centred on its count."""
    NC = 4 if cfg.sample_dim == 17 else 3
    D = cfg.sample_dim
    n = rows.shape[0]
    u = np.full((n, 8), 0.5, np.float32)
    umin = np.asarray(cfg.u_min, np.float32)[:NC]
    span = (np.asarray(cfg.u_max, np.float32)[:NC] - umin).astype(np.float32)
    live = span > 0
    ctrl = rows[:, D - 1 - NC:D - 1].astype(np.float32)
    uc = ((ctrl.astype(np.float64) - umin) / np.where(live, span, 1.0)).astype(np.float32)
    uc = np.where(live, uc, np.float32(0.5))
    for _ in range(8):
        c = umin + uc * span
        uc = np.where(live & (c < ctrl), np.nextafter(uc, np.float32(2.0)), uc)
        uc = np.where(live & (c > ctrl), np.nextafter(uc, np.float32(-1.0)), uc)
    assert (~live | (umin + uc * span == ctrl)).all(), "a control no uniform gives"
    u[:, :NC] = uc
    k = np.rint(rows[:, D - 1].astype(np.float64) / cfg.step_size)
    u[:, NC] = ((k - cfg.min_steps + 0.5) / (cfg.max_steps - cfg.min_steps + 1)).astype(np.float32)
    return u


def check_tree_properties(q, res, samples, parents, costs, path, n_edges=3000, seed=0):
    cfg = q.config
    D = cfg.sample_dim
    n = res["tree_size"]
    assert 1 <= n <= cfg.tree_capacity
    S, P, C = samples[:n], parents[:n], costs[:n]
    # every node but the root hangs off an earlier node
    assert P[0] == -1
    assert ((P[1:] >= 0) & (P[1:] < np.arange(1, n))).all()
    # rows are finite, inside the workspace and the velocity bounds
    assert np.isfinite(S).all()
    assert ((S[:, :3] >= cfg.ws_min) & (S[:, :3] <= cfg.ws_max)).all()
    vel = slice(3, 6) if D == 10 else slice(6, 9)
    assert ((S[1:, vel] >= cfg.v_min) & (S[1:, vel] <= cfg.v_max)).all()
    # durations are whole step counts within [min_steps, max_steps]
    k = S[1:, D - 1] / np.float32(cfg.step_size)
    assert np.allclose(k, np.rint(k), atol=1e-4)
    assert ((np.rint(k) >= cfg.min_steps) & (np.rint(k) <= cfg.max_steps)).all()
    # costs are the goal distances in the kernel's FP32 order (the root's is 0)
    g = np.asarray(q.goal, np.float32)
    d = [S[1:, j] - g[j] for j in range(3)]
    ref_cost = np.sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2])
    assert C[0] == 0.0
    assert np.array_equal(C[1:].view(np.uint32), ref_cost.astype(np.float32).view(np.uint32))
    # a success ends in the goal ball, and its path is the parent chain
    if res["status"] == 1:
        gi = res["goal_index"]
        assert 0 <= gi < n and C[gi] < cfg.goal_radius
        chain = [gi]
        while P[chain[-1]] >= 0:
            chain.append(int(P[chain[-1]]))
        assert res["path_len"] == len(chain)
        assert np.array_equal(path.view(np.uint32), S[chain].view(np.uint32))
    # edges re-propagated by the oracle's FP32 restatement from the parent
    # with the child's controls and step count give the child bit for bit,
    # collision-free; for the double integrator also within 1e-5 of FP64 (the
    # quadrotor's Euler-angle kinematics make FP32 and FP64 part near
    # theta = +-pi/2, where tan and 1/cos blow up: a property of the model)
    rng = np.random.default_rng(seed)
    kids = rng.choice(np.arange(1, n), size=min(n_edges, n - 1), replace=False)
    u = reconstruct_uniforms(cfg, S[kids])
    x32, valid32, _, _ = O.propagate_f32(cfg, S[P[kids]], u, q.obstacles)
    assert valid32.all(), kids[valid32 == 0][:5]
    assert np.array_equal(x32.view(np.uint32), S[kids].view(np.uint32)), kids[(x32 != S[kids]).any(axis=1)][:5]
    if D == 10:
        x1, valid = O.propagate_f64(cfg, S[P[kids]], u, q.obstacles)
        tol = REL_TOL * np.maximum(np.abs(S[kids]), state_scales(cfg))
        assert (np.abs(x1 - S[kids]) <= tol).all(), np.argwhere(np.abs(x1 - S[kids]) > tol)[:5]
        for i in np.flatnonzero(valid == 0):
            assert O.verdict_margin_f64(cfg, S[P[kids[i]]], u[i], q.obstacles) < 1e-6, kids[i]


@pytest.mark.parametrize("which", ["di_single_T100k", "quad_T2M"])
def test_full_size_single_query_properties(which):
    """The single double-integrator query (T = 100k) and the large quadrotor
    query (T = 2M, 8 samples per node, 200 boxes, 16^3 / 4^3 grid)."""
    q = W.double_integrator_query(seed=4) if which == "di_single_T100k" else W.quadrotor_query(seed=2)
    res, samples, parents, costs, path = plan_gpu(q)
    assert res["status"] in (1, 2, 3), res
    check_tree_properties(q, res, samples, parents, costs, path)


def test_full_size_batch_properties():
    """The 256-query double-integrator batch (50 boxes, T = 50k each): every
    query's tree, checked on a sample of its queries including the slowest."""
    qs = W.double_integrator_batch(256, n_obstacles=50, seed=1, tree_capacity=50_000)
    b, res = _batch(qs)
    slowest = int(np.argmax([r["iterations"] for r in res]))
    for i in sorted({0, 1, 127, 255, slowest}):
        s, p, c = b.copy_tree(i)
        check_tree_properties(qs[i], res[i], s, p, c, b.copy_path(i), n_edges=1000, seed=i)
    assert all(r["status"] == 1 for r in res)
    b.close()


def test_full_size_mixed_batch_properties():
    """The 1024-query mixed batch (half double integrator, half quadrotor;
    5..1000 boxes, 8^3..32^3 grids, T 10k..500k): both models' trees, the
    largest of each and the slowest queries among those checked."""
    qs = W.mixed_batch(1024, seed=1)
    b, res = _batch(qs)
    pick = set()
    for model_odd in (0, 1):  # even slots double integrator, odd ones quadrotor
        idx = [i for i in range(len(qs)) if i % 2 == model_odd]
        pick.add(max(idx, key=lambda i: res[i]["tree_size"]))
        pick.add(max(idx, key=lambda i: res[i]["iterations"]))
        pick.update(idx[:2])
    for i in sorted(pick):
        s, p, c = b.copy_tree(i)
        check_tree_properties(qs[i], res[i], s, p, c, b.copy_path(i), n_edges=1000, seed=i)
    b.close()
