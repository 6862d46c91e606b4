"""The CPU oracle against the golden vectors made from the reference's own
propagation / collision / region code (tests/golden/make_golden.py) and the
published Philox4x32-10 known-answer vectors."""
import json

import numpy as np
import pytest

from kgmt_gb300.config import (DI_RULE_REFERENCE, MODEL_DUBINS_AIRPLANE, MODEL_UNICYCLE, double_integrator_single,
                               dubins_airplane, quadrotor_large, unicycle)
from oracle import oracle as O

# state tolerance: |delta| <= 1e-5 * max(|ref|, scale) per component
REL_TOL = 1e-5


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
        s[6:9] = 1.0
        s[9] = cfg.step_size
    else:
        s[3:6] = np.pi
        s[6:9] = cfg.v_max
        s[9:12] = 1.0
        s[12:16] = 1.0
        s[16] = cfg.step_size
    return s


def test_philox_known_answers(golden_dir):
    for v in json.loads((golden_dir / "philox_kat.json").read_text()):
        assert O.philox(v["ctr"], v["key"]) == v["out"]


def test_uniform_range_and_order():
    u = O.sample_uniforms(12345, 7, 3)
    assert u.dtype == np.float32 and np.all(u > 0) and np.all(u <= 1)
    # ko_u01 maps 0xFFFFFFFF to exactly 1 and 0 to 2^-24
    assert float(O.load().ko_u01(0xFFFFFFFF)) == 1.0
    assert float(O.load().ko_u01(0)) == 2.0 ** -24


def test_di_reference_formula_bit_exact(golden_dir):
    g = np.load(golden_dir / "ref_di.npz")
    cfg = double_integrator_single().replace(di_rule=DI_RULE_REFERENCE)
    x1, valid, _, _ = O.propagate_f32(cfg, g["x0"], g["u"], g["obstacles"])
    assert np.array_equal(valid, g["valid"])
    assert np.array_equal(x1.view(np.uint32), g["x1"].view(np.uint32))


def test_di_fp64_oracle_tracks_reference(golden_dir):
    g = np.load(golden_dir / "ref_di.npz")
    cfg = double_integrator_single().replace(di_rule=DI_RULE_REFERENCE)
    x1, valid = O.propagate_f64(cfg, g["x0"], g["u"], g["obstacles"])
    same = valid == g["valid"]
    # a verdict may differ only where the FP64 trajectory passes within 1e-6
    # of a bound or a box face (none does in this fixture)
    for i in np.flatnonzero(~same):
        assert O.verdict_margin_f64(cfg, g["x0"][i], g["u"][i], g["obstacles"]) < 1e-6, i
    tol = REL_TOL * np.maximum(np.abs(x1), state_scales(cfg))
    assert np.all(np.abs(x1[same] - g["x1"][same]) <= tol[same])


def test_quad_matches_reference_within_tolerance(golden_dir):
    """Quadrotor (statePropagator.cu:246-370): the FP32 mirror and the FP64
    restatement against the reference's propagateAndCheckQuadRungeKutta fed
    the same uniforms.  Every verdict agrees except where the FP64 trajectory
    passes within 1e-6 of a bound or a box face (none does here)."""
    g = np.load(golden_dir / "ref_quad.npz")
    cfg = quadrotor_large().replace(min_steps=1, max_steps=15)
    for fn in (O.propagate_f32, O.propagate_f64):
        out = fn(cfg, g["x0"], g["u"], g["obstacles"])
        x1, valid = out[0], out[1]
        same = valid == g["valid"]
        for i in np.flatnonzero(~same):
            assert O.verdict_margin_f64(cfg, g["x0"][i], g["u"][i], g["obstacles"]) < 1e-6, (fn.__name__, i)
        tol = REL_TOL * np.maximum(np.abs(g["x1"]), state_scales(cfg))
        bad = np.abs(x1[same] - g["x1"][same]) > tol[same]
        assert not bad.any(), (fn.__name__, np.argwhere(bad)[:5])


@pytest.mark.parametrize("fixture,cfg", [("ref_dubins.npz", dubins_airplane(seed=3)), ("ref_unicycle.npz", unicycle(seed=3))])
def test_new_models_match_reference_within_tolerance(golden_dir, fixture, cfg):
    """Dubins airplane (statePropagator.cu:147-244) and unicycle (13-74): the
    FP32 mirror (portable sine/cosine) and the FP64 restatement against the
    reference's own code fed the same uniforms.  Verdicts agree except where
    the FP64 trajectory passes within 1e-6 of a bound or a box face."""
    g = np.load(golden_dir / fixture)
    for fn in (O.propagate_f32, O.propagate_f64):
        out = fn(cfg, g["x0"], g["u"], g["obstacles"])
        x1, valid = out[0], out[1]
        same = valid == g["valid"]
        for i in np.flatnonzero(~same):
            assert O.verdict_margin_f64(cfg, g["x0"][i], g["u"][i], g["obstacles"]) < 1e-6, (fn.__name__, i)
        tol = REL_TOL * np.maximum(np.abs(g["x1"]), state_scales(cfg))
        bad = np.abs(x1[same] - g["x1"][same]) > tol[same]
        assert not bad.any(), (fn.__name__, np.argwhere(bad)[:5])
    assert 0.2 < g["valid"].mean() < 0.9  # the fixture exercises both verdicts


def test_planar_regions():
    """W_DIM 2 (unicycle): r1 = ix * L + iy (Graph.cu:105-113 with two
    workspace digits), fine cell jx * F + jy; the heading plays no part."""
    cfg = unicycle()
    L, F = cfg.coarse_len, cfg.fine_len
    rng = np.random.default_rng(5)
    for _ in range(500):
        x = np.zeros(7, np.float32)
        x[:2] = rng.uniform(-0.05, 1.05, 2)
        x[2] = rng.uniform(-10, 10)
        ix, iy = [min(max(int(np.float32(L) * x[d] / np.float32(1.0)), 0), L - 1) if x[d] >= 0 else 0 for d in range(2)]
        r1 = O.region(cfg, x)
        assert r1 == ix * L + iy
        r2 = O.subregion(cfg, x, r1)
        assert 0 <= r2 < F * F
        y = x.copy()
        y[2] = 0.0
        assert O.region(cfg, y) == r1 and O.subregion(cfg, y, r1) == r2


def test_collision_verdicts_bit_exact(golden_dir):
    g = np.load(golden_dir / "ref_collision.npz")
    ours = np.array([O.segment_valid(a, b, g["obstacles"]) for a, b in zip(g["p0"], g["p1"])], np.uint8)
    assert np.array_equal(ours, g["valid"])


@pytest.mark.parametrize("name,cfg", [("di", double_integrator_single()), ("quad", quadrotor_large())])
def test_region_ids_bit_exact(golden_dir, name, cfg):
    g = np.load(golden_dir / "ref_region.npz")
    x = g[f"{name}_x"]
    ours = np.array([O.region(cfg, xi) for xi in x], np.int32)
    assert np.array_equal(ours, g[f"{name}_r1"])
