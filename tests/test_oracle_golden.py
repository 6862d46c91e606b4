"""The CPU oracle against the golden vectors made from the reference's own
propagation / collision / region code (tests/golden/make_golden.py) and the
published Philox4x32-10 known-answer vectors."""
import json

import numpy as np
import pytest

from kgmt_gb300.config import DI_RULE_REFERENCE, double_integrator_single, quadrotor_large
from oracle import oracle as O

# state tolerance: |delta| <= 1e-5 * max(|ref|, scale) per component
REL_TOL = 1e-5


def state_scales(cfg):
    D = cfg.sample_dim
    s = np.ones(D)
    s[:3] = cfg.ws_max - cfg.ws_min
    if D == 10:
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
    assert same.mean() > 0.995
    tol = REL_TOL * np.maximum(np.abs(x1), state_scales(cfg))
    assert np.all(np.abs(x1[same] - g["x1"][same]) <= tol[same])


def test_quad_matches_reference_within_tolerance(golden_dir):
    g = np.load(golden_dir / "ref_quad.npz")
    cfg = quadrotor_large().replace(min_steps=1, max_steps=15)
    for fn in (O.propagate_f32, O.propagate_f64):
        out = fn(cfg, g["x0"], g["u"], g["obstacles"])
        x1, valid = out[0], out[1]
        same = valid == g["valid"]
        assert same.mean() > 0.99, fn.__name__
        tol = REL_TOL * np.maximum(np.abs(g["x1"]), state_scales(cfg))
        bad = np.abs(x1[same] - g["x1"][same]) > tol[same]
        assert not bad.any(), (fn.__name__, np.argwhere(bad)[:5])


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
