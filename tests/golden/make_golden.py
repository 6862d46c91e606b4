"""Generate the golden vectors in tests/golden/ from the reference's own code.

Run with the path of a checkout of the reference's sources:

    python tests/golden/make_golden.py --ref /path/to/reference

It compiles the reference's propagation, collision and region functions for
the host (oracle/ref/Makefile -> oracle/_ref/*.so), feeds them seeded inputs
(the uniforms every curand_uniform() call returns are the Philox uniforms of
the oracle), and stores inputs and outputs as .npz fixtures.  The fixtures are
committed; the tests never need the reference.

Fixtures:
  ref_di.npz     reference DI propagation (statePropagator.cu:76-142), its
                 position formula (statePropagator.cu:97-99) as written
  ref_quad.npz   reference quadrotor propagation (statePropagator.cu:246-370)
  ref_dubins.npz reference Dubins-airplane propagation (statePropagator.cu:147-244)
  ref_unicycle.npz reference unicycle propagation (statePropagator.cu:13-74)
  ref_collision.npz  isMotionValid verdicts (collisionCheck.cu:3-10, 49-61)
  ref_region.npz getRegion ids (Graph.cu:99-153), 8^3 and 16^3 grids
  philox_kat.json published Philox4x32-10 known-answer vectors (Random123)
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from kgmt_gb300 import workloads as W  # noqa: E402
from kgmt_gb300.config import DI_RULE_REFERENCE, double_integrator_single, quadrotor_large  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent
REF_LIB = ROOT / "oracle" / "_ref"


def fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def load_ref(ref: str):
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle" / "ref"), f"REF={ref}"], check=True)
    libs = {}
    for name in ("di", "quad", "dubins", "uni", "graph_di", "graph_quad"):
        lib = C.CDLL(str(REF_LIB / f"libref_{name}.so"))
        libs[name] = lib
    for k in ("di", "quad", "dubins", "uni"):
        libs[k].ref_propagate.argtypes = [C.POINTER(C.c_float)] * 3 + [C.c_int, C.POINTER(C.c_float)]
        libs[k].ref_motion_valid.argtypes = [C.POINTER(C.c_float)] * 3 + [C.c_int]
    for k in ("graph_di", "graph_quad"):
        libs[k].ref_get_region.argtypes = [C.POINTER(C.c_float)]
    return libs


def uniforms(seed, n, itr=1):
    u = np.stack([O.sample_uniforms(seed, i, itr) for i in range(n)]).astype(np.float32)
    return u


def make_dynamics(lib, cfg, x0, u, obs):
    D = cfg.sample_dim
    n = x0.shape[0]
    x1 = np.zeros((n, D), np.float32)
    valid = np.zeros(n, np.uint8)
    obs = np.ascontiguousarray(obs, np.float32)
    for i in range(n):
        a = np.ascontiguousarray(x0[i])
        w = np.ascontiguousarray(u[i])
        y = np.zeros(D, np.float32)
        valid[i] = lib.ref_propagate(fp(a), fp(w), fp(obs), obs.shape[0], fp(y))
        x1[i] = y
    return x1, valid


def di_fixture(lib):
    cfg = double_integrator_single(seed=3).replace(di_rule=DI_RULE_REFERENCE)
    q = W.double_integrator_query(seed=3)
    rng = np.random.Generator(np.random.Philox(key=20240601))
    n = 2000
    x0 = np.zeros((n, 10), np.float32)
    x0[:, :3] = rng.uniform(0.0, 1.0, (n, 3))
    x0[:, 3:6] = rng.uniform(-0.3, 0.3, (n, 3))
    u = uniforms(777, n)
    # edge cases: k = 1 and k = max steps, zero velocity at the workspace corner,
    # a start exactly on an obstacle face, velocity exactly at the bound
    u[0, 3] = 2.0 ** -24  # k = 1
    u[1, 3] = 1.0 - 2.0 ** -24  # k = 6
    x0[2, :6] = [0.0, 0.0, 0.0, 0.0, 0.0, 0.0]
    b = q.obstacles[0]
    x0[3, :3] = [b[3], (b[1] + b[4]) / 2, (b[2] + b[5]) / 2]  # on the +x face
    x0[3, 3:6] = [0.2, 0.0, 0.0]
    x0[4, 3:6] = [0.3, -0.3, 0.3]
    u[:, 3] = np.minimum(u[:, 3], np.float32(1.0 - 2.0 ** -24))  # u == 1 gives MAX+1 steps in the reference
    x1, valid = make_dynamics(lib, cfg, x0, u, q.obstacles)
    np.savez_compressed(OUT / "ref_di.npz", x0=x0, u=u, obstacles=q.obstacles, x1=x1, valid=valid)
    return valid.mean()


def quad_fixture(lib):
    cfg = quadrotor_large(seed=3).replace(min_steps=1, max_steps=15)
    q = W.quadrotor_query(seed=3)
    rng = np.random.Generator(np.random.Philox(key=20240602))
    n = 1000
    x0 = np.zeros((n, 17), np.float32)
    x0[:, :3] = rng.uniform(0.1, 0.9, (n, 3))
    x0[:, 3:6] = rng.uniform(-0.5, 0.5, (n, 3))
    x0[:, 6:9] = rng.uniform(-0.2, 0.2, (n, 3))
    x0[:, 9:12] = rng.uniform(-1.0, 1.0, (n, 3))
    u = uniforms(778, n)
    u[:, 4] = np.minimum(u[:, 4], np.float32(1.0 - 2.0 ** -24))
    u[0, 4] = 2.0 ** -24
    x0[1, 3:12] = 0.0
    x1, valid = make_dynamics(lib, cfg, x0, u, q.obstacles)
    np.savez_compressed(OUT / "ref_quad.npz", x0=x0, u=u, obstacles=q.obstacles, x1=x1, valid=valid)
    return valid.mean()


def dubins_fixture(lib):
    q = W.dubins_query(seed=3, n_obstacles=40)
    rng = np.random.Generator(np.random.Philox(key=20240605))
    n = 1500
    x0 = np.zeros((n, 10), np.float32)
    x0[:, :3] = rng.uniform(0.1, 0.9, (n, 3))
    x0[:, 3] = rng.uniform(-np.pi, np.pi, n)
    x0[:, 4] = rng.uniform(-1.0, 1.0, n)
    x0[:, 5] = rng.uniform(0.0, 0.3, n)
    u = uniforms(779, n)
    u[:, 3] = np.minimum(u[:, 3], np.float32(1.0 - 2.0 ** -24))
    u[0, 3] = 2.0 ** -24  # k = 1
    u[1, 3] = 1.0 - 2.0 ** -24  # k = 10
    x0[2, 5] = 0.0  # at rest
    x0[3, 4] = 1.04  # pitch near its bound
    x1, valid = make_dynamics(lib, q.config, x0, u, q.obstacles)
    np.savez_compressed(OUT / "ref_dubins.npz", x0=x0, u=u, obstacles=q.obstacles, x1=x1, valid=valid)
    return valid.mean()


def unicycle_fixture(lib):
    # the reference's unicycle compiles with W_DIM 3 here: its step boxes lie
    # in z = 0, so boxes spanning z in [-1, 1] give the planar verdict
    q = W.unicycle_query(seed=3, n_obstacles=40)
    obs = q.obstacles.copy()
    obs[:, 2], obs[:, 5] = -1.0, 1.0
    rng = np.random.Generator(np.random.Philox(key=20240606))
    n = 1500
    x0 = np.zeros((n, 7), np.float32)
    x0[:, :2] = rng.uniform(0.1, 0.9, (n, 2))
    x0[:, 2] = rng.uniform(-np.pi, np.pi, n)
    x0[:, 3] = rng.uniform(0.0, 0.3, n)
    u = uniforms(780, n)
    u[:, 3] = np.minimum(u[:, 3], np.float32(1.0 - 2.0 ** -24))
    u[0, 3] = 2.0 ** -24
    u[1, 3] = 1.0 - 2.0 ** -24
    x0[2, 3] = 0.0
    x1, valid = make_dynamics(lib, q.config, x0, u, obs)
    np.savez_compressed(OUT / "ref_unicycle.npz", x0=x0, u=u, obstacles=obs, x1=x1, valid=valid)
    return valid.mean()


def collision_fixture(lib):
    rng = np.random.Generator(np.random.Philox(key=20240603))
    start = np.float32([0.05, 0.05, 0.05])
    goal = np.float32([0.95, 0.95, 0.95])
    obs = W.random_boxes(rng, 20, 0.05, 0.15, start, goal, 0.05)
    n = 3000
    p0 = rng.uniform(0, 1, (n, 3)).astype(np.float32)
    p1 = (p0 + rng.uniform(-0.1, 0.1, (n, 3))).astype(np.float32)
    # segments that end exactly on a face, or lie in a face plane
    for i in range(0, 300):
        b = obs[i % obs.shape[0]]
        d = i % 3
        p1[i] = p0[i]
        p1[i, d] = b[d]  # box edge touches the min face along axis d
        p0[i, (d + 1) % 3] = (b[(d + 1) % 3] + b[(d + 1) % 3 + 3]) / 2
        p0[i, (d + 2) % 3] = (b[(d + 2) % 3] + b[(d + 2) % 3 + 3]) / 2
        p1[i, (d + 1) % 3] = p0[i, (d + 1) % 3]
        p1[i, (d + 2) % 3] = p0[i, (d + 2) % 3]
        if i % 2:
            p1[i, d] = np.nextafter(b[d], np.float32(2.0))  # one ulp inside
    valid = np.zeros(n, np.uint8)
    o = np.ascontiguousarray(obs)
    for i in range(n):
        a = np.ascontiguousarray(p0[i])
        c = np.ascontiguousarray(p1[i])
        valid[i] = lib.ref_motion_valid(fp(a), fp(c), fp(o), o.shape[0])
    np.savez_compressed(OUT / "ref_collision.npz", p0=p0, p1=p1, obstacles=obs, valid=valid)
    return valid.mean()


def region_fixture(libs):
    rng = np.random.Generator(np.random.Philox(key=20240604))
    out = {}
    for name, L, D in (("di", 8, 10), ("quad", 16, 17)):
        n = 3000
        x = np.zeros((n, D), np.float32)
        x[:, :3] = rng.uniform(-0.1, 1.1, (n, 3))
        grid = np.arange(0, L + 1, dtype=np.float32) / np.float32(L)
        for i in range(600):
            x[i, :3] = rng.choice(grid, 3)  # exactly on cell boundaries
        for i in range(600, 700):
            x[i, :3] = rng.choice(np.float32([-5.0, -1e-7, 0.0, 1.0, 1.0000001, 7.0]), 3)
        r = np.zeros(n, np.int32)
        lib = libs[f"graph_{name}"]
        for i in range(n):
            r[i] = lib.ref_get_region(fp(np.ascontiguousarray(x[i])))
        out[f"{name}_x"] = x
        out[f"{name}_r1"] = r
    np.savez_compressed(OUT / "ref_region.npz", **out)


def philox_kat():
    # Published Philox4x32-10 known-answer vectors (Random123 kat_vectors).
    kat = [
        dict(ctr=[0, 0, 0, 0], key=[0, 0], out=[0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
        dict(ctr=[0xFFFFFFFF] * 4, key=[0xFFFFFFFF] * 2, out=[0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
        dict(ctr=[0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], key=[0xA4093822, 0x299F31D0],
             out=[0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
    ]
    (OUT / "philox_kat.json").write_text(json.dumps(kat, indent=1))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="checkout of the reference's sources (read only)")
    args = ap.parse_args()
    libs = load_ref(args.ref)
    assert libs["di"].ref_model() == 1 and libs["quad"].ref_model() == 3
    assert libs["dubins"].ref_model() == 2 and libs["uni"].ref_model() == 0
    print("di valid fraction", di_fixture(libs["di"]))
    print("quad valid fraction", quad_fixture(libs["quad"]))
    print("dubins valid fraction", dubins_fixture(libs["dubins"]))
    print("unicycle valid fraction", unicycle_fixture(libs["uni"]))
    print("collision valid fraction", collision_fixture(libs["di"]))
    region_fixture(libs)
    philox_kat()
    for p in sorted(OUT.glob("*.npz")):
        print(p.name, p.stat().st_size)


if __name__ == "__main__":
    main()
