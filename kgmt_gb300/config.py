"""Runtime planner configuration.

The reference configures everything at compile time through the macros of
``include/config/config.h`` (model at config.h:209, tree capacity :211, step
size :213, steps :214, goal threshold :216, grid lengths :239-245, epsilon
:262, quad constants :283-307).  Here the same quantities are fields of one
runtime struct, mirrored field for field by ``kgmt_config`` in
``include/kgmt.h``.

Grids are workspace-only: ``coarse_len``^W coarse regions, each split into
``fine_len``^W fine cells (at most 64 fine cells per region), W = 3, or 2 for
the planar unicycle.
"""
from __future__ import annotations

import dataclasses
import math
from dataclasses import dataclass, field

MODEL_UNICYCLE = 0  # reference MODEL 0 (planar)
MODEL_DOUBLE_INTEGRATOR = 1  # reference MODEL 1
MODEL_DUBINS_AIRPLANE = 2  # reference MODEL 2
MODEL_QUADROTOR = 3  # reference MODEL 3
MODELS = (MODEL_UNICYCLE, MODEL_DOUBLE_INTEGRATOR, MODEL_DUBINS_AIRPLANE, MODEL_QUADROTOR)

DI_RULE_RK4 = 0
DI_RULE_REFERENCE = 1  # statePropagator.cu:97-99 position formula

STATUS_RUNNING = 0
STATUS_SUCCESS = 1
STATUS_ITER_LIMIT = 2
STATUS_CAPACITY = 3
STATUS_CANCELLED = 4
STATUS_NAMES = {0: "running", 1: "success", 2: "iteration-limit", 3: "capacity", 4: "cancelled"}

MAX_SAMPLE_DIM = 17


def sample_dim(model: int) -> int:
    """SAMPLE_DIM of config.h: state + control + duration (unicycle 7, double
    integrator 10, Dubins airplane 10, quadrotor 17)."""
    return {MODEL_QUADROTOR: 17, MODEL_UNICYCLE: 7}.get(model, 10)


def state_dim(model: int) -> int:
    return {MODEL_QUADROTOR: 12, MODEL_UNICYCLE: 4}.get(model, 6)


def ws_dims(model: int) -> int:
    """W_DIM: 2 for the planar unicycle, else 3."""
    return 2 if model == MODEL_UNICYCLE else 3


@dataclass
class PlannerConfig:
    model: int = MODEL_DOUBLE_INTEGRATOR
    di_rule: int = DI_RULE_RK4
    tree_capacity: int = 100_000
    samples_per_node: int = 4
    max_iterations: int = 200
    min_steps: int = 1
    max_steps: int = 6
    step_size: float = 0.05
    goal_radius: float = 0.05
    epsilon: float = 1e-2
    ws_min: float = 0.0
    ws_max: float = 1.0
    coarse_len: int = 8
    fine_len: int = 2
    v_min: float = -0.3
    v_max: float = 0.3
    u_min: tuple = (-1.0, -1.0, -1.0, 0.0)
    u_max: tuple = (1.0, 1.0, 1.0, 0.0)
    nu: float = 10e-3
    mu: float = 2e-6
    ix: float = 1.0
    iy: float = 1.0
    iz: float = 2.0
    gravity: float = -9.81
    mass_inv: float = 1.0
    seed: int = 0
    pitch_min: float = -math.pi / 3  # Dubins airplane
    pitch_max: float = math.pi / 3
    wheelbase: float = 1.0  # unicycle (UNI_LENGTH)
    reserved: int = 0

    @property
    def sample_dim(self) -> int:
        return sample_dim(self.model)

    @property
    def ws_dims(self) -> int:
        return ws_dims(self.model)

    @property
    def regions(self) -> int:
        return self.coarse_len ** self.ws_dims

    @property
    def fine_per_region(self) -> int:
        return self.fine_len ** self.ws_dims

    def replace(self, **kw) -> "PlannerConfig":
        return dataclasses.replace(self, **kw)

    def validate(self) -> None:
        if self.model not in MODELS:
            raise ValueError(f"unknown model {self.model}")
        if self.tree_capacity < 2:
            raise ValueError("tree_capacity must be >= 2")
        if self.samples_per_node < 1:
            raise ValueError("samples_per_node must be >= 1")
        if not 1 <= self.min_steps <= self.max_steps:
            raise ValueError("need 1 <= min_steps <= max_steps")
        if self.fine_len ** self.ws_dims > 64 or self.fine_len < 1 or self.coarse_len < 1:
            raise ValueError("grid: coarse_len >= 1 and 1 <= fine_len^W <= 64")


def double_integrator_single(seed: int = 1) -> PlannerConfig:
    """3-D double integrator, unit cube, 8^3/2^3 grid, T=100k, S=4, 200 iters.

    dt = 0.05 and k = 1..6 steps give durations 0.05..0.30 s; |v| <= 0.3 per
    axis, accelerations uniform in [-1, 1]^3, goal radius 0.05.
    """
    return PlannerConfig(seed=seed)


def quadrotor_large(seed: int = 1) -> PlannerConfig:
    """12-D quadrotor, unit cube, 16^3/4^3 grid, T=2M, S=8, dt=0.02.

    k = 3..15 steps gives durations 0.06..0.30 s (0.05 is not a multiple of
    dt).  The reference's quad constants (config.h:283-307) are for a 100-unit
    workspace; lengths, velocities, gravity and thrust are scaled by 1/100,
    angles, torques and inertias are kept.
    """
    return PlannerConfig(
        model=MODEL_QUADROTOR,
        tree_capacity=2_000_000,
        samples_per_node=8,
        max_iterations=200,
        min_steps=3,
        max_steps=15,
        step_size=0.02,
        goal_radius=0.05,
        coarse_len=16,
        fine_len=4,
        v_min=-0.3,
        v_max=0.3,
        u_min=(0.0, -math.pi, -math.pi, -math.pi),
        u_max=(0.3, math.pi, math.pi, math.pi),
        gravity=-0.0981,
        seed=seed,
    )


def double_integrator_batched(seed: int = 1) -> PlannerConfig:
    """Per-query config of the 256-query homogeneous batch (T=50k)."""
    return PlannerConfig(tree_capacity=50_000, seed=seed)


def dubins_airplane(seed: int = 1) -> PlannerConfig:
    """Dubins airplane with the constants of the reference's Dubins block of
    config.h (MODEL 2): dt 0.1, 1..10 steps, |v| in [0, 0.3], a in [-0.3,
    0.3], yaw and pitch rates in [-pi/4, pi/4], pitch in [-pi/3, pi/3],
    T=200k, 300 iterations; the grid is workspace-only (8^3/2^3)."""
    q = math.pi / 4
    return PlannerConfig(model=MODEL_DUBINS_AIRPLANE, tree_capacity=200_000, samples_per_node=4, max_iterations=300,
                         min_steps=1, max_steps=10, step_size=0.1, coarse_len=8, fine_len=2, v_min=0.0, v_max=0.3,
                         u_min=(-0.3, -q, -q, 0.0), u_max=(0.3, q, q, 0.0), seed=seed)


def unicycle(seed: int = 1) -> PlannerConfig:
    """Planar unicycle with the reference's UNI_* constants (config.h MODEL 0
    block): steering in [-pi/2, pi/2], dt draw in [0.1, 2.0], length 1,
    a in [-0.2, 0.2]; dt 0.1 and 1..10 steps, unit square, 8^2/4^2 grid,
    T=100k."""
    return PlannerConfig(model=MODEL_UNICYCLE, tree_capacity=100_000, samples_per_node=4, max_iterations=200,
                         min_steps=1, max_steps=10, step_size=0.1, coarse_len=8, fine_len=4,
                         u_min=(-0.2, -math.pi / 2, 0.1, 0.0), u_max=(0.2, math.pi / 2, 2.0, 0.0), wheelbase=1.0,
                         seed=seed)
