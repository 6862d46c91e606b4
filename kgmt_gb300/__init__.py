"""GB300-native KGMT planning loop: CUDA kernels behind a C ABI
(include/kgmt.h), with Python and C++ host APIs that keep the reference
planner's surface."""
from .config import (DI_RULE_REFERENCE, DI_RULE_RK4, MODEL_DOUBLE_INTEGRATOR, MODEL_DUBINS_AIRPLANE, MODEL_QUADROTOR,
                     MODEL_UNICYCLE, PlannerConfig, double_integrator_batched, double_integrator_single, dubins_airplane,
                     quadrotor_large, sample_dim, unicycle)

__all__ = ["PlannerConfig", "MODEL_UNICYCLE", "MODEL_DOUBLE_INTEGRATOR", "MODEL_DUBINS_AIRPLANE", "MODEL_QUADROTOR",
           "DI_RULE_RK4", "DI_RULE_REFERENCE", "double_integrator_single", "quadrotor_large", "double_integrator_batched",
           "dubins_airplane", "unicycle", "sample_dim", "KGMT", "BatchPlanner", "Server", "propagate_samples"]


def __getattr__(name):
    if name in ("KGMT", "BatchPlanner", "Server", "propagate_samples"):
        from . import planner
        return getattr(planner, name)
    raise AttributeError(name)
