"""ctypes binding of libkgmt.so (include/kgmt.h).

There is no fallback: if the library is missing or no CUDA device is present,
calls fail with an exception carrying ``kgmt_last_error()``.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

from .config import PlannerConfig

PKG = Path(__file__).resolve().parent
# KGMT_LIBRARY selects another build of the same ABI (e.g. the bounds-checked
# _lib/libkgmt_checked.so)
LIB_PATH = Path(os.environ["KGMT_LIBRARY"]) if os.environ.get("KGMT_LIBRARY") else PKG / "_lib" / "libkgmt.so"

KGMT_OK = 0
STATUS_NAMES = {0: "OK", 1: "INVALID_ARG", 2: "OOM", 3: "CAPACITY", 4: "TIMEOUT", 5: "CUDA", 6: "NO_DEVICE", 7: "NOT_READY",
                8: "INTERNAL"}
MAX_SAMPLE_DIM = 17


class KgmtError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"kgmt error {STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


class KgmtConfig(C.Structure):
    _fields_ = [
        ("model", C.c_int32), ("di_rule", C.c_int32), ("tree_capacity", C.c_uint32), ("samples_per_node", C.c_uint32),
        ("max_iterations", C.c_uint32), ("min_steps", C.c_uint32), ("max_steps", C.c_uint32), ("step_size", C.c_float),
        ("goal_radius", C.c_float), ("epsilon", C.c_float), ("ws_min", C.c_float), ("ws_max", C.c_float),
        ("coarse_len", C.c_uint32), ("fine_len", C.c_uint32), ("v_min", C.c_float), ("v_max", C.c_float),
        ("u_min", C.c_float * 4), ("u_max", C.c_float * 4), ("nu", C.c_float), ("mu", C.c_float), ("ix", C.c_float),
        ("iy", C.c_float), ("iz", C.c_float), ("gravity", C.c_float), ("mass_inv", C.c_float), ("seed", C.c_uint64),
        ("pitch_min", C.c_float), ("pitch_max", C.c_float), ("wheelbase", C.c_float), ("reserved", C.c_uint32),
    ]


class KgmtResult(C.Structure):
    _fields_ = [("status", C.c_int32), ("iterations", C.c_uint32), ("tree_size", C.c_uint32), ("goal_index", C.c_int32),
                ("path_len", C.c_uint32), ("samples_drawn", C.c_uint32), ("solve_ms", C.c_float), ("latency_ms", C.c_float),
                ("ticket", C.c_uint64), ("goal_cost", C.c_float), ("reserved", C.c_uint32)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class KgmtBatchOptions(C.Structure):
    _fields_ = [("max_queries", C.c_uint32), ("iters_per_graph", C.c_uint32), ("propagate_block", C.c_uint32),
                ("use_graph", C.c_uint32), ("profile_kernels", C.c_uint32)]


class KgmtBatchStats(C.Structure):
    _fields_ = [("kernel_launches", C.c_uint64), ("steps_executed", C.c_uint64), ("obstacle_tests", C.c_uint64),
                ("samples", C.c_uint64), ("fp32_ops", C.c_uint64), ("iterations_launched", C.c_uint32),
                ("launches_propagate", C.c_uint32), ("launches_tail", C.c_uint32), ("launches_append", C.c_uint32),
                ("ms_propagate", C.c_float), ("ms_tail", C.c_float), ("ms_append", C.c_float),
                ("iterations_tail", C.c_uint32), ("reserved", C.c_uint32), ("fp32_ops_tail", C.c_uint64),
                ("samples_tail", C.c_uint64)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class KgmtAutotuneResult(C.Structure):
    _fields_ = [("propagate_block", C.c_uint32), ("samples_per_node", C.c_uint32), ("queries_per_s", C.c_float),
                ("success_rate", C.c_float), ("base_queries_per_s", C.c_float), ("base_success_rate", C.c_float)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class KgmtIteration(C.Structure):
    """kgmt_iteration: what one iteration of a traced plan left behind."""
    _fields_ = [("itr", C.c_uint32), ("tree_size", C.c_uint32), ("frontier_size", C.c_uint32), ("expanded", C.c_uint32),
                ("next_frontier_size", C.c_uint32), ("goal_index", C.c_int32), ("path_len", C.c_uint32),
                ("capacity", C.c_uint32), ("sample_dim", C.c_uint32), ("regions", C.c_uint32),
                ("samples", C.POINTER(C.c_float)), ("parents", C.POINTER(C.c_int32)), ("counter", C.POINTER(C.c_int32)),
                ("valid", C.POINTER(C.c_int32)), ("score", C.POINTER(C.c_float)), ("frontier", C.POINTER(C.c_uint8)),
                ("repeat", C.POINTER(C.c_uint32)), ("path", C.POINTER(C.c_float))]


ITERATION_HOOK = C.CFUNCTYPE(None, C.POINTER(KgmtIteration), C.c_void_p)


class KgmtServerOptions(C.Structure):
    _fields_ = [("max_slots", C.c_uint32), ("memory_budget", C.c_uint64), ("iters_per_step", C.c_uint32),
                ("propagate_block", C.c_uint32)]


def to_c(cfg: PlannerConfig) -> KgmtConfig:
    k = KgmtConfig()
    for name, _ in KgmtConfig._fields_:
        v = getattr(cfg, name)
        if name in ("u_min", "u_max"):
            setattr(k, name, (C.c_float * 4)(*[float(x) for x in v]))
        else:
            setattr(k, name, v)
    return k


# every function the header declares, with its signature
_vp = C.c_void_p
_u32, _i32, _f = C.c_uint32, C.c_int32, C.c_float
_fp, _u8p, _i32p, _u32p = C.POINTER(C.c_float), C.POINTER(C.c_uint8), C.POINTER(C.c_int32), C.POINTER(C.c_uint32)
_cfgp, _resp = C.POINTER(KgmtConfig), C.POINTER(KgmtResult)
SIGNATURES = {
    "kgmt_version": (C.c_char_p, []),
    "kgmt_last_error": (C.c_char_p, []),
    "kgmt_config_default": (_i32, [_i32, _cfgp]),
    "kgmt_config_validate": (_i32, [_cfgp]),
    "kgmt_query_bytes": (C.c_size_t, [_cfgp, _u32]),
    "kgmt_sample_dim": (_i32, [_i32]),
    "kgmt_create": (_i32, [_cfgp, _vp, C.POINTER(_vp)]),
    "kgmt_destroy": (None, [_vp]),
    "kgmt_plan": (_i32, [_vp, _vp, _vp, _vp, _u32]),
    "kgmt_get_result": (_i32, [_vp, _resp]),
    "kgmt_copy_tree": (_i32, [_vp, _vp, _vp, _vp, _u32]),
    "kgmt_copy_path": (_i32, [_vp, _vp, _u32, _u32p]),
    "kgmt_device_tree": (_i32, [_vp, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp)]),
    "kgmt_plan_traced": (_i32, [_vp, _vp, _vp, _vp, _u32, ITERATION_HOOK, _vp]),
    "kgmt_batch_create": (_i32, [C.POINTER(KgmtBatchOptions), _vp, C.POINTER(_vp)]),
    "kgmt_batch_destroy": (None, [_vp]),
    "kgmt_plan_batch": (_i32, [_vp, _u32, _cfgp, _vp, _vp, _vp, _vp, _vp, _resp]),
    "kgmt_plan_batch_device": (_i32, [_vp, _u32, _cfgp, _vp, _vp, _vp, _vp, _vp, _resp]),
    "kgmt_batch_get_stats": (_i32, [_vp, C.POINTER(KgmtBatchStats)]),
    "kgmt_batch_copy_tree": (_i32, [_vp, _u32, _vp, _vp, _vp, _u32]),
    "kgmt_batch_copy_path": (_i32, [_vp, _u32, _vp, _u32, _u32p]),
    "kgmt_batch_autotune": (_i32, [_vp, _u32, _cfgp, _vp, _vp, _vp, _vp, _vp, _u32p]),
    "kgmt_batch_autotune_full": (_i32, [_vp, _u32, _cfgp, _vp, _vp, _vp, _vp, _vp, C.POINTER(KgmtAutotuneResult)]),
    "kgmt_server_create": (_i32, [C.POINTER(KgmtServerOptions), _vp, C.POINTER(_vp)]),
    "kgmt_server_destroy": (None, [_vp]),
    "kgmt_server_submit": (_i32, [_vp, _cfgp, _vp, _vp, _vp, _u32, C.POINTER(C.c_uint64)]),
    "kgmt_server_step": (_i32, [_vp, _u32p, _u32p]),
    "kgmt_server_poll": (_i32, [_vp, _resp, _u32, _u32p]),
    "kgmt_server_cancel": (_i32, [_vp, C.c_uint64]),
    "kgmt_propagate_samples": (_i32, [_cfgp, _vp, _vp, _vp, _u32, _u32, _vp, _vp, _vp, _vp, _vp]),
    "kgmt_plan_noalloc": (_i32, [_cfgp, _vp, _vp, _vp, _u32, _vp, _vp, _vp, _u32, _vp, _u32, _resp, _vp]),
    "kgmt_selftest_bounded_wait": (_i32, [_u32, _u32p]),
}

_lib = None


def load(build_if_missing: bool = True):
    """Loads libkgmt.so (building it in-tree when missing and nvcc exists)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        if not build_if_missing:
            raise KgmtError(8, f"{LIB_PATH} is missing; run python -m kgmt_gb300.build")
        from .build import build
        build()
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(code: int) -> None:
    if code != KGMT_OK:
        raise KgmtError(code, load().kgmt_last_error().decode())


def ptr(x) -> int | None:
    """Raw address of a numpy array, torch tensor or int (None stays NULL)."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    return x.ctypes.data
