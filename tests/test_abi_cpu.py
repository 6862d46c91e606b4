"""Host-side checks of the C ABI that need no GPU: the library loads, exports
every function include/kgmt.h declares, the ctypes mirrors have the C layout,
config validation and sizing work, and planning calls fail loudly (no CPU
fallback) when no device is present."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from kgmt_gb300 import _abi
from kgmt_gb300.build import build
from kgmt_gb300.config import PlannerConfig, double_integrator_single, dubins_airplane, quadrotor_large, unicycle

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "kgmt.h"


@pytest.fixture(scope="module")
def lib():
    build()
    return _abi.load()


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"KGMT_API\s+[\w\s\*]*?\b(kgmt_\w+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert len(names) >= 25
    assert {"kgmt_create", "kgmt_plan", "kgmt_plan_batch", "kgmt_server_step", "kgmt_propagate_samples"} <= set(names)


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", str(_abi.LIB_PATH)], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (kgmt_\w+)", out))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing
    # and the binding knows each of them
    assert set(declared_functions()) == set(_abi.SIGNATURES)


def test_struct_layouts_match_c(tmp_path):
    src = tmp_path / "sizes.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "kgmt.h"\nint main(void){printf("%zu %zu %zu %zu %zu %zu %zu\\n",'
                   "sizeof(kgmt_config), sizeof(kgmt_result), sizeof(kgmt_batch_options), sizeof(kgmt_batch_stats),"
                   "sizeof(kgmt_server_options), offsetof(kgmt_config, seed), offsetof(kgmt_result, ticket));return 0;}\n")
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", f"-I{ROOT / 'include'}", str(src), "-o", str(exe)], check=True)
    got = list(map(int, subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()))
    want = [C.sizeof(_abi.KgmtConfig), C.sizeof(_abi.KgmtResult), C.sizeof(_abi.KgmtBatchOptions),
            C.sizeof(_abi.KgmtBatchStats), C.sizeof(_abi.KgmtServerOptions), _abi.KgmtConfig.seed.offset,
            _abi.KgmtResult.ticket.offset]
    assert got == want


def test_cpp_wrapper_and_cli_compile(tmp_path, lib):
    # the header-only wrapper compiles as plain C++ and the CLI was linked
    src = tmp_path / "w.cpp"
    src.write_text('#include "kgmt.hpp"\nint main(){ kgmt_config c = kgmt::default_config(); return c.model == 1 ? 0 : 1; }\n')
    subprocess.run(["g++", "-std=c++17", f"-I{ROOT / 'include'}", str(src), "-o", str(tmp_path / "w"),
                    f"-L{_abi.LIB_PATH.parent}", "-lkgmt", f"-Wl,-rpath,{_abi.LIB_PATH.parent}"], check=True)
    r = subprocess.run([str(tmp_path / "w")])
    assert r.returncode == 0
    assert (_abi.LIB_PATH.parent / "kgmt_plan").exists()


def test_obstacle_csv_reader_throws_instead_of_exiting(tmp_path, lib):
    """kgmt::read_obstacles_csv replaces readObstaclesFromCSV
    (helper.cu:13-39), which calls exit(1): a missing file, a token that is
    not a number and a partial box row each raise an exception the caller can
    handle; well-formed files give 2W floats per box."""
    (tmp_path / "ok3.csv").write_text("0.1, 0.2, 0.3, 0.4, 0.5, 0.6\n0.5,0.5,0.5,0.7,0.7,0.7\n")
    (tmp_path / "ok2.csv").write_text("0.1,0.2,0.3,0.4\n")
    (tmp_path / "text.csv").write_text("0.1,0.2,abc,0.4,0.5,0.6\n")
    (tmp_path / "short.csv").write_text("0.1,0.2,0.3,0.4,0.5,0.6\n0.1,0.2,0.3\n")
    src = tmp_path / "csv.cpp"
    src.write_text(r"""#include "kgmt.hpp"
#include <cstdio>
static int kind(const char* path, int w) {
    try { return (int)kgmt::read_obstacles_csv(path, w).size(); }
    catch(const std::invalid_argument&) { return -2; }
    catch(const std::runtime_error&) { return -1; }
}
int main(int, char** argv) {
    std::string d = argv[1];
    std::printf("%d %d %d %d %d\n", kind((d + "/ok3.csv").c_str(), 3), kind((d + "/ok2.csv").c_str(), 2),
                kind((d + "/missing.csv").c_str(), 3), kind((d + "/text.csv").c_str(), 3), kind((d + "/short.csv").c_str(), 3));
    return 0;
}
""")
    subprocess.run(["g++", "-std=c++17", f"-I{ROOT / 'include'}", str(src), "-o", str(tmp_path / "csv"),
                    f"-L{_abi.LIB_PATH.parent}", "-lkgmt", f"-Wl,-rpath,{_abi.LIB_PATH.parent}"], check=True)
    r = subprocess.run([str(tmp_path / "csv"), str(tmp_path)], capture_output=True, text=True, check=True)
    assert r.stdout.split() == ["12", "4", "-1", "-2", "-1"]


def test_config_defaults_and_validation(lib):
    c = _abi.KgmtConfig()
    assert lib.kgmt_config_default(1, C.byref(c)) == 0
    ours = _abi.to_c(double_integrator_single())
    for name, _ in _abi.KgmtConfig._fields_:
        if name in ("u_min", "u_max"):
            assert list(getattr(c, name))[:3] == list(getattr(ours, name))[:3]
        elif name != "seed":
            assert getattr(c, name) == pytest.approx(getattr(ours, name)), name
    assert lib.kgmt_config_default(3, C.byref(c)) == 0
    q = _abi.to_c(quadrotor_large())
    assert (c.coarse_len, c.fine_len, c.tree_capacity, c.min_steps, c.max_steps) == (16, 4, 2_000_000, 3, 15)
    assert c.gravity == pytest.approx(q.gravity)
    assert lib.kgmt_config_default(7, C.byref(c)) == 1
    # the Dubins airplane and unicycle defaults are the Python presets
    for model, preset in ((2, dubins_airplane()), (0, unicycle())):
        assert lib.kgmt_config_default(model, C.byref(c)) == 0
        ours = _abi.to_c(preset)
        for name, _ in _abi.KgmtConfig._fields_:
            if name in ("u_min", "u_max"):
                assert list(getattr(c, name))[:3] == pytest.approx(list(getattr(ours, name))[:3]), (model, name)
            elif name not in ("seed", "nu", "mu", "ix", "iy", "iz", "gravity", "mass_inv", "di_rule"):
                assert getattr(c, name) == pytest.approx(getattr(ours, name)), (model, name)
        assert lib.kgmt_config_validate(C.byref(c)) == 0
        assert lib.kgmt_sample_dim(model) == preset.sample_dim
    bad = [dict(model=4), dict(model=-1), dict(tree_capacity=1), dict(samples_per_node=0), dict(min_steps=0),
           dict(min_steps=7, max_steps=6), dict(fine_len=5), dict(ws_max=0.0), dict(step_size=0.0), dict(coarse_len=0),
           dict(di_rule=3), dict(model=0, fine_len=9), dict(model=0, wheelbase=0.0), dict(model=2, pitch_min=1.0, pitch_max=0.0)]
    for kw in bad:
        k = _abi.to_c(PlannerConfig().replace(**kw))
        assert lib.kgmt_config_validate(C.byref(k)) == 1, kw
        assert lib.kgmt_last_error().decode().startswith("invalid config")
    assert lib.kgmt_config_validate(C.byref(_abi.to_c(PlannerConfig()))) == 0


def test_query_bytes(lib):
    k = _abi.to_c(double_integrator_single())
    b0 = lib.kgmt_query_bytes(C.byref(k), 0)
    b10 = lib.kgmt_query_bytes(C.byref(k), 10)
    # tree + unexplored rows dominate: capacity x (2 x 40 B + 6 x 4 B + 1 B)
    assert 100_000 * 105 <= b0 <= 100_000 * 125
    assert b10 > b0
    assert lib.kgmt_sample_dim(1) == 10 and lib.kgmt_sample_dim(3) == 17
    assert lib.kgmt_sample_dim(0) == 7 and lib.kgmt_sample_dim(2) == 10 and lib.kgmt_sample_dim(4) == -1
    # the unicycle's 7-float rows (T = 100k, as the double integrator's 10)
    u = _abi.to_c(unicycle())
    bu = lib.kgmt_query_bytes(C.byref(u), 0)
    assert 100_000 * 80 <= bu < b0 - 100_000 * 2 * 12 + 1


def test_no_device_fails_loudly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    k = _abi.to_c(double_integrator_single())
    h = C.c_void_p()
    assert lib.kgmt_create(C.byref(k), None, C.byref(h)) == 6  # KGMT_ERR_NO_DEVICE
    assert "CUDA" in lib.kgmt_last_error().decode() or "device" in lib.kgmt_last_error().decode()
    with pytest.raises(_abi.KgmtError):
        from kgmt_gb300.planner import KGMT
        KGMT(double_integrator_single())
    bits = C.c_uint32(0)
    assert lib.kgmt_selftest_bounded_wait(1000, C.byref(bits)) == 6


def test_null_arguments_rejected(lib):
    assert lib.kgmt_create(None, None, None) == 1
    assert lib.kgmt_plan(None, None, None, None, 0) == 1
    assert lib.kgmt_plan_batch(None, 0, None, None, None, None, None, None, None) == 1
    assert lib.kgmt_server_poll(None, None, 0, None) == 1
    assert lib.kgmt_server_cancel(None, 1) == 1
    st = _abi.KgmtBatchStats()
    assert lib.kgmt_batch_get_stats(None, C.byref(st)) == 1
    bits = C.c_uint32(0)
    assert lib.kgmt_selftest_bounded_wait(1000, None) == 1
    assert lib.kgmt_selftest_bounded_wait(0, C.byref(bits)) == 1
