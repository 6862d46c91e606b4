"""Builds libkgmt.so (the CUDA planner behind include/kgmt.h) in-tree.

    python -m kgmt_gb300.build [--force] [--verbose]

Each translation unit is compiled for sm_103a in parallel, then linked into
``kgmt_gb300/_lib/libkgmt.so``.  ``-fmad=false`` keeps every float multiply
and add separately rounded (the planner's integer results -- region ids,
verdicts, parents -- are defined by that rounding); host code is compiled
with ``-ffp-contract=off`` for the same reason.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "_lib"
BUILD_DIR = PKG / "_build"
LIB = OUT_DIR / "libkgmt.so"
# the same sources with KGMT_CHECK_BOUNDS: the kernels test their scattered
# indices and report a failure as KGMT_ERR_INTERNAL (a sanitizer stand-in)
LIB_CHECKED = OUT_DIR / "libkgmt_checked.so"
SOURCES = ["kgmt_kernels.cu", "kgmt_engine.cu", "kgmt_abi.cu", "kgmt_noalloc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found")
    return cand


def common_flags() -> list[str]:
    return ["-std=c++17", "-O3", "-lineinfo", "-fmad=false", *ARCH, "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden",
            f"-I{ROOT / 'include'}", "--expt-relaxed-constexpr"]


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> Path:
    BUILD_DIR.mkdir(exist_ok=True)
    OUT_DIR.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "kgmt.h"]
    objs, objs_checked = [], []
    jobs = []
    for src in SOURCES:
        s = CSRC / src
        o = BUILD_DIR / (s.stem + ".o")
        oc = BUILD_DIR / (s.stem + "_checked.o")
        objs.append(o)
        objs_checked.append(oc)
        if force or _stale(o, [s, *headers]):
            cmd = [nvcc(), *common_flags(), "-c", str(s), "-o", str(o)]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
        if force or _stale(oc, [s, *headers]):
            jobs.append([nvcc(), *common_flags(), "-DKGMT_CHECK_BOUNDS", "-c", str(s), "-o", str(oc)])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
        for cmd, r in zip(jobs, results):
            if verbose or ptxas_info:
                print(" ".join(cmd))
                print(r.stdout, r.stderr)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    for lib, os_ in ((LIB, objs), (LIB_CHECKED, objs_checked)):
        if force or jobs or _stale(lib, os_):
            tmp = lib.with_suffix(".so.tmp")
            cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, os_), "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
            os.replace(tmp, lib)
    build_cli(force=force)
    return LIB


CLI_SRC = PKG / "cli" / "kgmt_plan.cpp"
CLI = OUT_DIR / "kgmt_plan"


def build_cli(force: bool = False) -> Path:
    """The C++ command-line driver (kgmt_gb300/cli/kgmt_plan.cpp), linked
    against libkgmt.so and the CUDA runtime."""
    deps = [CLI_SRC, ROOT / "include" / "kgmt.hpp", ROOT / "include" / "kgmt.h", LIB]
    if not force and not _stale(CLI, deps):
        return CLI
    cuda = Path(nvcc()).resolve().parent.parent
    cmd = ["g++", "-O2", "-std=c++17", f"-I{ROOT / 'include'}", f"-I{cuda / 'include'}", str(CLI_SRC), "-o", str(CLI),
           f"-L{OUT_DIR}", "-lkgmt", f"-L{cuda / 'lib64'}", "-lcudart", "-Wl,-rpath,$ORIGIN", f"-Wl,-rpath,{cuda / 'lib64'}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"CLI build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return CLI


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--ptxas-info", action="store_true", help="print registers / spills / shared memory per kernel")
    a = ap.parse_args(argv)
    print(build(force=a.force or a.ptxas_info, verbose=a.verbose, ptxas_info=a.ptxas_info))
    return 0


if __name__ == "__main__":
    sys.exit(main())
