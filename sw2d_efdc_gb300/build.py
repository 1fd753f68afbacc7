"""Build the SW2D GB300 library in-tree (sw2d_efdc_gb300/_lib/libsw2d.so).

Every CUDA translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``); nvcc cross-compiles without a
GPU.  The FP64 step is compiled with ``--fmad=false`` so that it performs the
same roundings as the CPU oracle.  Translation units compile in parallel.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
LIB = os.path.join(OUT_DIR, "libsw2d.so")
CLI = os.path.join(OUT_DIR, "sw2d_cli")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include"),
          "-I", CSRC]

# translation unit -> extra flags
UNITS = {
    "sw2d_fp64.cu": ["--fmad=false", "-Xptxas", "-v"],
    "sw2d_fp32.cu": ["-Xptxas", "-v"],
    "sw2d_engine.cu": [],
    "sw2d_batch.cu": [],
    "sw2d_api.cu": [],
    "sw2d_noalloc.cu": ["--fmad=false", "-Xptxas", "-v"],
    "sw2d_efdc_io.cu": [],
    "sw2d_case_prep.cu": ["-Xcompiler", "-ffp-contract=off"],
    "sw2d_lake_dev.cu": ["--fmad=false"],
}
HEADERS = ["sw2d_internal.h", "sw2d_math.h", "sw2d_fp32.h", "sw2d_engine.h"]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return p


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(unit: str) -> tuple[str, str]:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(OBJ_DIR, unit.replace(".cu", ".o"))
    deps = [src, os.path.join(ROOT, "include", "sw2d.h"), os.path.join(ROOT, "include", "sw2d_batch.h"),
                  os.path.join(ROOT, "include", "sw2d_noalloc.h"), os.path.join(ROOT, "include", "sw2d_test.h")] + \
        [os.path.join(CSRC, h) for h in HEADERS]
    if not _stale(obj, deps + [__file__]):
        return obj, ""
    cmd = [nvcc()] + ARCH + COMMON + UNITS[unit] + ["-c", src, "-o", obj + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (unit, r.stdout, r.stderr))
    os.replace(obj + ".tmp", obj)
    return obj, r.stderr


def build(verbose: bool = False) -> str:
    os.makedirs(OBJ_DIR, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        results = list(ex.map(_compile, list(UNITS)))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            if log:
                print(log)
    if _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
        os.replace(LIB + ".tmp", LIB)
    build_cli()
    return LIB


def build_cli() -> str:
    """The case driver (csrc/sw2d_cli.cpp): host C++ linked against
    libsw2d.so beside it (rpath $ORIGIN) and the CUDA runtime (the device
    copies of the lake-edge pre-pass)."""
    src = os.path.join(CSRC, "sw2d_cli.cpp")
    deps = [src, LIB, os.path.join(ROOT, "include", "sw2d.h"), __file__]
    if _stale(CLI, deps):
        cxx = shutil.which("g++") or "g++"
        cuda = os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))
        cmd = [cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-Wall", "-I", os.path.join(ROOT, "include"),
               "-I", os.path.join(cuda, "include"), src, "-o", CLI + ".tmp", "-L", OUT_DIR, "-lsw2d",
               "-L", os.path.join(cuda, "lib64"), "-lcudart", "-Wl,-rpath,$ORIGIN", "-pthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("sw2d_cli build failed:\n%s\n%s" % (r.stdout, r.stderr))
        os.replace(CLI + ".tmp", CLI)
    return CLI


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
