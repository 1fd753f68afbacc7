"""Build recipe for the test oracle (test infrastructure only).

Two products, both outside the shipped library:

* ``oracle/_build/libsw2d_oracle.so`` -- the CPU restatement of the SW2D
  explicit step (``sw2d_oracle.c``), plain C, compiled with
  ``-ffp-contract=off`` so that every floating-point operation is the single
  IEEE operation the source spells out, on x86 and on Arm alike.
* ``oracle/_ref/libsw2dref.so`` -- the reference's own kernels and host
  helpers, compiled unmodified on the CPU.  The range from ``init_inf`` up to
  (not including) ``make_gefdc_inputs`` of ``SW2D-EFDC.cu`` is copied at build
  time into ``oracle/_ref/ref_kernels.inc`` (git-ignored, never committed)
  and compiled behind ``ref_shim.h`` with ``ref_driver.cpp``.  This needs the
  reference checkout; where it is absent, a previously extracted
  ``ref_kernels.inc`` is reused if present.
* ``oracle/_ref/libsw2dref_gpu.so`` -- the same extracted kernels compiled
  by nvcc for sm_103a and driven by ``ref_gpu_driver.cu`` with the
  reference's own launch configuration: the "reference GPU" timing line.

Run as ``python oracle/build.py`` or call :func:`build_all`.
"""
from __future__ import annotations

import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
# The reference checkout: $SW2D_REFERENCE_ROOT, else a checkout named
# "reference" beside this repository (../reference from the repo root).
REFERENCE_ROOT = os.environ.get("SW2D_REFERENCE_ROOT",
                                os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))
REFERENCE_CU = os.path.join(REFERENCE_ROOT, "SW2D-EFDC.cu")

ORACLE_LIB = os.path.join(BUILD_DIR, "libsw2d_oracle.so")
REF_LIB = os.path.join(REF_DIR, "libsw2dref.so")
REF_GPU_LIB = os.path.join(REF_DIR, "libsw2dref_gpu.so")
REF_INC = os.path.join(REF_DIR, "ref_kernels.inc")

# First and one-past-last lines of the extracted range, matched by prefix.
_REF_BEGIN = "__global__ void init_inf("
_REF_END = "__host__ void make_gefdc_inputs("


def _fma_flags() -> list[str]:
    """Hardware FMA for explicit fma() calls only (contraction stays off)."""
    if platform.machine() in ("x86_64", "AMD64"):
        try:
            with open("/proc/cpuinfo") as f:
                if " fma " in f.read():
                    return ["-mfma"]
        except OSError:
            pass
    return []


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))


def _newer(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources if os.path.exists(s))


def build_oracle(force: bool = False) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    srcs = [os.path.join(HERE, "sw2d_oracle.c"), os.path.join(HERE, "sw2d_oracle.h")]
    math_h = os.path.join(HERE, "..", "sw2d_efdc_gb300", "csrc", "sw2d_math.h")
    if not force and _newer(ORACLE_LIB, srcs + [math_h]):
        return ORACLE_LIB
    cmd = ["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-fopenmp", "-I", os.path.join(HERE, "..", "sw2d_efdc_gb300", "csrc")]
    cmd += _fma_flags()
    cmd += [srcs[0], "-o", ORACLE_LIB + ".tmp", "-lm"]
    _run(cmd)
    os.replace(ORACLE_LIB + ".tmp", ORACLE_LIB)
    return ORACLE_LIB


def extract_reference() -> bool:
    """Copy the kernel range of the reference source into oracle/_ref/."""
    if not os.path.exists(REFERENCE_CU):
        return os.path.exists(REF_INC)
    os.makedirs(REF_DIR, exist_ok=True)
    with open(REFERENCE_CU, "r", encoding="latin-1") as f:
        lines = f.readlines()
    begin = next(i for i, l in enumerate(lines) if l.startswith(_REF_BEGIN))
    end = next(i for i, l in enumerate(lines) if l.startswith(_REF_END))
    text = "".join(lines[begin:end])
    if os.path.exists(REF_INC):
        with open(REF_INC, "r", encoding="latin-1") as f:
            if f.read() == text:
                return True
    with open(REF_INC, "w", encoding="latin-1") as f:
        f.write(text)
    return True


def build_reference(force: bool = False) -> str | None:
    if not extract_reference():
        return None
    srcs = [os.path.join(HERE, "ref_driver.cpp"), os.path.join(HERE, "ref_shim.h"), REF_INC]
    if not force and _newer(REF_LIB, srcs):
        return REF_LIB
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-fopenmp", "-w", "-I", HERE, "-I", REF_DIR, srcs[0], "-o", REF_LIB + ".tmp"]
    _run(cmd)
    os.replace(REF_LIB + ".tmp", REF_LIB)
    return REF_LIB


def build_reference_gpu(force: bool = False) -> str | None:
    """The same extracted kernels compiled by nvcc for sm_103a behind
    ref_gpu_driver.cu (the reference's launch configuration and host loop):
    the "reference GPU" timing line."""
    if not extract_reference():
        return None
    srcs = [os.path.join(HERE, "ref_gpu_driver.cu"), os.path.join(HERE, "ref_case.h"), REF_INC]
    if not force and _newer(REF_GPU_LIB, srcs):
        return REF_GPU_LIB
    nvcc = os.environ.get("NVCC", "nvcc")
    if not os.path.exists(nvcc) and subprocess.run(["which", nvcc], capture_output=True).returncode != 0:
        nvcc = "/usr/local/cuda/bin/nvcc"
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
           "-shared", "-w", "-I", HERE, "-I", REF_DIR, srcs[0], "-o", REF_GPU_LIB + ".tmp"]
    _run(cmd)
    os.replace(REF_GPU_LIB + ".tmp", REF_GPU_LIB)
    return REF_GPU_LIB


def build_all(force: bool = False) -> dict:
    out = {"oracle": build_oracle(force)}
    try:
        out["reference"] = build_reference(force)
    except RuntimeError as e:  # the reference build is optional on machines without it
        out["reference"] = None
        out["reference_error"] = str(e)
    try:
        out["reference_gpu"] = build_reference_gpu(force)
    except (RuntimeError, OSError) as e:
        out["reference_gpu"] = None
        out["reference_gpu_error"] = str(e)
    return out


if __name__ == "__main__":
    res = build_all(force="--force" in sys.argv)
    print(res)
