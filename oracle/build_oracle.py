"""Builds the CPU oracle (test infrastructure): oracle/build/libgi_oracle.so.

g++ -O3 with OpenMP and -ffp-contract=off: no multiply-add contraction, so the
fp32 restatement evaluates exactly the operation sequence written in the source
(the same sequence the CUDA kernels evaluate).  No -march=native: the result is
the same on x86-64 and AArch64 hosts.

The reference itself cannot be compiled here: its renderer needs the absent
dependencies/LegitVulkan submodule, Vulkan and GLFW, so there is no
oracle/_ref build.
"""
from __future__ import annotations

import platform
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT_DIR = HERE / "build"
LIB = OUT_DIR / "libgi_oracle.so"
SOURCES = [HERE / "gi_oracle.cpp"]
HEADERS = [HERE / "glsl.h", HERE / "sampler.h", HERE.parent / "legitengine_gb300" / "csrc" / "gi_math.h",
           HERE.parent / "include" / "legit_gi.h"]


def build(verbose: bool = False) -> Path:
    OUT_DIR.mkdir(exist_ok=True)
    deps = SOURCES + HEADERS
    if LIB.exists() and all(LIB.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return LIB
    flags = ["-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math"]
    if platform.machine() in ("x86_64", "AMD64"):
        flags.append("-mfma")  # fmaf as one instruction; fmaf is correctly rounded either way
    cmd = ["g++"] + flags + [str(s) for s in SOURCES] + ["-o", str(LIB)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
