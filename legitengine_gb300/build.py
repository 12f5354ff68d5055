"""Builds the CUDA library in-tree: legitengine_gb300/lib/libgi_gb300.so.

Every translation unit is compiled for sm_103a only, in parallel, then linked
with the static CUDA runtime.  Numerics flags are part of the library's
contract: ``--fmad=false`` (no multiply-add contraction) and no fast-math on
the device, ``-ffp-contract=off`` on the host, so that the fp32 arithmetic
follows the fixed evaluation order documented in csrc/gi_device.cuh.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIB_DIR = PKG / "lib"
LIB = LIB_DIR / "libgi_gb300.so"
CLI = LIB_DIR / "gi_render_scene"  # headless scene renderer (csrc/gi_render_scene.cpp) on the C ABI

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["gi_mips.cu", "gi_march.cu", "gi_filters.cu", "gi_inputs.cu", "gi_renderer.cu", "gi_mlp.cu", "gi_mlp_tc.cu", "gi_batch.cu"]
CPP_SOURCES = ["gi_host.cpp", "gi_scene.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _common_flags() -> list[str]:
    return [
        "-O3", "-std=c++17", "-lineinfo", "--fmad=false",
        "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden",
        f"-I{ROOT / 'include'}", f"-I{CSRC}",
    ]


def _compile(src: Path, extra: list[str]) -> Path:
    out = OBJ / (src.name + ".o")
    deps = [src] + sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [ROOT / "include" / "legit_gi.h"]
    if out.exists() and all(out.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return out
    cmd = [nvcc()] + ARCH + _common_flags() + extra + ["-c", str(src), "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return out


def build(verbose: bool = False, ptxas_info: bool = False) -> Path:
    """Compiles and links the library; returns its path."""
    OBJ.mkdir(exist_ok=True)
    LIB_DIR.mkdir(exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    jobs = [(CSRC / s, extra) for s in CU_SOURCES] + [(CSRC / s, ["-x", "cu"] if False else []) for s in CPP_SOURCES]
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda a: _compile(*a), jobs))
    if not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart=static", "-o", str(LIB)] + [str(o) for o in objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    src = CSRC / "gi_render_scene.cpp"
    deps = [src, LIB, ROOT / "include" / "legit_gi.h"]
    if not CLI.exists() or any(d.stat().st_mtime > CLI.stat().st_mtime for d in deps):
        cmd = [nvcc(), "-O2", "-std=c++17", f"-I{ROOT / 'include'}", str(src), "-o", str(CLI), f"-L{LIB_DIR}",
               "-lgi_gb300", "-Xlinker", "-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"CLI build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="-v" in sys.argv)
