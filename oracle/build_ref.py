"""Builds oracle/_ref/libgi_ref.so: the reference's own GLSL passes compiled as
C++ (test infrastructure: it checks the oracle's restatement, nothing ships it).

The reference renders with Vulkan and its host needs an absent submodule, so its
passes cannot run as the reference runs them.  Its fragment shaders, however, are
plain GLSL 450 arithmetic, and GLSL's vector/matrix language is what the
reference's own vendored glm (dependencies/glm, 0.9.9) mirrors in C++.  This
recipe reads each shader where it lies in the reference checkout and rewrites it
mechanically into a C++ struct -- the shader text itself is not edited by hand:

  1. `#version` / `#extension` lines are dropped;
  2. a uniform block `layout(...) uniform Name { members };` becomes its members;
  3. `layout(...)` and the storage qualifiers `uniform`, `in`, `out` of global
     declarations are dropped (samplers, varyings and outputs become members);
  4. function parameters `out T x` / `inout T x` become `T& x`, `in T x` becomes `T x`;
  5. GLSL array constructors `T name[] = T[](a, b, ...)` become `T name[] = {a, b, ...}`;
  6. unsuffixed floating literals (`2.0`, `10e-1`) get C++'s float suffix, as GLSL
     literals are single precision;
  7. a compound assignment of a scalar to a swizzle (`v.xyz /= s;`) takes the
     scalar as a vector (`v.xyz /= vec3(s);`), which glm's swizzle proxies need;
  8. optionally, the march's `const int dirsCount = 4;` takes the value the test
     asks for (the reference's constant generalised, as the library's `dirs`).

oracle/ref_shim.h supplies glm, the built-ins with GLSL's implicit conversions,
sampler2D with oracle/sampler.h's Vulkan sampler formulas and gl_FragCoord;
oracle/ref_runner.cpp runs the shaders per pixel behind a C API.  The rewritten
sources and the library go to oracle/_ref/ (git-ignored).  Without the reference
checkout (a machine that has only this repository) nothing is built.

Run: python oracle/build_ref.py [REFERENCE_ROOT]
(REFERENCE_ROOT: the argument, else LEGIT_REFERENCE_ROOT, else the default below).
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from pathlib import Path

DEFAULT_REFERENCE_ROOT = "/root/reference"

HERE = Path(__file__).resolve().parent
OUT_DIR = HERE / "_ref"
GEN_DIR = OUT_DIR / "gen"
LIB = OUT_DIR / "libgi_ref.so"
GLM_INCLUDE = "dependencies/glm/include"
GLSL = "bin/data/Shaders/glsl"
# struct name -> (shader under GLSL, output variable, march directions substituted)
SHADERS = {
    "MipLevelBuilder": ("Common/mipLevelBuilder.frag", None),
    "BlurLayerBuilder": ("Common/blurLayerBuilder.frag", None),
    "Deinterleave": ("Common/deinterleave.frag", None),
    "Interleave": ("Common/interleave.frag", None),
    "IndirectLighting": ("SSVGI/indirectLighting.frag", None),
    "IndirectLightingDirs": ("SSVGI/indirectLighting.frag", "REF_DIRS"),
    "FinalGatherer": ("Common/finalGatherer.frag", None),
    "DirectLighting": ("Common/directLighting.frag", None),
    "Denoiser": ("Common/denoiser.frag", None),
}


def reference_root(arg: str | None = None) -> Path:
    if arg:
        return Path(arg)
    return Path(os.environ.get("LEGIT_REFERENCE_ROOT", DEFAULT_REFERENCE_ROOT))


def available(root: Path | None = None) -> bool:
    root = root or reference_root()
    return (root / GLSL / "SSVGI/indirectLighting.frag").is_file() and (root / GLM_INCLUDE / "glm/glm.hpp").is_file()


_FLOAT_LIT = re.compile(r"(?<![\w.])(\d+\.\d*(?:[eE][+-]?\d+)?|\.\d+(?:[eE][+-]?\d+)?|\d+[eE][+-]?\d+)(?![\w.])")
_SWIZ_SCALAR = re.compile(r"(\.\s*)([xyzwrgba]{2,4})(\s*)([*/+-]=)\s*([^;]+);")


def translate(src: str, name: str, dirs_macro: str | None) -> str:
    """The rewrites 1-8 of the module docstring; returns the struct's C++ source."""
    s = src.replace("\r\n", "\n")
    s = re.sub(r"^\s*#\s*(version|extension)\b.*$", "", s, flags=re.M)                        # 1
    s = re.sub(r"layout\s*\([^)]*\)\s*uniform\s+\w+\s*\{([^}]*)\}\s*;", r"\1", s)            # 2
    s = re.sub(r"layout\s*\([^)]*\)\s*", "", s)                                               # 3
    s = re.sub(r"^(\s*)(uniform|in|out)\s+(?=\w+\s+\w+\s*;)", r"\1", s, flags=re.M)
    s = re.sub(r"([(,]\s*)(?:out|inout)\s+(\w+)\s+(\w+)", r"\1\2& \3", s)                    # 4
    s = re.sub(r"([(,]\s*)in\s+(\w+)\s+(\w+)", r"\1\2 \3", s)
    s = re.sub(r"(\w+)\s+(\w+)\s*\[\s*\]\s*=\s*\1\s*\[\s*\]\s*\(((?:[^;])*?)\)\s*;",          # 5
               r"\1 \2[] = {\3};", s)
    s = _FLOAT_LIT.sub(lambda m: m.group(1) + "f", s)                                         # 6
    s = _SWIZ_SCALAR.sub(lambda m: f"{m.group(1)}{m.group(2)}{m.group(3)}{m.group(4)} "        # 7
                                   f"vec{len(m.group(2))}({m.group(5).strip()});", s)
    if dirs_macro:                                                                            # 8
        s, n = re.subn(r"const\s+int\s+dirsCount\s*=\s*4\s*;", f"const int dirsCount = {dirs_macro};", s)
        if n != 1:
            raise RuntimeError("build_ref: the march's dirsCount constant was not found")
    return f"struct {name} : FragmentShader {{\n{s}\n}};\n"


def build(root: str | Path | None = None, verbose: bool = False) -> Path | None:
    """Translates and compiles; returns the library path, or None without the reference."""
    root = reference_root(str(root) if root else None)
    if not available(root):
        if verbose:
            print(f"build_ref: no reference checkout at {root}; oracle/_ref not built")
        return None
    GEN_DIR.mkdir(parents=True, exist_ok=True)
    sources = {name: root / GLSL / rel for name, (rel, _) in SHADERS.items()}
    deps = list(sources.values()) + [Path(__file__), HERE / "ref_shim.h", HERE / "ref_runner.cpp",
                                     HERE / "sampler.h", HERE / "glsl.h"]
    if LIB.exists() and all(LIB.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return LIB
    for name, (rel, macro) in SHADERS.items():
        text = translate(sources[name].read_text(), name, macro)
        (GEN_DIR / f"{name}.inc").write_text(f"// generated by oracle/build_ref.py from {GLSL}/{rel}\n" + text)
    flags = ["-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-w",
             f"-I{root / GLM_INCLUDE}", f"-I{HERE}", f"-I{GEN_DIR}"]
    cmd = ["g++"] + flags + [str(HERE / "ref_runner.cpp"), "-o", str(LIB)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build_ref failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr[-6000:]}")
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    out = build(sys.argv[1] if len(sys.argv) > 1 else None, verbose=True)
    sys.exit(0 if out else 1)
