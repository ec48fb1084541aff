"""Build recipe of the CPU oracle (test infrastructure).

* ``oracle/_build/liboracle.so`` — the C++ restatement of the wavefront pass
  (pt_oracle.cpp), built without FMA contraction so its float arithmetic
  rounds exactly like the CUDA kernels.
* ``oracle/_ref/libref_bsdf.so`` — only where the reference tree is present:
  the reference's own shader math (math.hlsl, material/utils.hlsl,
  material/lit.hlsl, utils/frame.hlsl, utils/sampling.hlsl) compiled with g++
  through ``ref_shim/hlsl_shim.h``.  The sources are read in place; the only
  rewrite is ``out T x`` / ``inout T x`` -> ``T& x`` (HLSL output parameters).
  The generated translation unit and the library stay under ``oracle/_ref/``,
  which is not committed.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
REFERENCE_ROOT = "/root/reference"
REF_SHADERS = [
    "bisemutum/shaders/core/utils/math.hlsl",
    "bisemutum/shaders/core/material/utils.hlsl",
    "bisemutum/shaders/core/material/lit.hlsl",
    "bisemutum/shaders/core/utils/frame.hlsl",
    "bisemutum/shaders/core/utils/sampling.hlsl",
]
CXXFLAGS = ["-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-pthread"]


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build_oracle(verbose: bool = False) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    src = os.path.join(HERE, "pt_oracle.cpp")
    out = os.path.join(BUILD_DIR, "liboracle.so")
    if _stale(out, [src, __file__]):
        cmd = ["g++", *CXXFLAGS, src, "-o", out + ".tmp"]
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)
        os.replace(out + ".tmp", out)
    return out


def _translate_hlsl(text: str) -> str:
    text = re.sub(r"^\s*#\s*(pragma once|include).*$", "", text, flags=re.M)
    text = re.sub(r"\b(?:inout|out)\s+(\w+)\s+(\w+)", r"\1& \2", text)
    return text


def build_reference(verbose: bool = False) -> str | None:
    """Compiles the reference's shader math; returns None when the reference tree is absent."""
    srcs = [os.path.join(REFERENCE_ROOT, p) for p in REF_SHADERS]
    if not all(os.path.exists(s) for s in srcs):
        return None
    os.makedirs(REF_DIR, exist_ok=True)
    inc = os.path.join(REF_DIR, "ref_sources.inc")
    shim_dir = os.path.join(HERE, "ref_shim")
    body = "".join(f"// ---- {p} ----\n" + _translate_hlsl(open(s).read()) + "\n" for p, s in zip(REF_SHADERS, srcs))
    if not os.path.exists(inc) or open(inc).read() != body:
        with open(inc, "w") as f:
            f.write(body)
    out = os.path.join(REF_DIR, "libref_bsdf.so")
    deps = [inc, os.path.join(shim_dir, "ref_bsdf.cpp"), os.path.join(shim_dir, "hlsl_shim.h"), __file__]
    if _stale(out, deps):
        cmd = ["g++", *CXXFLAGS, "-w", "-I", shim_dir, "-I", REF_DIR, os.path.join(shim_dir, "ref_bsdf.cpp"),
               "-o", out + ".tmp"]
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)
        os.replace(out + ".tmp", out)
    return out


if __name__ == "__main__":
    print(build_oracle(verbose=True))
    print(build_reference(verbose=True))
    sys.exit(0)
