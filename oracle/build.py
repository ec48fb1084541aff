"""Build recipe of the CPU oracle (test infrastructure).

* ``oracle/_build/liboracle.so`` — the C++ restatement of the wavefront pass
  (pt_oracle.cpp), built without FMA contraction so its float arithmetic
  rounds exactly like the CUDA kernels.
* ``oracle/_ref/libref_bsdf.so`` — only where the reference tree is present:
  the reference's own shader math (math.hlsl, material/utils.hlsl,
  material/lit.hlsl, utils/frame.hlsl, utils/sampling.hlsl, the G-buffer
  packing functions of utils/pack.hlsl and renderer/gbuffer.hlsl, and the
  light evaluation of renderer/lights.hlsl with its light structs) compiled
  with g++ through ``ref_shim/hlsl_shim.h``.  The sources are read in place;
  the only rewrite is ``out T x`` / ``inout T x`` -> ``T& x`` (HLSL output
  parameters); of pack.hlsl, gbuffer.hlsl, lights_struct.hlsl and lights.hlsl
  only the named functions and structs are taken (the rest of those files uses
  HLSL the shim lacks: textures, samplers, the LTC integrals).
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
# where the reference tree is read from (BSM_REFERENCE_ROOT overrides the default location)
REFERENCE_ROOT = os.environ.get("BSM_REFERENCE_ROOT", "/root/reference")
REF_SHADERS = [
    "bisemutum/shaders/core/utils/math.hlsl",
    "bisemutum/shaders/core/material/utils.hlsl",
    "bisemutum/shaders/core/material/lit.hlsl",
    "bisemutum/shaders/core/utils/frame.hlsl",
    "bisemutum/shaders/core/utils/sampling.hlsl",
]
# (file, names of the functions / structs taken from it)
REF_EXTRACTS = [
    ("bisemutum/shaders/core/utils/pack.hlsl",
     ["pack_u32_to_unorm16x2", "unpack_u32_from_unorm16x2", "pack_color_rg11b10", "unpack_color_rg11b10",
      "oct_wrap", "oct_encode", "oct_decode", "pack_normal_and_tangent", "unpack_normal_and_tangent"]),
    ("bisemutum/shaders/renderer/gbuffer.hlsl", ["GBuffer", "pack_surface_to_gbuffer", "unpack_gbuffer_to_surface"]),
    ("bisemutum/shaders/renderer/lights_struct.hlsl", ["DirLightData", "PointLightData"]),
    ("bisemutum/shaders/renderer/lights.hlsl", ["dir_light_eval", "point_light_eval"]),
]
# -O3 without -march=native (the same build on x86 and Arm hosts) and without fast-math or FMA contraction:
# IEEE float semantics at every optimisation level, so results equal the kernels'
CXXFLAGS = ["-std=c++17", "-O3", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-pthread"]


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


def _extract(text: str, name: str) -> str:
    """The definition of function or struct `name`: from its declaration line to the matching brace."""
    m = re.search(r"^(struct\s+" + name + r"\b|[\w<>]+\s+" + name + r"\s*\()", text, flags=re.M)
    if m is None:
        raise RuntimeError(f"{name} not found")
    i = text.index("{", m.start())
    depth = 0
    for j in range(i, len(text)):
        depth += {"{": 1, "}": -1}.get(text[j], 0)
        if depth == 0:
            end = j + 1
            if text.startswith("struct", m.start()):
                end = text.index(";", end) + 1
            return text[m.start():end] + "\n"
    raise RuntimeError(f"unbalanced braces after {name}")


def build_reference(verbose: bool = False) -> str | None:
    """Compiles the reference's shader math; returns None when the reference tree is absent."""
    srcs = [os.path.join(REFERENCE_ROOT, p) for p in REF_SHADERS]
    extracts = [(os.path.join(REFERENCE_ROOT, p), p, names) for p, names in REF_EXTRACTS]
    if not all(os.path.exists(s) for s in srcs) or not all(os.path.exists(e[0]) for e in extracts):
        return None
    os.makedirs(REF_DIR, exist_ok=True)
    inc = os.path.join(REF_DIR, "ref_sources.inc")
    shim_dir = os.path.join(HERE, "ref_shim")
    body = "".join(f"// ---- {p} ----\n" + _translate_hlsl(open(s).read()) + "\n" for p, s in zip(REF_SHADERS, srcs))
    for path, p, names in extracts:
        text = _translate_hlsl(open(path).read())
        body += f"// ---- {p}: {', '.join(names)} ----\n" + "".join(_extract(text, n) for n in names)
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
