"""Build recipe of the native library ``libbsm_pt.so`` (in-tree, no pip install).

CUDA sources are compiled for sm_103a only, with ``--fmad=false`` so that the
path arithmetic rounds once per operation (the traversal's box test asks for
its fused multiply-adds explicitly).  Host C++ is compiled without FMA
contraction for the same reason.  Translation units build in parallel; the
link goes through nvcc (static CUDA runtime).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libbsm_pt.so")

NVCC = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
CUDA_INC = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(NVCC))), "include")
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", *GENCODE, "-lineinfo", "-O3", "--fmad=false", "-prec-div=true", "-prec-sqrt=true",
              "-ftz=false", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", INCLUDE]
CXX_FLAGS = ["-std=c++20", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-pthread", "-I", INCLUDE,
             "-I", CUDA_INC]


def _sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INCLUDE, "bsm_pt.h"))
    return cu, cpp, headers


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    cu, cpp, headers = _sources()
    this = os.path.abspath(__file__)
    jobs_list = []
    objs = []
    for f in cu:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if _stale(obj, [src, this, *headers]):
            jobs_list.append([NVCC, *NVCC_FLAGS, "-c", src, "-o", obj])
    for f in cpp:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if _stale(obj, [src, this, *headers]):
            jobs_list.append(["g++", *CXX_FLAGS, "-c", src, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r

    with cf.ThreadPoolExecutor(max_workers=jobs or max(2, os.cpu_count() or 2)) as ex:
        list(ex.map(run, jobs_list))
    if jobs_list or _stale(LIB, objs):
        run([NVCC, "-shared", *GENCODE, "-o", LIB + ".tmp", *objs, "-lpthread"])
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
