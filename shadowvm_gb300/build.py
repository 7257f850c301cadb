"""Builds the data-plane library in-tree: shadowvm_gb300/_build/libshadowvm_gb300.so.

Every translation unit is compiled by nvcc for sm_103a only (one -gencode), in
parallel, then linked into one shared library with a plain C ABI
(include/svm_capi.h).  No torch, no CMake.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libshadowvm_gb300.so")

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
          f"-I{os.path.join(ROOT, 'include')}", f"-I{CSRC}"]
CU_FLAGS = ["--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]

SOURCES = ["capi.cpp", "pipeline.cpp", "expr.cpp", "strdict.cpp", "kern_util.cu", "kern_dim.cu", "kern_star.cu", "kern_star_plan.cu", "kern_star_plan_mix.cu", "kern_star_plan_mix2.cu", "kern_star_plan_mix3.cu", "kern_star_plan_list.cu", "kern_mbatch.cu", "kern_load.cu",
           "kern_noalloc.cu"]
HEADERS = ["svm_internal.h", "kern_common.cuh", "kern_star_common.cuh", "kern_star_plan.cuh", "kernels.h", "ctx.h", "expr.h", "strdict.h"]


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "svm_capi.h")]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _compile(src: str, verbose: bool) -> str:
    path = os.path.join(CSRC, src)
    obj = os.path.join(OUT_DIR, src + ".o")
    if not _stale(obj, path):
        return obj
    cmd = [NVCC, *ARCH, *COMMON, "-c", path, "-o", obj + ".tmp"]
    if src.endswith(".cu"):
        cmd[1:1] = CU_FLAGS
    else:
        cmd += ["-x", "cu"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stderr.strip()):
        sys.stderr.write(r.stderr)
    os.replace(obj + ".tmp", obj)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [NVCC, *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
