"""Builds libswr_gb300.so in-tree with nvcc for sm_103a (no CMake, one -gencode).

Translation units compile in parallel; -fmad=false keeps every float operation on the exact
vis-buffer path unfused unless written as an explicit fma intrinsic.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libswr_gb300.so")
SOURCES = ["swr_api.cu", "swr_raster.cu", "swr_texture.cu", "swr_shade.cu", "swr_batch.cu", "swr_noalloc.cu",
           "swr_neural.cu", "swr_neural_api.cu", "swr_gbuffer.cu", "swr_ibl.cu", "swr_meshletize.cpp"]
HEADERS = ["swr_device.cuh", "swr_internal.h", "swr_tc.cuh", "swr_neural.h", "swr_sample.cuh", "swr_surface.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags():
    return [*ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
            "-Xptxas", "-warn-spills", "--expt-relaxed-constexpr"]


def build(force: bool = False, verbose: bool = False) -> str:
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    deps = srcs + [os.path.join(CSRC, h) for h in HEADERS]
    inc = os.path.join(HERE, "..", "include")
    deps += [os.path.join(inc, "swr_gb300.h")]
    deps += [os.path.join(inc, "swr", h) for h in ("hostmath.h", "approx14.h", "device.cuh", "raster_math.cuh", "shader.cuh")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    os.makedirs(BUILD_DIR, exist_ok=True)
    objs = [os.path.join(BUILD_DIR, os.path.splitext(s)[0] + ".o") for s in SOURCES]

    def compile_one(src, obj):
        cmd = [nvcc(), *_flags(), "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        logs = list(ex.map(compile_one, srcs, objs))
    if verbose:
        for l in logs:
            if l.strip():
                print(l)
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [nvcc(), *ARCH, "-shared", *objs, "-o", tmp, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
