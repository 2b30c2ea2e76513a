"""Builds tests/user_shader/hook_shaders.cu, the user shaders of the shader-hook tests, into
tests/user_shader/_build/libhook_shaders.so with nvcc for sm_103a, as a user of the library would:
the shaders include swr/shader.cuh and link against libswr_gb300.so."""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
SRC = os.path.join(HERE, "hook_shaders.cu")
OUT = os.path.join(HERE, "_build", "libhook_shaders.so")


def build(force: bool = False) -> str:
    from glimpsw_gb300 import build as lib_build

    lib = lib_build.build()
    inc = os.path.join(ROOT, "include")
    deps = [SRC, lib] + [os.path.join(inc, "swr", h) for h in ("shader.cuh", "raster_math.cuh", "device.cuh", "approx14.h")]
    deps.append(os.path.join(inc, "swr_gb300.h"))
    if not force and os.path.exists(OUT) and all(os.path.getmtime(OUT) >= os.path.getmtime(d) for d in deps):
        return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    libdir = os.path.dirname(lib)
    tmp = OUT + f".tmp{os.getpid()}"
    cmd = [lib_build.nvcc(), *lib_build.ARCH, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", "-I", inc, SRC,
           "-o", tmp, "-L", libdir, "-lswr_gb300", "-Xlinker", f"-rpath={libdir}", "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {SRC}:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, OUT)
    return OUT
