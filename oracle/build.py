"""Builds the CPU oracle (test infrastructure) into oracle/_build/liborc.so with g++.

Float semantics matter here: -ffp-contract=off keeps every a*b+c unfused except the explicit
std::fma calls that restate the reference's simd::fma, and no fast-math flag is used.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SOURCES = ["swr_oracle_raster.cpp", "swr_oracle_texture.cpp", "swr_oracle_resolve.cpp", "swr_oracle_ibl.cpp"]
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liborc.so")


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    deps = srcs + [os.path.join(HERE, h) for h in ("swr_oracle.h", "swr_oracle_common.h")]
    deps += [os.path.join(HERE, "..", "include", "swr", h) for h in ("hostmath.h", "approx14.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-Wall", "-Wextra", "-Wno-unused-parameter", *srcs, "-o", tmp, "-lpthread"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
