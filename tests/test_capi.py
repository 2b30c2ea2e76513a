"""CPU tests of the C-ABI library: it builds for sm_103a, loads, and exports every declared symbol.
No CUDA work is issued (no GPU is needed)."""
import ctypes
import os
import re

from glimpsw_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "swr_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(swr_[a-z0-9_]+)\s*\(", text)))


def test_library_builds_and_exports_every_declared_symbol():
    path = build.build()
    lib = ctypes.CDLL(path)
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from glimpsw_gb300 import api
    assert set(declared_functions()) <= set(api._SIGS)


def test_library_is_built_for_sm_103a_only():
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
