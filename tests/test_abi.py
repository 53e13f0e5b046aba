"""CPU checks of the C ABI library: it builds for sm_103a, loads, and exports every entry point
include/lyon_gpu.h declares (no compute calls: there is no GPU here)."""

import ctypes
import os
import re

from lyon_gb300 import _native, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    hdr = open(os.path.join(ROOT, "include", "lyon_gpu.h")).read()
    return sorted(set(re.findall(r"\b(lyon_(?:gpu|srv)_\w+)\s*\(", hdr)))


def test_library_exports_every_declared_symbol():
    path = build.build()
    lib = ctypes.CDLL(path)
    syms = declared_symbols()
    assert syms, "no declarations found"
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    assert set(_native.EXPORTED) >= set(syms)


def test_library_is_built_for_sm_103a():
    assert "-gencode" in build.ARCH and "arch=compute_103a,code=sm_103a" in build.ARCH
    assert "--fmad=false" in build.NVCC_FLAGS


def test_version_string():
    lib = _native.load()
    assert b"sm_103a" in lib.lyon_gpu_version()
