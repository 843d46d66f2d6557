"""The C ABI library builds for sm_103a, loads, and exports every entry point
include/omdg.h declares (no compute calls: there may be no GPU here)."""
import ctypes
import os
import re

from conftest import ROOT


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "omdg.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(omdg_\w+)\s*\(", text, re.M)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "omdg_create" in syms and "omdg_step" in syms
    assert len(syms) >= 30


def test_library_exports_every_declared_symbol(omdg_lib):
    lib = ctypes.CDLL(omdg_lib.LIB_PATH)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_covers_the_header(omdg_lib):
    missing = [s for s in declared_symbols() if s not in omdg_lib.SIGNATURES]
    assert not missing, missing


def test_library_is_built_for_sm103a(omdg_lib):
    from objectmd_gb300 import build

    assert "arch=compute_103a,code=sm_103a" in " ".join(build.ARCH)
    assert os.path.getsize(omdg_lib.LIB_PATH) > 0


def test_no_gpu_fails_loudly(omdg_lib):
    """Without a usable GPU the context cannot be created (no CPU fallback)."""
    import torch

    if torch.cuda.is_available():
        return
    try:
        omdg_lib.Context(0)
    except omdg_lib.OMDGError:
        return
    raise AssertionError("context creation succeeded without a GPU")
