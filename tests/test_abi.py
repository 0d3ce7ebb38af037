"""C ABI: the library builds for sm_103a and exports every entry point that
include/dpgpu.h declares (CPU only: no compute call)."""
import ctypes
import os
import re

from conftest import ROOT


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "dpgpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dp_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_boundary():
    syms = declared_symbols()
    for s in ("dp_init", "dp_destroy", "dp_physics_create", "dp_physics_upload",
              "dp_backward_mc", "dp_tomo_forward", "dp_tomo_jacobian", "dp_tomo_vjp"):
        assert s in syms


def test_library_exports_every_declared_symbol():
    import build as b  # diffpumas.jl_gb300/build.py
    lib_path = b.build()
    lib = ctypes.CDLL(lib_path)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    assert lib.dp_version() == 1
