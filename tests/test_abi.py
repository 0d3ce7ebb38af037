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


def test_launch_shape_choices_and_argument_checks():
    """The compiled CTA sizes of the persistent transport kernels (no device
    needed): 1024 (default), 768 and 512 threads for the mixed-precision
    transport, 256 for FP64; bad arguments are rejected before any device
    work."""
    import dpgpu
    assert dpgpu.mc_thread_choices("mixed") == [1024, 768, 512]
    assert dpgpu.mc_thread_choices("fp64") == [256]
    lib = dpgpu.load()
    assert lib.dp_mc_thread_choices(7, None, 0) == dpgpu._lib.DP_ERR_ARG
    assert lib.dp_set_mc_threads(None, 0, 1, 512) == dpgpu._lib.DP_ERR_ARG
    assert lib.dp_autotune(None, 0, 1, dpgpu._lib.AUTOTUNE_RUN(lambda u: 0), None, None, None,
                           0) == dpgpu._lib.DP_ERR_ARG
