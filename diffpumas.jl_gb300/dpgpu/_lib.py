"""ctypes binding of libdpgpu.so (the C ABI declared in include/dpgpu.h).

The shared library is built in-tree by diffpumas.jl_gb300/build.py.  There is
no fallback: if the library is missing or no CUDA device is visible, the calls
raise.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.normpath(os.path.join(HERE, "..", "_build", "libdpgpu.so"))

DP_OK, DP_ERR_ARG, DP_ERR_CUDA, DP_ERR_DOMAIN, DP_ERR_ALLOC, DP_ERR_STATE = 0, -1, -2, -3, -4, -5

COLUMNS = ["E", "logE", "csda_S", "csda_R", "csda_T", "mixed_S", "mixed_R", "strag", "ion",
           "brems", "pair", "photo", "xs", "lb1", "lbe", "ecut", "magrot", "mu0", "fspin"]
NCOL = len(COLUMNS)


class DpElement(C.Structure):
    _fields_ = [("Z", C.c_double), ("A", C.c_double), ("I", C.c_double),
                ("fraction", C.c_double)]


class DpMaterial(C.Structure):
    _fields_ = [("name", C.c_char_p), ("density", C.c_double), ("I", C.c_double),
                ("ZoA", C.c_double), ("n_elements", C.c_int),
                ("elements", C.POINTER(DpElement))]


class DpSettings(C.Structure):
    _fields_ = [("mass", C.c_double), ("ctau", C.c_double), ("cutoff", C.c_double),
                ("elastic_ratio", C.c_double)]


class DpMcParams(C.Structure):
    _fields_ = [("rock_thickness", C.c_double), ("rock_density", C.c_double),
                ("elevation", C.c_double), ("energy_min", C.c_double),
                ("energy_max", C.c_double), ("n_samples", C.c_long), ("seed", C.c_uint64),
                ("straggling", C.c_int), ("scattering", C.c_int),
                ("compute_gradient", C.c_int), ("energy_threshold_low", C.c_double),
                ("source_energy_max", C.c_double), ("primary_altitude", C.c_double),
                ("rock_material", C.c_int), ("air_material", C.c_int), ("precision", C.c_int),
                ("porous_material", C.c_int), ("porous_density", C.c_double),
                ("porous_thickness", C.c_double)]


class DpMcResult(C.Structure):
    _fields_ = [("flux", C.c_double), ("sigma", C.c_double), ("gradient", C.c_double),
                ("gradient_flux", C.c_double), ("source_energy_max", C.c_double),
                ("n_samples", C.c_long), ("n_status_nonzero", C.c_long)]


class DpMcConfig(C.Structure):
    _fields_ = [("straggling", C.c_int), ("scattering", C.c_int),
                ("energy_threshold_low", C.c_double), ("source_energy_max", C.c_double),
                ("seed", C.c_uint64), ("precision", C.c_int)]


class DpLos(C.Structure):
    _fields_ = [(k, C.c_double) for k in (
        "thickness", "thickness_max", "density", "density_max", "elevation", "elevation_max",
        "primary_altitude", "air_height", "energy_min", "energy_max")] + [("n_samples", C.c_long)] + \
        [("porous_thickness", C.c_double), ("porous_density", C.c_double)]


class DpLosResult(C.Structure):
    _fields_ = [("flux", C.c_double), ("sigma", C.c_double), ("gradient", C.c_double),
                ("gradient_flux", C.c_double), ("n_samples", C.c_long),
                ("n_status_nonzero", C.c_long)]


class DpDirBatch(C.Structure):
    _fields_ = [("n_dirs", C.c_long), ("cos_theta", C.c_void_p), ("remaining_rock", C.c_void_p),
                ("air_distance", C.c_void_p), ("valid", C.c_void_p), ("seg_ptr", C.c_void_p),
                ("seg_medium", C.c_void_p), ("seg_density", C.c_void_p),
                ("seg_length", C.c_void_p), ("sample_ptr", C.c_void_p), ("energy", C.c_void_p),
                ("charge", C.c_void_p), ("weight", C.c_void_p), ("energy_min", C.c_double),
                ("energy_max", C.c_double), ("rock_medium", C.c_int), ("air_medium", C.c_int),
                ("rock_density", C.c_double), ("detector_elevation", C.c_double)]


class DpCsdaConfig(C.Structure):
    _fields_ = [("rock_material", C.c_int), ("water_material", C.c_int),
                ("air_material", C.c_int), ("porous_material", C.c_int),
                ("rock_density", C.c_double), ("water_density", C.c_double),
                ("porous_density", C.c_double), ("porous_top_thickness", C.c_double),
                ("detector_elevation", C.c_double), ("primary_altitude", C.c_double),
                ("correction", C.c_int), ("kappa_strag", C.c_double), ("kappa_hard", C.c_double),
                ("resid_a", C.c_double), ("resid_b", C.c_double), ("resid_c", C.c_double),
                ("resid_d", C.c_double), ("material_correction", C.c_int),
                ("material_linear", C.c_double), ("material_quadratic", C.c_double)]


class DpCsdaBatch(C.Structure):
    _fields_ = [("n_bins", C.c_long), ("cos_theta", C.c_void_p), ("remaining_rock", C.c_void_p),
                ("surface_exit_z", C.c_void_p), ("valid", C.c_void_p), ("seg_ptr", C.c_void_p),
                ("seg_cell", C.c_void_p), ("seg_length", C.c_void_p), ("n_energy", C.c_int),
                ("energy", C.c_void_p), ("charge", C.c_void_p), ("weight", C.c_void_p)]


class DpVoxelVolume(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("x_edges", C.c_void_p),
                ("y_edges", C.c_void_p), ("z_edges", C.c_void_p)]


class DpElevationMap(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("x0", C.c_double), ("y0", C.c_double),
                ("dx", C.c_double), ("dy", C.c_double), ("z", C.c_void_p)]


class DpTerrain(C.Structure):
    _fields_ = [("map", DpElevationMap), ("xy_scale", C.c_double),
                ("detector_elevation", C.c_double), ("step", C.c_double),
                ("max_distance", C.c_double)]


class DpTetraMesh(C.Structure):
    _fields_ = [("n_points", C.c_long), ("points", C.c_void_p), ("n_tets", C.c_long),
                ("tets", C.c_void_p)]


class DpMcShape(C.Structure):
    _fields_ = [("threads", C.c_int), ("staging", C.c_int), ("order", C.c_int),
                ("sync", C.c_int)]


class DpSolveParams(C.Structure):
    _fields_ = [("method", C.c_int), ("n_iter", C.c_int), ("cg_iter", C.c_int),
                ("precision", C.c_int), ("relaxation", C.c_double), ("lm_damping", C.c_double),
                ("box_lo", C.c_double), ("box_hi", C.c_double), ("prior_weight", C.c_double),
                ("smooth_strength", C.c_double), ("no_speculation", C.c_int),
                ("optimizer", C.c_int), ("fixed_linearization", C.c_int), ("lr", C.c_double)]


class DpGrid(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("x0", C.c_double),
                ("y0", C.c_double), ("z0", C.c_double), ("dx", C.c_double),
                ("dy", C.c_double), ("dz", C.c_double)]


class DpRay(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("ox", "oy", "oz", "ux", "uy", "uz", "cos_theta")]


class DpTomoParams(C.Structure):
    _fields_ = [("rock_material", C.c_int), ("air_material", C.c_int), ("side_cell", C.c_int),
                ("side_density", C.c_double), ("primary_altitude", C.c_double),
                ("n_nodes", C.c_int), ("node_energy", C.c_void_p),
                ("node_charge", C.c_void_p), ("node_weight", C.c_void_p),
                ("precision", C.c_int)]


_P = C.c_void_p
_D = C.c_double
_I = C.c_int
_L = C.c_long
_VP = C.c_void_p

# int run(void* user): the workload dp_autotune times
AUTOTUNE_RUN = C.CFUNCTYPE(C.c_int, C.c_void_p)

# name -> (restype, argtypes); pointers to arrays are passed as c_void_p.
PROTOTYPES = {
    "dp_version": (_I, []),
    "dp_init": (_I, [_I, C.POINTER(_P)]),
    "dp_destroy": (_I, [_P]),
    "dp_last_error": (C.c_char_p, [_P]),
    "dp_set_stream": (_I, [_P, _VP]),
    "dp_get_stream": (_VP, [_P]),
    "dp_set_timing": (_I, [_P, _I]),
    "dp_kernel_time": (_I, [_P, C.c_char_p, C.POINTER(_D)]),
    "dp_kernel_stats": (_I, [_P, C.c_char_p, C.POINTER(_D), C.POINTER(C.c_longlong)]),
    "dp_launch_count": (C.c_longlong, [_P]),
    "dp_scratch_bytes": (C.c_longlong, [_P]),
    "dp_set_blocking": (_I, [_P, _I]),
    "dp_sync": (_I, [_P]),
    "dp_set_debug_limits": (_I, [_P, _I, _I, _I]),
    "dp_mc_thread_choices": (_I, [_I, _VP, _I]),
    "dp_set_mc_threads": (_I, [_P, _I, _I, _I]),
    "dp_get_mc_threads": (_I, [_P, _I, _I, C.POINTER(_I)]),
    "dp_autotune": (_I, [_P, _I, _I, AUTOTUNE_RUN, _VP, C.POINTER(_I), _VP, _I]),
    "dp_set_mc_shape": (_I, [_P, _I, _I, C.POINTER(DpMcShape)]),
    "dp_get_mc_shape": (_I, [_P, _I, _I, C.POINTER(DpMcShape)]),
    "dp_autotune_shape": (_I, [_P, _I, _I, AUTOTUNE_RUN, _VP, C.POINTER(DpMcShape),
                               C.POINTER(DpMcShape), _VP, _I, C.POINTER(_I)]),
    "dp_physics_upload": (_I, [_P, C.POINTER(DpSettings), _I, _I, _VP, _VP, C.POINTER(_P)]),
    "dp_physics_create": (_I, [_P, C.POINTER(DpSettings), _I, _VP, _I, _D, _D, C.POINTER(_P)]),
    "dp_physics_create_dedx": (_I, [_P, C.POINTER(DpSettings), _I, _VP, _VP, C.POINTER(_P)]),
    "dp_tables_from_dedx": (_I, [C.POINTER(DpSettings), _I, _VP, _VP, C.POINTER(_I), _VP, _L]),
    "dp_physics_save": (_I, [_P, C.c_char_p]),
    "dp_physics_load": (_I, [_P, C.c_char_p, C.POINTER(_P)]),
    "dp_physics_settings": (_I, [_P, C.POINTER(DpSettings)]),
    "dp_physics_material_name": (_I, [_P, _I, C.c_char_p, _I]),
    "dp_physics_free": (_I, [_P]),
    "dp_physics_info": (_I, [_P, C.POINTER(_I), C.POINTER(_I)]),
    "dp_physics_column": (_I, [_P, _I, _I, _VP]),
    "dp_physics_material_index": (_I, [_P, C.c_char_p]),
    "dp_backward_mc": (_I, [_P, _P, C.POINTER(DpMcParams), C.POINTER(DpMcResult)]),
    "dp_csda_flux_samples": (_I, [_P, _P, C.POINTER(DpMcParams), _L, _VP, _VP, _VP, _VP, _VP,
                                  _VP]),
    "dp_csda_flux_samples_dev": (_I, [_P, _P, C.POINTER(DpMcParams), _L, _VP, _VP, _VP, _VP,
                                      _VP, _VP]),
    "dp_mc_samples": (_I, [_P, C.POINTER(DpMcParams), _L, _VP, _VP, _VP]),
    "dp_csda_direct_samples": (_I, [_P, _P, C.POINTER(DpMcParams), _L, _VP, _VP, _VP, _VP, _VP]),
    "dp_mixture_prepare": (_I, [_P, _P, _I, _VP, _VP, C.POINTER(_P)]),
    "dp_mixture_free": (_I, [_P]),
    "dp_mixture_kernel": (_I, [_P, _I, _VP, _I, C.POINTER(_I), C.POINTER(_D)]),
    "dp_mc_histories": (_I, [_P, _P, _P, _P, C.POINTER(DpMcConfig), _L, _VP, _VP, _VP, _VP, _VP,
                             _VP, _VP, _I, C.c_uint64, _VP, _VP, _VP, _VP]),
    "dp_mc_los": (_I, [_P, _P, _P, _P, C.POINTER(DpMcConfig), _L, _VP, _I, _VP]),
    "dp_mc_los_dev": (_I, [_P, _P, _P, _P, C.POINTER(DpMcConfig), _L, _VP, _L, _I, _VP]),
    "dp_mc_los_layers": (_I, [_P, _P, _P, _P, _P, C.POINTER(DpMcConfig), _L, _VP, _I, _VP]),
    "dp_mc_los_layers_dev": (_I, [_P, _P, _P, _P, _P, C.POINTER(DpMcConfig), _L, _VP, _L, _I,
                                  _VP]),
    "dp_dir_csda": (_I, [_P, _P, C.POINTER(DpCsdaConfig), C.POINTER(DpCsdaBatch), _L, _VP, _VP,
                         _VP, _VP, _I]),
    "dp_dir_csda_dev": (_I, [_P, _P, C.POINTER(DpCsdaConfig), C.POINTER(DpCsdaBatch), _L, _VP,
                             _VP, _VP, _VP, _I]),
    "dp_dir_media_create": (_I, [_P, _P, _I, C.POINTER(_P), C.POINTER(_P)]),
    "dp_voxel_trace": (_I, [_P, C.POINTER(DpVoxelVolume), _L, _VP, _VP, _VP, _VP, _VP, _VP,
                            C.c_int64, _VP, _VP]),
    "dp_map_elevation": (_I, [C.POINTER(DpElevationMap), _L, _VP, _VP, _VP, _VP]),
    "dp_map_gradient": (_I, [C.POINTER(DpElevationMap), _L, _VP, _VP, _VP, _VP, _VP]),
    "dp_surface_exit": (_I, [C.POINTER(DpTerrain), _L, _VP, _VP, _VP, _VP, _VP]),
    "dp_ray_triangle": (_I, [_VP, _VP, _VP, _VP, _VP, C.POINTER(_D), _VP]),
    "dp_tetra_neighbors": (_I, [C.POINTER(DpTetraMesh), _VP]),
    "dp_tetra_trace": (_I, [_P, C.POINTER(DpTetraMesh), _VP, C.POINTER(DpTerrain), _L, _VP, _VP,
                            _VP, _VP, _VP, C.c_int64, _VP, _VP, _VP, _VP, _VP]),
    "dp_dir_media_free": (_I, [_P]),
    "dp_dir_mc": (_I, [_P, _P, _P, C.POINTER(DpDirBatch), C.POINTER(DpMcConfig), _VP, _VP, _VP,
                       _VP]),
    "dp_dir_mc_dev": (_I, [_P, _P, _P, C.POINTER(DpDirBatch), _L, C.POINTER(DpMcConfig), _VP]),
    "dp_tomo_forward": (_I, [_P, _P, C.POINTER(DpGrid), C.POINTER(DpTomoParams), _VP, _L, _VP,
                             _VP]),
    "dp_tomo_jacobian": (_I, [_P, _P, C.POINTER(DpGrid), C.POINTER(DpTomoParams), _VP, _L, _VP,
                              _VP, _VP, _VP, _VP, C.c_int64, C.POINTER(C.c_int64)]),
    "dp_tomo_vjp": (_I, [_P, _P, C.POINTER(DpGrid), C.POINTER(DpTomoParams), _VP, _L, _VP, _VP,
                         _VP, _VP]),
    "dp_tomo_vjp_dev": (_I, [_P, _P, C.POINTER(DpGrid), C.POINTER(DpTomoParams), _VP, _L, _VP,
                             _VP, _VP, _VP]),
    "dp_tomo_paths_create": (_I, [_P, C.POINTER(DpGrid), _L, _VP, _I, C.POINTER(_P)]),
    "dp_tomo_paths_create_dev": (_I, [_P, C.POINTER(DpGrid), _L, _VP, _I, C.POINTER(_P)]),
    "dp_tomo_paths_free": (_I, [_P]),
    "dp_tomo_paths_info": (_I, [_P, C.POINTER(_L), C.POINTER(C.c_int64), C.POINTER(_I)]),
    "dp_tomo_paths_csr": (_I, [_P, _VP, _VP, _VP]),
    "dp_tomo_eval_dev": (_I, [_P, _P, _P, C.POINTER(DpTomoParams), _VP, _VP, _VP, _VP, _VP, _I]),
    "dp_tomo_eval": (_I, [_P, _P, _P, C.POINTER(DpTomoParams), _VP, _VP, _VP, _VP, _VP]),
    "dp_tomo_eval_noalloc_dev": (_I, [_P, _P, _P, C.POINTER(DpTomoParams), _VP, _VP, _VP, _VP]),
    "dp_tomo_solve_dev": (_I, [_P, _P, _P, C.POINTER(DpTomoParams), _VP, _VP, _VP,
                               C.POINTER(DpSolveParams), _VP]),
    "dp_tomo_forward_plain_dev": (_I, [_P, _P, C.POINTER(DpGrid), C.POINTER(DpTomoParams), _VP,
                                       _L, _VP, _VP]),
}

_lib = None


def load():
    """Loads libdpgpu.so and declares every prototype; raises if missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libdpgpu.so not built ({LIB_PATH}); run "
                               "python diffpumas.jl_gb300/build.py")
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in PROTOTYPES.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


class DpError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"libdpgpu error {code}: {msg}")
        self.code = code
        self.msg = msg


class DomainError(DpError):
    """DP_ERR_DOMAIN: where the reference throws DomainError (an energy outside
    the prepared tables, src/MixedTransport.jl:44-45,155,196) or errors on an
    invalid hard-event weight (:186); the message is the reference's."""


def check(rc, ctx=None):
    if rc != DP_OK:
        msg = load().dp_last_error(ctx).decode() if ctx else ""
        if rc == DP_ERR_ARG:
            raise ValueError(msg or "invalid argument")
        if rc == DP_ERR_DOMAIN:
            raise DomainError(rc, msg)
        raise DpError(rc, msg)
    return rc
