"""dpgpu -- Python host mirror of the DiffPumas.jl hot-path API on libdpgpu.

Names and keyword arguments follow the reference (src/DiffPumas.jl exports):
create_physics, get_material_index, run_backward_mc, compute_flux_differentiable,
compute_flux_gradient, csda_energy_quadrature, and the voxel-density
tomography forward / Jacobian / vector-Jacobian product.  Every computation
runs in libdpgpu's CUDA kernels; there is no CPU fallback.
"""
import ctypes as C
import math
import threading
from collections import namedtuple

import numpy as np

from . import _lib
from ._lib import (COLUMNS, DomainError, DpElement, DpError, DpGrid, DpLos, DpLosResult,
                   DpMaterial, DpMcConfig, DpMcParams, DpMcResult, DpRay, DpSettings,
                   DpTomoParams, check, load)

PRECISION = {"fp64": 0, "mixed": 1}
MUON_MASS = 0.10565839
MUON_C_TAU = 658.654
PRIMARY_ALTITUDE = 3e4
DEFAULT_CUTOFF = 5e-2
DEFAULT_ELASTIC_RATIO = 5e-2


# ----------------------------------------------------------------- context
class Context:
    """One CUDA stream on one device (dp_ctx)."""

    def __init__(self, device=0):
        lib = load()
        h = C.c_void_p()
        rc = lib.dp_init(device, C.byref(h))
        if rc != 0:
            raise _lib.DpError(rc, f"dp_init failed on device {device}")
        self.h = h
        self.device = device

    def close(self):
        if getattr(self, "h", None):
            load().dp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default = None
_lock = threading.Lock()


def default_context():
    global _default
    with _lock:
        if _default is None:
            _default = Context(0)
        return _default


# ----------------------------------------------------------------- launch shapes
KERNEL_MC, KERNEL_DIR = 0, 1  # two-layer transport, fixed-path transport
_FAMILY = {"mc": KERNEL_MC, "dir": KERNEL_DIR, KERNEL_MC: KERNEL_MC, KERNEL_DIR: KERNEL_DIR}
_PRECISION = {"fp64": 0, "mixed": 1, 0: 0, 1: 1}


def _ctx_of(obj):
    """The dp_ctx handle of a Context or of an object holding one (.ctx)."""
    ctx = obj if isinstance(obj, Context) else getattr(obj, "ctx", None)
    if not isinstance(ctx, Context):
        raise TypeError("expected a Context or an object with a .ctx Context")
    return ctx.h


def mc_thread_choices(precision="mixed"):
    """CTA sizes the persistent transport kernels are compiled for (the
    first is the default)."""
    buf = (C.c_int * 8)()
    n = load().dp_mc_thread_choices(_PRECISION[precision], C.cast(buf, C.c_void_p), 8)
    check(n if n < 0 else 0)
    return [buf[i] for i in range(n)]


def set_mc_threads(ctx, family, precision, threads):
    """CTA size of the persistent transport kernels of `family` ("mc" or
    "dir") at `precision` on this context; 0 restores the default."""
    h = _ctx_of(ctx)
    check(load().dp_set_mc_threads(h, _FAMILY[family], _PRECISION[precision], int(threads)), h)


def set_debug_limits(ctx, step_cap=None, event_cap=None, wait_iters=None):
    """dp_set_debug_limits: lowers this context's loop caps (transport steps
    of a history, hard events of a mixed step) and the poll count of the
    table-staging waits, for tests of the failure paths.  None restores the
    default.  A history that reaches a limit ends with its DP_ST_* bit and the
    call reports DP_ERR_STATE."""
    h = _ctx_of(ctx)
    v = lambda x: -1 if x is None else int(x)
    check(load().dp_set_debug_limits(h, v(step_cap), v(event_cap), v(wait_iters)), h)


def set_mc_shape(ctx, family, precision, threads=0, staging=None, order=None, sync=None):
    """dp_set_mc_shape: CTA size (0: default), table staging (0: shared
    memory when the media fit, 1: read through L1/L2), hand-out order (0:
    longest first, 1: index order) and lockstep mask (bit k: the warps of a
    CTA take the steps of phase k together) of the persistent transport
    kernels; None keeps the context's value."""
    from ._lib import DpMcShape
    h = _ctx_of(ctx)
    cur = get_mc_shape(ctx, family, precision)
    staging = cur["staging"] if staging is None else staging
    order = cur["order"] if order is None else order
    sync = cur["sync"] if sync is None else sync
    sh = DpMcShape(int(threads), int(staging), int(order), int(sync))
    check(load().dp_set_mc_shape(h, _FAMILY[family], _PRECISION[precision], C.byref(sh)), h)


def _shape_dict(s):
    return {"threads": s.threads, "staging": s.staging, "order": s.order, "sync": s.sync}


def get_mc_shape(ctx, family, precision):
    from ._lib import DpMcShape
    h = _ctx_of(ctx)
    sh = DpMcShape()
    check(load().dp_get_mc_shape(h, _FAMILY[family], _PRECISION[precision], C.byref(sh)), h)
    return _shape_dict(sh)


def autotune_shape(ctx, family, precision, run):
    """dp_autotune_shape: CTA size, then table staging, then hand-out order,
    then (mixed precision) the lockstep mask, each chosen by timing run() (the
    caller's workload on this context) once untimed and once timed per
    candidate.  Keeps the best on the context and returns (best shape,
    [(shape, ms), ...])."""
    from ._lib import DpMcShape
    h = _ctx_of(ctx)
    lib = load()
    errors = []

    def cb(_user):
        try:
            run()
            return 0
        except Exception as e:  # reported after dp_autotune_shape returns
            errors.append(e)
            return _lib.DP_ERR_STATE

    fn = _lib.AUTOTUNE_RUN(cb)
    best = DpMcShape()
    tried = (DpMcShape * 16)()
    ms = (C.c_double * 16)()
    n = C.c_int()
    rc = lib.dp_autotune_shape(h, _FAMILY[family], _PRECISION[precision], fn, None,
                               C.byref(best), tried, C.cast(ms, C.c_void_p), 16, C.byref(n))
    if errors:
        raise errors[0]
    check(rc, h)
    return _shape_dict(best), [(_shape_dict(tried[i]), ms[i]) for i in range(min(n.value, 16))]


def get_mc_threads(ctx, family, precision):
    h = _ctx_of(ctx)
    t = C.c_int()
    check(load().dp_get_mc_threads(h, _FAMILY[family], _PRECISION[precision], C.byref(t)), h)
    return t.value


def autotune(ctx, family, precision, run):
    """dp_autotune: times run() (the caller's workload on this context) once
    per compiled CTA size of (family, precision) after an untimed run, keeps
    the fastest on the context and returns (threads, {threads: ms})."""
    h = _ctx_of(ctx)
    lib = load()
    choices = mc_thread_choices(precision)
    errors = []

    def cb(_user):
        try:
            run()
            return 0
        except Exception as e:  # reported after dp_autotune returns
            errors.append(e)
            return _lib.DP_ERR_STATE

    fn = _lib.AUTOTUNE_RUN(cb)
    best = C.c_int()
    ms = (C.c_double * len(choices))()
    rc = lib.dp_autotune(h, _FAMILY[family], _PRECISION[precision], fn, None, C.byref(best),
                         C.cast(ms, C.c_void_p), len(choices))
    if errors:
        raise errors[0]
    check(rc, h)
    return best.value, {t: ms[i] for i, t in enumerate(choices)}


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


# ----------------------------------------------------------------- materials
class Material:
    """Elemental recipe (src/Materials.jl BaseMaterial): elements as
    (Z, A, I[GeV], mass fraction)."""

    def __init__(self, name, density, I, elements, ZoA=0.0):
        self.name, self.density, self.I, self.ZoA = name, float(density), float(I), float(ZoA)
        self.elements = [tuple(map(float, e)) for e in elements]

    def to_c(self):
        arr = (DpElement * len(self.elements))(*[DpElement(*e) for e in self.elements])
        m = DpMaterial(self.name.encode(), self.density, self.I, self.ZoA, len(self.elements),
                       C.cast(arr, C.POINTER(DpElement)))
        return m, arr


# src/Materials.jl:35-127
_EL = {"H": (1.0, 1.00794, 19.2e-9), "C": (6.0, 12.0107, 78.0e-9), "N": (7.0, 14.0067, 82.0e-9),
       "O": (8.0, 15.9994, 95.0e-9), "Na": (11.0, 22.9898, 149.0e-9),
       "Mg": (12.0, 24.305, 156.0e-9), "Al": (13.0, 26.9815, 166.0e-9),
       "Si": (14.0, 28.0855, 173.0e-9), "K": (19.0, 39.0983, 190.0e-9),
       "Ca": (20.0, 40.078, 191.0e-9), "Fe": (26.0, 55.845, 286.0e-9),
       "Ar": (18.0, 39.948, 188.0e-9)}


def _recipe(name, density, I, comp):
    return Material(name, density, I, [(*_EL[s], f) for s, f in comp])


STANDARD_ROCK = _recipe("StandardRock", 2650.0, 136.4e-9,
                        [("O", 0.466), ("Si", 0.277), ("Al", 0.081), ("Fe", 0.050),
                         ("Ca", 0.036), ("Na", 0.028), ("Mg", 0.021), ("K", 0.026)])
AIR = _recipe("Air", 1.205, 85.7e-9, [("N", 0.755), ("O", 0.232), ("Ar", 0.013)])
WATER = _recipe("Water", 1000.0, 75.0e-9, [("H", 0.1119), ("O", 0.8881)])


# ----------------------------------------------------------------- physics
class Physics:
    """Device-resident physics tables (dp_physics)."""

    def __init__(self, handle, ctx, names, settings):
        self.h, self.ctx, self.names, self.settings = handle, ctx, list(names), settings
        n_mat, n = C.c_int(), C.c_int()
        load().dp_physics_info(self.h, C.byref(n_mat), C.byref(n))
        self.n_materials, self.n_energies = n_mat.value, n.value
        self.mass = settings.mass
        self.ctau = settings.ctau

    def __del__(self):
        try:
            if getattr(self, "h", None):
                load().dp_physics_free(self.h)
                self.h = None
        except Exception:
            pass

    @property
    def materials(self):
        return {n: i for i, n in enumerate(self.names)}

    def column(self, mat, col):
        out = np.zeros(self.n_energies)
        check(load().dp_physics_column(self.h, int(mat), COLUMNS.index(col), _ptr(out)),
              self.ctx.h)
        return out

    def table(self, mat):
        return {c: self.column(mat, c) for c in COLUMNS}


def _settings(mass=MUON_MASS, ctau=MUON_C_TAU, cutoff=DEFAULT_CUTOFF,
              elastic_ratio=DEFAULT_ELASTIC_RATIO):
    return DpSettings(mass, ctau, cutoff, elastic_ratio)


def create_physics(particle="MUON", *, n_energies=200, K_min=1e-3, K_max=1e9,
                   materials=(STANDARD_ROCK, AIR), cutoff=DEFAULT_CUTOFF,
                   elastic_ratio=DEFAULT_ELASTIC_RATIO, ctx=None):
    """create_physics (src/Physics.jl:534-599) with the empirical tables built
    on the host by libdpgpu, then uploaded to the device."""
    if particle != "MUON":
        raise ValueError("only MUON physics is provided")
    ctx = ctx or default_context()
    st = _settings(cutoff=cutoff, elastic_ratio=elastic_ratio)
    cs = [m.to_c() for m in materials]
    arr = (DpMaterial * len(cs))(*[c[0] for c in cs])
    h = C.c_void_p()
    check(load().dp_physics_create(ctx.h, C.byref(st), len(cs), C.cast(arr, C.c_void_p),
                                   n_energies, K_min, K_max, C.byref(h)), ctx.h)
    return Physics(h, ctx, [m.name for m in materials], st)


def _dedx_args(dedx_paths, materials):
    if len(dedx_paths) != len(materials):
        raise ValueError("one dE/dx file per material")
    cs = [m.to_c() for m in materials]
    arr = (DpMaterial * len(cs))(*[c[0] for c in cs])
    paths = (C.c_char_p * len(dedx_paths))(*[str(p).encode() for p in dedx_paths])
    return cs, arr, paths


def create_physics_dedx(dedx_paths, materials, *, cutoff=DEFAULT_CUTOFF,
                        elastic_ratio=DEFAULT_ELASTIC_RATIO, ctx=None):
    """create_physics with PUMAS dE/dx files (src/Physics.jl:146-273,
    src/DEDXLoader.jl:100-190): one file per material recipe, built on the
    host by libdpgpu and uploaded."""
    ctx = ctx or default_context()
    st = _settings(cutoff=cutoff, elastic_ratio=elastic_ratio)
    cs, arr, paths = _dedx_args(dedx_paths, materials)
    h = C.c_void_p()
    check(load().dp_physics_create_dedx(ctx.h, C.byref(st), len(cs), C.cast(arr, C.c_void_p),
                                        C.cast(paths, C.c_void_p), C.byref(h)), ctx.h)
    return Physics(h, ctx, [m.name for m in materials], st)


def tables_from_dedx(dedx_paths, materials, *, cutoff=DEFAULT_CUTOFF,
                     elastic_ratio=DEFAULT_ELASTIC_RATIO):
    """The dE/dx-file tables on the host only (no device): a list of dicts
    column name -> array, one per material."""
    st = _settings(cutoff=cutoff, elastic_ratio=elastic_ratio)
    cs, arr, paths = _dedx_args(dedx_paths, materials)
    n = C.c_int()
    lib = load()
    check(lib.dp_tables_from_dedx(C.byref(st), len(cs), C.cast(arr, C.c_void_p),
                                  C.cast(paths, C.c_void_p), C.byref(n), None, 0))
    cols = np.zeros((len(cs), len(COLUMNS), n.value))
    check(lib.dp_tables_from_dedx(C.byref(st), len(cs), C.cast(arr, C.c_void_p),
                                  C.cast(paths, C.c_void_p), C.byref(n), _ptr(cols), cols.size))
    return [{c: cols[m, k] for k, c in enumerate(COLUMNS)} for m in range(len(cs))]


def save_physics(physics, path):
    """Writes the portable table file (dp_physics_save)."""
    check(load().dp_physics_save(physics.h, str(path).encode()), physics.ctx.h)
    return path


def load_physics(path, ctx=None):
    """Reads a portable table file onto the device (dp_physics_load)."""
    ctx = ctx or default_context()
    lib = load()
    h = C.c_void_p()
    check(lib.dp_physics_load(ctx.h, str(path).encode(), C.byref(h)), ctx.h)
    st = DpSettings()
    check(lib.dp_physics_settings(h, C.byref(st)))
    n_mat = C.c_int()
    lib.dp_physics_info(h, C.byref(n_mat), None)
    names = []
    buf = C.create_string_buffer(1 << 16)
    for m in range(n_mat.value):
        k = lib.dp_physics_material_name(h, m, buf, len(buf))
        names.append(buf.value.decode() if k >= 0 else f"material{m + 1}")
    return Physics(h, ctx, names, st)


def upload_physics(tables, names, materials=None, *, mass=MUON_MASS, ctau=MUON_C_TAU,
                   cutoff=DEFAULT_CUTOFF, elastic_ratio=DEFAULT_ELASTIC_RATIO, ctx=None):
    """Uploads caller-built tables: `tables` is a list (one per material) of
    dicts column-name -> array on one shared energy grid."""
    ctx = ctx or default_context()
    n = len(tables[0]["E"])
    cols = np.zeros((len(tables), len(COLUMNS), n))
    for m, t in enumerate(tables):
        for c, name in enumerate(COLUMNS):
            if name in t:
                cols[m, c] = t[name]
        if "logE" not in t:
            cols[m, 1] = np.log(cols[m, 0])
    st = DpSettings(mass, ctau, cutoff, elastic_ratio)
    rec = None
    keep = []
    if materials is not None:
        cs = [m.to_c() for m in materials]
        keep.append(cs)
        rec = (DpMaterial * len(cs))(*[c[0] for c in cs])
    h = C.c_void_p()
    cols = np.ascontiguousarray(cols)
    check(load().dp_physics_upload(ctx.h, C.byref(st), len(tables), n, _ptr(cols),
                                   C.cast(rec, C.c_void_p) if rec is not None else None,
                                   C.byref(h)), ctx.h)
    return Physics(h, ctx, names, st)


def get_material_index(physics, name):
    """1-based like the reference (src/Physics.jl:609); -1 when absent."""
    i = physics.materials.get(name)
    return -1 if i is None else i + 1


# ----------------------------------------------------------------- backward MC
MCResult = namedtuple("MCResult", "flux sigma gradient gradient_flux gradient_method "
                                  "source_energy_max")


def _mc_params(physics, rock_thickness, rock_density, elevation, energy_min, energy_max,
               n_samples, compute_gradient, seed, straggling, scattering,
               energy_threshold_low, source_energy_max, primary_altitude, precision="fp64",
               porous_material=-1, porous_density=0.0, porous_thickness=0.0):
    """dp_mc_params; porous_material is 1-based like the reference's (<= 0: none)."""
    rock = physics.materials.get("StandardRock", 0)
    air = physics.materials.get("Air", physics.n_materials - 1)
    return DpMcParams(float(rock_thickness), float(rock_density), float(elevation),
                      float(energy_min), float(energy_max if energy_max is not None else energy_min),
                      int(n_samples), int(seed) & 0xFFFFFFFFFFFFFFFF, int(bool(straggling)),
                      int(bool(scattering)), int(bool(compute_gradient)),
                      float(energy_threshold_low),
                      float(source_energy_max) if source_energy_max is not None else 0.0,
                      float(primary_altitude), rock, air, PRECISION[precision],
                      int(porous_material) - 1 if porous_material > 0 else -1,
                      float(porous_density), float(porous_thickness))


def compute_flux(physics, rock_density, rock_thickness, elevation, energy_min, energy_max, *,
                 n_samples=1000, seed=42, straggling=True, scattering=True,
                 energy_threshold_low=100.0, porous_material=-1, porous_density=0.0,
                 porous_thickness=0.0, primary_altitude=PRIMARY_ALTITUDE, precision="fp64"):
    """compute_flux (src/Geometry.jl:899-929): (flux, sigma) of the backward MC
    estimate over the two-layer column, with the optional shallow porous
    layer (porous_material is a 1-based material index; <= 0 or zero
    thickness: none)."""
    p = _mc_params(physics, rock_thickness, rock_density, elevation, energy_min, energy_max,
                   n_samples, False, seed, straggling, scattering, energy_threshold_low, None,
                   primary_altitude, precision, porous_material, porous_density,
                   porous_thickness)
    out = DpMcResult()
    check(load().dp_backward_mc(physics.ctx.h, physics.h, C.byref(p), C.byref(out)),
          physics.ctx.h)
    return out.flux, out.sigma


def run_backward_mc(physics, *, rock_thickness=100.0, rock_density=2650.0, elevation=45.0,
                    energy_min=1.0, energy_max=None, n_samples=10000, compute_gradient=False,
                    seed=42, straggling=True, scattering=True, energy_threshold_low=100.0,
                    source_energy_max=None, primary_altitude=PRIMARY_ALTITUDE,
                    precision="fp64"):
    """run_backward_mc (src/Geometry.jl:1286-1338).  Samples are drawn from a
    Philox stream keyed by (seed, sample id); straggling/scattering select the
    stochastic dual-mode transport, else deterministic CSDA."""
    p = _mc_params(physics, rock_thickness, rock_density, elevation, energy_min, energy_max,
                   n_samples, compute_gradient, seed, straggling, scattering,
                   energy_threshold_low, source_energy_max, primary_altitude, precision)
    out = DpMcResult()
    check(load().dp_backward_mc(physics.ctx.h, physics.h, C.byref(p), C.byref(out)),
          physics.ctx.h)
    g = (out.gradient, out.gradient_flux, "deterministic_csda_sample_average") \
        if compute_gradient else (None, None, None)
    return MCResult(out.flux, out.sigma, g[0], g[1], g[2], out.source_energy_max)


def mc_samples(physics, *, energy_min=1.0, energy_max=None, n_samples=10000, seed=42):
    """The (energy, charge, weight) triples run_backward_mc draws."""
    p = _mc_params(physics, 0, 0, 0, energy_min, energy_max, n_samples, False, seed, False,
                   False, 100.0, None, PRIMARY_ALTITUDE)
    E, q, w = (np.zeros(n_samples) for _ in range(3))
    check(load().dp_mc_samples(physics.ctx.h, C.byref(p), n_samples, _ptr(E), _ptr(q), _ptr(w)),
          physics.ctx.h)
    return E, q, w


def csda_flux_samples(physics, energy, charge, weight, *, rock_thickness, rock_density,
                      elevation, source_energy_max=None, primary_altitude=PRIMARY_ALTITUDE,
                      energy_threshold_low=100.0, steps=False, precision="fp64"):
    """Per-history w*flux and w*d flux/d rho of the deterministic CSDA surrogate
    ("fp64": the reference's operations; "mixed": the FP32 walk with float-pair
    range and altitude, final energy and flux in FP64)."""
    E, q, w = _f64(energy), _f64(charge), _f64(weight)
    n = len(E)
    c, d = np.zeros(n), np.zeros(n)
    st = np.zeros(n, np.int32) if steps else None
    p = _mc_params(physics, rock_thickness, rock_density, elevation, 1.0, None, n, True, 0,
                   False, False, energy_threshold_low, source_energy_max, primary_altitude,
                   precision)
    check(load().dp_csda_flux_samples(physics.ctx.h, physics.h, C.byref(p), n, _ptr(E), _ptr(q),
                                      _ptr(w), _ptr(c), _ptr(d),
                                      _ptr(st) if st is not None else None), physics.ctx.h)
    return (c, d, st) if steps else (c, d)


def compute_flux_differentiable(physics, rock_density, rock_thickness, elevation, energy_final,
                                charge, *, source_energy_max=None):
    """compute_flux_differentiable (src/Geometry.jl:958-986), CSDA."""
    c, _ = csda_flux_samples(physics, [energy_final], [charge], [1.0],
                             rock_thickness=rock_thickness, rock_density=rock_density,
                             elevation=elevation, source_energy_max=source_energy_max)
    return float(c[0])


def compute_flux_gradient(physics, rock_density, rock_thickness, elevation, energy_final, charge,
                          *, source_energy_max=None):
    """compute_flux_gradient (src/Geometry.jl:1007-1028): (flux, d flux/d rho)."""
    c, d = csda_flux_samples(physics, [energy_final], [charge], [1.0],
                             rock_thickness=rock_thickness, rock_density=rock_density,
                             elevation=elevation, source_energy_max=source_energy_max)
    return float(c[0]), float(d[0])


def csda_direct_samples(physics, energy, charge, weight, *, rock_thickness, rock_density,
                        elevation, primary_altitude=PRIMARY_ALTITUDE, rock_material=None,
                        air_material=None):
    """compute_flux_csda_direct (src/Geometry.jl:1126-1209) per sample:
    (w*flux, w*d flux/d rho) arrays.  Materials are 1-based (default
    StandardRock and Air)."""
    E, q, w = _f64(energy), _f64(charge), _f64(weight)
    p = _mc_params(physics, rock_thickness, rock_density, elevation, 1.0, 1.0, len(E), False, 0,
                   False, False, 100.0, None, primary_altitude)
    if rock_material is not None:
        p.rock_material = int(rock_material) - 1
    if air_material is not None:
        p.air_material = int(air_material) - 1
    c, d = np.zeros(len(E)), np.zeros(len(E))
    check(load().dp_csda_direct_samples(physics.ctx.h, physics.h, C.byref(p), len(E), _ptr(E),
                                        _ptr(q), _ptr(w), _ptr(c), _ptr(d)), physics.ctx.h)
    return c, d


def compute_flux_csda_direct(physics, rock_material, air_material, rock_density, rock_thickness,
                             elevation, energy_initial, charge, *,
                             primary_altitude=PRIMARY_ALTITUDE):
    """compute_flux_csda_direct (src/Geometry.jl:1126-1209): the flux of one
    sample (1-based materials)."""
    c, _ = csda_direct_samples(physics, [energy_initial], [charge], [1.0],
                               rock_thickness=rock_thickness, rock_density=rock_density,
                               elevation=elevation, primary_altitude=primary_altitude,
                               rock_material=rock_material, air_material=air_material)
    return float(c[0])


def compute_flux_gradient_csda(physics, rock_density, rock_thickness, elevation, energy_final,
                               charge):
    """compute_flux_gradient_csda (src/Geometry.jl:1253-1276): (flux, d flux/d rho)
    of the closed-form CSDA flux (StandardRock and Air)."""
    c, d = csda_direct_samples(physics, [energy_final], [charge], [1.0],
                               rock_thickness=rock_thickness, rock_density=rock_density,
                               elevation=elevation)
    return float(c[0]), float(d[0])


# ----------------------------------------------------------------- stochastic MC
class MaterialMixture:
    """A prepared propagation medium: one material or a runtime mixture with
    mass fractions (src/Types.jl:357-376), together with its MIXED transport
    kernel (prepare_mixed_kernel, src/MixedTransport.jl:51-97).  materials
    are 1-based indices like the reference's."""

    def __init__(self, physics, materials, fractions=None):
        mats = np.ascontiguousarray(np.atleast_1d(materials).astype(np.int32) - 1)
        fr = _f64(np.ones(len(mats)) if fractions is None else np.atleast_1d(fractions))
        self.physics = physics
        self.materials = [int(m) + 1 for m in mats]
        self.fractions = [float(f) / float(fr.sum()) for f in fr] if fr.sum() > 0 else list(fr)
        self.h = C.c_void_p()
        check(load().dp_mixture_prepare(physics.ctx.h, physics.h, len(mats), _ptr(mats), _ptr(fr),
                                        C.byref(self.h)), physics.ctx.h)

    def __del__(self):
        try:
            if getattr(self, "h", None):
                load().dp_mixture_free(self.h)
                self.h = None
        except Exception:
            pass

    def kernel(self):
        """The MIXED kernel columns: energies, stopping, sigma, range, hazard,
        proper, and the onset energy."""
        n, onset = C.c_int(), C.c_double()
        load().dp_mixture_kernel(self.h, 0, None, 0, C.byref(n), C.byref(onset))
        out = {}
        for j, name in enumerate(("energies", "stopping", "sigma", "range", "hazard", "proper")):
            a = np.zeros(n.value)
            load().dp_mixture_kernel(self.h, j, _ptr(a), n.value, None, None)
            out[name] = a
        out["onset"] = onset.value
        return out


def prepare_mixed_kernel(physics, material):
    """prepare_mixed_kernel (src/MixedTransport.jl:51-97) of a 1-based material
    index or a MaterialMixture; returns the kernel columns."""
    m = material if isinstance(material, MaterialMixture) else MaterialMixture(physics, material)
    return m.kernel()


def _mc_config(seed, straggling, scattering, energy_threshold_low, source_energy_max, precision):
    return DpMcConfig(int(bool(straggling)), int(bool(scattering)), float(energy_threshold_low),
                      float(source_energy_max) if source_energy_max is not None else 0.0,
                      int(seed) & 0xFFFFFFFFFFFFFFFF, PRECISION[precision])


def mc_histories(physics, rock, air, energy, charge, weight, *, thickness, density, elevation,
                 primary_altitude=PRIMARY_ALTITUDE, seed=42, id0=0, straggling=True,
                 scattering=True, energy_threshold_low=100.0, source_energy_max=None,
                 precision="fp64"):
    """Explicit stochastic histories (compute_flux_single with an rng,
    src/Geometry.jl:694-757): per-history w*flux, status bits, step counts and
    final states (n x 4: energy, altitude, u_z, transport weight).  Geometry
    arguments are scalars or per-history arrays."""
    E, q, w = _f64(energy), _f64(charge), _f64(weight)
    n = len(E)
    geo = [np.atleast_1d(_f64(v)) for v in (thickness, density, elevation, primary_altitude)]
    stride = int(any(len(g) > 1 for g in geo))
    if stride:
        geo = [_f64(np.broadcast_to(g, (n,))) for g in geo]
    c, Ef = np.zeros(n), np.zeros((n, 4))
    st, ns = np.zeros(n, np.int32), np.zeros(n, np.int32)
    cfg = _mc_config(seed, straggling, scattering, energy_threshold_low, source_energy_max,
                     precision)
    check(load().dp_mc_histories(physics.ctx.h, physics.h, rock.h, air.h, C.byref(cfg), n, _ptr(E),
                                 _ptr(q), _ptr(w), _ptr(geo[0]), _ptr(geo[1]), _ptr(geo[2]),
                                 _ptr(geo[3]), stride, int(id0), _ptr(c), _ptr(st), _ptr(ns),
                                 _ptr(Ef)), physics.ctx.h)
    return c, st, ns, Ef


LOS_FIELDS = ("thickness", "thickness_max", "density", "density_max", "elevation",
              "elevation_max", "primary_altitude", "air_height", "energy_min", "energy_max",
              "n_samples", "porous_thickness", "porous_density")


def make_los(n_samples, *, thickness, density, elevation, energy_min, energy_max=None,
             thickness_max=0.0, density_max=0.0, elevation_max=0.0,
             primary_altitude=PRIMARY_ALTITUDE, air_height=0.0, porous_thickness=0.0,
             porous_density=0.0):
    """Array of dp_los records (arguments are scalars or arrays of one length);
    porous_thickness / porous_density describe the shallow porous layer that
    backward_mc_batch(porous=...) adds at the top of each rock column."""
    vals = dict(thickness=thickness, thickness_max=thickness_max, density=density,
                density_max=density_max, elevation=elevation, elevation_max=elevation_max,
                primary_altitude=primary_altitude, air_height=air_height, energy_min=energy_min,
                energy_max=energy_min if energy_max is None else energy_max, n_samples=n_samples,
                porous_thickness=porous_thickness, porous_density=porous_density)
    n = max(len(np.atleast_1d(v)) for v in vals.values())
    arr = (DpLos * n)()
    cols = {k: np.broadcast_to(np.atleast_1d(v), (n,)) for k, v in vals.items()}
    for i in range(n):
        for k in LOS_FIELDS:
            setattr(arr[i], k, int(cols[k][i]) if k == "n_samples" else float(cols[k][i]))
    return arr


def backward_mc_batch(physics, los, *, rock, air, seed=42, straggling=True, scattering=True,
                      energy_threshold_low=100.0, source_energy_max=None, precision="mixed",
                      compute_gradient=False, porous=None):
    """Batched stochastic backward MC over lines of sight (one persistent
    launch): per line of sight flux, sigma, n_samples, n_status_nonzero and,
    with compute_gradient, the CSDA surrogate's gradient_flux and gradient
    (d flux / d density of the line).  porous: a MaterialMixture for the
    shallow porous layer of each line (its porous_thickness and
    porous_density, src/Geometry.jl:617-635); no gradient then."""
    n = len(los)
    out = (DpLosResult * n)()
    cfg = _mc_config(seed, straggling, scattering, energy_threshold_low, source_energy_max,
                     precision)
    check(load().dp_mc_los_layers(physics.ctx.h, physics.h, rock.h,
                                  porous.h if porous is not None else None, air.h,
                                  C.byref(cfg), n, C.cast(los, C.c_void_p),
                                  int(bool(compute_gradient)), C.cast(out, C.c_void_p)),
          physics.ctx.h)
    keys = ("flux", "sigma", "n_samples", "n_status_nonzero") + \
        (("gradient", "gradient_flux") if compute_gradient else ())
    return {k: np.array([getattr(r, k) for r in out]) for k in keys}


from .directional import (CellSegment, DirBatch, DirectionalPath, DirMedia,  # noqa: E402
                          EnergySample,
                          CsdaBatch, MaterialConfig, SiteConfig, VoxelVolume, flat_surface,
                          precompute_paths, trace_path,
                          assemble_forward_and_jacobian,
                          build_cell_properties_for_mc, compute_directional_flux_csda,
                          compute_directional_flux_mc, csda_flux_batch,
                          directional_flux_and_grad_csda, directional_flux_mc_batch,
                          get_csda_correction, get_csda_material_correction,
                          mc_cell_mixture_and_density, sample_energy_set, set_csda_correction,
                          set_csda_material_correction)


from .inverse import (EdgePrior, SmoothnessPrior, apply_laplacian_smoothing,  # noqa: E402
                      edge_gradient, edge_hessian, gauss_newton_reconstruct,
                      gradient_descent_reconstruct, laplacian_gradient, make_csda_operator,
                      mlem_reconstruct, mse, prior_value, rmse, sart_reconstruct)
from .calibration import (calibrate_csda_correction,  # noqa: E402
                          calibrate_csda_material_correction, column_water_fraction,
                          csda_geom_multiplier, csda_material_multiplier, load_csda_corrections,
                          path_rock_length, save_csda_corrections)
from .directional import cell_density  # noqa: E402
from .topography import (ElevationMap, Terrain, TetraVolume,  # noqa: E402
                         compute_shallow_mask, ray_triangle_intersect, trace_tetra_paths)
from .uncertainty import (SystematicSourceResult, TransportUncertaintyResult,  # noqa: E402
                          TransportVariation, compute_flux_uncertainty,
                          estimate_transport_uncertainty, relative_uncertainty_percent)
from .posterior import (laplace_posterior, null_model_tests, profile_inventory,  # noqa: E402
                        profiled_log_observation_operator)


# ----------------------------------------------------------------- tomography
def csda_energy_quadrature(n, energy_min, energy_max):
    """Log-midpoint nodes with charge 0 and half weights (src/Tomography.jl:263-274)."""
    if n <= 0:
        raise ValueError("CSDA quadrature requires at least one energy node")
    if not (math.isfinite(energy_min) and math.isfinite(energy_max) and 0 < energy_min < energy_max):
        raise ValueError("CSDA quadrature requires finite 0 < energy_min < energy_max")
    lo = math.log(energy_min)
    span = math.log(energy_max) - lo
    E = np.array([math.exp(lo + span * (i - 0.5) / n) for i in range(1, n + 1)])
    return E, np.zeros(n), 0.5 * E * span




class VoxelGrid:
    """Regular density grid; cell c = i + nx*(j + ny*k) (x fastest)."""

    def __init__(self, nx, ny, nz, origin, pitch):
        self.nx, self.ny, self.nz = int(nx), int(ny), int(nz)
        self.origin = tuple(map(float, origin))
        self.pitch = tuple(map(float, pitch)) if np.ndim(pitch) else (float(pitch),) * 3

    @property
    def ncell(self):
        return self.nx * self.ny * self.nz

    def to_c(self):
        return DpGrid(self.nx, self.ny, self.nz, *self.origin, *self.pitch)


def make_rays(origins, zenith_deg, azimuth_deg):
    """Rays from detector points: direction (sin t sin p, sin t cos p, cos t)
    (the direction convention of examples/diff_flux_cube.jl:326-333)."""
    o = np.asarray(origins, np.float64).reshape(-1, 3)
    th, ph = np.deg2rad(np.asarray(zenith_deg, np.float64)), np.deg2rad(np.asarray(azimuth_deg, np.float64))
    r = np.zeros((len(o), 7))
    r[:, :3] = o
    st = np.sin(th)
    r[:, 3] = st * np.sin(ph)
    r[:, 4] = st * np.cos(ph)
    r[:, 5] = np.cos(th)
    r[:, 6] = np.cos(th)
    return r


class TomoModel:
    """Voxel-density CSDA forward model with its adjoint on one grid."""

    def __init__(self, physics, grid, nodes, *, rock="StandardRock", air="Air", side_cell=-1,
                 side_density=2650.0, primary_altitude=PRIMARY_ALTITUDE, precision="fp64"):
        self.physics, self.grid = physics, grid
        self.nE, self.nq, self.nw = (_f64(x) for x in nodes)
        self.params = DpTomoParams(physics.materials[rock], physics.materials[air],
                                   int(side_cell), float(side_density), float(primary_altitude),
                                   len(self.nE), _ptr(self.nE).value, _ptr(self.nq).value,
                                   _ptr(self.nw).value, PRECISION[precision])
        self._g = grid.to_c()

    def _args(self, rho, rays):
        rho = _f64(rho).ravel()
        if rho.size != self.grid.ncell:
            raise ValueError("density array does not match the grid")
        rays = _f64(rays).reshape(-1, 7)
        return rho, rays

    def forward(self, rho, rays):
        rho, rays = self._args(rho, rays)
        out = np.zeros(len(rays))
        check(load().dp_tomo_forward(self.physics.ctx.h, self.physics.h, C.byref(self._g),
                                     C.byref(self.params), _ptr(rho), len(rays), _ptr(rays),
                                     _ptr(out)), self.physics.ctx.h)
        return out

    def jacobian(self, rho, rays):
        """(flux, row_ptr, col, val): one entry per traversed segment (col -1:
        the side-exit remainder when its density is a fixed value)."""
        rho, rays = self._args(rho, rays)
        n = len(rays)
        flux = np.zeros(n)
        rp = np.zeros(n + 1, np.int64)
        cap = n * (self.grid.nx + self.grid.ny + self.grid.nz + 66)
        col = np.zeros(cap, np.int32)
        val = np.zeros(cap)
        nnz = C.c_int64()
        check(load().dp_tomo_jacobian(self.physics.ctx.h, self.physics.h, C.byref(self._g),
                                      C.byref(self.params), _ptr(rho), n, _ptr(rays), _ptr(flux),
                                      _ptr(rp), _ptr(col), _ptr(val), cap, C.byref(nnz)),
              self.physics.ctx.h)
        k = nnz.value
        return flux, rp, col[:k].copy(), val[:k].copy()

    def vjp(self, rho, rays, cot):
        """(flux, J^T cot) with a deterministic reduction."""
        rho, rays = self._args(rho, rays)
        cot = _f64(cot)
        flux = np.zeros(len(rays))
        grad = np.zeros(self.grid.ncell)
        check(load().dp_tomo_vjp(self.physics.ctx.h, self.physics.h, C.byref(self._g),
                                 C.byref(self.params), _ptr(rho), len(rays), _ptr(rays),
                                 _ptr(cot), _ptr(flux), _ptr(grad)), self.physics.ctx.h)
        return flux, grad


class TomoPaths:
    """Rays traced once into device-resident segment lists (dp_paths); every
    evaluation then works on device tensors (torch CUDA tensors, float64).
    This is the resident form used by iterative solvers and benchmarks."""

    def __init__(self, physics, grid, rays, nodes, *, rock="StandardRock", air="Air",
                 side_cell=-1, side_density=2650.0, primary_altitude=PRIMARY_ALTITUDE):
        import torch
        self.physics, self.grid = physics, grid
        dev = torch.device("cuda", physics.ctx.device)
        self.dev = dev
        rays = _f64(rays).reshape(-1, 7)
        self.n_rays = len(rays)
        self.rays = torch.tensor(rays.ravel(), dtype=torch.float64, device=dev)
        self.nodes = [torch.tensor(_f64(x), dtype=torch.float64, device=dev) for x in nodes]
        self.params = DpTomoParams(physics.materials[rock], physics.materials[air],
                                   int(side_cell), float(side_density), float(primary_altitude),
                                   len(nodes[0]), *(t.data_ptr() for t in self.nodes), 0)
        self._g = grid.to_c()
        h = C.c_void_p()
        torch.cuda.synchronize(dev)
        check(load().dp_tomo_paths_create_dev(physics.ctx.h, C.byref(self._g), self.n_rays,
                                              self.rays.data_ptr(), int(side_cell), C.byref(h)),
              physics.ctx.h)
        self.h = h
        n, nnz, mx = C.c_long(), C.c_int64(), C.c_int()
        load().dp_tomo_paths_info(self.h, C.byref(n), C.byref(nnz), C.byref(mx))
        self.nnz, self.max_segments = nnz.value, mx.value

    def __del__(self):
        try:
            if getattr(self, "h", None):
                load().dp_tomo_paths_free(self.h)
                self.h = None
        except Exception:
            pass

    def csr(self):
        rp = np.zeros(self.n_rays + 1, np.int64)
        col = np.zeros(max(self.nnz, 1), np.int32)
        ln = np.zeros(max(self.nnz, 1))
        load().dp_tomo_paths_csr(self.h, _ptr(rp), _ptr(col), _ptr(ln))
        return rp, col[:self.nnz], ln[:self.nnz]

    def eval_host(self, rho, cot=None, *, precision="mixed", nodes=None):
        """Host arrays in and out through dp_tomo_eval (copies inside the call)."""
        rho = _f64(rho).ravel()
        nE, nq, nw = (_f64(x) for x in (nodes or [t.cpu().numpy() for t in self.nodes]))
        self._host_nodes = (nE, nq, nw)
        p = DpTomoParams(self.params.rock_material, self.params.air_material,
                         self.params.side_cell, self.params.side_density,
                         self.params.primary_altitude, len(nE), _ptr(nE).value, _ptr(nq).value,
                         _ptr(nw).value, PRECISION[precision])
        flux = np.zeros(self.n_rays)
        grad = np.zeros(self.grid.ncell) if cot is not None else None
        cot = _f64(cot) if cot is not None else None
        check(load().dp_tomo_eval(self.physics.ctx.h, self.physics.h, self.h, C.byref(p),
                                  _ptr(rho), _ptr(cot) if cot is not None else None, _ptr(flux),
                                  _ptr(grad) if grad is not None else None, None),
              self.physics.ctx.h)
        return flux, grad

    def eval(self, rho, cot=None, *, precision="mixed", flux=None, grad=None, jac=None):
        """rho (and cot) are float64 CUDA tensors; returns (flux, grad|None, jac|None)."""
        import torch
        if flux is None:
            flux = torch.empty(self.n_rays, dtype=torch.float64, device=self.dev)
        if cot is not None and grad is None:
            grad = torch.empty(self.grid.ncell, dtype=torch.float64, device=self.dev)
        p = lambda t: t.data_ptr() if t is not None else None
        check(load().dp_tomo_eval_dev(self.physics.ctx.h, self.physics.h, self.h,
                                      C.byref(self.params), p(rho), p(cot), p(flux), p(grad),
                                      p(jac), PRECISION[precision]), self.physics.ctx.h)
        return flux, grad, jac

    def solve(self, obs, rho0, *, method="gn", n_iter=12, weight=None, cg_iter=10,
              relaxation=0.2, lm_damping=1e-3, box=(500.0, 3500.0), precision="mixed",
              prior_weight=0.0, smooth_strength=0.1, speculation=True, optimizer="pgd",
              relinearize=True, lr=None):
        """Inversion loop on the device (src/Tomography_inverse.jl): "sart"
        (sart_reconstruct, Jacobian re-evaluated per iterate), "gn"
        (gauss_newton_reconstruct with matrix-free CG), "mlem" (mlem_reconstruct
        on the model linearised at the iterate, A = -J) or "gd"
        (gradient_descent_reconstruct, optimizer "pgd", "adam" or "gd").
        relinearize=False linearises MLEM and GD once at rho0.  obs, weight and
        rho0 are float64 CUDA tensors; returns (rho, misfit history; NaN past
        an early stop)."""
        import torch
        from ._lib import DpSolveParams
        rho = rho0.clone()
        sp = DpSolveParams({"sart": 0, "gn": 1, "mlem": 2, "gd": 3}[method], int(n_iter),
                           int(cg_iter), PRECISION[precision], float(relaxation),
                           float(lm_damping), float(box[0]), float(box[1]), float(prior_weight),
                           float(smooth_strength), 0 if speculation else 1,
                           {"pgd": 0, "adam": 1, "gd": 2}[optimizer], 0 if relinearize else 1,
                           float(lr) if lr is not None else 0.0)
        hist = np.zeros(n_iter + 1)
        torch.cuda.synchronize(self.dev)
        check(load().dp_tomo_solve_dev(self.physics.ctx.h, self.physics.h, self.h,
                                       C.byref(self.params), obs.data_ptr(),
                                       weight.data_ptr() if weight is not None else None,
                                       rho.data_ptr(), C.byref(sp), _ptr(hist)),
              self.physics.ctx.h)
        return rho, hist
