"""ctypes binding of the FP64 oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py.  The product (diffpumas.jl_gb300) never imports it.
"""
import ctypes as C
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_D = C.c_double
_I = C.c_int
_L = C.c_long
_P = C.c_void_p
_DP = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_IP = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")

MUON_MASS = 0.10565839
MUON_C_TAU = 658.654

# Column ids of a material table (oracle/capi.cpp column()).
COLUMNS = ["E", "logE", "csda_S", "csda_R", "csda_T", "mixed_S", "mixed_R", "strag",
           "ion", "brems", "pair", "photo", "xs", "lb1", "lbe", "elastic_cutoff",
           "magrot", "mu0", "fspin"]
BREMS, PAIR, PHOTO, IONI = 0, 1, 2, 3


def build():
    import subprocess
    subprocess.check_call(["make", "-s", "-C", HERE])


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_physics_new.restype = _P
        L.orc_physics_new.argtypes = [_D, _D, _D, _D]
        L.orc_physics_free.argtypes = [_P]
        L.orc_add_material_empirical.restype = _I
        L.orc_add_material_empirical.argtypes = [_P, C.c_char_p, _D, _D, _I, _DP, _DP, _DP, _DP,
                                                 _I, _D, _D, _I]
        L.orc_add_material_dedx.restype = _I
        L.orc_add_material_dedx.argtypes = [_P, C.c_char_p, C.c_char_p, _D, _D, _I, _DP, _DP,
                                            _DP, _DP, _I]
        L.orc_add_material_columns.restype = _I
        L.orc_add_material_columns.argtypes = [_P, C.c_char_p, _D, _D, _I, C.POINTER(C.POINTER(_D))]
        L.orc_table_size.restype = _I
        L.orc_table_size.argtypes = [_P, _I]
        L.orc_table_column.restype = _I
        L.orc_table_column.argtypes = [_P, _I, _I, _DP]
        L.orc_dcs.restype = _D
        L.orc_dcs.argtypes = [_I, _D, _D, _D, _D, _D, _D]
        L.orc_dcs_integral.restype = _D
        L.orc_dcs_integral.argtypes = [_I, _D, _D, _D, _D, _D, _D, _D, _I, _I]
        L.orc_dilog.restype = _D
        L.orc_dilog.argtypes = [_D]
        L.orc_flux_gccly.restype = _D
        L.orc_flux_gccly.argtypes = [_D, _D, _D]
        L.orc_electronic_stopping.restype = _D
        L.orc_electronic_stopping.argtypes = [C.c_char_p, _D, _D, _I, _DP, _DP, _DP, _DP, _D, _D]
        L.orc_lookup.restype = _D
        L.orc_lookup.argtypes = [_P, _I, _I, _D]
        L.orc_csda_energy.restype = _D
        L.orc_csda_energy.argtypes = [_P, _I, _D]
        L.orc_flux_single_csda.argtypes = [_P, _I, _I, _D, _D, _D, _D, _D, _D, _D,
                                           C.POINTER(_D), C.POINTER(_D), C.POINTER(_L)]
        L.orc_backward_mc_csda.argtypes = [_P, _I, _I, _D, _D, _D, _D, _D, _L, _DP, _DP, _DP,
                                           _DP, _DP, _I]
        L.orc_flux_csda_direct.argtypes = [_P, _I, _I, _D, _D, _D, _D, _D, _D,
                                           C.POINTER(_D), C.POINTER(_D)]
        L.orc_trace_ray.restype = _I
        L.orc_trace_ray.argtypes = [_IP, _DP, _DP, _I, _IP, _DP, C.POINTER(_D)]
        L.orc_tomo_forward.argtypes = [_P, _I, _I, _IP, _DP, _DP, _D, _D, _L, _DP, _I, _DP, _DP,
                                       _DP, _DP, _I]
        L.orc_tomo_vjp.argtypes = [_P, _I, _I, _IP, _DP, _DP, _D, _D, _L, _DP, _I, _DP, _DP, _DP,
                                   _DP, _DP, _DP, _I]
        L.orc_tomo_ray_grad.restype = _I
        L.orc_tomo_ray_grad.argtypes = [_P, _I, _I, _IP, _DP, _DP, _D, _D, _DP, _I, _DP, _DP,
                                        _DP, C.POINTER(_D), _I, _IP, _DP, C.POINTER(_D)]
        _U64 = C.c_uint64
        L.orc_mc_histories.argtypes = [_P, _I, _IP, _DP, _I, _L, _DP, _DP, _DP, _DP, _I, _DP, _DP,
                                       _DP, _U64, _U64, _I, _I, _D, _D, _DP, _IP,
                                       np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS"),
                                       _DP, _I, _I, _DP, _DP]
        _I64P = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
        L.orc_dir_histories.argtypes = [_P, _I, _IP, _IP, _DP, _I, _D, _I, _D, _L, _DP, _DP, _DP,
                                        _I64P, _IP, _DP, _DP, _I64P, _DP, _DP, _DP, _U64, _U64,
                                        _I, _D, _D, _DP, _IP, _I64P, _DP, _I]
        _U8P = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
        L.orc_dir_csda.argtypes = [_P, _IP, _DP, _DP, _DP, _L, _DP, _DP, _DP, _IP, _I64P, _IP,
                                   _DP, _L, _U8P, _DP, _I, _DP, _DP, _DP, _DP, C.c_void_p, _I]
        L.orc_mc_segment_step.restype = _D
        L.orc_mc_segment_step.argtypes = [_D, _D]
        L.orc_dir_segment.restype = _I
        L.orc_dir_segment.argtypes = [_P, _I, _IP, _DP, _DP, _D, _D, _I, _D, _D, _U64, _U64, _I,
                                      _DP, C.POINTER(_I)]
        L.orc_mixed_kernel.restype = _I
        L.orc_mixed_kernel.argtypes = [_P, _I, _IP, _DP, _I, _DP, C.POINTER(_D)]
        L.orc_mixed_step.restype = _I
        L.orc_mixed_step.argtypes = [_D, _D, _D, _I, _DP, _I, _DP, _D, _DP, _D, _D, _D, _U64,
                                     _U64, _I, _DP, C.POINTER(_I)]
        L.orc_reverse_del.restype = _I
        L.orc_reverse_del.argtypes = [_D, _D, _D, _I, _DP, _I, _DP, _D, _D, _I, _U64, _U64, _I,
                                      _DP, _DP, C.POINTER(_I)]
        _lib = L
    return _lib


def _arr(x):
    return np.ascontiguousarray(x, dtype=np.float64)


class Material:
    """Elemental recipe (src/Materials.jl BaseMaterial)."""

    def __init__(self, name, density, I, elements):
        self.name, self.density, self.I = name, float(density), float(I)
        self.Z = _arr([e[0] for e in elements])
        self.A = _arr([e[1] for e in elements])
        self.Iel = _arr([e[2] for e in elements])
        self.frac = _arr([e[3] for e in elements])


# src/Materials.jl:35-127 built-in recipes
_EL = {"H": (1.0, 1.00794, 19.2e-9), "C": (6.0, 12.0107, 78.0e-9), "N": (7.0, 14.0067, 82.0e-9),
       "O": (8.0, 15.9994, 95.0e-9), "Na": (11.0, 22.9898, 149.0e-9),
       "Mg": (12.0, 24.305, 156.0e-9), "Al": (13.0, 26.9815, 166.0e-9),
       "Si": (14.0, 28.0855, 173.0e-9), "K": (19.0, 39.0983, 190.0e-9),
       "Ca": (20.0, 40.078, 191.0e-9), "Fe": (26.0, 55.845, 286.0e-9),
       "Ar": (18.0, 39.948, 188.0e-9)}


def _mk(name, density, I, comp):
    return Material(name, density, I, [(*_EL[s], f) for s, f in comp])


STANDARD_ROCK = _mk("StandardRock", 2650.0, 136.4e-9,
                    [("O", 0.466), ("Si", 0.277), ("Al", 0.081), ("Fe", 0.050), ("Ca", 0.036),
                     ("Na", 0.028), ("Mg", 0.021), ("K", 0.026)])
AIR = _mk("Air", 1.205, 85.7e-9, [("N", 0.755), ("O", 0.232), ("Ar", 0.013)])
WATER = _mk("Water", 1000.0, 75.0e-9, [("H", 0.1119), ("O", 0.8881)])


class Physics:
    def __init__(self, mass=MUON_MASS, ctau=MUON_C_TAU, cutoff=0.05, elastic_ratio=0.05):
        self.h = lib().orc_physics_new(mass, ctau, cutoff, elastic_ratio)
        self.names = []

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_physics_free(self.h)
            self.h = None

    def add_empirical(self, m, n=200, Kmin=1e-3, Kmax=1e9, coulomb=False):
        self.names.append(m.name)
        return lib().orc_add_material_empirical(self.h, m.name.encode(), m.density, m.I,
                                                len(m.Z), m.Z, m.A, m.Iel, m.frac, n, Kmin, Kmax,
                                                int(coulomb))

    def add_dedx(self, path, m, coulomb=False):
        self.names.append(m.name)
        return lib().orc_add_material_dedx(self.h, path.encode(), m.name.encode(), m.density,
                                           m.I, len(m.Z), m.Z, m.A, m.Iel, m.frac, int(coulomb))

    def add_columns(self, name, density, ZoA, cols):
        """cols: dict column-name -> array (missing columns are zero)."""
        n = len(cols["E"])
        arrs = [_arr(cols.get(c, np.zeros(n))) for c in COLUMNS]
        if "logE" not in cols:
            arrs[1] = np.log(arrs[0])
        ptrs = (C.POINTER(_D) * 19)(*[a.ctypes.data_as(C.POINTER(_D)) for a in arrs])
        self._keep = getattr(self, "_keep", []) + [arrs]
        self.names.append(name)
        return lib().orc_add_material_columns(self.h, name.encode(), density, ZoA, n, ptrs)

    def column(self, mat, name):
        n = lib().orc_table_size(self.h, mat)
        out = np.zeros(n)
        lib().orc_table_column(self.h, mat, COLUMNS.index(name), out)
        return out

    def table(self, mat):
        return {c: self.column(mat, c) for c in COLUMNS}

    def lookup(self, mat, col, K):
        return lib().orc_lookup(self.h, mat, COLUMNS.index(col), K)


def default_physics(materials=(STANDARD_ROCK, AIR), n=200, Kmin=1e-3, Kmax=1e9, coulomb=False):
    """create_physics(MUON) with the empirical tables (src/Physics.jl:534)."""
    p = Physics()
    for m in materials:
        p.add_empirical(m, n, Kmin, Kmax, coulomb)
    return p


def dcs_integral(proc, Z, A, I, mass, K, xlo, xhi, mode, npoints=180):
    return lib().orc_dcs_integral(proc, Z, A, I, mass, K, xlo, xhi, mode, npoints)


def dcs(proc, Z, A, I, m, K, q):
    return lib().orc_dcs(proc, Z, A, I, m, K, q)


def flux_gccly(c, K, q):
    return lib().orc_flux_gccly(c, K, q)


def flux_single_csda(p, rock, air, thickness, rho, elevation, energy, charge,
                     threshold=1e9, primary_altitude=3e4):
    f, d, s = _D(), _D(), _L()
    lib().orc_flux_single_csda(p.h, rock, air, thickness, rho, elevation, energy, charge,
                               threshold, primary_altitude, C.byref(f), C.byref(d), C.byref(s))
    return f.value, d.value, s.value


def backward_mc_csda(p, rock, air, thickness, rho, elevation, E, q, w, threshold=1e9,
                     primary_altitude=3e4, threads=0):
    E, q, w = _arr(E), _arr(q), _arr(w)
    c, d = np.zeros(len(E)), np.zeros(len(E))
    threads = threads or os.cpu_count()
    lib().orc_backward_mc_csda(p.h, rock, air, thickness, rho, elevation, threshold,
                               primary_altitude, len(E), E, q, w, c, d, threads)
    return c, d


def flux_csda_direct(p, rock, air, rho, thickness, elevation, energy, charge, H=3e4):
    f, d = _D(), _D()
    lib().orc_flux_csda_direct(p.h, rock, air, rho, thickness, elevation, energy, charge, H,
                               C.byref(f), C.byref(d))
    return f.value, d.value


def trace_ray(dims, geom, ray, cap=4096):
    cells = np.zeros(cap, np.int32)
    lens = np.zeros(cap)
    z = _D()
    n = lib().orc_trace_ray(np.asarray(dims, np.int32), _arr(geom), _arr(ray), cap, cells, lens,
                            C.byref(z))
    return cells[:n].copy(), lens[:n].copy(), z.value


def tomo_forward(p, rock, air, dims, geom, rho, rho_side, rays, nodes, H=3e4, threads=0):
    rays = _arr(rays).reshape(-1, 7)
    out = np.zeros(len(rays))
    E, q, w = (_arr(x) for x in nodes)
    threads = threads or os.cpu_count()
    lib().orc_tomo_forward(p.h, rock, air, np.asarray(dims, np.int32), _arr(geom),
                           _arr(rho).ravel(), rho_side, H, len(rays), rays.ravel(), len(E), E, q,
                           w, out, threads)
    return out


def tomo_vjp(p, rock, air, dims, geom, rho, rho_side, rays, nodes, cot, H=3e4, threads=0):
    """Forward flux and J^T cot by the oracle's reverse sweep (all threads)."""
    rays = _arr(rays).reshape(-1, 7)
    flux = np.zeros(len(rays))
    rho = _arr(rho).ravel()
    grad = np.zeros(rho.size)
    E, q, w = (_arr(x) for x in nodes)
    threads = threads or os.cpu_count()
    lib().orc_tomo_vjp(p.h, rock, air, np.asarray(dims, np.int32), _arr(geom), rho, rho_side, H,
                       len(rays), rays.ravel(), len(E), E, q, w, _arr(cot), flux, grad, threads)
    return flux, grad


def tomo_ray_grad(p, rock, air, dims, geom, rho, rho_side, ray, nodes, H=3e4, cap=4096):
    E, q, w = (_arr(x) for x in nodes)
    cells = np.zeros(cap, np.int32)
    grads = np.zeros(cap)
    f, ds = _D(), _D()
    n = lib().orc_tomo_ray_grad(p.h, rock, air, np.asarray(dims, np.int32), _arr(geom),
                                _arr(rho).ravel(), rho_side, H, _arr(ray), len(E), E, q, w,
                                C.byref(f), cap, cells, grads, C.byref(ds))
    return f.value, cells[:n].copy(), grads[:n].copy(), ds.value


# ------------------------------------------------------------ stochastic MC
# History status bits (oracle/mc.hpp)
ST_STEP_CAP, ST_EVENT_CAP, ST_DOMAIN_HI, ST_DOMAIN_LO, ST_ZERO_RATE, ST_BAD_WEIGHT = (
    1, 4, 8, 16, 32, 64)


class Kernel:
    """Explicit MIXED transport kernel (src/MixedTransport.jl MixedKernel):
    columns E, stop, sigma, range, hazard, proper; elements (Z, A, I, fraction)."""

    def __init__(self, E, stop, sigma, range_, hazard, proper, elements=(), onset=math.inf,
                 mass=MUON_MASS, ctau=MUON_C_TAU, cutoff=0.05):
        self.cols = _arr(np.concatenate([_arr(c) for c in (E, stop, sigma, range_, hazard,
                                                            proper)]))
        self.n = len(E)
        self.el = _arr(np.array(elements, dtype=np.float64).reshape(-1, 4)).ravel()
        self.n_el = len(elements)
        self.onset, self.mass, self.ctau, self.cutoff = onset, mass, ctau, cutoff


STATE_FIELDS = ("E", "w", "t", "x", "y", "z", "ux", "uy", "uz", "dist", "X")


def _state(**kw):
    d = dict(E=0.0, w=1.0, t=0.0, x=0.0, y=0.0, z=0.0, ux=0.0, uy=0.0, uz=-1.0, dist=0.0, X=0.0)
    d.update(kw)
    return _arr([d[f] for f in STATE_FIELDS])


def mixed_step(kern, state, density, distance, energy_limit=-1.0, seed=0, id=0, script=None):
    """transport_mixed_step: returns (dict state, status, consumed script values)."""
    st = _state(**state) if isinstance(state, dict) else _arr(state).copy()
    sc = _arr(script if script is not None else [0.0])
    used = _I()
    status = lib().orc_mixed_step(kern.mass, kern.ctau, kern.cutoff, kern.n, kern.cols, kern.n_el,
                                  kern.el if kern.n_el else _arr([0.0]), kern.onset, st,
                                  density, distance, energy_limit, seed, id,
                                  -1 if script is None else len(script), sc, C.byref(used))
    return dict(zip(STATE_FIELDS, st)), status, used.value


def reverse_del(kern, k, details=False, seed=0, id=0, script=None):
    """reverse_del_event: returns (energy, weight, process, element, status, consumed)."""
    out = np.zeros(4)
    sc = _arr(script if script is not None else [0.0])
    used = _I()
    status = lib().orc_reverse_del(kern.mass, kern.ctau, kern.cutoff, kern.n, kern.cols,
                                   kern.n_el, kern.el if kern.n_el else _arr([0.0]), kern.onset, k,
                                   int(details), seed, id,
                                   -1 if script is None else len(script), sc, out, C.byref(used))
    return out[0], out[1], int(out[2]), int(out[3]), status, used.value


def dir_histories(p, media, rock, rock_density, air, detector_elevation, cos_theta,
                  remaining_rock, air_distance, seg_ptr, seg_medium, seg_density, seg_length,
                  smp_ptr, E, q, w, seed, id0=0, straggling=True, threshold_low=100.0,
                  energy_limit=1e9, threads=0):
    """Fixed-path MC histories (compute_directional_flux_mc,
    src/Tomography.jl:826-1041).  media: list of (materials, fractions).
    Returns (2 w_i w flux per history, status, steps, final energy)."""
    nm = np.array([len(m[0]) for m in media], np.int32)
    mats = np.zeros((len(media), 4), np.int32)
    fr = np.zeros((len(media), 4))
    for k, (ms, fs) in enumerate(media):
        mats[k, :len(ms)] = ms
        fr[k, :len(fs)] = fs
    i64 = lambda a: np.ascontiguousarray(a, np.int64)
    smp_ptr = i64(smp_ptr)
    n = int(smp_ptr[-1])
    contrib, Ef = np.zeros(n), np.zeros(n)
    status = np.zeros(n, np.int32)
    steps = np.zeros(n, np.int64)
    lib().orc_dir_histories(p.h, len(media), nm, mats.ravel(), fr.ravel(), rock, rock_density,
                            air, detector_elevation, len(cos_theta), _arr(cos_theta),
                            _arr(remaining_rock), _arr(air_distance), i64(seg_ptr),
                            np.ascontiguousarray(seg_medium, np.int32), _arr(seg_density),
                            _arr(seg_length), smp_ptr, _arr(E), _arr(q), _arr(w), seed, id0,
                            int(straggling), threshold_low, energy_limit, contrib, status, steps,
                            Ef, threads or os.cpu_count())
    return contrib, status, steps, Ef


def dir_csda(p, cfg, dens, site, corr, cos_t, rem, exit_z, valid, seg_ptr, seg_cell, seg_len,
             shallow, wf, E, q, ew, grad=False, threads=0):
    """Water-fraction CSDA flux per path (compute_directional_flux_csda,
    src/Tomography.jl:667-727) and optionally d flux/d w per segment (the
    derivative with respect to the segment's cell at its first segment on the
    path, 0 at repeats).  cfg: 0-based rock, water, air, porous indices; dens:
    rock, water, porous densities and porous top thickness; site: detector
    elevation, primary altitude; corr: 10 correction settings."""
    i32 = lambda a: np.ascontiguousarray(a, np.int32)
    seg_ptr = np.ascontiguousarray(seg_ptr, np.int64)
    n = len(cos_t)
    flux = np.zeros(n)
    g = np.zeros(max(int(seg_ptr[-1]), 1))
    lib().orc_dir_csda(p.h, i32(cfg), _arr(dens), _arr(site), _arr(corr), n, _arr(cos_t),
                       _arr(rem), _arr(exit_z), i32(valid), seg_ptr, i32(seg_cell), _arr(seg_len),
                       len(wf), np.ascontiguousarray(shallow, np.uint8), _arr(wf), len(E), _arr(E),
                       _arr(q), _arr(ew), flux, g.ctypes.data if grad else None,
                       threads or os.cpu_count())
    return (flux, g[:int(seg_ptr[-1])]) if grad else flux


def mc_segment_step(remaining, max_step):
    """_mc_segment_step (src/Tomography.jl:873-874) as the oracle applies it."""
    return lib().orc_mc_segment_step(remaining, max_step)


DIR_STATE = ("energy", "weight", "distance", "grammage", "z", "uz")


def dir_segment(p, mats, state, density, distance, *, fracs=None, straggling=True,
                threshold_low=100.0, energy_limit=1e9, seed=0, id=0, script=None):
    """propagate_mc_uniform_segment (src/Tomography.jl:876-920) of one medium:
    returns (final state dict, status, script values consumed)."""
    mats = np.atleast_1d(np.asarray(mats, np.int32))
    fr = _arr(fracs if fracs is not None else np.ones(len(mats)))
    st = _arr([state.get(k, d) for k, d in zip(DIR_STATE, (0.0, 1.0, 0.0, 0.0, 0.0, -1.0))])
    sc = _arr(script if script is not None else [0.0])
    status = C.c_int()
    used = lib().orc_dir_segment(p.h, len(mats), mats, fr, st, density, distance, int(straggling),
                                 threshold_low, energy_limit, seed, id,
                                 len(script) if script is not None else 0, sc,
                                 C.byref(status))
    return dict(zip(DIR_STATE, st)), status.value, used


def mixed_kernel(p, mats, fracs=None):
    """prepare_mixed_kernel (src/MixedTransport.jl:51-97) of a material or mixture."""
    mats = np.asarray(mats, np.int32)
    fracs = _arr(fracs if fracs is not None else np.ones(len(mats)))
    onset = _D()
    n = lib().orc_mixed_kernel(p.h, len(mats), mats, fracs, 0, np.zeros(1), C.byref(onset))
    cols = np.zeros(6 * n)
    lib().orc_mixed_kernel(p.h, len(mats), mats, fracs, n, cols, C.byref(onset))
    c = cols.reshape(6, n)
    return dict(E=c[0], stop=c[1], sigma=c[2], range=c[3], hazard=c[4], proper=c[5],
                onset=onset.value)


def mc_histories(p, rock, air, thickness, density, elevation, H, E, q, w, seed, id0=0,
                 straggling=True, scattering=True, threshold_low=100.0, source_max=1e9,
                 rock_fracs=None, threads=0, porous=-1, porous_thickness=0.0,
                 porous_density=0.0):
    """Stochastic backward histories (the dual-mode loop of src/Geometry.jl:534-757).

    rock: a material index or a list of indices (mixture with rock_fracs);
    porous >= 0: the shallow porous layer of that material (porous_thickness,
    porous_density); geometry arguments are scalars or per-history arrays.
    Returns (contribution w*f, status, steps, final energy) per history."""
    rock = np.atleast_1d(np.asarray(rock, np.int32))
    fr = _arr(rock_fracs if rock_fracs is not None else np.ones(len(rock)))
    E, q, w = _arr(E), _arr(q), _arr(w)
    n = len(E)
    geo = [_arr(np.atleast_1d(v)) for v in (thickness, density, elevation, H, porous_thickness,
                                            porous_density)]
    per = int(any(len(g) > 1 for g in geo))
    if per:
        geo = [_arr(np.broadcast_to(g, (n,))) for g in geo]
    contrib, Ef = np.zeros(n), np.zeros(n)
    status = np.zeros(n, np.int32)
    steps = np.zeros(n, np.int64)
    threads = threads or os.cpu_count()
    lib().orc_mc_histories(p.h, len(rock), rock, fr, air, n, geo[0], geo[1], geo[2], geo[3], per,
                           E, q, w, seed, id0, int(straggling), int(scattering), threshold_low,
                           source_max, contrib, status, steps, Ef, threads, int(porous), geo[4],
                           geo[5])
    return contrib, status, steps, Ef


# ----------------------------------------------------------------- Philox draws
# The counter-based generator (Philox4x32-10, Salmon et al., SC'11) that keys
# every history's stream by (seed, history id), vectorised over histories.
# Block 0 holds run_backward_mc's energy and charge draw (src/Pumas.jl:195-207,
# src/Geometry.jl:863-875: kf = E_min exp(rk u1), w = 2 kf rk, q = +-1 with
# probability 1/2); blocks 1-2 hold the per-history geometry that a line of
# sight with ranges draws (thickness and density from block 1, elevation from
# block 2), uniform on each range.
_M0, _M1, _W0, _W1, _MASK = 0xD2511F53, 0xCD9E8D57, 0x9E3779B9, 0xBB67AE85, 0xFFFFFFFF


def philox(ids, block, seed):
    ids = np.asarray(ids, np.uint64)
    c0, c1 = ids & _MASK, ids >> np.uint64(32)
    c2 = np.full_like(c0, block)
    c3 = np.zeros_like(c0)
    k0, k1 = np.uint64(seed & _MASK), np.uint64((seed >> 32) & _MASK)
    m0, m1, mask = np.uint64(_M0), np.uint64(_M1), np.uint64(_MASK)
    for _ in range(10):
        p0, p1 = m0 * c0, m1 * c2
        c0, c1, c2, c3 = ((p1 >> np.uint64(32)) ^ c1 ^ k0, p1 & mask,
                          (p0 >> np.uint64(32)) ^ c3 ^ k1, p0 & mask)
        k0 = (k0 + np.uint64(_W0)) & mask
        k1 = (k1 + np.uint64(_W1)) & mask
    return c0, c1, c2, c3


def u01(a, b):
    return ((a >> np.uint64(5)).astype(np.float64) * 67108864.0 +
            (b >> np.uint64(6)).astype(np.float64)) / 9007199254740992.0


def energy_draws(seed, ids, emin, emax):
    """(E, q, w) of histories `ids` (Philox block 0)."""
    x, y, z, w = philox(ids, 0, seed)
    rk = math.log(emax / emin)
    E = emin * np.exp(rk * u01(x, y))
    return E, np.where(u01(z, w) > 0.5, 1.0, -1.0), 2.0 * E * rk


def los_geometry_draws(seed, ids, thickness, thickness_max, density, density_max, elevation,
                       elevation_max):
    """Per-history (thickness, density, elevation) of a line of sight with
    ranges (Philox blocks 1 and 2)."""
    x1, y1, z1, w1 = philox(ids, 1, seed)
    x2, y2, _, _ = philox(ids, 2, seed)
    t = thickness + (thickness_max - thickness) * u01(x1, y1)
    r = density + (density_max - density) * u01(z1, w1)
    e = elevation + (elevation_max - elevation) * u01(x2, y2)
    return t, r, e
