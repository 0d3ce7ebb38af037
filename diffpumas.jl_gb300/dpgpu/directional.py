"""Fixed-path stochastic MC of src/Tomography.jl (compute_directional_flux_mc,
:826-1041) on libdpgpu: the reference's types and helpers for one direction,
and a batched form that runs many directions in one launch."""
import ctypes as C
import math
from collections import namedtuple

import numpy as np

from ._lib import DpDirBatch, DpLosResult, check, load

# src/Tomography.jl:179-223 (material indices are 1-based like the reference's)
MaterialConfig = namedtuple("MaterialConfig", "rock_material water_material air_material "
                            "porous_material rock_density water_density porous_density "
                            "porous_top_thickness")
SiteConfig = namedtuple("SiteConfig", "detector_elevation primary_altitude")
EnergySample = namedtuple("EnergySample", "energy charge weight")
CellSegment = namedtuple("CellSegment", "cell_idx distance")
DirectionalPath = namedtuple("DirectionalPath", "zenith azimuth segments distance_in_volume "
                             "surface_distance remaining_rock_distance surface_exit_z valid")


def is_shallow_porous(shallow, matcfg):
    """src/Tomography.jl:299-301."""
    return bool(shallow) and matcfg.porous_material > 0 and matcfg.porous_top_thickness > 0.0


def cell_density(w, shallow, matcfg):
    """Density of a cell with water mass fraction w, the CSDA model's form
    (src/Tomography.jl:295-302): specific volumes add."""
    if is_shallow_porous(shallow, matcfg):
        return 1.0 / (0.5 * (1.0 - w) / matcfg.porous_density +
                      0.5 * (1.0 - w) / matcfg.rock_density + w / matcfg.water_density)
    return 1.0 / ((1.0 - w) / matcfg.rock_density + w / matcfg.water_density)


def mc_cell_mixture_and_density(w, shallow, matcfg):
    """Mixture recipe ((materials, fractions)) and density of a cell with water
    mass fraction w (src/Tomography.jl:826-845): specific volumes add."""
    w = float(w)
    if is_shallow_porous(shallow, matcfg):
        porous = rock = 0.5 * (1.0 - w)
        recipe = ((matcfg.porous_material, matcfg.rock_material, matcfg.water_material),
                  (porous, rock, w))
        density = 1.0 / (porous / matcfg.porous_density + rock / matcfg.rock_density +
                         w / matcfg.water_density)
        return recipe, density
    if w <= 1e-12:
        return ((matcfg.rock_material,), (1.0,)), float(matcfg.rock_density)
    recipe = ((matcfg.rock_material, matcfg.water_material), (1.0 - w, w))
    return recipe, 1.0 / ((1.0 - w) / matcfg.rock_density + w / matcfg.water_density)


def build_cell_properties_for_mc(physics, shallow_flags, water_fractions, matcfg):
    """Per-cell prepared mixtures and densities (src/Tomography.jl:847-861);
    cells with the same (shallow, w) share one MaterialMixture."""
    from . import MaterialMixture
    cache = {}
    materials, densities = [], np.zeros(len(water_fractions))
    for i, (s, w) in enumerate(zip(shallow_flags, water_fractions)):
        key = (bool(s), float(w))
        if key not in cache:
            (mats, fr), rho = mc_cell_mixture_and_density(w, s, matcfg)
            cache[key] = (MaterialMixture(physics, list(mats), list(fr)), rho)
        materials.append(cache[key][0])
        densities[i] = cache[key][1]
    return materials, densities


def sample_energy_set(n_samples, energy_min, energy_max, seed):
    """Log-uniform final energies with weight k ln(E_max/E_min) and charges +-1
    (src/Tomography.jl:236-248, src/Pumas.jl:195-207).  The draws come from
    numpy's seeded generator, not Julia's MersenneTwister."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(int(n_samples)):
        if energy_max <= energy_min:
            kf, w = float(energy_min), 1.0
        else:
            rk = math.log(energy_max / energy_min)
            kf = energy_min * math.exp(rk * rng.random())
            w = kf * rk
        out.append(EnergySample(kf, 1.0 if rng.random() > 0.5 else -1.0, w))
    return out


class DirMedia:
    """A media set of fixed-path runs (dp_dir_media): the prepared media in the
    order given (the kernel stages the leading ones in shared memory)."""

    def __init__(self, physics, media):
        self.physics, self.media = physics, list(media)
        arr = (C.c_void_p * len(self.media))(*[m.h.value for m in self.media])
        self.h = C.c_void_p()
        check(load().dp_dir_media_create(physics.ctx.h, physics.h, len(self.media), arr,
                                         C.byref(self.h)), physics.ctx.h)

    def __del__(self):
        try:
            if getattr(self, "h", None):
                load().dp_dir_media_free(self.h)
                self.h = None
        except Exception:
            pass


class DirBatch:
    """A batch of directions prepared for dp_dir_mc: the paths' segment
    arrays, the media set (the rock first, the cell mixtures by use, the air
    last; the kernel stages the leading media in shared memory) and the
    samples (explicit EnergySample lists, or counts drawn on the device).
    run() passes host arrays; to_device() + run_dev() keep them resident."""

    def __init__(self, physics, matcfg, site, paths, cell_materials, cell_densities,
                 energy_samples=None, *, n_samples=None, energy_min=None, energy_max=None):
        from . import MaterialMixture
        self.physics = physics
        n = self.n_dirs = len(paths)
        cos_t = np.array([math.cos(math.radians(p.zenith)) for p in paths])
        valid = np.array([1 if (p.valid and c > 0.0) else 0 for p, c in zip(paths, cos_t)],
                         np.int32)
        if energy_samples is None:
            n_smp = np.broadcast_to(np.asarray(n_samples, np.int64), (n,)).copy()
        else:
            n_smp = np.array([len(s) for s in energy_samples], np.int64)
        seg_ptr = np.zeros(n + 1, np.int64)
        cells, lens = [], []
        for d, p in enumerate(paths):
            segs = p.segments if valid[d] else []
            seg_ptr[d + 1] = seg_ptr[d] + len(segs)
            cells.extend(int(s.cell_idx) - 1 for s in segs)
            lens.extend(float(s.distance) for s in segs)
        cells = np.array(cells, np.int64)
        use = {}
        for d in range(n):
            for c in cells[seg_ptr[d]:seg_ptr[d + 1]]:
                m = cell_materials[c]
                use[id(m)] = (m, use.get(id(m), (m, 0))[1] + int(n_smp[d]))
        rock = MaterialMixture(physics, matcfg.rock_material)
        air = MaterialMixture(physics, matcfg.air_material)
        self.media = [rock] + [m for m, _ in sorted(use.values(), key=lambda t: -t[1])] + [air]
        index = {id(m): k for k, m in enumerate(self.media)}
        self.arrays = {
            "cos_theta": cos_t,
            "remaining_rock": np.array([p.remaining_rock_distance for p in paths], np.float64),
            "air_distance": np.array([max(0.0, site.primary_altitude - p.surface_exit_z) /
                                      max(c, 1e-3) for p, c in zip(paths, cos_t)]),
            "valid": valid, "seg_ptr": seg_ptr,
            "seg_medium": np.array([index[id(cell_materials[c])] for c in cells], np.int32),
            "seg_density": np.array([cell_densities[c] for c in cells], np.float64),
            "seg_length": np.array(lens, np.float64),
            "sample_ptr": np.concatenate([[0], np.cumsum(n_smp)]).astype(np.int64)}
        if energy_samples is not None:
            flat = [s for ss in energy_samples for s in ss]
            for k, j in (("energy", 0), ("charge", 1), ("weight", 2)):
                self.arrays[k] = np.array([s[j] for s in flat], np.float64)
        self.energy_min = float(energy_min) if energy_min is not None else 0.0
        self.energy_max = float(energy_max) if energy_max is not None else 0.0
        self.total = int(self.arrays["sample_ptr"][-1])
        self.rock_density = float(matcfg.rock_density)
        self.detector_elevation = float(site.detector_elevation)
        self.set = DirMedia(physics, self.media)
        self.dev = None

    def _struct(self, ptr):
        B = DpDirBatch()
        B.n_dirs = self.n_dirs
        for k in ("cos_theta", "remaining_rock", "air_distance", "valid", "seg_ptr", "seg_medium",
                  "seg_density", "seg_length", "sample_ptr", "energy", "charge", "weight"):
            setattr(B, k, ptr(k))
        B.energy_min, B.energy_max = self.energy_min, self.energy_max
        B.rock_medium, B.air_medium = 0, len(self.media) - 1
        B.rock_density, B.detector_elevation = self.rock_density, self.detector_elevation
        return B

    def host_bytes(self):
        """Bytes of the batch arrays a host call copies to the device."""
        return sum(a.nbytes for a in self.arrays.values())

    def run(self, seed=42, *, straggling=True, energy_threshold_low=100.0, precision="mixed",
            return_histories=False):
        from . import _mc_config, _ptr
        B = self._struct(lambda k: self.arrays[k].ctypes.data if k in self.arrays else None)
        out = (DpLosResult * self.n_dirs)()
        n = max(self.total, 1)
        contrib, status, final = np.zeros(n), np.zeros(n, np.int32), np.zeros((n, 2))
        cfg = _mc_config(seed, straggling, False, energy_threshold_low, None, precision)
        ctx = self.physics.ctx.h
        h = return_histories
        rc = load().dp_dir_mc(ctx, self.physics.h, self.set.h, C.byref(B), C.byref(cfg),
                              C.cast(out, C.c_void_p), _ptr(contrib) if h else None,
                              _ptr(status) if h else None, _ptr(final) if h else None)
        res = {k: np.array([getattr(r, k) for r in out])
               for k in ("flux", "sigma", "n_samples", "n_status_nonzero")}
        if h:
            res["contrib"], res["status"] = contrib[:self.total], status[:self.total]
            res["final"] = final[:self.total]
        try:
            check(rc, ctx)
        except Exception as e:
            e.result = res  # the per-history records of a run that flagged histories
            raise
        return res

    def to_device(self):
        """Copies the batch arrays to torch device tensors (kept on self.dev)."""
        import torch
        dev = torch.device("cuda", self.physics.ctx.device)
        self.dev = {k: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
                    for k, a in self.arrays.items()}
        self.dev_out = torch.zeros(self.n_dirs * C.sizeof(DpLosResult), dtype=torch.uint8,
                                   device=dev)
        return self

    def run_dev(self, seed=42, *, straggling=True, energy_threshold_low=100.0,
                precision="mixed"):
        """Enqueues one run on the resident arrays; results stay in dev_out."""
        from . import _mc_config
        B = self._struct(lambda k: self.dev[k].data_ptr() if k in self.dev else None)
        cfg = _mc_config(seed, straggling, False, energy_threshold_low, None, precision)
        ctx = self.physics.ctx.h
        check(load().dp_dir_mc_dev(ctx, self.physics.h, self.set.h, C.byref(B), self.total,
                                   C.byref(cfg), self.dev_out.data_ptr()), ctx)

    def results_dev(self):
        raw = bytearray(self.dev_out.cpu().numpy().tobytes())
        out = (DpLosResult * self.n_dirs).from_buffer(raw)
        return {k: np.array([getattr(r, k) for r in out])
                for k in ("flux", "sigma", "n_samples", "n_status_nonzero")}


def directional_flux_mc_batch(physics, matcfg, site, paths, cell_materials, cell_densities,
                              energy_samples=None, seed=42, *, straggling=True,
                              energy_threshold_low=100.0, scattering=False, precision="mixed",
                              n_samples=None, energy_min=None, energy_max=None,
                              return_histories=False):
    """compute_directional_flux_mc over many directions in one launch.

    energy_samples: one list of EnergySample per path, or None to draw
    n_samples per path (an int or one per path) on the device from
    [energy_min, energy_max] (sample_energy_set semantics).  Returns flux,
    sigma (NaN for invalid paths), n_samples and n_status_nonzero per path;
    with return_histories also the per-sample 2 w_i w flux_i and status."""
    if scattering:
        raise ValueError("Fixed RayPath MC supports energy-loss fluctuations only; "
                         "use Geometry for scattered boundary retracing")
    b = DirBatch(physics, matcfg, site, paths, cell_materials, cell_densities, energy_samples,
                 n_samples=n_samples, energy_min=energy_min, energy_max=energy_max)
    return b.run(seed, straggling=straggling, energy_threshold_low=energy_threshold_low,
                 precision=precision, return_histories=return_histories)


def compute_directional_flux_mc(physics, matcfg, site, path, cell_materials, cell_densities,
                                energy_samples, seed, *, straggling, energy_threshold_low,
                                scattering=False, precision="fp64"):
    """(flux, sigma) of one direction (src/Tomography.jl:979-1041)."""
    if scattering:
        raise ValueError("Fixed RayPath MC supports energy-loss fluctuations only; "
                         "use Geometry for scattered boundary retracing")
    if not all(s.charge in (-1.0, 1.0) for s in energy_samples):
        raise ValueError("MC requires physical charges ±1; CSDA quadrature nodes are not MC "
                         "samples")
    r = directional_flux_mc_batch(physics, matcfg, site, [path], cell_materials, cell_densities,
                                  [list(energy_samples)], seed, straggling=straggling,
                                  energy_threshold_low=energy_threshold_low, precision=precision)
    return float(r["flux"][0]), float(r["sigma"][0])


# ---------------------------------------------------- water-fraction CSDA model
# The CSDA corrections (src/Tomography.jl:136-175): process-wide settings as
# in the reference, read by every evaluation.
CsdaCorrection = namedtuple("CsdaCorrection", "enabled kappa_strag kappa_hard resid_a resid_b "
                            "resid_c resid_d")
CsdaMaterialCorrection = namedtuple("CsdaMaterialCorrection", "enabled linear quadratic")
_CORRECTION = CsdaCorrection(False, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0)
_MATERIAL_CORRECTION = CsdaMaterialCorrection(False, 0.0, 0.0)


def set_csda_correction(*, enabled=True, kappa_strag=0.0, kappa_hard=0.0, resid_a=0.0,
                        resid_b=0.0, resid_c=0.0, resid_d=0.0):
    """set_csda_correction! (src/Tomography.jl:145-153)."""
    global _CORRECTION
    _CORRECTION = CsdaCorrection(bool(enabled), float(kappa_strag), float(kappa_hard),
                                 float(resid_a), float(resid_b), float(resid_c), float(resid_d))
    return _CORRECTION


def get_csda_correction():
    return _CORRECTION


def set_csda_material_correction(*, enabled=True, linear=0.0, quadratic=0.0):
    """set_csda_material_correction! (src/Tomography.jl:168-172)."""
    global _MATERIAL_CORRECTION
    if not (math.isfinite(linear) and math.isfinite(quadratic)):
        raise ValueError("nonfinite material coefficients")
    _MATERIAL_CORRECTION = CsdaMaterialCorrection(bool(enabled), float(linear), float(quadratic))
    return _MATERIAL_CORRECTION


def get_csda_material_correction():
    return _MATERIAL_CORRECTION


def _csda_config(matcfg, site):
    from ._lib import DpCsdaConfig
    c, m = _CORRECTION, _MATERIAL_CORRECTION
    return DpCsdaConfig(matcfg.rock_material - 1, matcfg.water_material - 1,
                        matcfg.air_material - 1,
                        matcfg.porous_material - 1 if matcfg.porous_material > 0 else -1,
                        float(matcfg.rock_density), float(matcfg.water_density),
                        float(matcfg.porous_density), float(matcfg.porous_top_thickness),
                        float(site.detector_elevation), float(site.primary_altitude),
                        int(c.enabled), c.kappa_strag, c.kappa_hard, c.resid_a, c.resid_b,
                        c.resid_c, c.resid_d, int(m.enabled), m.linear, m.quadratic)


class CsdaBatch:
    """Directions and energy samples prepared for dp_dir_csda (the segment
    arrays of every path, the shared EnergySample list).  run() evaluates a
    water-fraction field through host arrays; to_device() + run_dev() keep
    everything resident (torch CUDA tensors)."""

    def __init__(self, physics, shallow_flags, matcfg, site, paths, energy_samples):
        self.physics, self.n_bins = physics, len(paths)
        n = self.n_bins
        seg_ptr = np.zeros(n + 1, np.int64)
        seg_ptr[1:] = np.cumsum([len(p.segments) for p in paths])
        self.arrays = {
            "cos_theta": np.array([math.cos(math.radians(p.zenith)) for p in paths]),
            "remaining_rock": np.array([p.remaining_rock_distance for p in paths], np.float64),
            "surface_exit_z": np.array([p.surface_exit_z for p in paths], np.float64),
            "valid": np.array([1 if p.valid else 0 for p in paths], np.int32),
            "seg_ptr": seg_ptr,
            "seg_cell": np.array([s.cell_idx - 1 for p in paths for s in p.segments], np.int32),
            "seg_length": np.array([s.distance for p in paths for s in p.segments], np.float64),
            "energy": np.array([x.energy for x in energy_samples], np.float64),
            "charge": np.array([x.charge for x in energy_samples], np.float64),
            "weight": np.array([x.weight for x in energy_samples], np.float64),
            "shallow": np.ascontiguousarray(np.asarray(shallow_flags, bool).astype(np.uint8))}
        self.n_seg = int(seg_ptr[-1])
        self.n_energy = len(energy_samples)
        self.n_cells = len(self.arrays["shallow"])
        self.matcfg, self.site = matcfg, site
        self.dev = None

    @property
    def config(self):
        """dp_csda_config with the corrections in force at the call (the
        reference reads them at every evaluation)."""
        return _csda_config(self.matcfg, self.site)

    def _struct(self, ptr):
        from ._lib import DpCsdaBatch
        return DpCsdaBatch(self.n_bins, ptr("cos_theta"), ptr("remaining_rock"),
                           ptr("surface_exit_z"), ptr("valid"), ptr("seg_ptr"), ptr("seg_cell"),
                           ptr("seg_length"), self.n_energy, ptr("energy"), ptr("charge"),
                           ptr("weight"))

    def host_bytes(self):
        return sum(a.nbytes for a in self.arrays.values())

    def run(self, water_fractions, *, jacobian=True, precision="fp64"):
        """(flux per bin, d flux / d w per segment or None), host arrays.
        After to_device() the paths stay resident: only the water fractions
        go up and the results come back."""
        from . import PRECISION
        from . import _ptr
        if len(water_fractions) != self.n_cells:
            raise ValueError("water_fractions and shallow_flags differ in length")
        if self.dev is not None:
            import torch
            dev = self.dev["cos_theta"].device
            w_t = torch.from_numpy(np.ascontiguousarray(water_fractions, np.float64)).to(dev)
            torch.cuda.synchronize(dev)
            f_t = torch.zeros(max(self.n_bins, 1), dtype=torch.float64, device=dev)
            j_t = torch.zeros(max(self.n_seg, 1), dtype=torch.float64, device=dev) if jacobian \
                else None
            self.run_dev(w_t, f_t, j_t, precision=precision)
            check(load().dp_sync(self.physics.ctx.h), self.physics.ctx.h)
            return (f_t.cpu().numpy()[:self.n_bins],
                    j_t.cpu().numpy()[:self.n_seg] if jacobian else None)
        A = self.arrays
        B = self._struct(lambda k: A[k].ctypes.data if A[k].size else None)
        wf = np.ascontiguousarray(water_fractions, np.float64)
        flux = np.zeros(max(self.n_bins, 1))
        jac = np.zeros(max(self.n_seg, 1))
        ctx = self.physics.ctx.h
        cfg = self.config
        check(load().dp_dir_csda(ctx, self.physics.h, C.byref(cfg), C.byref(B),
                                 len(wf), _ptr(A["shallow"]), _ptr(wf), _ptr(flux),
                                 _ptr(jac) if jacobian else None, PRECISION[precision]), ctx)
        return flux[:self.n_bins], (jac[:self.n_seg] if jacobian else None)

    def to_device(self):
        import torch
        dev = torch.device("cuda", self.physics.ctx.device)
        self.dev = {k: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
                    for k, a in self.arrays.items()}
        return self

    def run_dev(self, water_fractions, flux, jac=None, precision="fp64"):
        """Enqueues one evaluation on resident arrays: water_fractions, flux
        (n_bins) and jac (n_seg, optional) are float64 CUDA tensors."""
        from . import PRECISION
        if water_fractions.numel() != self.n_cells or flux.numel() < self.n_bins or (
                jac is not None and jac.numel() < self.n_seg):
            raise ValueError("device arrays too small for the batch")
        B = self._struct(lambda k: self.dev[k].data_ptr() if self.dev[k].numel() else None)
        ctx = self.physics.ctx.h
        cfg = self.config
        check(load().dp_dir_csda_dev(ctx, self.physics.h, C.byref(cfg), C.byref(B),
                                     self.n_cells, self.dev["shallow"].data_ptr(),
                                     water_fractions.data_ptr(), flux.data_ptr(),
                                     jac.data_ptr() if jac is not None else None,
                                     PRECISION[precision]), ctx)


def csda_flux_batch(physics, shallow_flags, matcfg, site, paths, water_fractions,
                    energy_samples, *, jacobian=True, precision="fp64"):
    """The water-fraction CSDA flux of every path (compute_directional_flux_csda,
    src/Tomography.jl:667-727; NaN for invalid paths) in one launch, and with
    jacobian=True d flux / d w per segment (segment order, CSR offsets
    seg_ptr; summed over a cell's segments, the cell's Jacobian entry).
    Returns flux, seg_ptr, seg_cell (0-based), seg_jac."""
    b = CsdaBatch(physics, shallow_flags, matcfg, site, paths, energy_samples)
    flux, jac = b.run(water_fractions, jacobian=jacobian, precision=precision)
    return flux, b.arrays["seg_ptr"], b.arrays["seg_cell"], (jac if jacobian else
                                                             np.zeros(b.n_seg))


def compute_directional_flux_csda(physics, shallow_flags, matcfg, site, path, water_fractions,
                                  energy_samples):
    """Forward CSDA flux for one angular bin (src/Tomography.jl:667-727)."""
    f, _, _, _ = csda_flux_batch(physics, shallow_flags, matcfg, site, [path], water_fractions,
                                 energy_samples, jacobian=False)
    return float(f[0])


def directional_flux_and_grad_csda(physics, shallow_flags, matcfg, site, path, water_fractions,
                                   energy_samples):
    """(flux, cellids, values): the flux and d flux / d w of the cells the
    path crosses, 1-based cell ids in order of first crossing
    (src/Tomography.jl:736-762); (NaN, [], []) for an invalid path."""
    if not path.valid or math.cos(math.radians(path.zenith)) <= 0.0:
        return float("nan"), [], np.zeros(0)
    f, _, cells, jac = csda_flux_batch(physics, shallow_flags, matcfg, site, [path],
                                       water_fractions, energy_samples)
    ids, vals = [], []
    pos = {}
    for c, v in zip(cells, jac):
        if c not in pos:
            pos[c] = len(ids)
            ids.append(int(c) + 1)
            vals.append(0.0)
        vals[pos[c]] += v
    return float(f[0]), ids, np.array(vals)


def assemble_forward_and_jacobian(physics, shallow_flags, matcfg, site, paths, water_fractions,
                                  energy_samples, *, n_cells, threaded=True, precision="fp64"):
    """Forward flux of every bin and the sparse Jacobian J[bin, cell] =
    d flux / d w (src/Tomography.jl:773-820), one launch for all bins; entries
    that are zero or not finite are dropped as the reference drops them."""
    import scipy.sparse as sp
    flux, seg_ptr, cells, jac = csda_flux_batch(physics, shallow_flags, matcfg, site, paths,
                                                water_fractions, energy_samples,
                                                precision=precision)
    rows = np.repeat(np.arange(len(paths)), np.diff(seg_ptr))
    J = sp.coo_matrix((jac, (rows, cells)), shape=(len(paths), n_cells)).tocsc()
    J.sum_duplicates()
    J.data[~np.isfinite(J.data)] = 0.0
    J.eliminate_zeros()
    return flux, J


# ------------------------------------------------------------------ voxel paths
class VoxelVolume:
    """A voxel volume (examples/lvd_tomography.jl:181-187): increasing cell
    edges along x, y and z (metres, the detector at the origin), cells x
    fastest."""

    def __init__(self, x_edges, y_edges, z_edges, shallow_mask=None):
        self.x_edges, self.y_edges, self.z_edges = (np.ascontiguousarray(e, np.float64)
                                                    for e in (x_edges, y_edges, z_edges))
        self.nx, self.ny, self.nz = len(self.x_edges) - 1, len(self.y_edges) - 1, len(self.z_edges) - 1
        n = self.nx * self.ny * self.nz
        self.shallow_mask = np.zeros(n, bool) if shallow_mask is None else np.asarray(shallow_mask, bool)

    @property
    def n_cells(self):
        return self.nx * self.ny * self.nz


def flat_surface(height):
    """A flat surface `height` metres above the detector, in the role of
    ray_surface_exit_distance: (slant distance, valid, exit z)."""
    def surface(zenith, azimuth):
        c = math.cos(math.radians(zenith))
        if c <= 0.0:
            return float("nan"), False, float("nan")
        return height / c, True, float(height)
    return surface


def precompute_paths(volume, zeniths, azimuths, surface, ctx=None):
    """DirectionalPath of every (zenith, azimuth) pair, zeniths outer
    (examples/lvd_tomography.jl:694-779, 835-861): the reference's march
    through a VoxelVolume, or its walk through a TetraVolume, cut at the
    surface exit that `surface(zenith, azimuth) -> (slant distance, valid,
    exit z)` gives: flat_surface(h) for a flat overburden, or a Terrain
    (elevation map; required by a TetraVolume)."""
    from ._lib import DpVoxelVolume
    from . import _ptr
    from .topography import Terrain, TetraVolume, trace_tetra_paths
    h = ctx.h if ctx is not None else None  # host work: no device context needed
    pairs = [(float(t), float(p)) for t in zeniths for p in azimuths]
    n = len(pairs)
    zen = np.array([t for t, _ in pairs])
    az = np.array([p for _, p in pairs])
    if isinstance(volume, TetraVolume):
        if not isinstance(surface, Terrain):
            raise ValueError("a tetrahedral volume is traced against a Terrain")
        seg_ptr, cells, lens, trav, dist, rem, ez, ok = trace_tetra_paths(volume, surface, zen, az)
        out = []
        for d, (t, p) in enumerate(pairs):
            if not ok[d]:
                out.append(DirectionalPath(t, p, [], float("nan"), float("nan"), float("nan"),
                                           float("nan"), False))
                continue
            segs = [CellSegment(int(c), float(l)) for c, l in
                    zip(cells[seg_ptr[d]:seg_ptr[d + 1]], lens[seg_ptr[d]:seg_ptr[d + 1]])]
            out.append(DirectionalPath(t, p, segs, float(trav[d]), float(dist[d]), float(rem[d]),
                                       float(ez[d]), True))
        return out
    if isinstance(surface, Terrain):
        sd, sz, sok = surface.surface_exit(zen, az)
        surf = [(float(a), bool(o), float(b)) for a, b, o in zip(sd, sz, sok)]
    else:
        surf = [surface(t, p) for t, p in pairs]
    dist = np.array([s[0] if s[1] else float("nan") for s in surf])
    V = DpVoxelVolume(volume.nx, volume.ny, volume.nz, volume.x_edges.ctypes.data,
                      volume.y_edges.ctypes.data, volume.z_edges.ctypes.data)
    seg_ptr = np.zeros(n + 1, np.int64)
    trav, rem = np.zeros(max(n, 1)), np.zeros(max(n, 1))
    lib = load()
    check(lib.dp_voxel_trace(h, C.byref(V), n, _ptr(zen), _ptr(az), _ptr(dist), _ptr(seg_ptr),
                             None, None, 0, None, None), h)
    m = int(seg_ptr[-1])
    cells, lens = np.zeros(max(m, 1), np.int32), np.zeros(max(m, 1))
    check(lib.dp_voxel_trace(h, C.byref(V), n, _ptr(zen), _ptr(az), _ptr(dist), _ptr(seg_ptr),
                             _ptr(cells), _ptr(lens), m, _ptr(trav), _ptr(rem)), h)
    out = []
    for d, (t, p) in enumerate(pairs):
        if not surf[d][1] or not math.isfinite(dist[d]):
            out.append(DirectionalPath(t, p, [], float("nan"), float("nan"), float("nan"),
                                       float("nan"), False))
            continue
        segs = [CellSegment(int(c) + 1, float(l)) for c, l in
                zip(cells[seg_ptr[d]:seg_ptr[d + 1]], lens[seg_ptr[d]:seg_ptr[d + 1]])]
        out.append(DirectionalPath(t, p, segs, float(trav[d]), float(dist[d]), float(rem[d]),
                                   float(surf[d][2]), True))
    return out


def trace_path(volume, zenith, azimuth, surface):
    """trace_path(::VoxelVolume) (examples/lvd_tomography.jl:738-779)."""
    return precompute_paths(volume, [zenith], [azimuth], surface)[0]
