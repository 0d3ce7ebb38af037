"""Seeded synthetic inputs of the benchmark configurations (no public dataset
is involved; every input is generated here from a seed).

tomography_c3 / tomography_c5: voxel density = smooth Gaussian random field
(FFT-filtered white noise, Gaussian covariance of the stated correlation
length) with spherical low-density cavities; detectors on the bottom face;
ray directions uniform in zenith and azimuth.
"""
import numpy as np

from . import VoxelGrid, csda_energy_quadrature, make_rays


def gaussian_random_field(shape, pitch, corr_length, mean, sd, rng):
    """Stationary field with covariance sd^2 exp(-r^2 / (2 corr_length^2))."""
    nz, ny, nx = shape
    white = rng.standard_normal(shape)
    kz = np.fft.fftfreq(nz, d=pitch) * 2 * np.pi
    ky = np.fft.fftfreq(ny, d=pitch) * 2 * np.pi
    kx = np.fft.rfftfreq(nx, d=pitch) * 2 * np.pi
    k2 = kz[:, None, None] ** 2 + ky[None, :, None] ** 2 + kx[None, None, :] ** 2
    # convolution with a Gaussian kernel of sd corr_length/sqrt(2) gives a
    # Gaussian covariance of sd corr_length
    s = corr_length / np.sqrt(2.0)
    spec = np.fft.rfftn(white, axes=(0, 1, 2)) * np.exp(-0.5 * k2 * s * s)
    field = np.fft.irfftn(spec, s=shape, axes=(0, 1, 2))
    field = (field - field.mean()) / field.std()
    return mean + sd * field


def density_field(nx, ny, nz, pitch, origin, *, seed, mean=2500.0, sd=150.0, corr_length=50.0,
                  n_cavities=3, cavity_density=1000.0, radius=(20.0, 40.0)):
    """Density on the grid as a (nz, ny, nx) array (x fastest when raveled)."""
    rng = np.random.default_rng(seed)
    rho = gaussian_random_field((nz, ny, nx), pitch, corr_length, mean, sd, rng)
    xs = origin[0] + (np.arange(nx) + 0.5) * pitch
    ys = origin[1] + (np.arange(ny) + 0.5) * pitch
    zs = origin[2] + (np.arange(nz) + 0.5) * pitch
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    rmax_fit = 0.45 * min(nx, ny, nz) * pitch
    for _ in range(n_cavities):
        r = min(rng.uniform(*radius), rmax_fit)
        c = [rng.uniform(origin[0] + r, origin[0] + nx * pitch - r),
             rng.uniform(origin[1] + r, origin[1] + ny * pitch - r),
             rng.uniform(origin[2] + r, origin[2] + nz * pitch - r)]
        rho[(X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2 <= r * r] = cavity_density
    return rho


def detector_rays(detectors, rays_per_detector, zenith_max, *, seed):
    rng = np.random.default_rng(seed)
    out = []
    for d in detectors:
        zen = rng.uniform(0.0, zenith_max, rays_per_detector)
        az = rng.uniform(0.0, 360.0, rays_per_detector)
        out.append(make_rays(np.tile(np.asarray(d, float), (rays_per_detector, 1)), zen, az))
    return np.concatenate(out)


def tomography_config(nx=64, ny=64, nz=32, pitch=10.0, n_detectors=4, rays_per_detector=1024,
                      n_nodes=32, seed=2024):
    """Voxel grid + density + rays + CSDA energy nodes (flux above 1 GeV).
    64x64x32 @ 10 m with 4 x 1024 rays is the batched forward+adjoint config;
    128x128x64 with 8 x 8192 rays the inversion-loop config."""
    origin = (-nx * pitch / 2, -ny * pitch / 2, 0.0)
    grid = VoxelGrid(nx, ny, nz, origin, pitch)
    rho = density_field(nx, ny, nz, pitch, origin, seed=seed)
    h = nx * pitch / 4
    if n_detectors == 4:
        dets = [(sx * h, sy * h, 0.0) for sx in (-1, 1) for sy in (-1, 1)]
    else:
        dets = [((i % 4 - 1.5) * h, (i // 4 - 0.5) * h, 0.0) for i in range(n_detectors)]
    rays = detector_rays(dets, rays_per_detector, 60.0, seed=seed + 1)
    nodes = csda_energy_quadrature(n_nodes, 1.0, 1e6)
    return grid, rho, rays, nodes


def voxel_walk(nx, ny, nz, origin, pitch, start, direction):
    """Cells (1-based, x fastest) and lengths of a ray from `start` through a
    voxel grid (exact cell-boundary walk), and the distance to the grid exit."""
    o = np.asarray(origin, float)
    p = np.asarray(start, float)
    u = np.asarray(direction, float)
    n = np.array([nx, ny, nz])
    # entry: the start is on or inside the grid
    cell = np.clip(np.floor((p - o) / pitch).astype(int), 0, n - 1)
    step = np.where(u > 0, 1, -1)
    with np.errstate(divide="ignore"):
        nxt = o + (cell + (u > 0)) * pitch
        t_max = np.where(u != 0, (nxt - p) / u, np.inf)
        t_delta = np.where(u != 0, pitch / np.abs(u), np.inf)
    t, segs = 0.0, []
    while True:
        a = int(np.argmin(t_max))
        t_next = float(t_max[a])
        if t_next > t:
            segs.append((int(cell[0] + nx * (cell[1] + ny * cell[2])) + 1, t_next - t))
        t = t_next
        cell[a] += step[a]
        if cell[a] < 0 or cell[a] >= n[a]:
            return segs, t
        t_max[a] += t_delta[a]


def directional_config(n_dirs=4096, nx=32, ny=32, nz=16, pitch=20.0, surface=600.0,
                       zenith_max=75.0, water_fraction=0.3, seed=2026):
    """Fixed-path MC directions in the manner of the reference's directional
    runs: a detector at the centre of the bottom face of a 640 m x 640 m x
    320 m voxel volume, directions uniform in zenith [0, zenith_max] and
    azimuth, cells of pure rock or of rock with the given water mass fraction
    (half each, seeded), rock beyond the volume up to a flat surface `surface`
    m above the detector.  Returns (paths as (zenith, azimuth, segments,
    in-volume distance, slant distance to the surface, remaining rock,
    surface exit z)), per-cell water fractions."""
    rng = np.random.default_rng(seed)
    origin = (-nx * pitch / 2, -ny * pitch / 2, 0.0)
    zen = np.degrees(np.arccos(rng.uniform(np.cos(np.radians(zenith_max)), 1.0, n_dirs)))
    az = rng.uniform(0.0, 360.0, n_dirs)
    out = []
    for z, a in zip(zen, az):
        th, ph = np.radians(z), np.radians(a)
        u = (np.sin(th) * np.sin(ph), np.sin(th) * np.cos(ph), np.cos(th))
        segs, t_exit = voxel_walk(nx, ny, nz, origin, pitch, (0.0, 0.0, 0.0), u)
        z_exit = t_exit * u[2]
        slant = surface / u[2]
        out.append((float(z), float(a), segs, t_exit, slant, max(0.0, slant - t_exit), surface))
    wf = np.where(rng.random(nx * ny * nz) < 0.5, water_fraction, 0.0)
    return out, wf
