"""The allocation-free tomography entry point, dp_tomo_eval_noalloc_dev.

Callers that may not allocate device memory during a call (a service with a
fixed device-memory budget, a plugin whose host process owns device memory
through its own pool) use this entry point: its Jacobian scratch is a fixed
array inside the library instead of the context's grow-on-demand scratch.
These tests call it through the C ABI and check it against the ordinary
mixed-precision entry point, dp_tomo_eval_dev, on two calls in a row (the
shared array keeps the previous call's contents, which must not leak into the
next result), with and without the adjoint, that the calls take no device
memory (neither the context's scratch nor the device's free memory moves),
and that oversized paths are refused.  The file sorts last so
that a run stopping at its first failure has run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(seed, rays_per_detector):
    import torch

    import dpgpu
    from dpgpu.workloads import tomography_config
    grid, rho, rays, nodes = tomography_config(seed=seed, rays_per_detector=rays_per_detector)
    phys = dpgpu.create_physics()
    paths = dpgpu.TomoPaths(phys, grid, rays, nodes, side_density=2500.0)
    dev = paths.dev
    t = lambda a: torch.tensor(np.ascontiguousarray(a, np.float64).ravel(), device=dev)
    return dpgpu, torch, phys, grid, paths, t(rho), t


def _noalloc(dpgpu, torch, phys, grid, paths, rho, cot, flux=None, grad=None):
    """One call; cot None evaluates the flux only (no adjoint, no grad)."""
    if flux is None:
        flux = torch.empty(paths.n_rays, dtype=torch.float64, device=paths.dev)
    if grad is None and cot is not None:
        grad = torch.empty(grid.ncell, dtype=torch.float64, device=paths.dev)
    ptr = lambda t: None if t is None else t.data_ptr()
    rc = dpgpu.load().dp_tomo_eval_noalloc_dev(phys.ctx.h, phys.h, paths.h, C.byref(paths.params),
                                               rho.data_ptr(), ptr(cot), flux.data_ptr(),
                                               ptr(grad))
    dpgpu.check(rc, phys.ctx.h)
    return flux.cpu().numpy(), None if grad is None else grad.cpu().numpy()


def test_noalloc_matches_allocating_entry_point_on_two_calls():
    dpgpu, torch, phys, grid, paths, rho, t = _setup(seed=31, rays_per_detector=512)
    rng = np.random.default_rng(5)
    for call in range(2):
        cot = t(rng.uniform(0.5, 1.5, paths.n_rays))
        f_ref, g_ref, _ = paths.eval(rho, cot, precision="mixed")
        f, g = _noalloc(dpgpu, torch, phys, grid, paths, rho, cot)
        # same kernels and the same summation order: equal to the mixed-precision
        # entry point within the tests' floating-point tolerance (bitwise in practice)
        np.testing.assert_allclose(f, f_ref.cpu().numpy(), rtol=1e-12, atol=0)
        np.testing.assert_allclose(g, g_ref.cpu().numpy(), rtol=1e-12,
                                   atol=1e-12 * np.abs(g_ref.cpu().numpy()).max())
        assert np.all(f > 0) and np.any(g != 0)


def test_noalloc_flux_only_and_takes_no_device_memory():
    """The flux-only form (no cotangent, no J^T r) equals the allocating
    entry point's flux on two calls in a row, and neither form of the call
    takes device memory: the context's scratch and the device's free memory
    are the same before and after each call.  Both kernels of the allocating
    path run first, so that the driver has loaded them and sized their local
    memory before the memory is read."""
    dpgpu, torch, phys, grid, paths, rho, t = _setup(seed=17, rays_per_detector=256)
    lib = dpgpu.load()
    rng = np.random.default_rng(9)
    cot = t(rng.uniform(0.5, 1.5, paths.n_rays))
    paths.eval(rho, cot, precision="mixed")
    f_ref = paths.eval(rho, None, precision="mixed")[0].cpu().numpy()
    flux = torch.empty(paths.n_rays, dtype=torch.float64, device=paths.dev)
    grad = torch.empty(grid.ncell, dtype=torch.float64, device=paths.dev)
    torch.cuda.synchronize()
    held = lib.dp_scratch_bytes(phys.ctx.h)
    free = torch.cuda.mem_get_info(paths.dev)[0]
    for call in range(2):
        f, g = _noalloc(dpgpu, torch, phys, grid, paths, rho, None, flux=flux)
        assert g is None
        np.testing.assert_allclose(f, f_ref, rtol=1e-12, atol=0)
        _noalloc(dpgpu, torch, phys, grid, paths, rho, cot, flux=flux, grad=grad)
        torch.cuda.synchronize()
        assert lib.dp_scratch_bytes(phys.ctx.h) == held
        assert torch.cuda.mem_get_info(paths.dev)[0] == free


def test_noalloc_refuses_paths_beyond_its_fixed_scratch():
    import dpgpu
    from dpgpu.workloads import tomography_config
    grid, rho, rays, nodes = tomography_config(nx=128, ny=128, nz=64, n_detectors=8,
                                               rays_per_detector=8192, seed=3)
    phys = dpgpu.create_physics()
    paths = dpgpu.TomoPaths(phys, grid, rays, nodes, side_density=2500.0)
    assert paths.nnz > 2 ** 21
    import torch
    t = lambda a: torch.tensor(np.ascontiguousarray(a, np.float64).ravel(), device=paths.dev)
    with pytest.raises(ValueError, match="fixed scratch"):
        _noalloc(dpgpu, torch, phys, grid, paths, t(rho), t(np.ones(paths.n_rays)))
