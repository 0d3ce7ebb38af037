"""Benchmark of the DiffPumas.jl hot path on GB300 through libdpgpu.

python bench.py [--gpus N] [--steps K] [--warmup W] [--workload c2|c3|c1] [--impl gpu|reference]

Workloads (seeded synthetic inputs):
  c2  (default) straggled backward MC with DEL/EHS hard events and Coulomb
      scattering through a runtime rock/water/air mixture (0.70/0.25/0.05)
      under 1 km of air; per-history thickness, density and elevation drawn
      on the device; 10^6 histories per step, FP32 transport with FP64
      positions, kinematics and compensated tally.  Unit: samples/s.
  c3  batched tomography forward + adjoint: 64x64x32 voxel grid at 10 m,
      smooth random density field with 3 cavities, 4 detectors x 1024 rays,
      32 CSDA energy nodes on [1, 1e6] GeV.  One step = per-ray flux and the
      density vector-Jacobian product J^T r over all rays.  Unit: rays/s.
  dir fixed-path stochastic MC (compute_directional_flux_mc): 4096
      directions x 1024 histories through a voxel volume of rock and
      rock+water cells, rock to the surface and air above; energies
      1e-3 - 1e9 GeV drawn on the device.  Unit: samples/s.
  wcsda water-fraction CSDA flux + sparse d flux/d w (the Tomography
      forward model and Jacobian) over the dir workload's 4096 directions,
      32 CSDA nodes.  Unit: rays/s.
  c1  backward MC, CSDA mode, StandardRock 2650 kg/m^3, 100 m, 45 deg,
      energies log-uniform 1-100 GeV, +-1 charges, 10^4 histories, with the
      density gradient.  One step = one run_backward_mc estimate.  Unit:
      samples/s.

The --impl reference arm times the CPU implementation of the same path (the
FP64 oracle restating the reference's Julia code, which cannot run here) on
all host cores.  Multi-GPU: the path has no exchange step, N ranks run
independent replicas (weak scaling).
"""
import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "diffpumas.jl_gb300"))

import numpy as np  # noqa: E402

METRIC = "MC samples/s & tomography rays/s (+dflux/drho) vs plain GPU at <=1e-4 rel err"
L2_BYTES = 129 * 2 ** 20


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return d["hbm_gbs"], "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except Exception:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, x):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------ workloads
def setup_c3(dp, torch, dev, precision="mixed"):
    from dpgpu.workloads import tomography_config
    grid, rho, rays, nodes = tomography_config()
    phys = dp.create_physics()
    model = dp.TomoModel(phys, grid, nodes, side_density=2500.0, precision=precision)
    cot = np.random.default_rng(1).uniform(0.5, 1.5, len(rays))
    paths = dp.TomoPaths(phys, grid, rays, nodes, side_density=2500.0)
    nseg = paths.nnz
    T = lambda a: torch.tensor(np.ascontiguousarray(a).ravel(), dtype=torch.float64, device=dev)
    d = {"rho": T(rho), "cot": T(cot),
         "flux": torch.zeros(len(rays), dtype=torch.float64, device=dev),
         "grad": torch.zeros(grid.ncell, dtype=torch.float64, device=dev)}
    lib = dp.load()

    def step_dev():
        paths.eval(d["rho"], d["cot"], precision=precision, flux=d["flux"], grad=d["grad"])

    h_flux = np.zeros(len(rays))
    h_grad = np.zeros(grid.ncell)
    rho_h, rays_h, cot_h = (np.ascontiguousarray(a, np.float64).ravel() for a in (rho, rays, cot))
    g = grid.to_c()
    nE, nq, nw = (np.ascontiguousarray(x, np.float64) for x in nodes)
    tp = dp.DpTomoParams(paths.params.rock_material, paths.params.air_material,
                         paths.params.side_cell, paths.params.side_density,
                         paths.params.primary_altitude, len(nE), nE.ctypes.data, nq.ctypes.data,
                         nw.ctypes.data, dp.PRECISION[precision])
    hp = lambda a: a.ctypes.data_as(C.c_void_p)

    def step_e2e():
        # reference-facing C ABI call with host buffers (dp_tomo_eval): rho and
        # r in, flux and J^T r out, copies inside the call (rays traced once
        # beforehand, as precompute_paths does)
        dp.check(lib.dp_tomo_eval(phys.ctx.h, phys.h, paths.h, C.byref(tp), hp(rho_h), hp(cot_h),
                                  hp(h_flux), hp(h_grad), None), phys.ctx.h)

    def plain_dev():
        dp.check(lib.dp_tomo_forward_plain_dev(phys.ctx.h, phys.h, C.byref(g),
                                               C.byref(paths.params), d["rho"].data_ptr(),
                                               len(rays), paths.rays.data_ptr(),
                                               d["flux"].data_ptr()), phys.ctx.h)

    n_rays = len(rays)
    # algorithmic bytes of the adjoint kernel per launch: per ray the row
    # pointers (16 B), cos theta (8 B) and the flux written (8 B); per
    # traversed segment the cell id (4 B), length (8 B), density gather (8 B)
    # and the Jacobian value written (4 B in mixed precision, 8 B in FP64).
    jb = 4 if precision == "mixed" else 8
    alg = n_rays * (16 + 8 + 8) + nseg * (4 + 8 + 8 + jb)
    # DRAM read+write bytes of one tomo_adjoint launch on this workload, from an
    # ncu capture of the kernel on this workload
    traffic = 3494400 if precision == "mixed" else None
    info = {"units": n_rays, "unit": "rays/s", "kernel": "tomo_adjoint", "alg_bytes": alg,
            "dominant": "tomo_adjoint", "dominant_bytes": alg,
            "traffic": traffic,
            "config": {"workload": "c3: tomography forward + adjoint, 64x64x32 @ 10 m, 4x1024 rays, "
                                   "32 energy nodes [1,1e6] GeV, flux + J^T r per step",
                       "grid": [64, 64, 32], "rays": n_rays, "energy_nodes": 32,
                       "segments": nseg, "precision": precision,
                       "paths": "traced once (resident), as precompute_paths does"},
            "h2d": 8 * (rho_h.size + cot_h.size + 3 * len(nodes[0])),
            "d2h": 8 * (n_rays + grid.ncell)}
    return step_dev, step_e2e, plain_dev, info, phys


def bench_checks():
    """FP64 oracle fluxes of the c2 and c4 workloads on the bench's own streams
    (written by tests/golden/make_bench_checks.py)."""
    with open(os.path.join(ROOT, "tests", "golden", "bench_checks.json")) as f:
        return json.load(f)


def los_results(dp, d_out, n):
    raw = d_out.cpu().numpy().tobytes()
    k = C.sizeof(dp.DpLosResult)
    return [dp.DpLosResult.from_buffer_copy(raw[i * k:(i + 1) * k]) for i in range(n)]


def _device_bytes(torch, dev, obj):
    raw = bytearray(C.string_at(C.addressof(obj), C.sizeof(obj)))
    return torch.frombuffer(raw, dtype=torch.uint8).to(dev)


C2_MIX = ([1, 3, 2], [0.70, 0.25, 0.05])  # rock, water, air (1-based material indices)
# Issue figures of the dominant transport kernels, from ncu captures of small
# cases of the same kernels (the bound that binds them: instruction issue)
# Issue-slot figures of the dominant kernels, from the ncu captures of the
# same builds (reduced cases of each workload; the launch tails weigh more there)
C2_ISSUE = {"issue_active": 0.4391, "lanes_per_inst": 18.17,
            "source": "ncu smsp__issue_active and smsp__thread_inst_executed_per_inst_executed, "
                      "mc_kernel<float,0,1024> (phase 0, lockstep, tables through L1/L2) on a "
                      "5e5-history c2 case"}
C4_ISSUE = {"issue_active": 0.3864, "lanes_per_inst": 21.21,
            "source": "ncu, mc_kernel<float,1,1024> (mc_mixed_hi, lockstep) on 819 of the c4 lines "
                      "(443,846 histories)"}
C1_ISSUE = {"issue_active": 0.206, "lanes_per_inst": 15.88,
            "source": "ncu, csda32_kernel on the c1 workload (one warp per scheduler, bound by "
                      "the dependent steps of each warp's longest history)"}


def c2_los(dp, n):
    return dp.make_los(n, thickness=20.0, thickness_max=500.0, density=2000.0, density_max=2800.0,
                       elevation=30.0, elevation_max=90.0, air_height=1000.0, energy_min=1.0,
                       energy_max=1e4)


def setup_c2(dp, torch, dev, precision="mixed", scale=1.0):
    """Straggled backward MC with DEL/EHS events and Coulomb scattering below
    100 GeV, mixed above, through rock (runtime mixture rock/water/air
    0.70/0.25/0.05) under 1 km of air; per history thickness U[20,500] m,
    density U[2000,2800] kg/m^3, elevation U[30,90] deg drawn on the device;
    final energies log-uniform 1 GeV - 10 TeV, +-1 charges; 10^6 histories."""
    phys = dp.create_physics(materials=(dp.STANDARD_ROCK, dp.AIR, dp.WATER))
    mix = dp.MaterialMixture(phys, *C2_MIX)
    air = dp.MaterialMixture(phys, 2)
    n = max(1, int(1_000_000 * scale))
    los = c2_los(dp, n)
    lib = dp.load()
    ctx = phys.ctx.h
    cfgs = {p: dp._mc_config(2026, True, True, 100.0, None, p) for p in ("mixed", "fp64")}
    d_los = _device_bytes(torch, dev, los)
    d_out = torch.zeros(C.sizeof(dp.DpLosResult), dtype=torch.uint8, device=dev)
    # the plain FP64 form runs a tenth of the histories (its rate per history
    # does not depend on their number)
    n_plain = max(1, n // 10)
    d_los_plain = _device_bytes(torch, dev, c2_los(dp, n_plain))

    def run_dev(p, nn=n, d=d_los):
        dp.check(lib.dp_mc_los_dev(ctx, phys.h, mix.h, air.h, C.byref(cfgs[p]), 1, d.data_ptr(),
                                   nn, 0, d_out.data_ptr()), ctx)

    def step_e2e():
        r = dp.backward_mc_batch(phys, los, rock=mix, air=air, seed=2026, precision=precision)
        assert r["n_status_nonzero"][0] == 0

    def check():
        # the step's answer against the FP64 oracle on the first 2e5 of the same
        # streams (statistical: the two estimates share those histories)
        torch.cuda.synchronize()
        r = los_results(dp, d_out, 1)[0]
        ref = bench_checks()["c2"]
        z = (r.flux - ref["flux"]) / math.hypot(r.sigma, ref["sigma"])
        assert r.n_status_nonzero == 0 and abs(z) < 3, (r.flux, r.sigma, ref)
        return {"flux": r.flux, "sigma": r.sigma, "oracle_flux": ref["flux"],
                "oracle_sigma": ref["sigma"], "oracle_histories": ref["n_histories"], "z": z,
                "pass": True}

    kernel = ("mc_init+mc_mixed_lo+mc_mixed_hi+mc_finish+mc_tally" if precision == "mixed"
              else "mc_init+mc_fp64_lo+mc_fp64_hi+mc_finish+mc_tally")
    info = {"units": n, "unit": "samples/s", "kernel": kernel, "family": "mc",
            **({"check": check} if scale == 1.0 else {}),
            # per history: contribution (8 B) and status (4 B) written by the
            # transport kernel and read back by the tally
            "alg_bytes": n * 24,
            # DRAM bytes (read + write) of one phase-0 launch from an ncu capture
            # at 5e5 histories (303 MB: records and the spilled stacks' write-back),
            # scaled by the histories
            "traffic": int(605 * n) if precision == "mixed" else None,
            "note": "SM-issue bound, not HBM: ncu smsp__issue_active 43.9% (phase 0, a "
                    "5e5-history case) with 18.2 of 32 lanes per instruction; DRAM traffic "
                    "is under 0.3% of the bandwidth",
            "config": {"workload": "c2: straggled MC with DEL/EHS + Coulomb scattering, rock mixture "
                                   "rock/water/air 0.70/0.25/0.05 (per-history thickness U[20,500] m, "
                                   "density U[2000,2800], elevation U[30,90] deg) under 1 km air, "
                                   "E 1 GeV-10 TeV, 1e6 histories",
                       "n_samples": n, "precision": precision, "tables": "create_physics(MUON), "
                       "rock+air+water, 200 nodes, with Coulomb columns"},
            "h2d": C.sizeof(dp.DpLos), "d2h": C.sizeof(dp.DpLosResult),
            # the phase-0 transport kernel (below the mode switch, every history):
            # 16 B of history parameters in and 16 B of result out per history
            "dominant": "mc_mixed_lo" if precision == "mixed" else "mc_fp64_lo",
            "dominant_bytes": n * 32,
            "issue": C2_ISSUE if precision == "mixed" else None,
            "plain_what": "FP64 transport (the reference's operations), same launch, "
                          f"{n_plain} histories", "plain_units": n_plain,
            "plain_reps": 1, "plain_warm": False}
    return ((lambda: run_dev(precision)), step_e2e,
            (lambda: run_dev("fp64", n_plain, d_los_plain)), info, phys)


def c4_los(dp, seed=4, n_los=16384):
    rng = np.random.default_rng(seed)
    depth = np.exp(rng.uniform(np.log(50.0), np.log(2000.0), n_los))
    rho = rng.uniform(2400.0, 2800.0, n_los)
    ns = rng.integers(64, 1025, n_los)
    return dp.make_los(ns, thickness=depth, density=rho, elevation=90.0, energy_min=1.0,
                       energy_max=1e4), int(ns.sum()), (depth, rho, ns)


def setup_c4(dp, torch, dev, precision="mixed", scale=1.0):
    """Batched backward MC over 16384 vertical lines of sight (depth
    log-uniform 50-2000 m, density U[2400,2800], 64-1024 histories each,
    StandardRock under air to 30 km), mixed transport everywhere (threshold at
    the 1 GeV lowest final energy, no scattering), plus the CSDA sample-average
    gradient per line of sight; one persistent launch per phase."""
    phys = dp.create_physics(materials=(dp.STANDARD_ROCK, dp.AIR))
    rock = dp.MaterialMixture(phys, 1)
    air = dp.MaterialMixture(phys, 2)
    los, total, _ = c4_los(dp, n_los=max(16, int(16384 * scale)))
    lib = dp.load()
    ctx = phys.ctx.h
    cfgs = {p: dp._mc_config(2027, True, False, 1.0, None, p) for p in ("mixed", "fp64")}
    d_los = _device_bytes(torch, dev, los)
    d_out = torch.zeros(len(los) * C.sizeof(dp.DpLosResult), dtype=torch.uint8, device=dev)
    n_los = len(los)

    def run_dev():
        dp.check(lib.dp_mc_los_dev(ctx, phys.h, rock.h, air.h, C.byref(cfgs[precision]), n_los,
                                   d_los.data_ptr(), total, 1, d_out.data_ptr()), ctx)

    def step_e2e():
        r = dp.backward_mc_batch(phys, los, rock=rock, air=air, seed=2027, scattering=False,
                                 energy_threshold_low=1.0, precision=precision,
                                 compute_gradient=True)
        assert r["n_status_nonzero"].sum() == 0

    # plain form: FP64 transport, one launch per line of sight, on the first
    # 4 lines (their rate stands for the batch)
    n_plain = 4
    sub = (dp.DpLos * n_plain)(*[los[i] for i in range(n_plain)])
    sub_n = sum(los[i].n_samples for i in range(n_plain))
    d_sub = _device_bytes(torch, dev, sub)
    one = C.sizeof(dp.DpLos)

    def plain_dev():
        for i in range(n_plain):
            dp.check(lib.dp_mc_los_dev(ctx, phys.h, rock.h, air.h, C.byref(cfgs["fp64"]), 1,
                                       d_sub.data_ptr() + i * one, sub[i].n_samples, 1,
                                       d_out.data_ptr()), ctx)

    def check():
        # 64 seeded lines of sight against the FP64 oracle over the same
        # histories (every history of each line, the same streams)
        torch.cuda.synchronize()
        res = los_results(dp, d_out, n_los)
        zs = []
        for ref in bench_checks()["c4"]["lines"]:
            r = res[ref["line"]]
            assert r.n_status_nonzero == 0 and r.n_samples == ref["n_histories"]
            zs.append((r.flux - ref["flux"]) / math.hypot(r.sigma, ref["sigma"]))
        zmax = float(np.abs(zs).max())
        assert zmax < 3, zs
        return {"lines": len(zs), "max_abs_z": zmax,
                "rms_z": float(np.sqrt(np.mean(np.square(zs)))), "pass": True}

    kernel = "mc_init+mc_mixed_lo+mc_mixed_hi+mc_finish+csda_mc32+mc_tally" if precision == "mixed" \
        else "mc_init+mc_fp64_lo+mc_fp64_hi+mc_finish+csda_mc+mc_tally"
    info = {"units": total, "unit": "samples/s", "kernel": kernel, "family": "mc",
            **({"check": check} if scale == 1.0 else {}),
            # per history: contribution and status written and read back,
            # CSDA contribution and derivative written and read back
            "alg_bytes": total * (24 + 32),
            # DRAM bytes of one mc_mixed_hi launch from an ncu capture of a tenth
            # of the lines of sight (562 MB for 882,273 histories), scaled by the
            # histories
            "traffic": int(637 * total) if precision == "mixed" else None,
            "note": "SM-issue bound, not HBM: ncu smsp__issue_active 38.6% (mixed transport, "
                    "lockstep)",
            "config": {"workload": "c4: 16384 vertical lines of sight, depth log-uniform 50-2000 m, "
                                   "density U[2400,2800], 64-1024 histories each (uneven), mixed "
                                   "transport everywhere, E 1 GeV-10 TeV, + CSDA d flux/d rho per "
                                   "line of sight",
                       "n_los": n_los, "n_samples": total, "precision": precision},
            "h2d": n_los * C.sizeof(dp.DpLos), "d2h": n_los * C.sizeof(dp.DpLosResult),
            # the transport kernel above the mode switch (every history here):
            # 16 B of history parameters in and 16 B of result out per history
            "dominant": "mc_mixed_hi" if precision == "mixed" else "mc_fp64_hi",
            "dominant_bytes": total * 32,
            "issue": C4_ISSUE if precision == "mixed" else None,
            "plain_what": "FP64 transport (+ FP64 CSDA gradient), one launch per line of sight, "
                          f"first {n_plain} lines", "plain_units": sub_n, "plain_reps": 1}
    return run_dev, step_e2e, plain_dev, info, phys


def setup_c5(dp, torch, dev, precision="mixed", scale=1.0):
    """Gauss-Newton inversion loop on a 128x128x64 grid (truth: the c3
    generator), 8 detectors x 8192 rays, synthetic Poisson counts at an
    exposure of ~10^3 counts per ray (tau = 10^3 / median flux), weights
    W = tau^2 / max(counts, 1) (inverse variance of the observed flux),
    smoothness prior 1e-5 sum_edges (rho_i - rho_j)^2; start rho = 2650.
    One step = 50 Gauss-Newton iterations (10 CG iterations per linear
    solve) from the same start; SART (50 iterations, smoothing sweeps) is run
    once after the timed region for the record."""
    from dpgpu.workloads import tomography_config
    grid, truth, rays, nodes = tomography_config(nx=128, ny=128, nz=64, n_detectors=8,
                                                 rays_per_detector=max(64, int(8192 * scale)))
    phys = dp.create_physics()
    paths = dp.TomoPaths(phys, grid, rays, nodes, side_density=2500.0)
    T = lambda a: torch.tensor(np.ascontiguousarray(a, np.float64).ravel(), device=dev)
    f_true, _, _ = paths.eval(T(truth), precision="fp64")
    f_true = f_true.cpu().numpy()
    tau = 1e3 / np.median(f_true)
    counts = np.random.default_rng(5).poisson(tau * f_true)
    obs, W = T(counts / tau), T(tau * tau / np.maximum(counts, 1))
    rho0 = T(np.full(grid.ncell, 2650.0))
    n_iter = 50
    state = {}

    def step():
        rho, hist = paths.solve(obs, rho0, method="gn", n_iter=n_iter, weight=W, cg_iter=10,
                                precision=precision, prior_weight=1e-5)
        state["rho"], state["hist"] = rho, hist

    def finish():
        rmse = lambda x: float(np.sqrt(np.mean((x - truth.ravel()) ** 2)))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rho_s, hist_s = paths.solve(obs, rho0, method="sart", n_iter=n_iter, precision=precision,
                                    prior_weight=1.0)
        torch.cuda.synchronize()
        sart_ms = (time.perf_counter() - t0) * 1e3 / n_iter
        return {"rmse_start": rmse(np.full(grid.ncell, 2650.0)),
                "gn": {"rmse": rmse(state["rho"].cpu().numpy()),
                       "misfit": [float(state["hist"][0]), float(state["hist"][-1])]},
                "sart": {"rmse": rmse(rho_s.cpu().numpy()), "ms_per_iteration": sart_ms,
                         "misfit": [float(hist_s[0]), float(hist_s[-1])]}}

    def e2e():
        step()
        state["rho_host"] = state["rho"].cpu().numpy()

    # algorithmic bytes of one Jacobian evaluation (the dominant kernel, about
    # one launch per iteration): per ray the row pointers, cos theta and the flux
    # written (32 B); per segment the cell id, length, density gather and the
    # FP32 Jacobian value written (24 B)
    jb = 4 if precision == "mixed" else 8
    info = {"units": n_iter, "unit": "iterations/s",
            "kernel": "tomo_adjoint+tomo_forward+tomo_transpose+gn_spmv+gn_colsum+gn_dot+gn_cg",
            "alg_bytes": len(rays) * 32 + paths.nnz * (20 + jb), "traffic": None,
            "dominant": "tomo_adjoint", "dominant_bytes": len(rays) * 32 + paths.nnz * (20 + jb),
            "config": {"workload": "c5: Gauss-Newton inversion, 128x128x64 @ 10 m, 8 x 8192 rays, "
                                   "Poisson counts ~1e3/ray, 50 iterations x 10 CG, start 2650",
                       "rays": len(rays), "segments": paths.nnz, "precision": precision},
            "h2d": 0, "d2h": 8 * grid.ncell, "finish": finish}
    return step, e2e, None, info, phys


DIR_E = (1e-3, 1e9)  # final-energy range of the reference's directional runs (GeV)


def dir_scene(dp, phys, n_dirs):
    """Fixed-path workload inputs: material config, site, paths and per-cell
    mixtures (rock or rock with 30 % water by mass)."""
    from dpgpu.workloads import directional_config
    raw, wf = directional_config(n_dirs)
    cfg = dp.MaterialConfig(1, 3, 2, -1, 2710.0, 1000.0, 0.0, 0.0)
    site = dp.SiteConfig(963.0, 30000.0)
    mats, dens = dp.build_cell_properties_for_mc(phys, np.zeros(len(wf), bool), wf, cfg)
    paths = [dp.DirectionalPath(z, a, [dp.CellSegment(c, l) for c, l in segs], tin, slant, rem,
                                sz, True) for z, a, segs, tin, slant, rem, sz in raw]
    return cfg, site, paths, mats, dens, wf


def setup_dir(dp, torch, dev, precision="mixed", scale=1.0):
    """Fixed-path stochastic MC (compute_directional_flux_mc) over 4096
    directions x 1024 histories: a 640 m x 640 m x 320 m voxel volume of
    rock and rock with 30 % water (by mass, half the cells each), rock to a
    flat surface 600 m above the detector (slant depths 0.6-2.3 km), air to
    30 km; final energies log-uniform 1e-3 - 1e9 GeV drawn on the device,
    straggling on, mode switch at 100 GeV, no scattering (the settings of the
    reference's directional timing runs)."""
    phys = dp.create_physics(materials=(dp.STANDARD_ROCK, dp.AIR, dp.WATER))
    n_dirs = max(16, int(4096 * scale))
    per = 1024
    cfg, site, paths, mats, dens, _ = dir_scene(dp, phys, n_dirs)
    batch = dp.DirBatch(phys, cfg, site, paths, mats, dens, None, n_samples=per,
                        energy_min=DIR_E[0], energy_max=DIR_E[1]).to_device()
    sub = dp.DirBatch(phys, cfg, site, paths[:16], mats, dens, None, n_samples=per,
                      energy_min=DIR_E[0], energy_max=DIR_E[1])
    one = [dp.DirBatch(phys, cfg, site, [p], mats, dens, None, n_samples=per,
                       energy_min=DIR_E[0], energy_max=DIR_E[1]).to_device() for p in paths[:16]]

    def step_dev():
        batch.run_dev(2028, precision=precision)

    def step_e2e():
        r = batch.run(2028, precision=precision)
        assert r["n_status_nonzero"].sum() == 0

    def plain_dev():
        for b in one:
            b.run_dev(2028, precision="fp64")

    name = "mixed" if precision == "mixed" else "fp64"
    info = {"units": batch.total, "unit": "samples/s", "family": "dir",
            "kernel": f"dir_init+dir_{name}_lo+dir_{name}_hi+dir_finish+mc_tally",
            # per history: contribution and status written and read back
            "alg_bytes": batch.total * 24,
            # DRAM bytes of one dir_mixed_hi launch from an ncu capture of a tenth
            # of the directions (611 MB for 418,816 histories), scaled by the histories
            "traffic": int(1458 * batch.total) if precision == "mixed" else None,
            "note": "SM-issue bound (one thread per history, table lookups in shared memory)",
            "config": {"workload": "dir: fixed-path MC (compute_directional_flux_mc), 4096 "
                                   "directions x 1024 histories, 32x32x16 cells @ 20 m of rock / "
                                   "rock+30% water, rock to a surface 600 m up, air to 30 km, "
                                   "E 1e-3-1e9 GeV, straggling, switch 100 GeV",
                       "n_dirs": n_dirs, "n_samples": batch.total, "precision": precision,
                       "segments": int(batch.arrays["seg_ptr"][-1]), "media": len(batch.media)},
            "h2d": batch.host_bytes(), "d2h": n_dirs * C.sizeof(dp.DpLosResult),
            "plain_what": "FP64 transport, one launch per direction, first 16 directions",
            "plain_units": sub.total, "plain_reps": 1}
    return step_dev, step_e2e, plain_dev, info, phys


def setup_wcsda(dp, torch, dev, precision="mixed", scale=1.0):
    """Water-fraction CSDA forward model with its sparse Jacobian
    (compute_directional_flux_csda + directional_flux_and_grad_csda for every
    bin, i.e. assemble_forward_and_jacobian) over the dir workload's 4096
    directions: 32x32x16 cells at 20 m, water fraction 0 or 0.3 per cell,
    rock to the surface 600 m up, air to 30 km, 32 CSDA quadrature nodes on
    [1, 1e6] GeV.  Mixed precision (FP32 walk, FP64 adjoint sums and flux);
    the plain form is the FP64 kernel, one launch per direction."""
    phys = dp.create_physics(materials=(dp.STANDARD_ROCK, dp.AIR, dp.WATER))
    n_dirs = max(16, int(4096 * scale))
    _, site, paths, _, _, wf = dir_scene(dp, phys, n_dirs)
    cfg = dp.MaterialConfig(1, 3, 2, -1, 2710.0, 1000.0, 0.0, 0.0)
    nodes = [dp.EnergySample(*x) for x in zip(*dp.csda_energy_quadrature(32, 1.0, 1e6))]
    sh = np.zeros(len(wf), bool)
    batch = dp.CsdaBatch(phys, sh, cfg, site, paths, nodes).to_device()
    w_t = torch.tensor(wf, dtype=torch.float64, device=dev)
    flux = torch.zeros(n_dirs, dtype=torch.float64, device=dev)
    jac = torch.zeros(max(batch.n_seg, 1), dtype=torch.float64, device=dev)
    one = [dp.CsdaBatch(phys, sh, cfg, site, [p], nodes).to_device() for p in paths[:16]]

    def step_dev():
        batch.run_dev(w_t, flux, jac, precision=precision)

    def step_e2e():
        f, _ = batch.run(wf, precision=precision)
        assert np.isfinite(f).all()

    def plain_dev():
        for b in one:
            b.run_dev(w_t, flux, jac, precision="fp64")

    info = {"units": n_dirs, "unit": "rays/s",
            "kernel": "dir_csda32_grad" if precision == "mixed" else "dir_csda_grad",
            # per bin: 40 B geometry + per segment 4 B cell + 8 B length + 8 B w
            # read and 8 B Jacobian value written
            "alg_bytes": n_dirs * 40 + batch.n_seg * 28,
            # DRAM bytes of one launch from an ncu capture of a tenth of the
            # directions (0.44 MB for 409: tables and paths stay in L2), scaled
            "traffic": int(1076 * n_dirs) if precision == "mixed" else None,
            "note": "SM issue / FP64 pipe bound, not HBM (tables in shared memory, paths in L2)",
            "config": {"workload": "wcsda: water-fraction CSDA flux + d flux/d w per bin, 4096 "
                                   "directions through 32x32x16 cells @ 20 m (w 0 / 0.3), rock to "
                                   "600 m, air to 30 km, 32 CSDA nodes [1, 1e6] GeV",
                       "n_bins": n_dirs, "segments": batch.n_seg, "precision": precision},
            "h2d": batch.host_bytes() + wf.nbytes, "d2h": 8 * (n_dirs + batch.n_seg),
            "plain_what": "FP64, one launch per direction, first 16 directions", "plain_units": 16,
            "plain_reps": 1}
    return step_dev, step_e2e, plain_dev, info, phys


# objective evaluations of one calibrate_csda_correction with the default
# grid: 'before', 41 + 4 x 9 grid points, the residual fit and 'after'
CALIB_EVALS = 80


def setup_calib(dp, torch, dev, precision="mixed", scale=1.0):
    """calibrate_csda_correction over the dir workload's 4096 directions
    against MC reference fluxes from the device fixed-path MC (1024 histories
    per direction, final energies 1e-3 - 1e9 GeV; made once, untimed).  One
    step is one calibration: the kappa_hard grid (41 + 4 x 9 points), the
    geometric residual fit and the before / after passes, 80 evaluations of
    the water-fraction CSDA model (32 quadrature nodes on the same energy
    range) over all bins, one launch each.  The plain form is the reference's
    loop structure on the device: FP64, one launch per bin and evaluation."""
    phys = dp.create_physics(materials=(dp.STANDARD_ROCK, dp.AIR, dp.WATER))
    n_dirs = max(16, int(4096 * scale))
    cfg, site, paths, mats, dens, wf = dir_scene(dp, phys, n_dirs)
    mc = dp.DirBatch(phys, cfg, site, paths, mats, dens, None, n_samples=1024,
                     energy_min=DIR_E[0], energy_max=DIR_E[1]).run(2029, precision="mixed")["flux"]
    nodes = [dp.EnergySample(*x) for x in zip(*dp.csda_energy_quadrature(32, *DIR_E))]
    sh = np.zeros(len(wf), bool)
    bins = list(range(1, n_dirs + 1))
    model = dp.CsdaBatch(phys, sh, cfg, site, paths, nodes).to_device()
    result = {}

    def calibrate(m):
        dp.set_csda_correction(enabled=False)
        ks, kh, st = dp.calibrate_csda_correction(phys, sh, cfg, site, paths, wf, nodes, mc, bins,
                                                  precision=precision, model=m)
        result.update(kappa_hard=kh, rel_before=st["rel_before"], rel_after=st["rel_after"])

    def step_dev():
        calibrate(model)

    def step_e2e():
        calibrate(None)  # the bins' batch is built and uploaded inside the call

    one = [dp.CsdaBatch(phys, sh, cfg, site, [p], nodes).to_device() for p in paths[:16]]
    w_t = torch.tensor(wf, dtype=torch.float64, device=dev)
    f1 = torch.zeros(1, dtype=torch.float64, device=dev)

    def plain_dev():
        for _ in range(CALIB_EVALS):
            for b in one:
                b.run_dev(w_t, f1, None, precision="fp64")

    info = {"units": 1, "unit": "calibrations/s",
            "kernel": "dir_csda32" if precision == "mixed" else "dir_csda",
            # per evaluation: 40 B geometry per bin, per segment 4 B cell,
            # 8 B length and 8 B w read, 8 B flux per bin written
            "alg_bytes": CALIB_EVALS * (n_dirs * 48 + model.n_seg * 20), "traffic": None,
            "note": "host-driven grid search: per evaluation one launch, the water fractions "
                    "up and the fluxes down",
            "config": {"workload": "calib: calibrate_csda_correction (kappa_hard grid 41 + 4x9, "
                                   "geometric residual fit) of the water-fraction CSDA model "
                                   "against device fixed-path MC fluxes, 4096 directions of the "
                                   "dir workload, 32 CSDA nodes [1e-3, 1e9] GeV",
                       "n_bins": n_dirs, "evaluations": CALIB_EVALS, "segments": model.n_seg,
                       "precision": precision},
            "h2d": model.host_bytes() + CALIB_EVALS * wf.nbytes,
            "d2h": CALIB_EVALS * 8 * n_dirs,
            "plain_what": "FP64, one launch per bin and evaluation, first 16 bins x 80 "
                          "evaluations", "plain_units": 16 / n_dirs, "plain_reps": 1,
            "finish": lambda: dict(result)}
    return step_dev, step_e2e, plain_dev, info, phys


def setup_c1(dp, torch, dev, precision="mixed"):
    """run_backward_mc in CSDA mode with the gradient.  "mixed": the FP32 walk
    with float-pair range, tangent and altitude, FP64 start offset, final
    energy and flux (within 1e-6 of the FP64 oracle, tested); "fp64": the
    reference's FP64 operations."""
    phys = dp.create_physics()
    n = 10000
    p = dp._mc_params(phys, 100.0, 2650.0, 45.0, 1.0, 100.0, n, True, 42, False, False, 100.0,
                      None, 3e4, precision)
    out = dp.DpMcResult()
    lib = dp.load()

    def step():
        dp.check(lib.dp_backward_mc(phys.ctx.h, phys.h, C.byref(p), C.byref(out)), phys.ctx.h)

    kernel = "csda_mc32" if precision == "mixed" else "csda_mc"
    info = {"units": n, "unit": "samples/s", "kernel": kernel, "alg_bytes": n * (24 + 16),
            # per history: (E, q, w) in and the contribution and its derivative out
            "dominant": kernel, "dominant_bytes": n * (24 + 16),
            # DRAM bytes of one csda32_kernel launch (ncu, this workload)
            "traffic": 89856 if precision == "mixed" else None,
            "issue": C1_ISSUE if precision == "mixed" else None,
            "config": {"workload": "c1: backward MC CSDA, StandardRock 100 m @ 45 deg, 2650 kg/m3, "
                                   "E 1-100 GeV, 1e4 histories, with d flux/d rho",
                       "n_samples": n, "precision": precision},
            "h2d": 0, "d2h": 8 * 7}
    return step, step, None, info, phys


# ------------------------------------------------------------------ arms
SETUP = {"c2": setup_c2, "c3": setup_c3, "c4": setup_c4, "c5": setup_c5, "c1": setup_c1,
         "dir": setup_dir, "wcsda": setup_wcsda, "calib": setup_calib}
UNITS = {"c2": "samples/s", "c3": "rays/s", "c4": "samples/s", "c5": "iterations/s",
         "c1": "samples/s", "dir": "samples/s", "wcsda": "rays/s", "calib": "calibrations/s"}
# the other configurations measured with the default (c2) run, each in full:
# value, e2e, roofline, cpu_baseline, plain form, clocks
SUB_WORKLOADS = ("c1", "c3", "c4", "c5")


def measure(args, workload, dp, torch, dev, world, rank, local, steps, warmup, cpu_budget):
    """One workload: warm-up, `steps` timed steps (device time, CUDA events on
    the context stream, L2 flushed between steps), the end-to-end form through
    the host-pointer C ABI, the plain FP64 form and, on rank 0, the bounded CPU
    baseline.  Returns the JSON line's fields."""
    setup = SETUP[workload]
    kw = {"scale": args.scale} if workload in ("c2", "c4", "c5", "dir", "wcsda", "calib") else {}
    kw["precision"] = args.precision
    step_dev, step_e2e, plain_dev, info, phys = setup(dp, torch, dev, **kw)
    if args.scale != 1.0:
        info["config"]["scale"] = args.scale
    fam = info.get("family")
    if fam and info["config"].get("precision") == "mixed":
        # CTA size of the persistent transport kernels: dp_autotune over the
        # compiled sizes on this very step (untimed), or the size given
        if args.mc_threads == "auto" and not args.profile_run:
            best, tried = dp.autotune_shape(phys, fam, "mixed", step_dev)
            info["config"]["cta_threads"] = best["threads"]
            info["config"]["launch_shape"] = best
            info["config"]["autotune_ms"] = [dict(s, ms=round(v, 2)) for s, v in tried]
        elif args.mc_threads != "auto":
            dp.set_mc_threads(phys, fam, "mixed", int(args.mc_threads))
            info["config"]["cta_threads"] = int(args.mc_threads)
    if args.profile_run:
        # capture mode for the profiler: warm-up steps and one step, nothing else
        for _ in range(warmup + 1):
            step_dev()
        torch.cuda.synchronize()
        return None
    lib = dp.load()
    ctx = phys.ctx.h
    stream = torch.cuda.ExternalStream(lib.dp_get_stream(ctx), device=dev)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)

    for _ in range(warmup):
        step_dev()
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        # keep the GPU busy with untimed steps for 0.5 s so that the 100 ms
        # clock samples cover the load, then the timed steps
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 0.5:
            step_dev()
            torch.cuda.synchronize()
        lib.dp_set_timing(ctx, 1)
        lib.dp_set_blocking(ctx, 0)  # enqueue steps back to back; errors checked by dp_sync
        launches0 = lib.dp_launch_count(ctx)
        events = []
        t_wall = time.perf_counter()
        for _ in range(steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                flush.zero_()  # L2 flush between timed steps (outside the events)
                e0.record(stream)
            step_dev()
            e1.record(stream)
            events.append((e0, e1))
        stream.synchronize()
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall
    dp.check(lib.dp_sync(ctx), ctx)
    lib.dp_set_blocking(ctx, 1)
    # the last timed step's answer against the oracle (before the other forms
    # overwrite its outputs)
    checked = info["check"]() if "check" in info else None
    times = [a.elapsed_time(b) for a, b in events]
    barrier(world)
    launches = lib.dp_launch_count(ctx) - launches0
    kms = 0.0
    breakdown, nlaunch = {}, {}
    for name in info["kernel"].split("+"):  # summed over the kernels of the timed step
        k, cnt = C.c_double(), C.c_longlong()
        lib.dp_kernel_stats(ctx, name.encode(), C.byref(k), C.byref(cnt))
        kms += k.value
        breakdown[name] = k.value / steps
        nlaunch[name] = cnt.value / steps
    lib.dp_set_timing(ctx, 0)
    ms = max_over_ranks(world, sum(times) / len(times))
    value = world * info["units"] / (ms * 1e-3)

    # end to end through the host-pointer C ABI (copies inside the timed region)
    for _ in range(max(1, warmup // 2)):
        step_e2e()
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(steps):
        step_e2e()
    torch.cuda.synchronize()
    e2e_ms = max_over_ranks(world, (time.perf_counter() - t0) * 1e3 / steps)

    # plain FP64 one-launch-per-ray form (speed-up denominator)
    plain = None
    if plain_dev is not None and not args.no_plain:
        if info.get("plain_warm", True):
            plain_dev()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        reps = info.get("plain_reps", 2)
        for _ in range(reps):
            plain_dev()
        torch.cuda.synchronize()
        plain_ms = (time.perf_counter() - t0) * 1e3 / reps
        plain = {"value": info.get("plain_units", info["units"]) / (plain_ms * 1e-3),
                 "unit": info["unit"],
                 "ms_per_step": plain_ms,
                 "what": info.get("plain_what", "plain FP64 one-launch-per-ray, forward only")}

    peak, peak_kind = peaks()
    # roofline of the dominant kernel: its algorithmic bytes per launch over its
    # average launch duration (CUDA events on the context stream, timed steps)
    dom = info.get("dominant") or max(breakdown, key=breakdown.get)
    dom_ms = breakdown.get(dom, 0.0) / max(1.0, nlaunch.get(dom, 1.0))
    dom_bytes = info.get("dominant_bytes", info["alg_bytes"])
    achieved = dom_bytes / (dom_ms * 1e-3) / 1e9 if dom_ms > 0 else None
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak if achieved else None,
            "traffic": info.get("traffic"), "kernel": dom, "kernel_ms": dom_ms,
            "launches_per_step": nlaunch.get(dom),
            "alg_bytes_per_launch": dom_bytes, "step_kernels_ms": kms / steps,
            "kernel_ms_each": breakdown, "peak_source": peak_kind}
    if info.get("issue"):
        roof["issue"] = info["issue"]
    if info.get("note"):
        roof["note"] = info["note"]
    line = {"metric": METRIC, "value": value, "unit": info["unit"], "n_gpus": world,
            "steps": steps, "warmup": warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64" if info["config"].get("precision") == "mixed" else "f64",
            "data": "synthetic (seeded)", "config": dict(info["config"], l2="flushed between steps",
                                                          parallelism=f"replicas x{world}"),
            "e2e": {"value": world * info["units"] / (e2e_ms * 1e-3), "unit": info["unit"],
                    "h2d_bytes_per_step": info["h2d"], "d2h_bytes_per_step": info["d2h"]},
            "roofline": roof,
            "gpu_launches": int(launches),
            "plain_gpu": plain,
            "speedup_vs_plain": (value / plain["value"]) if plain else None,
            "clocks": clk.summary(), "wall_s": t_wall}
    if "finish" in info:
        line["result"] = info["finish"]()
    if checked is not None:
        line["check"] = checked
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(workload, budget_s=cpu_budget)
    return line


def run_gpu(args):
    import torch
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    import dpgpu as dp
    dp._default = dp.Context(local)
    line = measure(args, args.workload, dp, torch, dev, world, rank, local, args.steps,
                   args.warmup, args.cpu_seconds)
    if line is None:
        return
    if args.workload == "c2" and not args.only:
        # every other configuration of the path, measured the same way with
        # fewer steps each (their steps are 0.2-630 ms)
        line["workloads"] = {}
        for w in SUB_WORKLOADS:
            sub = measure(args, w, dp, torch, dev, world, rank, local, min(args.steps, 10),
                          args.warmup, min(args.cpu_seconds, 5.0))
            line["workloads"][w] = {k: v for k, v in sub.items() if k != "metric"}
        if args.precision == "mixed":
            # c1 in the reference's FP64 operations too (its configuration
            # names FP64; the mixed form is the headline entry)
            sub = measure(argparse.Namespace(**{**vars(args), "precision": "fp64",
                                                "no_cpu": True}), "c1", dp, torch, dev, world,
                          rank, local, min(args.steps, 10), args.warmup, 0.0)
            line["workloads"]["c1"]["fp64"] = {k: sub[k] for k in
                                               ("value", "unit", "ms_per_step", "e2e", "dtype")}
        line["gpu_launches"] += sum(v["gpu_launches"] for v in line["workloads"].values())
    if rank == 0:
        print(json.dumps(line))


def cpu_baseline(workload, budget_s=15.0, threads=None):
    """The FP64 oracle on a bounded sample of the same workload, all host cores."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    threads = threads or os.cpu_count()
    if workload == "c3":
        from dpgpu.workloads import tomography_config
        grid, rho, rays, nodes = tomography_config()
        p = O.default_physics((O.STANDARD_ROCK, O.AIR))
        dims = np.array([grid.nx, grid.ny, grid.nz], np.int32)
        geom = np.array([*grid.origin, *grid.pitch])
        n, t0 = 0, time.perf_counter()
        while time.perf_counter() - t0 < budget_s:
            i = n % len(rays)
            chunk = rays[i:i + 512]
            O.tomo_vjp(p, 0, 1, dims, geom, rho, 2500.0, chunk, nodes, np.ones(len(chunk)),
                       threads=threads)
            n += len(chunk)
        dt = time.perf_counter() - t0
        return {"value": n / dt, "unit": "rays/s", "cores": threads, "kind": "port",
                "sample": f"{n} rays of the c3 workload (cycled), forward flux + reverse-sweep "
                          "J^T r (FP64 oracle, OpenMP)"}
    if workload == "c4":
        import dpgpu as dp
        p = O.default_physics((O.STANDARD_ROCK, O.AIR), coulomb=True)
        _, _, (depth, rho, ns) = c4_los(dp)
        rng = np.random.default_rng(1)
        n, t0, l = 0, time.perf_counter(), 0
        while time.perf_counter() - t0 < budget_s:
            m = int(ns[l])
            E = np.exp(rng.uniform(0, np.log(1e4), m))
            q = np.where(rng.uniform(size=m) > 0.5, 1.0, -1.0)
            w = 2 * E * np.log(1e4)
            O.mc_histories(p, [0], 1, depth[l], rho[l], 90.0, 3e4, E, q, w, seed=9, id0=n,
                           straggling=True, scattering=False, threshold_low=1.0, threads=threads)
            O.backward_mc_csda(p, 0, 1, depth[l], rho[l], 90.0, E, q, w, threads=threads)
            n += m
            l += 1
        dt = time.perf_counter() - t0
        return {"value": n / dt, "unit": "samples/s", "cores": threads, "kind": "port",
                "sample": f"{l} lines of sight ({n} histories) of the c4 workload: stochastic "
                          "transport + dual-number CSDA gradient (FP64 oracle, OpenMP)"}
    if workload == "c5":
        return cpu_baseline_c5(O, budget_s, threads)
    if workload == "dir":
        return cpu_baseline_dir(O, budget_s, threads)
    if workload == "wcsda":
        return cpu_baseline_wcsda(O, budget_s, threads)
    if workload == "calib":
        return cpu_baseline_calib(O, budget_s, threads)
    if workload == "c2":
        p = O.default_physics((O.STANDARD_ROCK, O.AIR, O.WATER), coulomb=True)
        rng = np.random.default_rng(0)
        n, t0 = 0, time.perf_counter()
        while time.perf_counter() - t0 < budget_s:
            m = 4096
            E = np.exp(rng.uniform(0, np.log(1e4), m))
            q = np.where(rng.uniform(size=m) > 0.5, 1.0, -1.0)
            t = rng.uniform(20.0, 500.0, m)
            O.mc_histories(p, [0, 2, 1], 1, t, rng.uniform(2000.0, 2800.0, m),
                           rng.uniform(30.0, 90.0, m), t + 1000.0, E, q, 2 * E * np.log(1e4),
                           seed=7, id0=n, rock_fracs=[0.70, 0.25, 0.05], threads=threads)
            n += m
        dt = time.perf_counter() - t0
        return {"value": n / dt, "unit": "samples/s", "cores": threads, "kind": "port",
                "sample": f"{n} histories of the c2 workload (FP64 oracle, OpenMP over histories)"}
    p = O.default_physics((O.STANDARD_ROCK, O.AIR))
    rng = np.random.default_rng(0)
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < budget_s:
        E = np.exp(rng.uniform(0, np.log(100.0), 2048))
        q = np.where(rng.uniform(size=2048) > 0.5, 1.0, -1.0)
        O.backward_mc_csda(p, 0, 1, 100.0, 2650.0, 45.0, E, q, 2 * E * np.log(100.0), threads=threads)
        n += 2048
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": "samples/s", "cores": threads, "kind": "port",
            "sample": f"{n} histories of the c1 workload with the dual-number gradient (FP64 oracle, OpenMP)"}


def cpu_baseline_c5(O, budget_s, threads):
    """One Gauss-Newton iteration of the c5 workload on the host: the oracle's
    flux and reverse-sweep Jacobian pass over all 65,536 rays (timed on a
    cycled sample of rays, OpenMP over rays, scaled to the full set) plus the
    10 conjugate-gradient iterations' products with the sparse Jacobian
    (scipy.sparse on a matrix of the c5 shape and segment count).  The
    reference's own solver forms the dense normal matrix, which for
    1,048,576 cells does not fit in memory, so its loop cannot be timed."""
    import scipy.sparse as sp
    from dpgpu.workloads import tomography_config
    grid, _, rays, nodes = tomography_config(nx=128, ny=128, nz=64, n_detectors=8,
                                             rays_per_detector=8192)
    p = O.default_physics((O.STANDARD_ROCK, O.AIR))
    dims = np.array([grid.nx, grid.ny, grid.nz], np.int32)
    geom = np.array([*grid.origin, *grid.pitch])
    rho = np.full(grid.ncell, 2650.0)
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < 0.7 * budget_s:
        i = (n * 7919) % len(rays)
        chunk = rays[i:i + 512]
        O.tomo_vjp(p, 0, 1, dims, geom, rho, 2500.0, chunk, nodes, np.ones(len(chunk)),
                   threads=threads)
        n += len(chunk)
    t_jac = (time.perf_counter() - t0) / n * len(rays)
    # the products of 10 CG iterations: W J p and J^T (W J p), on a matrix with
    # the c5 paths' shape and nonzeros (about 99 segments per ray)
    rng = np.random.default_rng(0)
    nnz_row = 99
    cols = rng.integers(0, grid.ncell, len(rays) * nnz_row)
    J = sp.csr_matrix((rng.uniform(-1, 0, cols.size), cols,
                       np.arange(0, cols.size + 1, nnz_row)), shape=(len(rays), grid.ncell))
    Jt = J.T.tocsr()
    x = rng.uniform(size=grid.ncell)
    w = rng.uniform(size=len(rays))
    reps, t1 = 0, time.perf_counter()
    while reps < 2 or time.perf_counter() - t1 < 0.3 * budget_s:
        Jt @ (w * (J @ x))
        reps += 1
    t_cg = 10 * (time.perf_counter() - t1) / reps
    return {"value": 1.0 / (t_jac + t_cg), "unit": "iterations/s", "cores": threads,
            "kind": "port",
            "sample": f"{n} rays of the c5 workload (cycled) through the oracle's flux + "
                      f"reverse-sweep J^T r (FP64, OpenMP), scaled to {len(rays)} rays "
                      f"({t_jac:.2f} s), plus 10 CG iterations of sparse products "
                      f"(scipy, {t_cg:.2f} s); the reference's dense normal solve does not fit"}


def cpu_baseline_dir(O, budget_s, threads):
    """The oracle's fixed-path MC over the dir workload's directions (cycled),
    1024 histories each with the device's Philox energy draws."""
    from dpgpu.workloads import directional_config
    raw, wf = directional_config(4096)
    p = O.default_physics((O.STANDARD_ROCK, O.AIR, O.WATER), coulomb=True)
    mix = 1.0 / (0.7 / 2710.0 + 0.3 / 1000.0)
    media = [([0], [1.0]), ([0, 2], [0.7, 0.3]), ([1], [1.0])]  # rock, rock+water, air
    per = 1024
    rk = np.log(DIR_E[1] / DIR_E[0])
    n, t0, d = 0, time.perf_counter(), 0
    while time.perf_counter() - t0 < budget_s:
        z, a, segs, tin, slant, rem, sz = raw[d % len(raw)]
        cells = np.array([c - 1 for c, _ in segs])
        wet = wf[cells] > 0
        ct = np.cos(np.radians(z))
        rng = np.random.default_rng(n)
        E = DIR_E[0] * np.exp(rk * rng.random(per))
        q = np.where(rng.random(per) > 0.5, 1.0, -1.0)
        O.dir_histories(p, media, 0, 2710.0, 2, 963.0, [ct], [rem],
                        [max(0.0, 30000.0 - sz) / max(ct, 1e-3)], [0, len(segs)],
                        wet.astype(np.int32), np.where(wet, mix, 2710.0),
                        [l for _, l in segs], [0, per], E, q, E * rk, seed=11, id0=n,
                        threads=threads)
        n += per
        d += 1
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": "samples/s", "cores": threads, "kind": "port",
            "sample": f"{d} directions x {per} histories of the dir workload (FP64 oracle, "
                      "OpenMP over histories)"}


def cpu_baseline_wcsda(O, budget_s, threads):
    """The oracle's water-fraction CSDA flux and d flux/d w (one dual-number
    pass per on-path cell, as the reference's forward-mode segment rules
    differentiate) over the wcsda directions, OpenMP over bins."""
    import dpgpu as dp
    from dpgpu.workloads import directional_config
    raw, wf = directional_config(4096)
    p = O.default_physics((O.STANDARD_ROCK, O.AIR, O.WATER))
    E, q, w = dp.csda_energy_quadrature(32, 1.0, 1e6)
    n, t0, i = 0, time.perf_counter(), 0
    while time.perf_counter() - t0 < budget_s:
        chunk = [raw[(i + k) % len(raw)] for k in range(64)]
        i += 64
        seg_ptr = np.concatenate([[0], np.cumsum([len(c[2]) for c in chunk])])
        O.dir_csda(p, [0, 2, 1, -1], [2710.0, 1000.0, 0.0, 0.0], [963.0, 30000.0], [0] * 10,
                   [np.cos(np.radians(c[0])) for c in chunk], [c[5] for c in chunk],
                   [c[6] for c in chunk], [1] * len(chunk), seg_ptr,
                   [s[0] - 1 for c in chunk for s in c[2]], [s[1] for c in chunk for s in c[2]],
                   np.zeros(len(wf), np.uint8), wf, E, q, w, grad=True, threads=threads)
        n += len(chunk)
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": "rays/s", "cores": threads, "kind": "port",
            "sample": f"{n} directions of the wcsda workload (cycled), flux + dual-number "
                      "d flux/d w (FP64 oracle, OpenMP over bins)"}


def cpu_baseline_calib(O, budget_s, threads):
    """The oracle's water-fraction CSDA flux (forward only) over the dir
    directions, OpenMP over bins; one calibration is 80 evaluations of all
    4096 bins."""
    import dpgpu as dp
    from dpgpu.workloads import directional_config
    raw, wf = directional_config(4096)
    p = O.default_physics((O.STANDARD_ROCK, O.AIR, O.WATER))
    E, q, w = dp.csda_energy_quadrature(32, *DIR_E)
    n, t0, i = 0, time.perf_counter(), 0
    while time.perf_counter() - t0 < budget_s:
        chunk = [raw[(i + k) % len(raw)] for k in range(256)]
        i += 256
        seg_ptr = np.concatenate([[0], np.cumsum([len(c[2]) for c in chunk])])
        O.dir_csda(p, [0, 2, 1, -1], [2710.0, 1000.0, 0.0, 0.0], [963.0, 30000.0],
                   [1, 1.0, 20.0, 0, 0, 0, 0, 0, 0.0, 0.0],
                   [np.cos(np.radians(c[0])) for c in chunk], [c[5] for c in chunk],
                   [c[6] for c in chunk], [1] * len(chunk), seg_ptr,
                   [s[0] - 1 for c in chunk for s in c[2]], [s[1] for c in chunk for s in c[2]],
                   np.zeros(len(wf), np.uint8), wf, E, q, w, threads=threads)
        n += len(chunk)
    dt = time.perf_counter() - t0
    return {"value": n / dt / (CALIB_EVALS * 4096), "unit": "calibrations/s", "cores": threads,
            "kind": "port",
            "sample": f"{n} bin evaluations of the calib workload (cycled; one calibration = "
                      f"{CALIB_EVALS} x 4096), corrected CSDA flux (FP64 oracle, OpenMP over bins)"}


def reference_line(args, workload, steps, warmup, budget):
    vals = []
    for _ in range(warmup):
        cpu_baseline(workload, budget_s=budget / 4)
    for _ in range(steps):
        vals.append(cpu_baseline(workload, budget_s=budget)["value"])
    cb = cpu_baseline(workload, budget_s=min(budget, 1.0))
    v = statistics.mean(vals)
    cb["value"] = v
    unit = UNITS[workload]
    return {"value": v, "unit": unit, "steps": steps, "warmup": warmup,
            "higher_is_better": True, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": workload,
                       "note": "reference is Julia (no toolchain on this box): FP64 oracle port "
                               "of its code path on all host cores"},
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_reference(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    line = {"metric": METRIC, "impl": "reference", "n_gpus": world, "scaling": "weak",
            "vs_baseline": None}
    line.update(reference_line(args, args.workload, args.steps, args.warmup, args.cpu_seconds))
    if args.workload == "c2" and not args.only:
        line["workloads"] = {w: reference_line(args, w, min(args.steps, 3), 1,
                                               min(args.cpu_seconds, 3.0))
                             for w in SUB_WORKLOADS}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--workload", default="c2",
                    choices=["c2", "c3", "c4", "c5", "c1", "dir", "wcsda", "calib"])
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=6.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--only", action="store_true",
                    help="c2: measure c2 alone (by default the line also holds c1, c3, c4 and "
                         "c5 under 'workloads')")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain one-launch-per-ray form")
    ap.add_argument("--scale", type=float, default=1.0,
                    help="c2/c4: fraction of the histories / lines of sight (profiling captures)")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"],
                    help="arithmetic of the timed kernels; fp64 runs the reference's "
                         "operations (parity mode)")
    ap.add_argument("--mc-threads", default="auto",
                    help="c2/c4/dir: CTA size of the transport kernels (1024, 768, 512) or "
                         "'auto' (dp_autotune before the warm-up; the default size, 1024, "
                         "under --profile-run)")
    ap.add_argument("--profile-run", action="store_true",
                    help="only warm-up steps and one step (for ncu captures); prints nothing")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
