"""Device failure paths: every device loop has a cap and every table-staging
wait a poll limit, and reaching one ends the loop with a status the call
reports; none of them faults or hangs the GPU.

The limits are lowered per context (dp_set_debug_limits) so that they run
out on small batches.  Each test checks the affected histories' DP_ST_* bit,
the call's error code and that the histories the limit did not touch are
bit for bit what an unlimited run gives (every history owns its Philox
stream), then restores the limits and checks that the context still works.

Reference throw sites: src/MixedTransport.jl:44-45 (mixed kernel domain),
:157,193 (100000 hard events), :186 (adjoint weight); the step cap and the
staging wait have no reference counterpart (the reference loops until a
boundary and stages nothing).
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ST_STEP_CAP, ST_EVENT_CAP, ST_DOMAIN_LO, ST_TABLE_WAIT = 1, 4, 16, 128
DP_ERR_DOMAIN, DP_ERR_STATE = -3, -5


@pytest.fixture(scope="module")
def dp():
    import dpgpu
    return dpgpu


@pytest.fixture(scope="module")
def orc_phys(oracle):
    return oracle.default_physics((oracle.STANDARD_ROCK, oracle.AIR), coulomb=True)


@pytest.fixture(scope="module")
def phys(dp, orc_phys):
    ctx = dp.Context(0)  # a context of its own: the limits never leak into other tests
    tabs = [orc_phys.table(i) for i in range(2)]
    return dp.upload_physics(tabs, ["StandardRock", "Air"], materials=(dp.STANDARD_ROCK, dp.AIR),
                             ctx=ctx)


@pytest.fixture(scope="module")
def media(dp, phys):
    return dp.MaterialMixture(phys, 1), dp.MaterialMixture(phys, 2)


def _histories(dp, phys, media, E, *, precision, thickness, threshold_low=100.0,
               scattering=True, seed=5):
    """dp_mc_histories through the C ABI, returning the code with the
    per-history results (the Python wrapper raises on a nonzero code)."""
    rock, air = media
    n = len(E)
    E = np.ascontiguousarray(E, np.float64)
    q = np.where(np.arange(n) % 2 == 0, 1.0, -1.0)
    w = 2 * E * np.log(1e4)
    geo = [np.array([v], np.float64) for v in (thickness, 2650.0, 60.0, thickness + 1000.0)]
    c, Ef = np.zeros(n), np.zeros((n, 4))
    st, ns = np.zeros(n, np.int32), np.zeros(n, np.int32)
    cfg = dp._mc_config(seed, True, scattering, threshold_low, None, precision)
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    rc = dp.load().dp_mc_histories(phys.ctx.h, phys.h, rock.h, air.h, C.byref(cfg), n, p(E), p(q),
                                   p(w), p(geo[0]), p(geo[1]), p(geo[2]), p(geo[3]), 0, 0, p(c),
                                   p(st), p(ns), p(Ef))
    msg = dp.load().dp_last_error(phys.ctx.h).decode() if rc else ""
    return rc, msg, c, st, ns


def _limited(dp, phys, **kw):
    class _Limits:
        def __enter__(self):
            dp.set_debug_limits(phys, **kw)

        def __exit__(self, *a):
            dp.set_debug_limits(phys)
    return _Limits()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_step_cap(dp, phys, media, precision):
    """Histories that need more steps than the cap end flagged
    DP_ST_STEP_CAP with no flux, the call returns DP_ERR_STATE, and the
    histories within the cap are unchanged."""
    E = np.exp(np.random.default_rng(1).uniform(0.0, np.log(300.0), 96))
    rc0, _, c0, st0, ns0 = _histories(dp, phys, media, E, precision=precision, thickness=120.0)
    assert rc0 == 0 and (st0 == 0).all()
    cap = int(np.median(ns0))
    with _limited(dp, phys, step_cap=cap):
        rc, msg, c, st, ns = _histories(dp, phys, media, E, precision=precision, thickness=120.0)
    over = ns0 > cap
    assert over.any() and (~over).any()
    assert rc == DP_ERR_STATE and "step cap" in msg
    assert ((st[over] & ST_STEP_CAP) != 0).all() and (c[over] == 0).all()
    assert (st[~over] == 0).all()
    np.testing.assert_array_equal(c[~over], c0[~over])
    np.testing.assert_array_equal(ns[~over], ns0[~over])
    rc1, _, c1, st1, _ = _histories(dp, phys, media, E, precision=precision, thickness=120.0)
    assert rc1 == 0 and (st1 == 0).all()
    np.testing.assert_array_equal(c1, c0)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_event_cap(dp, phys, media, precision):
    """With a cap of one pass of the mixed-step event loop
    (src/MixedTransport.jl:157-193: the pass that finds no event counts too),
    a mixed step that meets a hard event exceeds it: DP_ST_EVENT_CAP, the
    reference's message, DP_ERR_STATE.  Histories without a hard event are
    unchanged."""
    E = np.exp(np.random.default_rng(2).uniform(np.log(150.0), np.log(1500.0), 128))
    kw = dict(precision=precision, thickness=25.0, scattering=False)
    rc0, _, c0, st0, _ = _histories(dp, phys, media, E, **kw)
    assert rc0 == 0 and (st0 == 0).all()
    with _limited(dp, phys, event_cap=1):
        rc, msg, c, st, _ = _histories(dp, phys, media, E, **kw)
    hit = (st & ST_EVENT_CAP) != 0
    assert hit.any() and (~hit).any()
    assert rc == DP_ERR_STATE
    assert msg == "Mixed transport exceeded 100000 hard events; segment incomplete"
    assert (st[hit] == ST_EVENT_CAP).all() and (c[hit] == 0).all()
    assert (st[~hit] == 0).all()
    np.testing.assert_array_equal(c[~hit], c0[~hit])


def test_table_wait_runs_out(dp, phys, media):
    """A staging wait allowed no poll gives up in every block: each block
    still waits for its copy in flight, then ends its share of the histories
    flagged DP_ST_TABLE_WAIT; the call returns DP_ERR_STATE and the context
    works afterwards."""
    E = np.exp(np.random.default_rng(3).uniform(0.0, np.log(1e4), 512))
    shape = dp.get_mc_shape(phys, "mc", "mixed")
    dp.set_mc_shape(phys, "mc", "mixed", staging=0)  # tables in shared memory
    try:
        rc0, _, c0, st0, _ = _histories(dp, phys, media, E, precision="mixed", thickness=80.0)
        assert rc0 == 0 and (st0 == 0).all()
        with _limited(dp, phys, wait_iters=0):
            rc, msg, c, st, _ = _histories(dp, phys, media, E, precision="mixed", thickness=80.0)
        assert rc == DP_ERR_STATE and "table-staging" in msg
        assert (st == ST_TABLE_WAIT).all() and (c == 0).all()
        rc1, _, c1, st1, _ = _histories(dp, phys, media, E, precision="mixed", thickness=80.0)
        assert rc1 == 0 and (st1 == 0).all()
        np.testing.assert_array_equal(c1, c0)
    finally:
        dp.set_mc_shape(phys, "mc", "mixed", **shape)


def test_below_mixed_kernel_domain(dp, phys, media, oracle, orc_phys):
    """A mixed step that starts below the prepared energy grid
    (final energy 5e-4 GeV, grid from 1e-3 GeV, mode switch below it) is the
    reference's DomainError "Below prepared mixed kernel domain"
    (src/MixedTransport.jl:44): DP_ST_DOMAIN_LO, DP_ERR_DOMAIN with that
    message, as in the oracle.  The energies above the grid cannot be reached
    through this API: the source ceiling is checked against the grid
    (DP_ERR_ARG) and the transport stops at it, as the reference's
    (src/MixedTransport.jl:150-151, 196) does."""
    E = np.array([5e-4, 2.0, 7e-4, 30.0])
    rc, msg, c, st, _ = _histories(dp, phys, media, E, precision="fp64", thickness=10.0,
                                   threshold_low=1e-4, scattering=False)
    assert rc == DP_ERR_DOMAIN and msg == "Below prepared mixed kernel domain"
    low = E < 1e-3
    assert ((st[low] & ST_DOMAIN_LO) != 0).all() and (c[low] == 0).all()
    assert (st[~low] == 0).all() and (c[~low] > 0).all()
    q = np.where(np.arange(4) % 2 == 0, 1.0, -1.0)
    _, ost, _, _ = oracle.mc_histories(orc_phys, [0], 1, 10.0, 2650.0, 60.0, 1010.0, E, q,
                                       2 * E * np.log(1e4), seed=5, straggling=True,
                                       scattering=False, threshold_low=1e-4)
    np.testing.assert_array_equal(ost & ST_DOMAIN_LO, st & ST_DOMAIN_LO)
    with pytest.raises(dp.DomainError, match="Below prepared mixed kernel domain"):
        dp.mc_histories(phys, *media, E, q, 2 * E * np.log(1e4), thickness=10.0, density=2650.0,
                        elevation=60.0, primary_altitude=1010.0, seed=5, scattering=False,
                        energy_threshold_low=1e-4)


def test_csda_limits(dp, phys):
    """The CSDA history loop (run_backward_mc, straggling = scattering =
    false): a step cap below the histories' step counts and a staging wait
    allowed no poll both return DP_ERR_STATE; the context works afterwards."""
    E, q, w = dp.mc_samples(phys, energy_min=1.0, energy_max=100.0, n_samples=256, seed=3)
    geo = dict(rock_thickness=100.0, rock_density=2650.0, elevation=45.0)
    c0, d0 = dp.csda_flux_samples(phys, E, q, w, **geo)
    with _limited(dp, phys, step_cap=10):
        with pytest.raises(dp.DpError, match="step cap") as e:
            dp.csda_flux_samples(phys, E, q, w, **geo)
        assert e.value.code == DP_ERR_STATE
    with _limited(dp, phys, wait_iters=0):
        with pytest.raises(dp.DpError, match="table-staging") as e:
            dp.csda_flux_samples(phys, E, q, w, **geo)
        assert e.value.code == DP_ERR_STATE
    c1, d1 = dp.csda_flux_samples(phys, E, q, w, **geo)
    np.testing.assert_array_equal(c1, c0)
    np.testing.assert_array_equal(d1, d0)


def test_tomography_wait(dp, phys):
    """The tomography evaluation kernels (FP64 and mixed) stage their tables
    the same way: a wait allowed no poll returns DP_ERR_STATE."""
    from dpgpu.workloads import tomography_config
    grid, rho, rays, nodes = tomography_config(nx=8, ny=8, nz=4, rays_per_detector=8, seed=3)
    paths = dp.TomoPaths(phys, grid, rays, nodes, side_density=2500.0)
    cot = np.ones(len(rays))
    ref = {p: paths.eval_host(rho.ravel(), cot, precision=p, nodes=nodes) for p in ("fp64", "mixed")}
    for p in ("fp64", "mixed"):
        with _limited(dp, phys, wait_iters=0):
            with pytest.raises(dp.DpError) as e:
                paths.eval_host(rho.ravel(), cot, precision=p, nodes=nodes)
            assert e.value.code == DP_ERR_STATE
        f, g = paths.eval_host(rho.ravel(), cot, precision=p, nodes=nodes)
        np.testing.assert_array_equal(f, ref[p][0])
        np.testing.assert_array_equal(g, ref[p][1])
