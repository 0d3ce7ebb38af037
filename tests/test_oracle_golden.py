"""The oracle against the reference's golden data (CPU only)."""
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN


def _rows(path):
    for line in open(path):
        if line.startswith("#") or line.startswith("process") or line.startswith("material"):
            continue
        yield line.strip().split(",")


def test_radiative_moments_vs_official_pumas(oracle):
    """test/test_material_integrals.jl:7-29: 45 raw-DCS moments of the
    official PUMAS C library, rtol 1e-6 inside, 3e-4 (2e-5 at 1800 points)
    on the full hard band."""
    n = 0
    for f in _rows(os.path.join(GOLDEN, "pumas_radiative_moments.csv")):
        proc, E = int(f[0]), float(f[1])
        m, xl, xh = map(float, f[2:5])
        mode, ref = int(f[5]), float(f[6])
        v = oracle.dcs_integral(proc, 11.0, 22.0, 149e-9, m, E, xl, xh, mode)
        tol = 3e-4 if xh == 1.0 else 1e-6
        assert v == pytest.approx(ref, rel=tol)
        if xh == 1.0:
            v2 = oracle.dcs_integral(proc, 11.0, 22.0, 149e-9, m, E, xl, xh, mode, 1800)
            assert v2 == pytest.approx(ref, rel=2e-5)
        n += 1
    assert n == 45


def test_moment_identities(oracle):
    """test/test_material_integrals.jl:31-49: narrow band = local density,
    moment ordering of a positive measure."""
    M = oracle.MUON_MASS
    NA = 6.02214076e23
    for proc in (oracle.BREMS, oracle.PAIR, oracle.PHOTO):
        E, x, dx = 100.0, 0.2, 1e-5
        sigma = oracle.dcs_integral(proc, 11.0, 22.0, 149e-9, M, E, x - dx / 2, x + dx / 2, 0)
        dens = oracle.dcs(proc, 11.0, 22.0, 149e-9, M, E, x * E) * NA / (22.0 * 0.001)
        assert sigma / (E * dx) == pytest.approx(dens, rel=1e-7)
        m = [oracle.dcs_integral(proc, 11.0, 22.0, 149e-9, M, E, 0.1, 0.5, k) for k in range(3)]
        assert all(v > 0 for v in m)
        assert 0.1 * E * m[0] <= m[1] <= 0.5 * E * m[0]
        assert 0.1 * E * m[1] <= m[2] <= 0.5 * E * m[1]


def _bragg(els):
    tot = sum(e[3] for e in els)
    zoa = sum(e[0] / e[1] * e[3] / tot for e in els)
    return math.exp(sum(e[0] / e[1] * e[3] / tot * math.log(e[2]) for e in els) / zoa)


def revision_physics(oracle):
    """The revision physics: MDF recipes (examples/data/revision_physics/
    materials.xml as recorded in physics-metadata.toml) with the PUMAS dE/dx
    tables, cutoff 0.05, elastic ratio 0.05."""
    rk = [(11.0, 22.0, 136.4e-9, 1.0)]
    wat = [(8.0, 15.9993, 95e-9, 0.888106), (1.0, 1.0087, 19.2e-9, 0.111894)]
    air = [(7.0, 14.0072, 82e-9, 0.755267), (8.0, 15.9993, 95e-9, 0.231781),
           (18.0, 39.9481, 188e-9, 0.012827), (6.0, 12.0108, 78e-9, 0.000124)]
    p = oracle.Physics()
    d = os.path.join(GOLDEN, "dedx_muon")
    p.add_dedx(os.path.join(d, "standard_rock.txt"),
               oracle.Material("StandardRock", 2650.0, _bragg(rk), rk), coulomb=True)
    p.add_dedx(os.path.join(d, "air.txt"), oracle.Material("Air", 1.205, _bragg(air), air),
               coulomb=True)
    p.add_dedx(os.path.join(d, "water.txt"), oracle.Material("Water", 1000.0, 79.7e-9, wat),
               coulomb=True)
    return p


def test_revision_tables_vs_reference_outputs(oracle):
    """docs/revision_evidence/corrected_transport/physics-julia.csv: the
    reference's own property values at 10..1e5 GeV for rock and air: CSDA and
    restricted stopping power and range, proper time, straggling, hard cross
    section and the Coulomb first transport path; all 80 agree to 1e-12."""
    p = revision_physics(oracle)
    colmap = {"stopping_power_0": "csda_S", "stopping_power_1": "mixed_S", "range_0": "csda_R",
              "range_1": "mixed_R", "proper_time_0": "csda_T", "energy_straggling": "strag",
              "cross_section": "xs", "transport_path_1": "lb1"}
    mats = {"StandardRock": 0, "Air": 1}
    n = 0
    for m, E, prop, v in _rows(os.path.join(GOLDEN, "physics-julia.csv")):
        got = p.lookup(mats[m], colmap[prop], float(E))
        assert got == pytest.approx(float(v), rel=1e-12), (m, E, prop)
        n += 1
    assert n == 80


def test_electronic_stopping_vs_pumas_table(oracle):
    """The Fano/Bethe electronic stopping power of the standard-rock pseudo
    element against the ionisation column of the official PUMAS dE/dx table
    (printed to 4 digits)."""
    rk = oracle.Material("StandardRock", 2650.0, 136.4e-9, [(11.0, 22.0, 136.4e-9, 1.0)])
    L = oracle.lib()
    rows = [l.split() for l in open(os.path.join(GOLDEN, "dedx_muon", "standard_rock.txt"))]
    rows = [r for r in rows if len(r) == 11 and r[0][0].isdigit()]
    assert len(rows) == 193
    for r in rows[::8]:
        K, ion = float(r[0]) * 1e-3, float(r[2]) * 1e-4
        v = L.orc_electronic_stopping(b"Rk", 2650.0, 136.4e-9, 1, rk.Z, rk.A, rk.Iel, rk.frac,
                                      oracle.MUON_MASS, K)
        assert v == pytest.approx(ion, rel=6e-4)


def test_dilog(oracle):
    L = oracle.lib()
    assert L.orc_dilog(1.0) == pytest.approx(math.pi ** 2 / 6, rel=1e-15)
    assert L.orc_dilog(0.5) == pytest.approx(math.pi ** 2 / 12 - 0.5 * math.log(2) ** 2, rel=1e-14)
    assert L.orc_dilog(-1.0) == pytest.approx(-math.pi ** 2 / 12, rel=1e-15)
    # series check at small x
    x = 1e-3
    assert L.orc_dilog(x) == pytest.approx(sum(x ** k / k ** 2 for k in range(1, 12)), rel=1e-14)
