"""The product's host table builder from PUMAS dE/dx files
(create_material_table_from_dedx, src/Physics.jl:146-273; load_dedx_file,
src/DEDXLoader.jl:100-190), on the CPU: pinned to the reference's own
tabulated revision physics (docs/revision_evidence/corrected_transport/
physics-julia.csv) and equal to the oracle's restatement column by column."""
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN
from test_oracle_golden import _bragg, _rows, revision_physics

DEDX = os.path.join(GOLDEN, "dedx_muon")
RK = [(11.0, 22.0, 136.4e-9, 1.0)]
WAT = [(8.0, 15.9993, 95e-9, 0.888106), (1.0, 1.0087, 19.2e-9, 0.111894)]
AIR = [(7.0, 14.0072, 82e-9, 0.755267), (8.0, 15.9993, 95e-9, 0.231781),
       (18.0, 39.9481, 188e-9, 0.012827), (6.0, 12.0108, 78e-9, 0.000124)]


@pytest.fixture(scope="module")
def dp():
    import dpgpu
    return dpgpu


@pytest.fixture(scope="module")
def revision(dp):
    """The revision physics' recipes (physics-metadata.toml) with the PUMAS
    dE/dx tables, cutoff 0.05, elastic ratio 0.05, built by libdpgpu."""
    mats = [dp.Material("StandardRock", 2650.0, _bragg(RK), RK),
            dp.Material("Air", 1.205, _bragg(AIR), AIR),
            dp.Material("Water", 1000.0, 79.7e-9, WAT)]
    files = [os.path.join(DEDX, f) for f in ("standard_rock.txt", "air.txt", "water.txt")]
    return dp.tables_from_dedx(files, mats), mats, files


def _interp(t, col, K):
    """interpolate_table_fast (src/Physics.jl:660-687): linear in log E, clamped."""
    lE, y = t["logE"], t[col]
    x = math.log(K)
    if x <= lE[0]:
        return y[0]
    if x >= lE[-1]:
        return y[-1]
    i = int(np.searchsorted(lE, x, side="right")) - 1
    return y[i] + (x - lE[i]) / (lE[i + 1] - lE[i]) * (y[i + 1] - y[i])


def test_dedx_tables_vs_reference_outputs(revision):
    """The 80 property values of physics-julia.csv (rock and air at
    10..1e5 GeV: CSDA and restricted stopping power and range, proper time,
    straggling, hard cross section, Coulomb first transport path) from the
    product's builder, to 1e-12."""
    tabs, _, _ = revision
    colmap = {"stopping_power_0": "csda_S", "stopping_power_1": "mixed_S", "range_0": "csda_R",
              "range_1": "mixed_R", "proper_time_0": "csda_T", "energy_straggling": "strag",
              "cross_section": "xs", "transport_path_1": "lb1"}
    mats = {"StandardRock": 0, "Air": 1}
    n = 0
    for m, E, prop, v in _rows(os.path.join(GOLDEN, "physics-julia.csv")):
        got = _interp(tabs[mats[m]], colmap[prop], float(E))
        assert got == pytest.approx(float(v), rel=1e-12), (m, E, prop)
        n += 1
    assert n == 80


def test_dedx_tables_equal_the_oracle(revision, oracle):
    """Every column of the three materials against the oracle's restatement."""
    tabs, _, _ = revision
    p = revision_physics(oracle)
    ocols = {"ecut": "elastic_cutoff"}
    for m in range(3):
        o = p.table(m)
        for c, v in tabs[m].items():
            np.testing.assert_allclose(v, o[ocols.get(c, c)], rtol=1e-12, atol=0,
                                       err_msg=f"material {m} column {c}")


def test_dedx_errors(dp, revision, tmp_path):
    """Missing files, files without a data section and differing grids are
    argument errors."""
    _, mats, files = revision
    with pytest.raises(ValueError):
        dp.tables_from_dedx([files[0], str(tmp_path / "none.txt"), files[2]], mats)
    bad = tmp_path / "bad.txt"
    bad.write_text("no header here\n1 2 3 4 5 6 7 8 9 10 11\n")
    with pytest.raises(ValueError):
        dp.tables_from_dedx([files[0], str(bad), files[2]], mats)
    short = tmp_path / "short.txt"
    lines = open(files[1]).read().splitlines()
    short.write_text("\n".join(lines[:-5]) + "\n")
    with pytest.raises(ValueError):
        dp.tables_from_dedx([files[0], str(short), files[2]], mats)
    with pytest.raises(ValueError):
        dp.tables_from_dedx(files[:2], mats)
