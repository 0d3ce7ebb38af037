"""Physics tables on the device from PUMAS dE/dx files and through the
portable table file (the counterpart of the reference's .pumas
serialisation, src/Loader.jl:30-105)."""
import os

import numpy as np
import pytest

from test_physics_tables import AIR, DEDX, RK, WAT, _bragg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dp():
    import dpgpu
    return dpgpu


def test_dedx_physics_and_table_file_round_trip(dp, tmp_path):
    """dp_physics_create_dedx holds the host builder's columns bit for bit; a
    saved and reloaded table set keeps names, settings and every column bit
    for bit and gives the same run_backward_mc estimate; a damaged file is
    rejected."""
    mats = [dp.Material("StandardRock", 2650.0, _bragg(RK), RK),
            dp.Material("Air", 1.205, _bragg(AIR), AIR),
            dp.Material("Water", 1000.0, 79.7e-9, WAT)]
    files = [os.path.join(DEDX, f) for f in ("standard_rock.txt", "air.txt", "water.txt")]
    phys = dp.create_physics_dedx(files, mats)
    host = dp.tables_from_dedx(files, mats)
    for m in range(3):
        for c in dp.COLUMNS:
            np.testing.assert_array_equal(phys.column(m, c), host[m][c])
    path = str(tmp_path / "revision.dptab")
    dp.save_physics(phys, path)
    p2 = dp.load_physics(path)
    assert p2.names == ["StandardRock", "Air", "Water"]
    assert (p2.n_materials, p2.n_energies) == (3, phys.n_energies)
    assert (p2.settings.mass, p2.settings.cutoff) == (phys.settings.mass, phys.settings.cutoff)
    for m in range(3):
        for c in dp.COLUMNS:
            np.testing.assert_array_equal(p2.column(m, c), host[m][c])
    kw = dict(rock_thickness=120.0, rock_density=2650.0, elevation=60.0, energy_min=1.0,
              energy_max=1e3, n_samples=4000, seed=5)
    a = dp.run_backward_mc(phys, straggling=False, scattering=False, **kw)
    b = dp.run_backward_mc(p2, straggling=False, scattering=False, **kw)
    assert (a.flux, a.sigma) == (b.flux, b.sigma) and a.flux > 0
    raw = open(path, "rb").read()
    bad = tmp_path / "bad.dptab"
    bad.write_bytes(raw[: len(raw) // 2])
    with pytest.raises(ValueError):
        dp.load_physics(str(bad))
    bad.write_bytes(b"NOTATABLE" + raw[9:])
    with pytest.raises(ValueError):
        dp.load_physics(str(bad))


def test_empirical_physics_round_trip(dp, tmp_path):
    """create_physics (empirical tables) through the file: identical columns."""
    phys = dp.create_physics(n_energies=40, K_min=1e-3, K_max=1e6,
                             materials=(dp.STANDARD_ROCK, dp.AIR, dp.WATER))
    path = str(tmp_path / "emp.dptab")
    dp.save_physics(phys, path)
    p2 = dp.load_physics(path)
    assert p2.names == phys.names
    for m in range(3):
        for c in dp.COLUMNS:
            np.testing.assert_array_equal(p2.column(m, c), phys.column(m, c))
