"""Writes tests/golden/bench_checks.json: FP64 oracle fluxes of the bench's
c2 and c4 workloads on the bench's own Philox streams, which bench.py
compares its device answer against (its 'check' entry).

c2: the first 200,000 histories of the 10^6-history line of sight (seed
2026; per-history thickness, density and elevation drawn from Philox blocks
1-2, energy and charge from block 0), rock/water/air 0.70/0.25/0.05 under
1 km of air, straggling and scattering, mode switch at 100 GeV.
c4: 64 seeded lines of sight of the 16,384-line generator (seed 4), every
history of each (seed 2027, history id = running sample index), straggling
without scattering, mixed transport from 1 GeV.

Usage: python tests/golden/make_bench_checks.py   (about a minute on 8 cores)
"""
import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import pyoracle as O  # noqa: E402


def flux_sigma(c):
    f = float(c.mean())
    return f, math.sqrt(max(float((c * c).mean()) - f * f, 0.0) / len(c))


def c4_generator(seed=4, n_los=16384):
    rng = np.random.default_rng(seed)
    depth = np.exp(rng.uniform(np.log(50.0), np.log(2000.0), n_los))
    rho = rng.uniform(2400.0, 2800.0, n_los)
    ns = rng.integers(64, 1025, n_los)
    return depth, rho, ns


def main():
    out = {}
    p3 = O.default_physics((O.STANDARD_ROCK, O.AIR, O.WATER), coulomb=True)
    m = 200_000
    ids = np.arange(m)
    E, q, w = O.energy_draws(2026, ids, 1.0, 1e4)
    t, rho, el = O.los_geometry_draws(2026, ids, 20.0, 500.0, 2000.0, 2800.0, 30.0, 90.0)
    c, st, _, _ = O.mc_histories(p3, [0, 2, 1], 1, t, rho, el, t + 1000.0, E, q, w, seed=2026,
                                 rock_fracs=[0.70, 0.25, 0.05])
    assert (st == 0).all()
    f, s = flux_sigma(c)
    out["c2"] = {"flux": f, "sigma": s, "n_histories": m, "seed": 2026}
    p2 = O.default_physics((O.STANDARD_ROCK, O.AIR), coulomb=True)
    depth, rho, ns = c4_generator()
    off = np.concatenate([[0], np.cumsum(ns)])
    pick = np.sort(np.random.default_rng(64).choice(len(ns), 64, replace=False))
    lines = []
    for l in pick:
        ids = np.arange(off[l], off[l + 1])
        E, q, w = O.energy_draws(2027, ids, 1.0, 1e4)
        c, st, _, _ = O.mc_histories(p2, [0], 1, depth[l], rho[l], 90.0, 3e4, E, q, w, seed=2027,
                                     id0=int(off[l]), straggling=True, scattering=False,
                                     threshold_low=1.0)
        assert (st == 0).all()
        f, s = flux_sigma(c)
        lines.append({"line": int(l), "flux": f, "sigma": s, "n_histories": int(ns[l])})
    out["c4"] = {"lines": lines, "seed": 2027}
    with open(os.path.join(HERE, "bench_checks.json"), "w") as fh:
        json.dump(out, fh, indent=1)


if __name__ == "__main__":
    main()
