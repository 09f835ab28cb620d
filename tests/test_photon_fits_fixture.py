"""The oracle against the reference's only statistical fixture for this path,
assets/photon_fits.parquet (a slice in tests/golden/photon_fits_sample.json,
made by tests/golden/make_photon_fits_sample.py).

The fixture's det_fraction is the fraction of a point-like Cherenkov
emitter's photons detected by a module at distance d along +z, weighted by
absorption and the PMT acceptance, with the emitter's axis at the
observation angle from the module direction (modelling.jl:60-167, Cascadia
Basin water, Frank-Tamm spectrum 300-800 nm).  It was made with an older
propagation API that no longer exists (propagate_source, modelling.jl:135),
so it supports an order-of-magnitude check only: the oracle's weighted
fraction for a 0.21 m sphere must lie within a factor 3 of the fixture
(its median over the 11 nearest observation angles, which smooths the
fixture's own Monte Carlo noise), at points where the oracle sees at least
40 hits.
"""
import json
import os
from pathlib import Path

import numpy as np
import pytest

import neutrinotelescopes_gb300 as nt
from neutrinotelescopes_gb300 import workloads

GOLDEN = Path(__file__).resolve().parent / "golden" / "photon_fits_sample.json"
POINTS = [(10.0, 0.3), (10.0, 0.75), (10.0, 1.2), (10.0, 2.0), (25.0, 0.3), (25.0, 0.75), (25.0, 1.2),
          (50.0, 0.75)]


@pytest.fixture(scope="module")
def fixture_rows():
    return np.asarray(json.loads(GOLDEN.read_text())["rows"])


@pytest.mark.parametrize("d_want,a_want", POINTS)
def test_detected_fraction_matches_fixture(oracle_lib, fixture_rows, d_want, a_want):
    levels = np.unique(fixture_rows[:, 0])
    d = float(levels[np.argmin(np.abs(levels - d_want))])
    rows = fixture_rows[fixture_rows[:, 0] == d]
    rows = rows[np.argsort(rows[:, 1])]
    i = int(np.argmin(np.abs(rows[:, 1] - a_want)))
    a = float(rows[i, 1])
    want = float(np.median(rows[max(0, i - 5):i + 6, 2]))
    m = nt.make_cascadia_medium_properties(0.99)
    n = 3_000_000 if d < 20.0 else 6_000_000
    src = nt.PointlikeCherenkovEmitter((0.0, 0.0, 0.0), (np.sin(a), 0.0, np.cos(a)), 0.0, n)
    tgt = nt.DetectionSphere((0.0, 0.0, d), 0.21, 16, workloads.PMT_AREA, 1)
    setup = nt.PhotonPropSetup([src], [tgt], m, nt.CherenkovSpectrum((300.0, 800.0), 40, m))
    hits = oracle_lib.propagate_f32(setup, seed=7, threads=os.cpu_count() or 1)
    assert len(hits) >= 40, f"only {len(hits)} oracle hits at d={d:.1f} m, angle {a:.2f}"
    w = oracle_lib.total_weight(hits, setup, nt.p_one_pmt_acc)
    got = float(np.sum(w["abs_weight"] * w["wl_acc"])) / n
    assert want / 3 <= got <= 3 * want, f"d={d:.1f} m angle {a:.2f}: oracle {got:.3g}, fixture {want:.3g}"
