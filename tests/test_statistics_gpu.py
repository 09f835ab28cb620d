"""Statistical agreement of the CUDA propagation with the oracle's
single-precision mirror of the reference step law (photon_prop_cuda.jl:402-506),
on independent Philox keys: per-module hit rates within 3 sigma (Poisson) and
arrival-time distributions with a two-sample KS p-value above 0.01.

The GPU runs ten times the mirror's photons, so hit *rates* (hits per photon)
are compared: under equal rates the difference r_gpu - r_cpu of two Poisson
counts has variance p (1/n_gpu + 1/n_cpu) with p the pooled rate, and z is
that difference over its standard deviation.  Modules with at least 25 hits
in the two runs together enter the comparison (the normal approximation of
the Poisson difference holds there).  With up to 25 such modules every one
must lie within 3 sigma.  With more (the 10 x 10 string grid), some modules
fall outside 3 sigma by chance alone (0.27% each): there the number outside
3 sigma must not exceed the 99% quantile of that binomial count, none may lie
beyond 4.5 sigma, and the sum of z^2 must pass a chi-square test at p > 0.01.

Cases: the 1e6-photon point cone of the benchmark definition (one module, its
medium 0.85 HG(0.97) + 0.15 Rayleigh), the cascades on a 20-module POM string
in that medium, a cascade in the reference's own water (Cascadia Basin optics,
pure HG g = 0.99, 30-knot Frank-Tamm texture), and cascades on the 10 x 10
string grid with the kernel's 2-D grid walk (the mirror looks targets up in a
bucket grid, which gives the same hits as its scan over all 2000 modules).
"""
import os

import numpy as np
import pytest

import neutrinotelescopes_gb300 as nt
from neutrinotelescopes_gb300 import workloads

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1
Z_MAX = 3.0
MIN_COUNT = 25


@pytest.fixture(scope="module")
def orc(oracle_lib):
    return oracle_lib


def rate_z(ids_a, n_a, ids_b, n_b):
    """Per-module z of the hit-rate difference (a minus b) for modules with
    at least MIN_COUNT hits in both runs together; returns (module ids, z,
    counts a, counts b)."""
    ids = np.unique(np.concatenate([ids_a, ids_b]))
    ca = np.array([np.sum(ids_a == i) for i in ids], dtype=np.float64)
    cb = np.array([np.sum(ids_b == i) for i in ids], dtype=np.float64)
    keep = (ca + cb) >= MIN_COUNT
    ids, ca, cb = ids[keep], ca[keep], cb[keep]
    p = (ca + cb) / (n_a + n_b)
    z = (ca / n_a - cb / n_b) / np.sqrt(p * (1.0 / n_a + 1.0 / n_b))
    return ids, z, ca, cb


def assert_rates_agree(ids, z):
    from scipy import stats
    assert len(z) >= 1
    if len(z) <= 25:
        assert np.all(np.abs(z) < Z_MAX), dict(zip(ids.tolist(), np.round(z, 2).tolist()))
        return
    outside = int(np.sum(np.abs(z) >= Z_MAX))
    allowed = int(stats.binom.ppf(0.99, len(z), 2 * stats.norm.sf(Z_MAX)))
    assert outside <= allowed, f"{outside} of {len(z)} modules beyond 3 sigma (allowed {allowed})"
    assert np.max(np.abs(z)) < 4.5, f"max |z| {np.max(np.abs(z)):.2f}"
    chi2 = float(np.sum(z * z))
    assert stats.chi2.sf(chi2, len(z)) > 0.01, f"chi2 {chi2:.1f} over {len(z)} modules"


def run_pair(orc, gpu_setup, cpu_setup, binned=False, gpu_seed=101, cpu_seed=202):
    g = nt.propagate_photons(gpu_setup, seed=gpu_seed, reference_columns=False)
    n_g = sum(int(s.photons) for s in gpu_setup.sources)
    o = orc.propagate_f32(cpu_setup, seed=cpu_seed, threads=THREADS, binned=binned)
    n_o = sum(int(s.photons) for s in cpu_setup.sources)
    assert g.n_photons_simulated == n_g
    return g.records, n_g, o, n_o


def check_pair(g, n_g, o, n_o, min_hits):
    from scipy import stats
    assert len(o) >= min_hits, f"mirror found only {len(o)} hits"
    ids, z, ca, cb = rate_z(g["module_id"], n_g, o["module_id"], n_o)
    print(f"{len(ids)} modules, GPU {len(g)} hits / {n_g:.3g} photons, mirror {len(o)} / {n_o:.3g}, "
          f"max |z| {np.max(np.abs(z)):.2f}")
    assert_rates_agree(ids, z)
    assert stats.ks_2samp(g["time"], o["time"]).pvalue > 0.01
    # the brightest module on its own
    top = ids[np.argmax(cb)]
    assert stats.ks_2samp(g["time"][g["module_id"] == top], o["time"][o["module_id"] == top]).pvalue > 0.01


def test_point_cone_statistics(orc):
    # about 16 hits per 1e6 photons: 1e9 on the GPU, 1e8 in the mirror
    g, n_g, o, n_o = run_pair(orc, workloads.point_cone_setup(1_000_000_000), workloads.point_cone_setup(100_000_000))
    check_pair(g, n_g, o, n_o, min_hits=1000)


def test_cascade_string_statistics_benchmark_water(orc):
    # the benchmark's four cascades (1e3-1e5 GeV) on the 20-module string,
    # 0.85 HG(0.97) + 0.15 Rayleigh: 7.5e8 photons on the GPU, 1e8 in the mirror
    g, n_g, o, n_o = run_pair(orc, workloads.cascade_string_setup(4, photon_scale=0.1),
                              workloads.cascade_string_setup(4, photon_scale=0.1 / 7.5))
    check_pair(g, n_g, o, n_o, min_hits=20_000)


def _compat_setup(photons):
    m = nt.make_cascadia_medium_properties(0.99)
    lp = nt.LongitudinalParameterisation.from_energy(1e4, m, nt.PEMinus)
    src = nt.ExtendedCherenkovEmitter((4.0, 0.0, 140.0), (0.0, 0.6, 0.8), 0.0, photons, lp)
    targets = nt.string_of_modules(20, 15.0, pmt_area=workloads.PMT_AREA)
    return nt.PhotonPropSetup([src], targets, m, nt.CherenkovSpectrum((300.0, 800.0), 30, m))


def test_cascade_string_statistics_reference_water(orc):
    g, n_g, o, n_o = run_pair(orc, _compat_setup(400_000_000), _compat_setup(40_000_000))
    check_pair(g, n_g, o, n_o, min_hits=10_000)


def _grid_setup(photon_scale):
    targets = workloads.string_grid(10, 10, 50.0, 20, 15.0)
    srcs = workloads.cascade_sources(3, np.random.default_rng(5), photon_scale=photon_scale, string_z=(0.0, 285.0),
                                     distance=8.0)
    return nt.PhotonPropSetup(srcs, targets, nt.make_simple_water(), nt.InverseSquareSpectrum(300.0, 600.0))


def test_string_grid_statistics_with_grid_walk(orc):
    # 10 x 10 strings x 20 modules; the GPU setup walks the 2-D cell grid
    # (more than 8 columns), the mirror uses its bucket-grid lookup
    gs = _grid_setup(0.1)
    assert gs.plain_scan is False
    g, n_g, o, n_o = run_pair(orc, gs, _grid_setup(0.01), binned=True)
    check_pair(g, n_g, o, n_o, min_hits=10_000)
