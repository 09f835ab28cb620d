"""Host-side medium / spectrum / light-yield tables against the oracle's
restatement of medium.jl, spectrum.jl and lightyield.jl."""
import ctypes as C

import numpy as np
import pytest

import neutrinotelescopes_gb300 as nt
from neutrinotelescopes_gb300 import medium as M


def test_quan_fry_params_cascadia(oracle_lib):
    m = nt.make_cascadia_medium_properties(0.99)
    out = (C.c_double * 4)()
    oracle_lib.lib().ntpo_quan_fry_params(34.82, 1.8, 269.44088 / 1.01325, out)
    np.testing.assert_allclose(m.quan_fry_params, np.float32(np.array(out)), rtol=0)
    # values of the reference parameters (medium.jl:174-205 evaluated for Cascadia)
    assert m.quan_fry_params[0] == pytest.approx(1.32403, abs=1e-5)
    assert m.quan_fry_params[1] == pytest.approx(16.2626, abs=1e-4)


def test_group_velocity_and_dispersion_quirk(oracle_lib):
    m = nt.make_cascadia_medium_properties(0.99)
    p = (C.c_double * 4)(*m.quan_fry_params)
    wl = np.linspace(300, 800, 57)
    L = oracle_lib.lib()
    np.testing.assert_allclose(m.refractive_index(wl), [L.ntpo_refractive_index_fry(w, p) for w in wl], rtol=1e-14)
    np.testing.assert_allclose(m.group_velocity(wl), [L.ntpo_group_velocity(w, p) for w in wl], rtol=1e-13)
    # the reference's v_g at 400 nm with its dispersion and lambda_0 terms as written (medium.jl:293-318)
    assert m.group_velocity(np.array([400.0]))[0] == pytest.approx(0.22049, abs=2e-5)


def test_scattering_length(oracle_lib):
    m = nt.make_cascadia_medium_properties(0.99)
    wl = np.linspace(300, 800, 23)
    L = oracle_lib.lib()
    np.testing.assert_allclose(m.scattering_length(wl), [L.ntpo_scattering_length(w, 0.0075, 0.0075) for w in wl],
                               rtol=1e-13)
    assert m.scattering_length(np.array([400.0]))[0] == pytest.approx(37.69, abs=0.01)
    assert m.scattering_length(np.array([600.0]))[0] == pytest.approx(82.53, abs=0.01)


def test_density_and_radiation_length(oracle_lib):
    m = nt.make_cascadia_medium_properties(0.99)
    assert m.density == pytest.approx(oracle_lib.lib().ntpo_dippr105(1.8 + 273.15), rel=1e-14)
    lp = nt.LongitudinalParameterisation.from_energy(1e3, m, nt.PEMinus)
    assert lp.lrad == pytest.approx(36.08 / m.density * 10, rel=1e-12)
    assert lp.a == pytest.approx(2.01849 + 1.45469 * 3, rel=1e-6)


def test_absorption_table(oracle_lib):
    m = nt.make_cascadia_medium_properties(0.99)
    assert len(M.STRAW_ABS_WL) == 101
    assert M.STRAW_ABS_WL[0] == 300.0 and M.STRAW_ABS_WL[-1] == 800.0
    assert float(m.absorption_length(np.array([400.0]))[0]) == pytest.approx(14.5, abs=0.05)
    simple = nt.make_simple_water()
    assert float(simple.absorption_length(np.array([400.0]))[0]) == pytest.approx(30.0, rel=1e-5)
    assert len(simple.abs_wavelength) == 10


@pytest.mark.parametrize("medium", ["cascadia", "simple"])
def test_tables_match_formulas(medium):
    m = nt.make_cascadia_medium_properties(0.99) if medium == "cascadia" else nt.make_simple_water()
    tab = m.tabulate(300.0, 800.0, 1024)
    x = np.random.default_rng(1).uniform(300, 800, 5000)
    grid = np.linspace(300, 800, len(tab.ref_index))
    if medium == "simple":
        assert len(tab.ref_index) == 2  # constant quantities need two knots
    for name, f in (("ref_index", m.refractive_index), ("group_velocity", m.group_velocity),
                    ("scattering_length", m.scattering_length)):
        interp = np.interp(x, grid, getattr(tab, name).astype(np.float64))
        np.testing.assert_allclose(interp, f(x), rtol=2e-6, err_msg=name)


def test_frank_tamm_norm_matches_oracle(oracle_lib):
    m = nt.make_cascadia_medium_properties(0.99)
    p = (C.c_double * 4)(*m.quan_fry_params)
    for lo, hi in ((300.0, 800.0), (300.0, 600.0), (350.0, 351.0)):
        want = oracle_lib.lib().ntpo_frank_tamm_norm(lo, hi, p)
        assert nt.frank_tamm_norm((lo, hi), m.refractive_index) == pytest.approx(want, rel=1e-12)
    # photons per metre, 300-800 nm at n ~ 1.35: about 4.4e4 (2.3e5 photons/GeV over 5.32 m/GeV)
    y = nt.frank_tamm_norm((300.0, 800.0), m.refractive_index)
    assert 4.0e4 < y < 4.8e4


def test_cherenkov_spectrum_knots():
    m = nt.make_cascadia_medium_properties(0.99)
    sp = nt.CherenkovSpectrum((300.0, 800.0), 30, m)
    assert sp.knots.shape == (30,)
    assert sp.knots[0] == 300.0 and sp.knots[-1] == 800.0
    assert np.all(np.diff(sp.knots) > 0)
    # CDF at the knots is k/(n-1)
    norms, wls = nt.frank_tamm_inverted_cdf((300.0, 800.0), m)
    cdf = np.interp(sp.knots.astype(np.float64), wls, norms)
    np.testing.assert_allclose(cdf, np.linspace(0, 1, 30), atol=2e-6)


def test_total_lightyield_and_track_length():
    m = nt.make_cascadia_medium_properties(0.99)
    p = nt.Particle((0, 0, 0), (0, 0, 1), 0.0, 1e3, nt.PEMinus)
    assert nt.cherenkov_track_length(1e3, nt.PEMinus) == pytest.approx(5.3207078881 * 1e3 ** 1.00000211)
    y = nt.total_lightyield(p, m, (300.0, 800.0))
    assert 2.0e5 * 1e3 < y < 2.6e5 * 1e3


def test_longitudinal_profile_modes():
    # figures/long_profile_comp.png: profile modes ~3.1 m at 1e3 GeV and ~5.6 m at 1e6 GeV
    m = nt.make_cascadia_medium_properties(0.99)
    for e, mode in ((1e3, 3.1), (1e6, 5.6)):
        lp = nt.LongitudinalParameterisation.from_energy(e, m, nt.PEMinus)
        z = np.linspace(0.01, 20, 20000)
        zmax = z[np.argmax(nt.longitudinal_profile(z, lp))]
        assert zmax == pytest.approx((lp.a - 1) / lp.b * lp.lrad, rel=1e-3)
        assert zmax == pytest.approx(mode, abs=0.15)
