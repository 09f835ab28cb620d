"""Synthetic workloads of the benchmark and the tests, named by what they are.

point_cone:      1e6 photons from the origin on a 41.2 degree cone around +z,
                 1/lambda^2 spectrum on 300-600 nm, one 0.21 m sphere at
                 (0, 0, 10 m), simple water (n 1.35, group index 1.39, absorption
                 30 m at 400 nm, scattering 50 m, 0.85 HG(0.97) + 0.15 Rayleigh).
string_grid:     nx x ny vertical strings spaced `spacing` m on a square grid,
                 n_modules per string spaced dz m (the serving detector is
                 10 x 10 strings, 50 m, 20 modules 15 m apart; the hybrid
                 detector 10 x 10 strings, 50 m, 80 modules 15 m apart).
cascade_string:  electromagnetic cascades, energy log-uniform 1e3-1e5 GeV,
                 1.3e5 photons/GeV, gamma longitudinal profile a = 2 + 0.6 ln E,
                 b = 0.63, radiation length 0.36 m, isotropic direction, vertex
                 10 m from the string at a random azimuth and depth; a string of
                 20 modules 15 m apart with 16 PMTs each (POM layout, 75 mm PMT
                 diameter as the reference scripts use), PMT acceptance resampled
                 to 31 knots on 300-600 nm; simple water.
"""
from __future__ import annotations

import numpy as np

from .detection import DetectionSphere, p_one_pmt_acc, string_of_modules
from .lightyield import AxiconeEmitter, ExtendedCherenkovEmitter, LongitudinalParameterisation
from .medium import make_simple_water
from .photon_prop import PhotonPropSetup
from .spectrum import InverseSquareSpectrum

PMT_AREA = float(np.pi * (75e-3 / 2) ** 2)
SEED_BASE = 0x5EED0000


def point_cone_setup(photons: int = 1_000_000, **kw) -> PhotonPropSetup:
    src = AxiconeEmitter((0.0, 0.0, 0.0), (0.0, 0.0, 1.0), 0.0, photons, float(np.deg2rad(41.2)))
    tgt = DetectionSphere((0.0, 0.0, 10.0), 0.21, 16, PMT_AREA, 1)
    return PhotonPropSetup([src], [tgt], make_simple_water(), InverseSquareSpectrum(300.0, 600.0), **kw)


def cascade_sources(n: int, rng: np.random.Generator, e_min=1e3, e_max=1e5, photons_per_gev=1.3e5,
                    string_z=(0.0, 285.0), distance=10.0, photon_scale=1.0):
    out = []
    for _ in range(n):
        e = 10 ** rng.uniform(np.log10(e_min), np.log10(e_max))
        ct = rng.uniform(-1, 1)
        phi = rng.uniform(0, 2 * np.pi)
        st = np.sqrt(1 - ct * ct)
        direction = (st * np.cos(phi), st * np.sin(phi), ct)
        az = rng.uniform(0, 2 * np.pi)
        z = rng.uniform(string_z[0] + 50.0, string_z[1] - 50.0)
        pos = (distance * np.cos(az), distance * np.sin(az), z)
        lp = LongitudinalParameterisation(a=float(np.float32(2.0 + 0.6 * np.log(e))), b=0.63, lrad=0.36)
        out.append(ExtendedCherenkovEmitter(pos, direction, 0.0, int(photons_per_gev * e * photon_scale), lp))
    return out


def cascade_string_setup(n_cascades: int = 4, seed: int = 1, photon_scale: float = 1.0, **kw) -> PhotonPropSetup:
    rng = np.random.default_rng(seed)
    targets = string_of_modules(20, 15.0, pmt_area=PMT_AREA)
    srcs = cascade_sources(n_cascades, rng, photon_scale=photon_scale)
    return PhotonPropSetup(srcs, targets, make_simple_water(), InverseSquareSpectrum(300.0, 600.0),
                           wavelength_acceptance=p_one_pmt_acc.resampled(300.0, 600.0, 31), **kw)


def string_grid(nx: int = 10, ny: int = 10, spacing: float = 50.0, n_modules: int = 20, dz: float = 15.0,
                z0: float = 0.0):
    """MultiPMTDetector modules of nx * ny strings centred on x = y = 0, module ids 1..N."""
    targets = []
    for j in range(ny):
        for i in range(nx):
            x = (i - (nx - 1) / 2) * spacing
            y = (j - (ny - 1) / 2) * spacing
            targets += string_of_modules(n_modules, dz, x=x, y=y, z_start=z0, pmt_area=PMT_AREA,
                                         id_offset=len(targets))
    return targets


def serving_requests(n: int = 4096, seed: int = 2, rate_hz: float = 200.0, ph_lo: float = 1e4, ph_hi: float = 1e8,
                     cube: float = 100.0, centre=(0.0, 0.0, 142.5), photons_per_gev: float = 1.3e5):
    """Event requests of the serving workload: Poisson arrivals at rate_hz,
    photon counts log-uniform in [ph_lo, ph_hi], cascades (gamma profile a =
    2 + 0.6 ln E with E = photons / photons_per_gev, clamped to E >= 1 GeV so
    that a >= 2, b = 0.63, radiation length 0.36 m), isotropic direction,
    vertex uniform in a cube of side ``cube`` around ``centre``.
    Returns [(arrival_time_s, event_id, source)]."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate_hz, n))
    out = []
    for i in range(n):
        photons = int(10 ** rng.uniform(np.log10(ph_lo), np.log10(ph_hi)))
        e = max(photons / photons_per_gev, 1.0)
        ct = rng.uniform(-1, 1)
        phi = rng.uniform(0, 2 * np.pi)
        st = np.sqrt(1 - ct * ct)
        pos = tuple(c + rng.uniform(-cube / 2, cube / 2) for c in centre)
        lp = LongitudinalParameterisation(a=float(np.float32(2.0 + 0.6 * np.log(e))), b=0.63, lrad=0.36)
        src = ExtendedCherenkovEmitter(pos, (st * np.cos(phi), st * np.sin(phi), ct), 0.0, photons, lp)
        out.append((float(t[i]), i + 1, src))
    return out


def hybrid_setup(**kw) -> PhotonPropSetup:
    """The hybrid detector: 10 x 10 strings, 50 m apart, 80 modules 15 m apart (8000 POM modules x 16 PMTs),
    simple water."""
    return PhotonPropSetup([], string_grid(10, 10, 50.0, 80, 15.0), make_simple_water(),
                           InverseSquareSpectrum(300.0, 600.0),
                           wavelength_acceptance=p_one_pmt_acc.resampled(300.0, 600.0, 31), **kw)


def serving_setup(**kw) -> PhotonPropSetup:
    """The serving detector: 10 x 10 strings, 50 m apart, 20 modules 15 m apart, simple water."""
    return PhotonPropSetup([], string_grid(10, 10, 50.0, 20, 15.0), make_simple_water(),
                           InverseSquareSpectrum(300.0, 600.0),
                           wavelength_acceptance=p_one_pmt_acc.resampled(300.0, 600.0, 31), **kw)
