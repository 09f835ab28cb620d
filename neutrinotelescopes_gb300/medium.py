"""Water optics (src/photon_propagation/medium.jl of the reference).

A medium answers refractive_index / group_velocity / scattering_length /
absorption_length at a wavelength (nm) and carries the phase function
parameters.  ``tabulate`` turns it into the knot tables the device reads
(include/ntp.h, ntp_medium_desc): the kernel interpolates those per photon,
the oracle interpolates the same knots, and a table with 1024 knots over a
few hundred nm differs from the formulas by far less than float rounding.
"""
from __future__ import annotations

import csv
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from .utils import fast_linear_interp

C_VAC_M_NS = 0.299792458  # SpeedOfLightInVacuum in m/ns
DATA = Path(__file__).resolve().parent / "data"

DEFAULT_TABLE_KNOTS = 1024


def _read_csv(name: str) -> tuple[np.ndarray, np.ndarray]:
    with open(DATA / name) as f:
        rows = list(csv.reader(f))[1:]
    a = np.array([[float(x) for x in r] for r in rows if r])
    return a[:, 0], a[:, 1]


# STRAW absorption-length fit, assets/attenuation_length_straw_fit.parquet
STRAW_ABS_WL, STRAW_ABS_LEN = _read_csv("straw_abs_len.csv")


def dippr105(temperature_k: float, A=0.14395, B=0.0112, C=649.727, D=0.05107) -> float:
    """Water density (kg/m^3) from the DIPPR105 formula (medium.jl:26-48)."""
    return A / (B ** (1 + (1 - temperature_k / C) ** D))


def calc_quan_fry_params(salinity: float, temperature: float, pressure: float):
    """Parameters (a01, a2, a3, a4) of the Quan & Fry refractive index (medium.jl:174-205).

    salinity in permille, temperature in degC, pressure in atm.
    """
    n0, n1, n2, n3, n4, n5 = 1.31405, 1.45e-5, 1.779e-4, 1.05e-6, 1.6e-8, 2.02e-6
    n6, n7, n8, n9, n10 = 15.868, 0.01155, 0.00423, 4382, 1.1455e6
    a01 = n0 + (n2 - n3 * temperature + n4 * temperature ** 2) * salinity - n5 * temperature ** 2 + n1 * pressure
    a2 = n6 + n7 * salinity - n8 * temperature
    return a01, a2, -n9, n10


def refractive_index_fry(wavelength, params):
    """Phase refractive index of sea water, Quan & Fry (medium.jl:234-244)."""
    a01, a2, a3, a4 = params
    x = 1.0 / np.asarray(wavelength, dtype=np.float64)
    x2 = x * x
    return x * a2 + a01 + (x2 * a3 + x2 * x * a4)


def dispersion_fry(wavelength, params):
    """dn/dlambda as the reference writes it (medium.jl:293-298).

    The reference unpacks the four parameters into three names, so a2, a3, a4
    take the values of a01, a2, a3; that is reproduced.
    """
    a2, a3, a4 = params[0], params[1], params[2]
    w = np.asarray(wavelength, dtype=np.float64)
    x = 1.0 / w
    return (a2 + 2.0 * x * a3 + 3.0 * x ** 2 * a4) * -1.0 / w ** 2


def sca_len_part_conc(wavelength, vol_conc_small_part: float, vol_conc_large_part: float):
    """Scattering length (m) from particle concentrations (medium.jl:331-347)."""
    x = 550.0 / np.asarray(wavelength, dtype=np.float64)
    c = 0.0017 * x ** 4.3 + 1.34 * vol_conc_small_part * x ** 1.7 + 0.312 * vol_conc_large_part * x ** 0.3
    return 1.0 / c


@dataclass
class MediumTables:
    """Knot tables of a medium, ready for ntp_set_medium."""

    wl_min: float
    wl_max: float
    ref_index: np.ndarray
    group_velocity: np.ndarray
    scattering_length: np.ndarray
    abs_wavelength: np.ndarray
    abs_length: np.ndarray
    hg_g: float
    rayleigh_fraction: float


class MediumProperties:
    """Interface of a medium (MediumProperties, medium.jl:52)."""

    mean_scattering_angle: float = 0.0
    rayleigh_fraction: float = 0.0

    def refractive_index(self, wavelength):
        raise NotImplementedError

    def group_velocity(self, wavelength):
        raise NotImplementedError

    def scattering_length(self, wavelength):
        raise NotImplementedError

    def absorption_table(self) -> tuple[np.ndarray, np.ndarray]:
        """(wavelength nm, absorption length m) knots, linear interpolation."""
        raise NotImplementedError

    def absorption_length(self, wavelength):
        wl, al = self.absorption_table()
        return fast_linear_interp(np.asarray(wavelength, dtype=np.float32), wl.astype(np.float32),
                                  al.astype(np.float32))

    def cherenkov_angle(self, wavelength):
        """acos(1/n) (medium.jl:309-311)."""
        return np.arccos(1.0 / self.refractive_index(wavelength))

    def radiation_length(self) -> float:
        raise NotImplementedError

    def material_density(self) -> float:
        raise NotImplementedError

    def tabulate(self, wl_min: float, wl_max: float, n_knots: int = DEFAULT_TABLE_KNOTS) -> MediumTables:
        """Knot tables on [wl_min, wl_max]; a medium whose per-photon
        quantities do not vary with wavelength gets 2 knots (exact)."""
        wl = np.linspace(wl_min, wl_max, n_knots)
        awl, alen = self.absorption_table()
        tabs = [np.asarray(f(wl), dtype=np.float32) for f in
                (self.refractive_index, self.group_velocity, self.scattering_length)]
        if all(np.all(t == t[0]) for t in tabs):
            tabs = [t[:1].repeat(2) for t in tabs]
        return MediumTables(
            wl_min=float(wl_min),
            wl_max=float(wl_max),
            ref_index=tabs[0],
            group_velocity=tabs[1],
            scattering_length=tabs[2],
            abs_wavelength=np.asarray(awl, dtype=np.float32),
            abs_length=np.asarray(alen, dtype=np.float32),
            hg_g=float(self.mean_scattering_angle),
            rayleigh_fraction=float(self.rayleigh_fraction),
        )


@dataclass
class WaterProperties(MediumProperties):
    """Sea water after the reference (WaterProperties, medium.jl:70-125).

    salinity permille, pressure atm, temperature degC, particle volume
    concentrations ppm, radiation length g/cm^2.  The Quan-Fry parameters are
    rounded to float32 as the reference stores them in the medium's float type.
    Pure Henyey-Greenstein scattering with g = mean_scattering_angle.
    """

    salinity: float
    pressure: float
    temperature: float
    vol_conc_small_part: float
    vol_conc_large_part: float
    radiation_length_gcm2: float
    mean_scattering_angle: float
    rayleigh_fraction: float = 0.0
    density: float = field(init=False)
    quan_fry_params: tuple = field(init=False)

    def __post_init__(self):
        self.density = dippr105(self.temperature + 273.15)
        self.quan_fry_params = tuple(
            float(np.float32(p)) for p in calc_quan_fry_params(self.salinity, self.temperature, self.pressure))

    def refractive_index(self, wavelength):
        return refractive_index_fry(wavelength, self.quan_fry_params)

    def dispersion(self, wavelength):
        return dispersion_fry(wavelength, self.quan_fry_params)

    def group_velocity(self, wavelength):
        """c / (n - lambda_0 dn/dlambda) with lambda_0 = n * lambda, as medium.jl:313-318."""
        n = self.refractive_index(wavelength)
        l0 = n * np.asarray(wavelength, dtype=np.float64)
        return C_VAC_M_NS / (n - l0 * self.dispersion(wavelength))

    def scattering_length(self, wavelength):
        return sca_len_part_conc(wavelength, self.vol_conc_small_part, self.vol_conc_large_part)

    def absorption_table(self):
        return STRAW_ABS_WL, STRAW_ABS_LEN

    def radiation_length(self) -> float:
        return self.radiation_length_gcm2

    def material_density(self) -> float:
        return self.density


def make_cascadia_medium_properties(mean_scattering_angle: float = 0.99) -> WaterProperties:
    """Cascadia Basin water (make_cascadia_medium_properties, medium.jl:131-138)."""
    return WaterProperties(
        salinity=34.82,
        pressure=269.44088 / 1.01325,  # bar -> atm
        temperature=1.8,
        vol_conc_small_part=0.0075,
        vol_conc_large_part=0.0075,
        radiation_length_gcm2=36.08,
        mean_scattering_angle=float(np.float32(mean_scattering_angle)),
    )


@dataclass
class SimpleWater(MediumProperties):
    """Water with a constant phase and group index, a constant scattering
    length, an absorption table and a Henyey-Greenstein + Rayleigh mixture
    phase function."""

    n_phase: float = 1.35
    n_group: float = 1.39
    scattering_length_m: float = 50.0
    abs_wavelength: np.ndarray = None
    abs_length: np.ndarray = None
    mean_scattering_angle: float = 0.97
    rayleigh_fraction: float = 0.15
    radiation_length_m: float = 0.36

    def refractive_index(self, wavelength):
        return np.full(np.shape(wavelength), self.n_phase, dtype=np.float64)

    def group_velocity(self, wavelength):
        return np.full(np.shape(wavelength), C_VAC_M_NS / self.n_group, dtype=np.float64)

    def scattering_length(self, wavelength):
        return np.full(np.shape(wavelength), self.scattering_length_m, dtype=np.float64)

    def absorption_table(self):
        return np.asarray(self.abs_wavelength, dtype=np.float64), np.asarray(self.abs_length, dtype=np.float64)

    def radiation_length(self) -> float:
        return self.radiation_length_m

    def material_density(self) -> float:
        return 1000.0


def straw_shaped_absorption(n_knots: int, wl_min: float, wl_max: float, at_400: float):
    """n_knots equidistant knots of the STRAW absorption shape scaled so that
    the value at 400 nm is ``at_400`` metres."""
    wl = np.linspace(wl_min, wl_max, n_knots)
    shape = fast_linear_interp(wl, STRAW_ABS_WL, STRAW_ABS_LEN)
    ref = float(fast_linear_interp(np.array([400.0]), STRAW_ABS_WL, STRAW_ABS_LEN)[0])
    return wl, shape * (at_400 / ref)


def make_simple_water() -> SimpleWater:
    """The benchmark medium: n = 1.35, group index 1.39, absorption 30 m at
    400 nm (10-knot linear table over 300-600 nm, STRAW-shaped), scattering
    length 50 m, phase function 0.85 HG(g=0.97) + 0.15 Rayleigh."""
    wl, al = straw_shaped_absorption(10, 300.0, 600.0, 30.0)
    return SimpleWater(abs_wavelength=wl, abs_length=al)
