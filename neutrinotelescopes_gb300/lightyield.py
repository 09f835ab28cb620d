"""Photon sources and light yield (src/photon_propagation/lightyield.jl and
src/types.jl of the reference).

Emitters are plain records; ``to_c`` packs one into the 64-byte ntp_source of
include/ntp.h.
"""
from __future__ import annotations

import dataclasses
from dataclasses import dataclass
from math import gamma as _gamma_fn
from typing import Sequence

import numpy as np

from . import _abi
from .medium import MediumProperties
from .spectrum import frank_tamm_norm


# ---------------------------------------------------------------- particles
class ParticleType:
    pdg = 0


class PEPlus(ParticleType):
    pdg = -11


class PEMinus(ParticleType):
    pdg = 11


class PGamma(ParticleType):
    pdg = 22


@dataclass
class Particle:
    """A particle (types.jl:18-24): position m, direction, time ns, energy GeV."""

    position: Sequence[float]
    direction: Sequence[float]
    time: float
    energy: float
    type: type = PEMinus


# ------------------------------------------------------ longitudinal profile
@dataclass(frozen=True)
class LongitudinalParameters:
    alpha: float
    beta: float
    b: float


LongitudinalParametersEMinus = LongitudinalParameters(alpha=2.01849, beta=1.45469, b=0.63207)
LongitudinalParametersEPlus = LongitudinalParameters(alpha=2.00035, beta=1.45501, b=0.63008)
LongitudinalParametersGamma = LongitudinalParameters(alpha=2.83923, beta=1.34031, b=0.64526)

_LONG = {PEMinus: LongitudinalParametersEMinus, PEPlus: LongitudinalParametersEPlus,
         PGamma: LongitudinalParametersGamma}


def get_longitudinal_params(ptype) -> LongitudinalParameters:
    return _LONG[ptype]


def long_parameter_a_edep(energy: float, long_pars: LongitudinalParameters) -> float:
    """a = alpha + beta log10(E) (lightyield.jl:204-209)."""
    return long_pars.alpha + long_pars.beta * np.log10(energy)


@dataclass
class LongitudinalParameterisation:
    """Gamma-profile parameters of a cascade (lightyield.jl:139-158)."""

    a: float
    b: float
    lrad: float

    @classmethod
    def from_energy(cls, energy: float, medium: MediumProperties, long_pars) -> "LongitudinalParameterisation":
        if isinstance(long_pars, type):
            long_pars = get_longitudinal_params(long_pars)
        a = np.float32(long_parameter_a_edep(energy, long_pars))
        b = np.float32(long_pars.b)
        lrad = medium.radiation_length() / medium.material_density() * 10  # g/cm^2 / (kg/m^3) -> m
        return cls(float(a), float(b), float(lrad))


def longitudinal_profile(z, long_param: LongitudinalParameterisation):
    """Longitudinal shower profile pdf at depth z in m (lightyield.jl:221-230)."""
    t = np.asarray(z) / long_param.lrad
    a, b = long_param.a, long_param.b
    return b * ((t * b) ** (a - 1.0) * np.exp(-(t * b)) / _gamma_fn(a))


# ------------------------------------------------------------ track length
@dataclass(frozen=True)
class CherenkovTrackLengthParameters:
    alpha: float
    beta: float
    alpha_dev: float
    beta_dev: float


CherenkovTrackLengthParametersEMinus = CherenkovTrackLengthParameters(5.3207078881, 1.00000211, 0.0578170887, 0.5)
CherenkovTrackLengthParametersEPlus = CherenkovTrackLengthParameters(5.3211320598, 0.99999254, 0.0573419669, 0.5)
CherenkovTrackLengthParametersGamma = CherenkovTrackLengthParameters(5.3208540905, 0.99999877, 0.0578170887,
                                                                     5.66586567)
_TRACK = {PEMinus: CherenkovTrackLengthParametersEMinus, PEPlus: CherenkovTrackLengthParametersEPlus,
          PGamma: CherenkovTrackLengthParametersGamma}


def cherenkov_track_length(energy: float, ptype=PEMinus) -> float:
    """Cherenkov track length in m (lightyield.jl:350-353)."""
    p = _TRACK[ptype] if isinstance(ptype, type) else ptype
    return p.alpha * energy ** p.beta


def total_lightyield(particle: Particle, medium: MediumProperties, wl_range) -> float:
    """Expected photon count: Frank-Tamm norm times track length (lightyield.jl:356-366)."""
    return frank_tamm_norm(wl_range, medium.refractive_index) * cherenkov_track_length(particle.energy, particle.type)


STD_ANG_DIST_PARS = (4.27033, -6.02527, 0.29887, -0.00103)


def cherenkov_ang_dist(costheta, ref_index, pars=STD_ANG_DIST_PARS):
    """Angular distribution of Cherenkov photons of EM cascades (lightyield.jl:59-71)."""
    a, b, c, d = pars
    return a * np.exp(b * np.abs(np.asarray(costheta) - 1 / ref_index) ** c) + d


# ----------------------------------------------------------------- emitters
def _v3(v):
    return (float(v[0]), float(v[1]), float(v[2]))


class PhotonSource:
    photons: int
    kind: int

    def to_c(self) -> _abi.NtpSource:
        raise NotImplementedError


@dataclass
class PointlikeIsotropicEmitter(PhotonSource):
    """lightyield.jl:436-440"""

    position: Sequence[float]
    time: float
    photons: int
    kind = _abi.SRC_POINT_ISOTROPIC

    def to_c(self):
        return _abi.NtpSource(position=_v3(self.position), time=self.time, photons=int(self.photons), kind=self.kind)


@dataclass
class PointlikeTimeRangeEmitter(PhotonSource):
    """lightyield.jl:449-453"""

    position: Sequence[float]
    time_range: tuple
    photons: int
    kind = _abi.SRC_POINT_TIME_RANGE

    def to_c(self):
        return _abi.NtpSource(position=_v3(self.position), time=self.time_range[0], time_end=self.time_range[1],
                              photons=int(self.photons), kind=self.kind)


@dataclass
class AxiconeEmitter(PhotonSource):
    """lightyield.jl:421-427: photons on a cone of half-angle ``angle`` around ``direction``."""

    position: Sequence[float]
    direction: Sequence[float]
    time: float
    photons: int
    angle: float
    kind = _abi.SRC_AXICONE

    def to_c(self):
        return _abi.NtpSource(position=_v3(self.position), direction=_v3(self.direction), time=self.time,
                              angle=self.angle, photons=int(self.photons), kind=self.kind)


@dataclass
class PencilEmitter(PhotonSource):
    """lightyield.jl:429-434"""

    position: Sequence[float]
    direction: Sequence[float]
    time: float
    photons: int
    kind = _abi.SRC_PENCIL

    def to_c(self):
        return _abi.NtpSource(position=_v3(self.position), direction=_v3(self.direction), time=self.time,
                              photons=int(self.photons), kind=self.kind)


@dataclass
class ExtendedCherenkovEmitter(PhotonSource):
    """Cascade with a gamma longitudinal profile (lightyield.jl:463-481)."""

    position: Sequence[float]
    direction: Sequence[float]
    time: float
    photons: int
    long_param: LongitudinalParameterisation
    kind = _abi.SRC_EXTENDED_CHERENKOV

    @classmethod
    def from_particle(cls, particle: Particle, medium: MediumProperties, wl_range, oversample: float = 1.0,
                      rng: np.random.Generator | None = None) -> "ExtendedCherenkovEmitter":
        rng = rng or np.random.default_rng()
        long_param = LongitudinalParameterisation.from_energy(particle.energy, medium, particle.type)
        photons = int(rng.poisson(total_lightyield(particle, medium, wl_range) * oversample))
        return cls(particle.position, particle.direction, particle.time, photons, long_param)

    def to_c(self):
        return _abi.NtpSource(position=_v3(self.position), direction=_v3(self.direction), time=self.time,
                              photons=int(self.photons), kind=self.kind, long_a=self.long_param.a,
                              long_b=self.long_param.b, long_lrad=self.long_param.lrad)


@dataclass
class PointlikeCherenkovEmitter(PhotonSource):
    """lightyield.jl:491-509"""

    position: Sequence[float]
    direction: Sequence[float]
    time: float
    photons: int
    kind = _abi.SRC_POINT_CHERENKOV

    @classmethod
    def from_particle(cls, particle: Particle, medium: MediumProperties, wl_range,
                      rng: np.random.Generator | None = None) -> "PointlikeCherenkovEmitter":
        rng = rng or np.random.default_rng()
        photons = int(rng.poisson(total_lightyield(particle, medium, wl_range)))
        return cls(particle.position, particle.direction, particle.time, photons)

    def to_c(self):
        return _abi.NtpSource(position=_v3(self.position), direction=_v3(self.direction), time=self.time,
                              photons=int(self.photons), kind=self.kind)


@dataclass
class CherenkovTrackEmitter(PhotonSource):
    """Uniform emission along a track of ``length`` m (lightyield.jl:519-530).

    The reference's initialiser assigns a scalar angle to the direction
    (photon_prop_cuda.jl:197) and so cannot run; photons here leave on the
    Cherenkov cone around the track, as for PointlikeCherenkovEmitter.
    """

    position: Sequence[float]
    direction: Sequence[float]
    time: float
    length: float
    photons: int
    kind = _abi.SRC_CHERENKOV_TRACK

    def to_c(self):
        return _abi.NtpSource(position=_v3(self.position), direction=_v3(self.direction), time=self.time,
                              length=self.length, photons=int(self.photons), kind=self.kind)


def split_source(source: PhotonSource, parts: int) -> list:
    """Split into ``parts`` sources, the last taking the remainder (lightyield.jl:372-401)."""
    if source.photons < parts:
        raise ValueError("Cannot split source. Fewer photons than parts")
    ph_split, remainder = divmod(int(source.photons), parts)
    return [dataclasses.replace(source, photons=ph_split + (remainder if i == parts - 1 else 0))
            for i in range(parts)]


def oversample_source(source: PhotonSource, factor: float) -> PhotonSource:
    """Same source with photons multiplied by ``factor`` (lightyield.jl:410-420)."""
    return dataclasses.replace(source, photons=int(source.photons * factor))
