"""Photon wavelength spectra (src/photon_propagation/spectrum.jl of the reference)."""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import _abi
from .utils import integrate_gauss_quad

FINE_STRUCTURE = 7.2973525693e-3  # CODATA2018


def frank_tamm(wavelength, ref_index):
    """Frank-Tamm photon density per unit length and wavelength (spectrum.jl:32-34)."""
    return 2 * np.pi * FINE_STRUCTURE / np.asarray(wavelength) ** 2 * (1 - 1 / np.asarray(ref_index) ** 2)


def frank_tamm_norm(wl_range, ref_index_func) -> float:
    """Cherenkov photons per metre in wl_range, nm (spectrum.jl:42-45)."""
    return integrate_gauss_quad(lambda wl: frank_tamm(wl, ref_index_func(wl)), wl_range[0], wl_range[1]) * 1e9


def frank_tamm_inverted_cdf(wl_range, medium, step_size: float = 1.0):
    """(cdf values, wavelengths) on a step_size grid (spectrum.jl:55-71)."""
    wl_steps = np.arange(wl_range[0], wl_range[1] + step_size / 2, step_size)
    n = lambda wl: medium.refractive_index(wl)
    full = frank_tamm_norm(wl_range, n)
    norms = np.zeros(len(wl_steps))
    for i in range(1, len(wl_steps)):
        norms[i] = frank_tamm_norm((wl_range[0], wl_steps[i]), n) / full
    order = np.argsort(norms, kind="stable")
    return norms[order], wl_steps[order]


class Spectrum:
    def desc(self) -> tuple[_abi.NtpSpectrumDesc, object]:
        """ntp_spectrum_desc and the array it points to (kept alive by the caller)."""
        raise NotImplementedError

    @property
    def wl_range(self) -> tuple[float, float]:
        raise NotImplementedError


@dataclass
class Monochromatic(Spectrum):
    """Single wavelength (spectrum.jl:21-23)."""

    wavelength: float

    @property
    def wl_range(self):
        return (self.wavelength - 1.0, self.wavelength + 1.0)

    def desc(self):
        d = _abi.NtpSpectrumDesc(kind=_abi.SPEC_MONOCHROMATIC, n_knots=0, wavelength=self.wavelength)
        return d, None


class CherenkovSpectrum(Spectrum):
    """Cherenkov spectrum as an inverse-CDF table (spectrum.jl:89-108).

    ``CherenkovSpectrum(wl_range, interp_steps, medium)`` builds the knots as the
    reference does: the Frank-Tamm CDF on a 1 nm grid (10-point Gauss-Legendre
    per interval), linearly interpolated at interp_steps equidistant
    probabilities.  The reference reads the knots through a CUDA texture with
    linear filtering and normalised coordinates; ``semantics='texture'``
    (default) reproduces that lookup, ``'linear'`` interpolates the knots
    exactly as an inverse CDF.
    """

    def __init__(self, wl_range, interp_steps: int = 30, medium=None, *, knots=None, semantics: str = "texture"):
        self._wl_range = (float(wl_range[0]), float(wl_range[1]))
        if knots is None:
            norms, wl_steps = frank_tamm_inverted_cdf(self._wl_range, medium)
            u = np.linspace(0.0, 1.0, interp_steps)
            knots = np.interp(u, norms, wl_steps)
        self.knots = np.ascontiguousarray(knots, dtype=np.float32)
        if semantics not in ("texture", "linear"):
            raise ValueError("semantics must be 'texture' or 'linear'")
        self.semantics = semantics

    @property
    def wl_range(self):
        return self._wl_range

    def desc(self):
        kind = _abi.SPEC_TABLE_TEXTURE if self.semantics == "texture" else _abi.SPEC_TABLE_LINEAR
        d = _abi.NtpSpectrumDesc(kind=kind, n_knots=len(self.knots), icdf_knots=_abi.fptr(self.knots))
        return d, self.knots


@dataclass
class InverseSquareSpectrum(Spectrum):
    """dN/dlambda proportional to 1/lambda^2 on [lo, hi] (Frank-Tamm with a
    constant refractive index), sampled by its exact inverse CDF."""

    lo: float = 300.0
    hi: float = 600.0

    @property
    def wl_range(self):
        return (self.lo, self.hi)

    def desc(self):
        d = _abi.NtpSpectrumDesc(kind=_abi.SPEC_INV_SQUARE, n_knots=0, wl_min=self.lo, wl_max=self.hi)
        return d, None
