"""Optical modules and detector layouts (src/photon_propagation/detection.jl of the reference)."""
from __future__ import annotations

from dataclasses import dataclass
from itertools import product
from typing import Sequence

import numpy as np

from . import _abi
from .medium import _read_csv
from .utils import calc_rot_matrix, cart_to_sph, fast_linear_interp, sph_to_cart


class PhotonTarget:
    position: Sequence[float]
    radius: float
    module_id: int


@dataclass
class DetectionSphere(PhotonTarget):
    """Spherical module read out as one unit (detection.jl:29-36)."""

    position: Sequence[float]
    radius: float
    n_pmts: int
    pmt_area: float
    module_id: int = 1


@dataclass
class MultiPMTDetector(PhotonTarget):
    """Spherical module with PMTs at (theta, phi) columns of ``pmt_coordinates``
    (2 x N, detection.jl:39-46)."""

    position: Sequence[float]
    radius: float
    pmt_area: float
    pmt_coordinates: np.ndarray
    module_id: int = 1


def get_pmt_count(target) -> int:
    return 1 if isinstance(target, DetectionSphere) else int(np.shape(target.pmt_coordinates)[1])


def make_pom_pmt_coordinates(dtype=np.float32) -> np.ndarray:
    """(theta, phi) of the 16 PMTs of a POM (detection.jl:107-134).

    Four rings at 90-57.5, 90-25, 90+25, 90+57.5 degrees (azimuths offset by
    pi/4 on the outer rings), then the module rotated so that e_z goes to e_x.
    """
    coords = np.zeros((2, 16), dtype=np.float64)
    coords[0, 0:4] = np.deg2rad(90 - 57.5)
    coords[1, 0:4] = np.pi / 4 + np.arange(4) * np.pi / 2
    coords[0, 4:8] = np.deg2rad(90 - 25)
    coords[1, 4:8] = np.arange(4) * np.pi / 2
    coords[0, 8:12] = np.deg2rad(90 + 25)
    coords[1, 8:12] = np.arange(4) * np.pi / 2
    coords[0, 12:16] = np.deg2rad(90 + 57.5)
    coords[1, 12:16] = np.pi / 4 + np.arange(4) * np.pi / 2
    R = calc_rot_matrix([0.0, 0.0, 1.0], [1.0, 0.0, 0.0])
    for j in range(16):
        cart = R @ sph_to_cart(coords[0, j], coords[1, j])
        coords[:, j] = cart_to_sph(*cart)
    return coords.astype(dtype)


def area_acceptance(position, target) -> float:
    """Fraction of the module surface covered by PMTs (detection.jl:139-146)."""
    if isinstance(target, DetectionSphere):
        total = np.float32(target.n_pmts) * np.float32(target.pmt_area)
        return float(total) / (4 * np.pi * float(np.float32(target.radius) ** 2))
    return 1.0


_ACC_WL, _ACC = _read_csv("pmt_acceptance.csv")


class PMTWavelengthAcceptance:
    """Linear interpolation of a PMT's wavelength acceptance (detection.jl:148-163)."""

    def __init__(self, xs, ys):
        self.xs = np.asarray(xs, dtype=np.float64)
        self.ys = np.asarray(ys, dtype=np.float64)

    def __call__(self, wavelength):
        return fast_linear_interp(np.asarray(wavelength, dtype=np.float64), self.xs, self.ys)

    def resampled(self, lo: float, hi: float, n: int) -> "PMTWavelengthAcceptance":
        xs = np.linspace(lo, hi, n)
        return PMTWavelengthAcceptance(xs, self(xs))


# assets/PMTAcc.csv, 200-800 nm, peak 0.27 near 400 nm
p_one_pmt_acc = PMTWavelengthAcceptance(_ACC_WL, _ACC)


def make_detector_cube(nx, ny, nz, spacing_vert, spacing_hor):
    """Positions on a cubic grid (detection.jl:167-178)."""
    out = np.zeros((nx * ny * nz, 3))
    for i, j, k in product(range(nx), range(ny), range(nz)):
        ix = i + nx * (j + ny * k)
        out[ix] = [-0.5 * spacing_hor * nx + i * spacing_hor, -0.5 * spacing_hor * ny + j * spacing_hor,
                   -0.5 * spacing_vert * nz + k * spacing_vert]
    return out


def make_detector_hex(n_side: int, n_z: int, spacing_hor: float, spacing_vert: float, truncate: int = 0):
    """Positions of a hexagonal string layout (detection.jl:181-204)."""
    positions = []
    z_positions = np.arange(0, n_z * spacing_vert + spacing_vert / 2, spacing_vert)
    for irow in range(0, n_side - truncate + 1):
        i_this_row = 2 * (n_side - 1) - irow
        x_pos = np.linspace(-(i_this_row - 1) / 2 * spacing_hor, (i_this_row - 1) / 2 * spacing_hor, i_this_row)
        y = irow * spacing_hor * np.sqrt(3) / 2
        for x, z in product(x_pos, z_positions):
            positions.append([x, y, z])
        if irow != 0:
            y = -irow * spacing_hor * np.sqrt(3) / 2
            for x, z in product(x_pos, z_positions):
                positions.append([x, y, z])
    return np.array(positions)


def make_targets(positions, n_pmts: int, pmt_area: float):
    """DetectionSphere of radius 0.21 m at each position (detection.jl:208-210)."""
    return [DetectionSphere(tuple(p), 0.21, n_pmts, pmt_area, i + 1) for i, p in enumerate(positions)]


def string_of_modules(n_modules: int, dz: float, x: float = 0.0, y: float = 0.0, z_start: float = 0.0,
                      radius: float = 0.21, pmt_area: float = np.pi * (75e-3 / 2) ** 2, id_offset: int = 0,
                      pmt_coordinates=None):
    """A vertical string of MultiPMTDetector modules (as positions_on_line in
    scripts/simulate_event_full_test.jl:12-31)."""
    coords = make_pom_pmt_coordinates() if pmt_coordinates is None else pmt_coordinates
    return [MultiPMTDetector((x, y, z_start + i * dz), radius, pmt_area, coords, i + 1 + id_offset)
            for i in range(n_modules)]


def pack_targets(targets) -> tuple[np.ndarray, np.ndarray]:
    """ntp_target records and the (theta, phi) PMT coordinate table."""
    recs = (_abi.NtpTarget * max(len(targets), 1))()
    coords: list[np.ndarray] = []
    layout_offsets: dict[int, int] = {}
    n_coords = 0
    for i, t in enumerate(targets):
        r = recs[i]
        r.position = tuple(float(v) for v in t.position)
        r.radius = float(t.radius)
        r.module_id = int(t.module_id)
        r.pmt_area = float(t.pmt_area)
        if isinstance(t, MultiPMTDetector):
            pc = np.asarray(t.pmt_coordinates, dtype=np.float32)
            key = id(t.pmt_coordinates)
            if key not in layout_offsets:
                layout_offsets[key] = n_coords
                coords.append(pc.T.reshape(-1))
                n_coords += pc.shape[1]
            r.kind = _abi.TARGET_MULTI_PMT
            r.n_pmts = pc.shape[1]
            r.pmt_offset = layout_offsets[key]
        else:
            r.kind = _abi.TARGET_SPHERE
            r.n_pmts = int(t.n_pmts)
            r.pmt_offset = 0
    flat = np.ascontiguousarray(np.concatenate(coords) if coords else np.zeros(0), dtype=np.float32)
    return recs, flat
