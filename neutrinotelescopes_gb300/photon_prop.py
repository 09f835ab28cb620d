"""The propagation interface of the reference (PhotonPropagationCuda,
src/photon_propagation/photon_prop_cuda.jl), on top of libntp.so.

``PhotonPropSetup`` + ``propagate_photons`` + ``make_hits_from_photons`` +
``calc_total_weight`` + ``calc_time_residual`` keep the reference's names,
argument meaning and column names; the hit table is a numpy record array
(64-byte ``ntp_hit`` records) with extra columns added by the
post-processing calls, instead of a DataFrame.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np

from . import _abi
from .detection import DetectionSphere, MultiPMTDetector, p_one_pmt_acc, pack_targets
from .medium import MediumProperties
from .spectrum import Spectrum

PhotonHit = _abi.HIT_DTYPE  # PhotonHit, photon_prop_cuda.jl:391-399 (+ source_index, photon_index)


def _check(lib, ctx, status: int) -> None:
    if status != _abi.NTP_OK:
        msg = lib.ntp_last_error(ctx)
        raise _abi.NtpError(status, msg.decode() if msg else "")


class HitTable:
    """Hits with named columns (the reference's DataFrame of PhotonHit).

    ``records`` is the structured array of ntp_hit; derived columns
    (pmt_id, total_weight, tres, ...) live in ``extra``.
    """

    def __init__(self, records: np.ndarray, n_photons_simulated: int = 0, extra: dict | None = None):
        self.records = records
        self.n_photons_simulated = int(n_photons_simulated)
        self.extra: dict[str, np.ndarray] = dict(extra or {})
        self._swap = False

    def __len__(self) -> int:
        return len(self.records)

    @property
    def columns(self) -> list[str]:
        return list(self.records.dtype.names) + list(self.extra)

    def __getitem__(self, key):
        if isinstance(key, str):
            if key in self.extra:
                return self.extra[key]
            if self._swap and key in ("direction", "initial_direction"):
                key = "initial_direction" if key == "direction" else "direction"
            return self.records[key]
        sub = HitTable(self.records[key], self.n_photons_simulated, {k: v[key] for k, v in self.extra.items()})
        sub._swap = self._swap
        return sub

    def __setitem__(self, key: str, value) -> None:
        value = np.asarray(value)
        if len(value) != len(self):
            raise ValueError("column length mismatch")
        self.extra[key] = value

    def sorted_by_photon(self) -> "HitTable":
        order = np.lexsort((self.records["photon_index"], self.records["source_index"]))
        return self[order]

    def to_dict(self) -> dict:
        return {c: self[c] for c in self.columns}


@dataclass
class PhotonPropSetup:
    """Sources, targets, medium and spectrum of one propagation
    (PhotonPropSetup, photon_prop_cuda.jl:34-45).

    Options beyond the reference: ``max_steps`` (15 in the reference kernel),
    ``hit_policy`` ('first' = first target in list order, as the reference;
    'nearest'), ``exact_pole_rotation`` (apply the true rotation where the
    reference's rot_from_ez_fast uses copysign at |a_z| = 1), ``device`` and
    ``wavelength_acceptance`` (PMT acceptance table; default assets/PMTAcc.csv)
    and ``plain_scan`` (test every target at every step instead of culling by
    vertical columns; same hits, slower).
    """

    sources: list
    targets: list
    medium: MediumProperties
    spectrum: Spectrum
    max_steps: int = 15
    hit_policy: str = "first"
    exact_pole_rotation: bool = False
    device: int = 0
    medium_knots: int = 1024
    wavelength_acceptance: object = None
    plain_scan: bool = False
    _ctx: object = field(default=None, init=False, repr=False)
    _uploaded: tuple = field(default=(), init=False, repr=False)

    def __post_init__(self):
        if not isinstance(self.sources, (list, tuple)):
            self.sources = [self.sources]
        if not isinstance(self.targets, (list, tuple)):
            self.targets = [self.targets]
        self.sources = list(self.sources)
        self.targets = list(self.targets)

    # -- device context -------------------------------------------------
    def context(self):
        """(library, ntp_ctx*) with medium, spectrum, targets and acceptance uploaded."""
        lib = _abi.load_library()
        if self._ctx is None:
            ctx = C.c_void_p()
            st = lib.ntp_create(self.device, C.byref(ctx))
            if st != _abi.NTP_OK:
                raise _abi.NtpError(st, lib.ntp_last_error(None).decode())
            self._ctx = ctx
        key = (id(self.medium), id(self.spectrum), tuple(id(t) for t in self.targets), self.medium_knots,
               id(self.wavelength_acceptance))
        if key != self._uploaded:
            self._upload(lib)
            self._uploaded = key
        return lib, self._ctx

    def _upload(self, lib) -> None:
        ctx = self._ctx
        lo, hi = self.spectrum.wl_range
        tab = self.medium.tabulate(lo, hi, self.medium_knots)
        keep = [np.ascontiguousarray(a, dtype=np.float32) for a in
                (tab.ref_index, tab.group_velocity, tab.scattering_length, tab.abs_wavelength, tab.abs_length)]
        md = _abi.NtpMediumDesc(n_knots=len(keep[0]), wl_min=tab.wl_min, wl_max=tab.wl_max,
                                ref_index=_abi.fptr(keep[0]), group_velocity=_abi.fptr(keep[1]),
                                scattering_length=_abi.fptr(keep[2]), n_abs_knots=len(keep[3]),
                                abs_wavelength=_abi.fptr(keep[3]), abs_length=_abi.fptr(keep[4]),
                                hg_g=tab.hg_g, rayleigh_fraction=tab.rayleigh_fraction)
        _check(lib, ctx, lib.ntp_set_medium(ctx, C.byref(md)))
        sd, _knots = self.spectrum.desc()
        _check(lib, ctx, lib.ntp_set_spectrum(ctx, C.byref(sd)))
        recs, coords = pack_targets(self.targets)
        _check(lib, ctx, lib.ntp_set_targets(ctx, recs, len(self.targets), _abi.fptr(coords),
                                             len(coords) // 2))
        acc = self.wavelength_acceptance or p_one_pmt_acc
        awl = np.ascontiguousarray(acc.xs, dtype=np.float64)
        aval = np.ascontiguousarray(acc.ys, dtype=np.float64)
        dp = C.POINTER(C.c_double)
        _check(lib, ctx, lib.ntp_set_wavelength_acceptance(ctx, awl.ctypes.data_as(dp), aval.ctypes.data_as(dp),
                                                           len(awl)))

    def close(self) -> None:
        if self._ctx is not None:
            _abi.load_library().ntp_destroy(self._ctx)
            self._ctx = None
            self._uploaded = ()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def prop_opts(self, stream: int | None = None) -> _abi.NtpPropOpts:
        if self.hit_policy not in ("first", "nearest"):
            raise ValueError("hit_policy must be 'first' or 'nearest'")
        return _abi.NtpPropOpts(
            max_steps=self.max_steps,
            hit_policy=_abi.HIT_FIRST_IN_LIST if self.hit_policy == "first" else _abi.HIT_NEAREST,
            flags=(_abi.FLAG_EXACT_POLE_ROTATION if self.exact_pole_rotation else 0)
            | (_abi.FLAG_PLAIN_SCAN if self.plain_scan else 0),
            stream=stream,
        )


def pack_sources(sources: Sequence) -> C.Array:
    arr = (_abi.NtpSource * max(len(sources), 1))()
    for i, s in enumerate(sources):
        arr[i] = s.to_c()
    return arr


def _default_capacity(total: int) -> int:
    return int(min(max(total // 100, 1 << 16), 1 << 26))


def propagate_photons(setup: PhotonPropSetup, *, seed: int = 0, capacity: int | None = None,
                      reference_columns: bool = True) -> HitTable:
    """Propagate every photon of every source; returns the hits
    (propagate_photons, photon_prop_cuda.jl:804-817).

    The hit count is exact: if the first buffer is too small the run is
    repeated with an exact-size buffer (same seed, hence the same hits).
    With ``reference_columns`` and a single target, the ``direction`` and
    ``initial_direction`` columns are exchanged as the reference's
    single-target kernel writes them (photon_prop_cuda.jl:591-592).
    """
    lib, ctx = setup.context()
    srcs = pack_sources(setup.sources)
    total = sum(int(s.photons) for s in setup.sources)
    cap = _default_capacity(total) if capacity is None else int(capacity)
    opts = setup.prop_opts()
    while True:
        out = np.empty(max(cap, 1), dtype=_abi.HIT_DTYPE)
        n_hits, n_sim = C.c_uint64(), C.c_uint64()
        st = lib.ntp_propagate(ctx, srcs, len(setup.sources), C.c_uint64(seed & (2 ** 64 - 1)), C.byref(opts),
                               out.ctypes.data, cap, 0, C.byref(n_hits), C.byref(n_sim))
        if st == _abi.NTP_ERR_OVERFLOW and capacity is None:
            cap = int(n_hits.value)
            continue
        _check(lib, ctx, st)
        break
    table = HitTable(out[: n_hits.value], n_sim.value)
    table._swap = reference_columns and len(setup.targets) == 1
    return table


def make_hits_from_photons(hits: HitTable, setup: PhotonPropSetup, target_orientation) -> HitTable:
    """Hits that land inside a PMT, with a ``pmt_id`` column (1-based)
    (make_hits_from_photons, photon_prop_cuda.jl:884-904)."""
    lib, ctx = setup.context()
    R = np.ascontiguousarray(np.asarray(target_orientation, dtype=np.float64).reshape(3, 3))
    recs = np.ascontiguousarray(hits.records)
    pmt = np.zeros(len(recs), dtype=np.int32)
    _check(lib, ctx, lib.ntp_make_hits(ctx, recs.ctypes.data, len(recs), R.ctypes.data_as(C.POINTER(C.c_double)),
                                       pmt.ctypes.data, 0, None))
    mask = pmt > 0
    out = hits[mask]
    out.extra["pmt_id"] = pmt[mask]
    return out


def calc_total_weight(hits: HitTable, setup: PhotonPropSetup) -> HitTable:
    """Adds area_acc, wl_acc, abs_weight, ref_ix and total_weight columns
    (calc_total_weight!, photon_prop_cuda.jl:850-882)."""
    lib, ctx = setup.context()
    recs = np.ascontiguousarray(hits.records)
    n = len(recs)
    cols = {k: np.zeros(n, dtype=np.float64) for k in ("area_acc", "wl_acc", "abs_weight", "total_weight")}
    _check(lib, ctx, lib.ntp_calc_total_weight(ctx, recs.ctypes.data, n, cols["area_acc"].ctypes.data,
                                               cols["wl_acc"].ctypes.data, cols["abs_weight"].ctypes.data,
                                               cols["total_weight"].ctypes.data, 0, None))
    for k, v in cols.items():
        hits.extra[k] = v
    hits.extra["ref_ix"] = np.asarray(setup.medium.refractive_index(recs["wavelength"].astype(np.float64)))
    return hits


calc_total_weight_ = calc_total_weight


def calc_time_residual(hits: HitTable, setup: PhotonPropSetup) -> HitTable:
    """Adds the ``tres`` column: time minus the direct-light time from the
    first source to each module (calc_time_residual!, photon_prop_cuda.jl:906-924)."""
    lib, ctx = setup.context()
    recs = np.ascontiguousarray(hits.records)
    n = len(recs)
    tres = np.zeros(n, dtype=np.float64)
    src = (C.c_float * 3)(*[float(v) for v in setup.sources[0].position])
    n800 = float(np.float32(np.asarray(setup.medium.refractive_index(np.array([800.0])))[0]))
    _check(lib, ctx, lib.ntp_calc_time_residual(ctx, recs.ctypes.data, n, src, n800, tres.ctypes.data, 0, None))
    hits.extra["tres"] = tres
    return hits


calc_time_residual_ = calc_time_residual


def pmt_summary(hits: HitTable, setup: PhotonPropSetup, target_orientation, *, n_bins: int = 0,
                t_range=(-20.0, 1500.0), time_residual: bool = True) -> dict:
    """Per (target, PMT) weight sums, hit counts and weighted time histograms
    in double precision (ntp_pmt_summary): the fusion of
    make_hits_from_photons, calc_total_weight and calc_time_residual with the
    per-(module, PMT) grouping of resample_simulation.  Arrays are indexed
    [target index, pmt - 1 (, bin)]."""
    lib, ctx = setup.context()
    max_pmts = max([t.pmt_coordinates.shape[1] if isinstance(t, MultiPMTDetector) else 1 for t in setup.targets]
                   or [1])
    n_t = len(setup.targets)
    recs = np.ascontiguousarray(hits.records)
    R = np.ascontiguousarray(np.asarray(target_orientation, dtype=np.float64).reshape(3, 3))
    n800 = float(np.float32(np.asarray(setup.medium.refractive_index(np.array([800.0])))[0]))
    spec = _abi.NtpSummarySpec(max_pmts=max_pmts, n_bins=n_bins, t_min=t_range[0], t_max=t_range[1],
                               use_time_residual=int(time_residual),
                               source_position=tuple(float(v) for v in setup.sources[0].position) if setup.sources
                               else (0.0, 0.0, 0.0), n800=n800)
    wsum = np.zeros((n_t, max_pmts))
    count = np.zeros((n_t, max_pmts))
    hist = np.zeros((n_t, max_pmts, max(n_bins, 1)))
    _check(lib, ctx, lib.ntp_pmt_summary(ctx, recs.ctypes.data, len(recs), R.ctypes.data_as(C.POINTER(C.c_double)),
                                         C.byref(spec), wsum.ctypes.data, count.ctypes.data,
                                         hist.ctypes.data if n_bins > 0 else None, 0, None))
    out = {"weight_sum": wsum, "hit_count": count}
    if n_bins > 0:
        out["time_hist"] = hist
        out["bin_edges"] = np.linspace(t_range[0], t_range[1], n_bins + 1)
    return out


def resample_simulation(hits: HitTable, setup: PhotonPropSetup, *, downsample: float = 1.0, seed: int = 0,
                        time_col: str = "time") -> dict:
    """Poisson-resampled hits per (module, PMT) (resample_simulation with
    per_pmt = true, pmt_frontend/pipeline.jl:86-116) on the device.

    ``hits`` needs the ``pmt_id`` column (make_hits_from_photons) and
    ``total_weight`` (calc_total_weight); ``time_col`` names the time that is
    kept ("time", or "tres" after calc_time_residual).  Returns columns
    pmt_id, module_id, the time column and hit_index (row in ``hits``),
    grouped by (module, PMT).
    """
    lib, ctx = setup.context()
    max_pmts = max([t.pmt_coordinates.shape[1] if isinstance(t, MultiPMTDetector) else 1 for t in setup.targets]
                   or [1])
    recs = np.ascontiguousarray(hits.records)
    n = len(recs)
    pmt = np.ascontiguousarray(hits["pmt_id"], dtype=np.int32)
    w = np.ascontiguousarray(hits["total_weight"], dtype=np.float64)
    tv = np.ascontiguousarray(hits[time_col], dtype=np.float64)
    cap = max(n, 1)
    g = np.zeros(cap, dtype=np.int32)
    t = np.zeros(cap)
    hi = np.zeros(cap, dtype=np.uint64)
    n_out = C.c_uint64()
    _check(lib, ctx, lib.ntp_resample(ctx, recs.ctypes.data, n, pmt.ctypes.data, w.ctypes.data, tv.ctypes.data,
                                      max_pmts, float(downsample), C.c_uint64(seed & (2 ** 64 - 1)), g.ctypes.data,
                                      t.ctypes.data, hi.ctypes.data, cap, C.byref(n_out), 0, None))
    k = n_out.value
    g, t, hi = g[:k], t[:k], hi[:k]
    order = np.lexsort((hi, g))
    g, t, hi = g[order], t[order], hi[order]
    module_ids = np.array([tg.module_id for tg in setup.targets], dtype=np.uint32)
    return {"pmt_id": (g % max_pmts + 1).astype(np.int32), "module_id": module_ids[g // max_pmts],
            time_col: t, "hit_index": hi}
