"""Python access to the CPU oracle (oracle/libntp_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by the
CPU-baseline leg of bench.py, always as the reference the GPU results are
compared with or as the timed CPU reference, never as the product path.  Parity status and its limits are stated
at the top of ntp_oracle.c.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

from neutrinotelescopes_gb300 import _abi

HERE = Path(__file__).resolve().parent
LIB = HERE / "libntp_oracle.so"
_lib = None


def build() -> Path:
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    r = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        d, u32, u64, i32, vp = C.c_double, C.c_uint32, C.c_uint64, C.c_int, C.c_void_p
        dp = C.POINTER(C.c_double)
        L.ntpo_philox4x32_10.argtypes = [C.POINTER(u32), C.POINTER(u32), C.POINTER(u32)]
        L.ntpo_u01_f64.argtypes = [u32]
        L.ntpo_u01_f64.restype = d
        common = [C.POINTER(_abi.NtpSource), i32, C.POINTER(_abi.NtpMediumDesc), C.POINTER(_abi.NtpSpectrumDesc),
                  C.POINTER(_abi.NtpTarget), i32, u64, C.POINTER(_abi.NtpPropOpts), u64, u64, vp, u64]
        L.ntpo_propagate_f64.argtypes = common
        L.ntpo_propagate_f64.restype = u64
        L.ntpo_propagate_f64_binned.argtypes = common
        L.ntpo_propagate_f64_binned.restype = u64
        L.ntpo_propagate_f32.argtypes = common + [i32]
        L.ntpo_propagate_f32.restype = u64
        L.ntpo_propagate_f32_binned.argtypes = common + [i32]
        L.ntpo_propagate_f32_binned.restype = u64
        L.ntpo_make_hits.argtypes = [vp, u64, C.POINTER(_abi.NtpTarget), i32, C.POINTER(C.c_float), dp, vp]
        L.ntpo_total_weight.argtypes = [vp, u64, C.POINTER(_abi.NtpTarget), i32, C.POINTER(C.c_float),
                                        C.POINTER(C.c_float), i32, dp, dp, i32, vp, vp, vp, vp]
        L.ntpo_time_residual.argtypes = [vp, u64, C.POINTER(_abi.NtpTarget), i32, C.POINTER(C.c_float), C.c_float,
                                         vp]
        L.ntpo_check_intersection.argtypes = [dp, d, dp, dp, d, dp]
        L.ntpo_check_intersection.restype = i32
        L.ntpo_check_intersection_f32.argtypes = [C.POINTER(C.c_float), C.c_float, C.POINTER(C.c_float),
                                                  C.POINTER(C.c_float), C.c_float, C.POINTER(C.c_float)]
        L.ntpo_check_intersection_f32.restype = i32
        L.ntpo_rot_from_ez.argtypes = [dp, dp, i32, dp]
        L.ntpo_rot_to_ez.argtypes = [dp, dp, dp]
        L.ntpo_sph_to_cart.argtypes = [d, d, dp]
        L.ntpo_cart_to_sph.argtypes = [dp, dp, dp]
        L.ntpo_apply_rot.argtypes = [dp, dp, dp, dp]
        L.ntpo_gauss_legendre_10.argtypes = [dp, dp]
        L.ntpo_quan_fry_params.argtypes = [d, d, d, dp]
        L.ntpo_refractive_index_fry.argtypes = [d, dp]
        L.ntpo_refractive_index_fry.restype = d
        L.ntpo_dispersion_fry.argtypes = [d, dp]
        L.ntpo_dispersion_fry.restype = d
        L.ntpo_group_velocity.argtypes = [d, dp]
        L.ntpo_group_velocity.restype = d
        L.ntpo_scattering_length.argtypes = [d, d, d]
        L.ntpo_scattering_length.restype = d
        L.ntpo_dippr105.argtypes = [d]
        L.ntpo_dippr105.restype = d
        L.ntpo_frank_tamm_norm.argtypes = [d, d, dp]
        L.ntpo_frank_tamm_norm.restype = d
        L.ntpo_sample_wavelengths.argtypes = [C.POINTER(_abi.NtpSpectrumDesc), u64, u32, u64, dp]
        L.ntpo_sample_gamma.argtypes = [C.c_float, C.c_float, u64, u32, u64, dp]
        L.ntpo_poisson.argtypes = [d, u64, u32]
        L.ntpo_poisson.restype = d
        L.ntpo_resample.argtypes = [vp, u64, vp, vp, vp, C.POINTER(_abi.NtpTarget), i32, i32, d, u64, vp, vp, vp, u64]
        L.ntpo_resample.restype = u64
        L.ntpo_hg_costheta.argtypes = [d, d]
        L.ntpo_hg_costheta.restype = d
        L.ntpo_rayleigh_costheta.argtypes = [d]
        L.ntpo_rayleigh_costheta.restype = d
        _lib = L
    return _lib


def _d3(v):
    return (C.c_double * 3)(*[float(x) for x in v])


def philox(ctr, key) -> tuple:
    out = (C.c_uint32 * 4)()
    lib().ntpo_philox4x32_10((C.c_uint32 * 4)(*ctr), (C.c_uint32 * 2)(*key), out)
    return tuple(out)


def check_intersection(center, radius, pos, direction, step):
    d = C.c_double()
    hit = lib().ntpo_check_intersection(_d3(center), radius, _d3(pos), _d3(direction), step, C.byref(d))
    return bool(hit), (d.value if hit else float("nan"))


def rot_from_ez_fast(a, v, exact_pole=False):
    out = (C.c_double * 3)()
    lib().ntpo_rot_from_ez(_d3(a), _d3(v), int(exact_pole), out)
    return np.array(out)


def rot_to_ez_fast(a, v):
    out = (C.c_double * 3)()
    lib().ntpo_rot_to_ez(_d3(a), _d3(v), out)
    return np.array(out)


def sph_to_cart(theta, phi):
    out = (C.c_double * 3)()
    lib().ntpo_sph_to_cart(theta, phi, out)
    return np.array(out)


def cart_to_sph(v):
    t, p = C.c_double(), C.c_double()
    lib().ntpo_cart_to_sph(_d3(v), C.byref(t), C.byref(p))
    return t.value, p.value


def apply_rot(a, b, v):
    out = (C.c_double * 3)()
    lib().ntpo_apply_rot(_d3(a), _d3(b), _d3(v), out)
    return np.array(out)


class World:
    """C descriptors of one setup (medium / spectrum / targets), for oracle calls."""

    def __init__(self, setup):
        lo, hi = setup.spectrum.wl_range
        tab = setup.medium.tabulate(lo, hi, setup.medium_knots)
        self._keep = [np.ascontiguousarray(a, dtype=np.float32) for a in
                      (tab.ref_index, tab.group_velocity, tab.scattering_length, tab.abs_wavelength, tab.abs_length)]
        k = self._keep
        self.medium = _abi.NtpMediumDesc(n_knots=len(k[0]), wl_min=tab.wl_min, wl_max=tab.wl_max,
                                         ref_index=_abi.fptr(k[0]), group_velocity=_abi.fptr(k[1]),
                                         scattering_length=_abi.fptr(k[2]), n_abs_knots=len(k[3]),
                                         abs_wavelength=_abi.fptr(k[3]), abs_length=_abi.fptr(k[4]),
                                         hg_g=tab.hg_g, rayleigh_fraction=tab.rayleigh_fraction)
        self.spectrum, self._knots = setup.spectrum.desc()
        from neutrinotelescopes_gb300.detection import pack_targets
        self.targets, self.pmt_coords = pack_targets(setup.targets)
        self.n_targets = len(setup.targets)
        self.opts = setup.prop_opts()
        from neutrinotelescopes_gb300.photon_prop import pack_sources
        self.sources = pack_sources(setup.sources)
        self.n_sources = len(setup.sources)
        self.total = sum(int(s.photons) for s in setup.sources)


def _f64_range(w, seed, b, e, cap, binned=False):
    cap = cap or max(1024, (e - b) // 20)
    fn = lib().ntpo_propagate_f64_binned if binned else lib().ntpo_propagate_f64
    while True:
        out = np.zeros(cap, dtype=_abi.HIT_DTYPE)
        n = fn(w.sources, w.n_sources, C.byref(w.medium), C.byref(w.spectrum), w.targets, w.n_targets, seed,
               C.byref(w.opts), b, e, out.ctypes.data, cap)
        if n <= cap:
            return out[:n]
        cap = int(n)


def propagate_f64(setup, seed=0, gid_begin=0, gid_end=None, cap=None, threads=1, binned=False) -> np.ndarray:
    """Double-precision oracle run over photons [gid_begin, gid_end); hits
    ordered by photon.  threads > 1 splits the range into pieces run on that
    many host threads (each a ctypes call, which releases the GIL) and joins
    them in order: the same hits as one call.  binned=True looks targets up
    in a bucket grid instead of scanning all of them (same hits)."""
    w = World(setup)
    gid_end = w.total if gid_end is None else min(gid_end, w.total)
    if threads <= 1 or gid_end - gid_begin < 4096:
        return _f64_range(w, seed, gid_begin, gid_end, cap, binned)
    from concurrent.futures import ThreadPoolExecutor
    n_pieces = 4 * threads
    edges = np.linspace(gid_begin, gid_end, n_pieces + 1).astype(np.int64)
    with ThreadPoolExecutor(max_workers=threads) as ex:
        parts = list(ex.map(lambda i: _f64_range(w, seed, int(edges[i]), int(edges[i + 1]), None, binned),
                            range(n_pieces)))
    return np.concatenate(parts) if parts else np.zeros(0, dtype=_abi.HIT_DTYPE)


def propagate_f32(setup, seed=0, gid_begin=0, gid_end=None, threads=1, cap=None, binned=False) -> np.ndarray:
    """Single-precision mirror (OpenMP); hits unordered.  binned=True looks
    targets up in a bucket grid instead of scanning all of them (same hits;
    for detectors of thousands of modules)."""
    w = World(setup)
    gid_end = w.total if gid_end is None else gid_end
    cap = cap or max(1024, (gid_end - gid_begin) // 20)
    fn = lib().ntpo_propagate_f32_binned if binned else lib().ntpo_propagate_f32
    while True:
        out = np.zeros(cap, dtype=_abi.HIT_DTYPE)
        n = fn(w.sources, w.n_sources, C.byref(w.medium), C.byref(w.spectrum), w.targets, w.n_targets, seed,
               C.byref(w.opts), gid_begin, gid_end, out.ctypes.data, cap, threads)
        if n <= cap:
            return out[:n]
        cap = int(n)


def make_hits(hits: np.ndarray, setup, orientation) -> np.ndarray:
    from neutrinotelescopes_gb300.detection import pack_targets
    tg, coords = pack_targets(setup.targets)
    R = np.ascontiguousarray(np.asarray(orientation, dtype=np.float64).reshape(9))
    hits = np.ascontiguousarray(hits)
    pmt = np.zeros(len(hits), dtype=np.int32)
    lib().ntpo_make_hits(hits.ctypes.data, len(hits), tg, len(setup.targets), _abi.fptr(coords),
                         R.ctypes.data_as(C.POINTER(C.c_double)), pmt.ctypes.data)
    return pmt


def total_weight(hits: np.ndarray, setup, acceptance) -> dict:
    from neutrinotelescopes_gb300.detection import pack_targets
    tg, _ = pack_targets(setup.targets)
    awl, alen = setup.medium.absorption_table()
    awl = np.ascontiguousarray(awl, dtype=np.float32)
    alen = np.ascontiguousarray(alen, dtype=np.float32)
    xs = np.ascontiguousarray(acceptance.xs, dtype=np.float64)
    ys = np.ascontiguousarray(acceptance.ys, dtype=np.float64)
    hits = np.ascontiguousarray(hits)
    n = len(hits)
    cols = {k: np.zeros(n) for k in ("area_acc", "wl_acc", "abs_weight", "total_weight")}
    dp = C.POINTER(C.c_double)
    lib().ntpo_total_weight(hits.ctypes.data, n, tg, len(setup.targets), _abi.fptr(awl), _abi.fptr(alen), len(awl),
                            xs.ctypes.data_as(dp), ys.ctypes.data_as(dp), len(xs), cols["area_acc"].ctypes.data,
                            cols["wl_acc"].ctypes.data, cols["abs_weight"].ctypes.data,
                            cols["total_weight"].ctypes.data)
    return cols


def time_residual(hits: np.ndarray, setup, n800: float) -> np.ndarray:
    from neutrinotelescopes_gb300.detection import pack_targets
    tg, _ = pack_targets(setup.targets)
    hits = np.ascontiguousarray(hits)
    out = np.zeros(len(hits))
    src = (C.c_float * 3)(*[float(v) for v in setup.sources[0].position])
    lib().ntpo_time_residual(hits.ctypes.data, len(hits), tg, len(setup.targets), src, n800, out.ctypes.data)
    return out


def sample_wavelengths(spectrum, n, seed=0, src_index=0) -> np.ndarray:
    d, _keep = spectrum.desc()
    out = np.zeros(n)
    lib().ntpo_sample_wavelengths(C.byref(d), seed, src_index, n, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def sample_gamma(shape, scale, n, seed=0, src_index=0) -> np.ndarray:
    out = np.zeros(n)
    lib().ntpo_sample_gamma(shape, scale, seed, src_index, n, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def resample(hits: np.ndarray, pmt: np.ndarray, weight: np.ndarray, setup, max_pmts: int, downsample: float = 1.0,
             seed: int = 0, time=None) -> dict:
    from neutrinotelescopes_gb300.detection import pack_targets
    tg, _ = pack_targets(setup.targets)
    hits = np.ascontiguousarray(hits)
    pmt = np.ascontiguousarray(pmt, dtype=np.int32)
    weight = np.ascontiguousarray(weight, dtype=np.float64)
    tv = None if time is None else np.ascontiguousarray(time, dtype=np.float64)
    cap = max(1, len(hits))
    g = np.zeros(cap, dtype=np.int32)
    t = np.zeros(cap)
    h = np.zeros(cap, dtype=np.uint64)
    n = lib().ntpo_resample(hits.ctypes.data, len(hits), pmt.ctypes.data, weight.ctypes.data,
                            None if tv is None else tv.ctypes.data, tg, len(setup.targets), max_pmts, downsample, seed,
                            g.ctypes.data, t.ctypes.data, h.ctypes.data, cap)
    return {"group": g[:n], "time": t[:n], "hit": h[:n]}
