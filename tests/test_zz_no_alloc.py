"""ntp_propagate_noalloc, the entry point for callers that cannot allocate
device memory (a data-taking process that reserves its device memory at
start-up, or a framework whose buffers come from its own pool): it must give
the same hits as ntp_propagate on the same inputs, on two calls in a row (the
second call reuses the library's fixed scratch array, which must be reset).
Called through the C ABI with ctypes; the test allocates the output buffer
itself, as such a caller would.  Collected last so that a run stopping at the
first failure has run every other test."""
import ctypes as C

import numpy as np
import pytest

import neutrinotelescopes_gb300 as nt
from neutrinotelescopes_gb300 import _abi, workloads
from neutrinotelescopes_gb300.detection import pack_targets
from neutrinotelescopes_gb300.photon_prop import pack_sources

pytestmark = pytest.mark.gpu


def _descriptors(setup):
    lo, hi = setup.spectrum.wl_range
    tab = setup.medium.tabulate(lo, hi, setup.medium_knots)
    keep = [np.ascontiguousarray(a, dtype=np.float32) for a in
            (tab.ref_index, tab.group_velocity, tab.scattering_length, tab.abs_wavelength, tab.abs_length)]
    md = _abi.NtpMediumDesc(n_knots=len(keep[0]), wl_min=tab.wl_min, wl_max=tab.wl_max,
                            ref_index=_abi.fptr(keep[0]), group_velocity=_abi.fptr(keep[1]),
                            scattering_length=_abi.fptr(keep[2]), n_abs_knots=len(keep[3]),
                            abs_wavelength=_abi.fptr(keep[3]), abs_length=_abi.fptr(keep[4]),
                            hg_g=tab.hg_g, rayleigh_fraction=tab.rayleigh_fraction)
    sd, knots = setup.spectrum.desc()
    tg, coords = pack_targets(setup.targets)
    return md, sd, tg, (keep, knots, coords)


def _sorted(records):
    return records[np.lexsort((records["photon_index"], records["source_index"]))]


def _memory_state(torch):
    torch.cuda.synchronize()
    free, _total = torch.cuda.mem_get_info()
    return free, torch.cuda.memory_allocated(), torch.cuda.memory_reserved()


def test_noalloc_matches_propagate_twice():
    import torch
    setup = workloads.cascade_string_setup(2, photon_scale=3e-3)
    seeds = (11, 12)
    # the expected hits first: ntp_propagate allocates (its context), the
    # entry point under test must not
    want = {seed: nt.propagate_photons(setup, seed=seed, reference_columns=False).sorted_by_photon().records
            for seed in seeds}
    lib = _abi.load_library()
    md, sd, tg, _keep = _descriptors(setup)
    srcs = pack_sources(setup.sources)
    cap = 1 << 20
    buf = torch.zeros((cap, 64), dtype=torch.uint8, device="cuda")
    states = []
    for seed in seeds:
        nh, ns = C.c_uint64(), C.c_uint64()
        opts = setup.prop_opts()
        st = lib.ntp_propagate_noalloc(C.byref(md), C.byref(sd), tg, len(setup.targets), srcs, len(setup.sources),
                                       seed, C.byref(opts), buf.data_ptr(), cap, C.byref(nh), C.byref(ns))
        assert st == _abi.NTP_OK, lib.ntp_last_error(None)
        # device memory after the call: free bytes (cudaMemGetInfo) and the
        # torch allocator's counters; the first call may load the library's
        # fixed scratch array, so the check compares the calls after it
        states.append(_memory_state(torch))
        got = _sorted(buf[: nh.value].cpu().numpy().view(_abi.HIT_DTYPE).reshape(-1))
        assert ns.value == sum(s.photons for s in setup.sources)
        assert len(got) == len(want[seed]) > 100
        np.testing.assert_array_equal(got, want[seed])
    before = states[0]
    nh, ns = C.c_uint64(), C.c_uint64()
    for _ in range(3):
        st = lib.ntp_propagate_noalloc(C.byref(md), C.byref(sd), tg, len(setup.targets), srcs, len(setup.sources),
                                       seeds[0], C.byref(setup.prop_opts()), buf.data_ptr(), cap, C.byref(nh),
                                       C.byref(ns))
        assert st == _abi.NTP_OK
        assert _memory_state(torch) == before
    assert states[1] == before
    setup.close()


def test_noalloc_rejects_oversized_and_host_buffers():
    src = nt.PointlikeIsotropicEmitter((0.0, 0.0, 0.0), 0.0, 1000)
    many = [nt.DetectionSphere((float(i), 0.0, 5.0), 0.2, 1, 1.0, i + 1) for i in range(4097)]
    setup = nt.PhotonPropSetup([src], many, nt.make_simple_water(), nt.Monochromatic(400.0))
    lib = _abi.load_library()
    md, sd, tg, _keep = _descriptors(setup)
    nh, ns = C.c_uint64(), C.c_uint64()
    host = np.zeros(16, dtype=_abi.HIT_DTYPE)
    st = lib.ntp_propagate_noalloc(C.byref(md), C.byref(sd), tg, len(many), pack_sources([src]), 1, 0, None,
                                   host.ctypes.data, 16, C.byref(nh), C.byref(ns))
    assert st == _abi.NTP_ERR_INVALID and b"n_targets" in lib.ntp_last_error(None)
    st = lib.ntp_propagate_noalloc(C.byref(md), C.byref(sd), tg, 4, pack_sources([src]), 1, 0, None,
                                   host.ctypes.data, 16, C.byref(nh), C.byref(ns))
    assert st == _abi.NTP_ERR_INVALID and b"device memory" in lib.ntp_last_error(None)


def test_noalloc_rejects_bad_medium_and_spectrum():
    src = nt.PointlikeIsotropicEmitter((0.0, 0.0, 0.0), 0.0, 1000)
    setup = nt.PhotonPropSetup([src], [nt.DetectionSphere((0.0, 0.0, 5.0), 0.2, 1, 1.0, 1)], nt.make_simple_water(),
                               nt.InverseSquareSpectrum(300.0, 600.0))
    lib = _abi.load_library()
    md, sd, tg, keep = _descriptors(setup)
    nh, ns = C.c_uint64(), C.c_uint64()
    ref_index = keep[0][0]
    ref_index[1] = 0.9  # n <= 1
    st = lib.ntp_propagate_noalloc(C.byref(md), C.byref(sd), tg, 1, pack_sources([src]), 1, 0, None, None, 0,
                                   C.byref(nh), C.byref(ns))
    assert st == _abi.NTP_ERR_INVALID and b"n > 1" in lib.ntp_last_error(None)
    ref_index[1] = ref_index[0]
    bad = np.array([300.0, -1.0, 600.0], dtype=np.float32)
    sd_bad = _abi.NtpSpectrumDesc(kind=_abi.SPEC_TABLE_LINEAR, n_knots=3, icdf_knots=_abi.fptr(bad))
    st = lib.ntp_propagate_noalloc(C.byref(md), C.byref(sd_bad), tg, 1, pack_sources([src]), 1, 0, None, None, 0,
                                   C.byref(nh), C.byref(ns))
    assert st == _abi.NTP_ERR_INVALID and b"knots" in lib.ntp_last_error(None)
    # a good call (no photons, nothing to write) clears the thread's error text
    none = nt.PointlikeIsotropicEmitter((0.0, 0.0, 0.0), 0.0, 0)
    st = lib.ntp_propagate_noalloc(C.byref(md), C.byref(sd), tg, 1, pack_sources([none]), 1, 0, None, None, 0,
                                   C.byref(nh), C.byref(ns))
    assert st == _abi.NTP_OK and lib.ntp_last_error(None) == b""


def test_noalloc_rejects_a_buffer_on_another_device():
    import torch
    if torch.cuda.device_count() < 2:
        pytest.skip("needs two GPUs")
    setup = workloads.point_cone_setup(1000)
    lib = _abi.load_library()
    md, sd, tg, _keep = _descriptors(setup)
    buf = torch.zeros((16, 64), dtype=torch.uint8, device="cuda:1")
    torch.cuda.set_device(0)
    nh, ns = C.c_uint64(), C.c_uint64()
    st = lib.ntp_propagate_noalloc(C.byref(md), C.byref(sd), tg, 1, pack_sources(setup.sources), 1, 0, None,
                                   buf.data_ptr(), 16, C.byref(nh), C.byref(ns))
    assert st == _abi.NTP_ERR_INVALID and b"device 1" in lib.ntp_last_error(None)
