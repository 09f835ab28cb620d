"""Parity of the CUDA propagation kernel with the CPU oracle, through the C ABI.

Per-photon replay: the kernel and the double-precision oracle draw the same
Philox stream, so every photon can be compared individually.  Tolerances:
position, time and distance to 1e-4 relative, directions to 1e-4 absolute
(unit vectors; at most one photon in 10^4, and at least one, may reach
1e-3: after hundreds of metres and several scatters a near-backward scatter,
where sin theta is ill-conditioned in single precision, can carry one
direction slightly past 1e-4), wavelength to 1e-5 relative.  A position is the sum of the
photon's step vectors, so its rounding error scales with the path length:
positions are compared relative to the larger of the position norm and the
distance travelled (a photon of the point-cone case ends 10 m from the origin
after up to 15 scatters and several hundred metres).
Where the photon enters the sphere at a grazing angle the entry distance
amplifies a lateral error by 1/cos(incidence): the position / time / distance
bound of such a hit is widened by that factor (capped at 50), with
cos(incidence) taken from the oracle's hit.  A photon whose hit/miss decision
falls within float rounding of the sphere edge or the step end can come out
differently in float and double; at most 0.5% of the hit photons (and at
least 3) may differ in the set of hit photons.  The widened bound is
reported: at most 1% of the matched photons (and at least 3) may need it,
i.e. have an error above the unwidened 1e-4 bound.
"""
import ctypes as C
import os

import numpy as np
import pytest

import neutrinotelescopes_gb300 as nt
from neutrinotelescopes_gb300 import _abi, workloads
from neutrinotelescopes_gb300.photon_prop import pack_sources

pytestmark = pytest.mark.gpu

POS_RTOL = 1e-4
DIR_ATOL = 1e-4
WL_RTOL = 1e-5


def gpu_hits(setup, seed=0):
    h = nt.propagate_photons(setup, seed=seed, reference_columns=False)
    return h.sorted_by_photon().records


def incidence_slack(hits, setup):
    """1 / cos(incidence) at each hit (capped at 50), from the hit position,
    final direction and the module centre."""
    centres = {t.module_id: (np.asarray(t.position, dtype=np.float64), float(t.radius)) for t in setup.targets}
    out = np.ones(len(hits))
    for i, h in enumerate(hits):
        c, r = centres[int(h["module_id"])]
        n = (h["position"].astype(np.float64) - c) / r
        out[i] = 1.0 / max(abs(float(np.dot(n, h["direction"]))), 0.02)
    return out


def compare_replay(g, o, min_hits=20, setup=None):
    assert len(o) >= min_hits, f"oracle found only {len(o)} hits"
    kg = g["source_index"].astype(np.uint64) << np.uint64(40) | g["photon_index"]
    ko = o["source_index"].astype(np.uint64) << np.uint64(40) | o["photon_index"]
    common, ig, io = np.intersect1d(kg, ko, return_indices=True)
    n_diff = len(kg) + len(ko) - 2 * len(common)
    a, b = g[ig], o[io]
    same_module = float(np.mean(a["module_id"] == b["module_id"])) if len(b) else 1.0
    same = a["module_id"] == b["module_id"]
    a, b = a[same], b[same]
    slack = incidence_slack(b, setup) if setup is not None else np.ones(len(b))
    dp = np.linalg.norm(a["position"].astype(np.float64) - b["position"], axis=1)
    scale = np.maximum(np.maximum(np.linalg.norm(b["position"].astype(np.float64), axis=1),
                                  b["dist_travelled"].astype(np.float64)), 1.0)
    # along-path error of the entry point: at most the lateral bound times the slack
    dl = POS_RTOL * scale * slack
    vg = np.maximum(b["dist_travelled"] / np.maximum(b["time"], 1e-9), 0.05)
    ddist = np.abs(a["dist_travelled"] - b["dist_travelled"])
    dtime = np.abs(a["time"].astype(np.float64) - b["time"])
    # photons that need the grazing-incidence widening: above the plain bound
    dl0 = POS_RTOL * scale
    widened = ((dp > dl0) | (ddist > POS_RTOL * b["dist_travelled"] + dl0 + 1e-4)
               | (dtime > POS_RTOL * np.abs(b["time"]) + dl0 / vg + 1e-3))
    n_widened = int(np.sum(widened))
    dang = float(np.max(np.abs(a["direction"].astype(np.float64) - b["direction"]))) if len(b) else 0.0
    print(f"replay: {len(common)} matched, {n_diff} differ in hit/miss ({len(kg) - len(common)} kernel only, "
          f"{len(ko) - len(common)} oracle only), {n_widened} need the widened bound "
          f"(max slack used {float(np.max(slack[widened])) if n_widened else 1.0:.2f}); max relative position "
          f"error {float(np.max(dp / scale)) if len(b) else 0.0:.2e}, max direction error {dang:.2e}")
    assert n_diff <= max(3, int(0.005 * len(ko))), f"{n_diff} photons differ in hit/miss out of {len(ko)}"
    # the photons that differ must not favour one side: a float rounding
    # that biased the hit test would lose (or gain) hits systematically
    n_g_only, n_o_only = len(kg) - len(common), len(ko) - len(common)
    assert abs(n_g_only - n_o_only) <= 3.0 * np.sqrt(n_g_only + n_o_only) + 3, (n_g_only, n_o_only)
    assert same_module >= 0.995
    assert np.all(dp <= POS_RTOL * scale * slack), f"max rel pos err {np.max(dp / scale / slack):.3g}"
    assert np.all(ddist <= POS_RTOL * b["dist_travelled"] + dl + 1e-4)
    assert np.all(dtime <= POS_RTOL * np.abs(b["time"]) + dl / vg + 1e-3)
    derr = np.maximum(np.abs(a["direction"].astype(np.float64) - b["direction"]).max(axis=1),
                      np.abs(a["initial_direction"].astype(np.float64) - b["initial_direction"]).max(axis=1))
    n_dir_over = int(np.sum(derr > DIR_ATOL))
    assert n_dir_over <= max(1, int(1e-4 * len(b))), f"{n_dir_over} directions beyond {DIR_ATOL}"
    assert np.all(derr <= 10 * DIR_ATOL), float(np.max(derr))
    np.testing.assert_allclose(a["wavelength"], b["wavelength"], rtol=WL_RTOL)
    assert n_widened <= max(3, int(0.01 * len(b))), f"{n_widened} of {len(b)} photons need the widened bound"
    return len(common)


def iso_close_setup(photons=200_000, **kw):
    src = nt.PointlikeIsotropicEmitter((0.0, 0.0, 0.0), 0.0, photons)
    tgt = nt.DetectionSphere((0.0, 0.0, 5.0), 1.0, 16, workloads.PMT_AREA, 7)
    return nt.PhotonPropSetup([src], [tgt], nt.make_simple_water(), nt.InverseSquareSpectrum(300.0, 600.0), **kw)


def cascade_small_setup(photons=200_000, **kw):
    m = nt.make_cascadia_medium_properties(0.99)
    lp = nt.LongitudinalParameterisation.from_energy(1e4, m, nt.PEMinus)
    src = nt.ExtendedCherenkovEmitter((4.0, 0.0, 140.0), (0.0, 0.6, 0.8), 0.0, photons, lp)
    targets = nt.string_of_modules(20, 15.0, pmt_area=workloads.PMT_AREA)
    return nt.PhotonPropSetup([src], targets, m, nt.CherenkovSpectrum((300.0, 800.0), 30, m), **kw)


def mixed_setup(**kw):
    srcs = [
        nt.PencilEmitter((0.0, 0.0, -3.0), (0.0, 0.0, 1.0), 1.0, 30_000),
        nt.PointlikeTimeRangeEmitter((0.5, 0.0, 0.0), (0.0, 20.0), 40_000),
        nt.PointlikeCherenkovEmitter((0.0, -2.0, 0.0), (0.0, 0.8, 0.6), 0.0, 40_000),
        nt.CherenkovTrackEmitter((1.0, 1.0, -5.0), (0.0, 0.0, 1.0), 0.0, 10.0, 40_000),
        nt.AxiconeEmitter((0.0, 0.0, 0.0), (0.0, 0.0, 1.0), 0.0, 40_000, 0.7),
    ]
    targets = [nt.DetectionSphere((0.0, 0.0, 3.0), 0.8, 16, workloads.PMT_AREA, 11),
               nt.DetectionSphere((0.0, 0.0, 6.0), 1.2, 16, workloads.PMT_AREA, 12),
               nt.DetectionSphere((2.0, 1.0, 2.0), 0.7, 16, workloads.PMT_AREA, 13)]
    m = nt.make_cascadia_medium_properties(0.99)
    return nt.PhotonPropSetup(srcs, targets, m, nt.CherenkovSpectrum((300.0, 800.0), 30, m, semantics="linear"), **kw)


@pytest.fixture(scope="module")
def orc(oracle_lib):
    return oracle_lib


def test_replay_isotropic_close_sphere(orc):
    s = iso_close_setup()
    n = compare_replay(gpu_hits(s, seed=3), orc.propagate_f64(s, seed=3), min_hits=1000, setup=s)
    assert n > 1000


@pytest.mark.parametrize("seed", [11, 12])
def test_replay_point_cone(orc, seed):
    # The 1e6-photon point cone (41.2 degrees about +z, one R = 0.21 m module
    # 10 m up the axis) is missed by direct light and gives about 16 hits per
    # 1e6 photons.  1e8 photons under one Philox key are 100 such runs; every
    # hit photon is replayed by the FP64 oracle (the whole range, on all host
    # cores), so both directions of the hit set are checked.
    s = workloads.point_cone_setup(100_000_000)
    g = nt.propagate_photons(s, seed=seed, reference_columns=False, capacity=1 << 16).sorted_by_photon().records
    o = orc.propagate_f64(s, seed=seed, threads=os.cpu_count() or 1)
    assert compare_replay(g, o, min_hits=1000, setup=s) >= 1000


def test_replay_cascade_on_pom_string(orc):
    s = cascade_small_setup()
    compare_replay(gpu_hits(s, seed=5), orc.propagate_f64(s, seed=5), min_hits=50, setup=s)


@pytest.mark.parametrize("policy,exact", [("first", False), ("nearest", False), ("first", True)])
def test_replay_mixed_sources(orc, policy, exact):
    s = mixed_setup(hit_policy=policy, exact_pole_rotation=exact)
    compare_replay(gpu_hits(s, seed=17), orc.propagate_f64(s, seed=17), min_hits=1000, setup=s)


def test_replay_string_grid_with_grid_walk(orc):
    # 10 x 10 strings x 20 modules, three cascades near the centre (2.2e7
    # photons): the kernel culls by columns and walks its 2-D cell grid, the
    # FP64 oracle looks targets up in its bucket grid (the same hits as its
    # scan over all 2000 modules); every hit photon is replayed
    targets = workloads.string_grid(10, 10, 50.0, 20, 15.0)
    srcs = workloads.cascade_sources(3, np.random.default_rng(5), photon_scale=0.0025, string_z=(0.0, 285.0),
                                     distance=8.0)
    s = nt.PhotonPropSetup(srcs, targets, nt.make_simple_water(), nt.InverseSquareSpectrum(300.0, 600.0))
    o = orc.propagate_f64(s, seed=31, threads=os.cpu_count() or 1, binned=True)
    assert compare_replay(gpu_hits(s, seed=31), o, min_hits=10_000, setup=s) >= 10_000
    s.close()


def test_column_culling_matches_plain_scan():
    # culling by vertical columns keeps exactly the hits of the full scan
    for policy in ("first", "nearest"):
        a = cascade_small_setup(400_000, hit_policy=policy)
        b = cascade_small_setup(400_000, hit_policy=policy, plain_scan=True)
        ha, hb = gpu_hits(a, seed=8), gpu_hits(b, seed=8)
        assert len(ha) > 100
        assert ha.tobytes() == hb.tobytes()
    s = workloads.cascade_string_setup(2, photon_scale=2e-4)
    t = workloads.cascade_string_setup(2, photon_scale=2e-4, plain_scan=True)
    ha, hb = gpu_hits(s, seed=3), gpu_hits(t, seed=3)
    assert len(ha) > 100 and ha.tobytes() == hb.tobytes()


def test_grid_culling_matches_plain_scan_on_string_grid():
    # 10 x 10 strings, 20 modules each: the 2-D grid walk keeps exactly the hits of the full scan
    targets = workloads.string_grid(10, 10, 50.0, 20, 15.0)
    rng = np.random.default_rng(5)
    srcs = workloads.cascade_sources(3, rng, photon_scale=2e-4, string_z=(0.0, 285.0), distance=8.0)
    m = nt.make_simple_water()
    for policy in ("first", "nearest"):
        a = nt.PhotonPropSetup(srcs, targets, m, nt.InverseSquareSpectrum(300.0, 600.0), hit_policy=policy)
        b = nt.PhotonPropSetup(srcs, targets, m, nt.InverseSquareSpectrum(300.0, 600.0), hit_policy=policy,
                               plain_scan=True)
        ha, hb = gpu_hits(a, seed=21), gpu_hits(b, seed=21)
        assert len(ha) > 100
        assert ha.tobytes() == hb.tobytes()
        a.close()
        b.close()


def test_grid_walk_matches_plain_scan_on_irregular_strings():
    # 16 strings at random positions (no lattice): the cell walk, not the
    # lattice form, culls; both policies keep exactly the hits of the full scan
    rng = np.random.default_rng(9)
    targets = []
    for k in range(16):
        x, y = rng.uniform(-60.0, 60.0, 2)
        targets += nt.string_of_modules(12, 15.0, x=float(x), y=float(y), z_start=0.0, pmt_area=workloads.PMT_AREA,
                                        id_offset=len(targets))
    srcs = workloads.cascade_sources(3, np.random.default_rng(6), photon_scale=2e-4, string_z=(0.0, 165.0),
                                     distance=8.0)
    m = nt.make_simple_water()
    for policy in ("first", "nearest"):
        a = nt.PhotonPropSetup(srcs, targets, m, nt.InverseSquareSpectrum(300.0, 600.0), hit_policy=policy)
        b = nt.PhotonPropSetup(srcs, targets, m, nt.InverseSquareSpectrum(300.0, 600.0), hit_policy=policy,
                               plain_scan=True)
        ha, hb = gpu_hits(a, seed=23), gpu_hits(b, seed=23)
        assert len(ha) > 100
        assert ha.tobytes() == hb.tobytes()
        a.close()
        b.close()


def test_axicone_pole_quirk_half_cone():
    # rot_from_ez_fast at a = e_z (utils.jl:230-232): every photon of a cone about +z has y >= 0
    src = nt.AxiconeEmitter((0.0, 0.0, 0.0), (0.0, 0.0, 1.0), 0.0, 100_000, 0.7)
    tgt = nt.DetectionSphere((0.0, 0.0, 1.0), 0.9, 1, 1.0, 1)
    s = nt.PhotonPropSetup([src], [tgt], nt.make_simple_water(), nt.Monochromatic(400.0))
    h = gpu_hits(s)
    first = h[h["dist_travelled"] < 0.5]  # unscattered, straight into the sphere
    assert len(first) > 1000
    assert np.all(first["initial_direction"][:, 1] >= 0)
    s2 = nt.PhotonPropSetup([src], [tgt], nt.make_simple_water(), nt.Monochromatic(400.0), exact_pole_rotation=True)
    h2 = gpu_hits(s2)
    assert np.mean(h2["initial_direction"][:, 1] < 0) > 0.4


def test_deterministic_rerun():
    s = iso_close_setup(100_000)
    a, b = gpu_hits(s, seed=9), gpu_hits(s, seed=9)
    assert a.tobytes() == b.tobytes()
    c = gpu_hits(s, seed=10)
    assert len(c) != len(a) or c.tobytes() != a.tobytes()


def test_overflow_reports_exact_count():
    s = iso_close_setup(100_000)
    full = gpu_hits(s, seed=4)
    assert len(full) > 100
    with pytest.raises(_abi.NtpError) as e:
        nt.propagate_photons(s, seed=4, capacity=50)
    assert e.value.status == _abi.NTP_ERR_OVERFLOW
    lib, ctx = s.context()
    out = np.zeros(50, dtype=_abi.HIT_DTYPE)
    nh, ns = C.c_uint64(), C.c_uint64()
    st = lib.ntp_propagate(ctx, pack_sources(s.sources), 1, 4, C.byref(s.prop_opts()), out.ctypes.data, 50, 0,
                           C.byref(nh), C.byref(ns))
    assert st == _abi.NTP_ERR_OVERFLOW and nh.value == len(full) and ns.value == 100_000
    keys = set(zip(full["source_index"], full["photon_index"]))
    assert all((r["source_index"], r["photon_index"]) in keys for r in out)


def test_empty_and_no_target_inputs():
    s = iso_close_setup(0)
    h = nt.propagate_photons(s)
    assert len(h) == 0 and h.n_photons_simulated == 0
    src = nt.PointlikeIsotropicEmitter((0.0, 0.0, 0.0), 0.0, 50_000)
    s2 = nt.PhotonPropSetup([src], [], nt.make_simple_water(), nt.Monochromatic(400.0))
    h2 = nt.propagate_photons(s2)
    assert len(h2) == 0 and h2.n_photons_simulated == 50_000


def test_invalid_arguments():
    s = iso_close_setup(1000)
    lib, ctx = s.context()
    srcs = pack_sources(s.sources)
    srcs[0].kind = 99
    nh, ns = C.c_uint64(), C.c_uint64()
    out = np.zeros(10, dtype=_abi.HIT_DTYPE)
    st = lib.ntp_propagate(ctx, srcs, 1, 0, None, out.ctypes.data, 10, 0, C.byref(nh), C.byref(ns))
    assert st == _abi.NTP_ERR_INVALID and b"unknown kind" in lib.ntp_last_error(ctx)
    bad = nt.PhotonPropSetup([nt.PointlikeIsotropicEmitter((0, 0, 0), 0.0, 10)],
                             [nt.DetectionSphere((0, 0, 1), -1.0, 1, 1.0, 1)], nt.make_simple_water(),
                             nt.Monochromatic(400.0))
    with pytest.raises(_abi.NtpError):
        nt.propagate_photons(bad)
    dup = nt.PhotonPropSetup([nt.PointlikeIsotropicEmitter((0, 0, 0), 0.0, 10)],
                             [nt.DetectionSphere((0, 0, 1), 0.2, 1, 1.0, 1), nt.DetectionSphere((0, 0, 2), 0.2, 1, 1.0, 1)],
                             nt.make_simple_water(), nt.Monochromatic(400.0))
    with pytest.raises(_abi.NtpError, match="duplicate module_id"):
        nt.propagate_photons(dup)


def test_run_stats_counts_steps():
    s = iso_close_setup(100_000)
    h = nt.propagate_photons(s, seed=1)
    lib, ctx = s.context()
    st = _abi.NtpRunStats()
    assert lib.ntp_get_run_stats(ctx, C.byref(st)) == 0
    assert st.photons == 100_000 and st.hits == len(h)
    # photons that hit stop early; the others take all 15 steps
    assert 100_000 * 1 <= st.photon_steps <= 100_000 * 15
    assert st.photon_steps > (100_000 - len(h)) * 15


def test_make_hits_matches_oracle(orc):
    s = cascade_small_setup(1_000_000)
    h = nt.propagate_photons(s, seed=21, reference_columns=False)
    R = nt.utils.random_rotation(np.random.default_rng(3))
    lib, ctx = s.context()
    recs = np.ascontiguousarray(h.records)
    pmt = np.zeros(len(recs), dtype=np.int32)
    assert lib.ntp_make_hits(ctx, recs.ctypes.data, len(recs), np.ascontiguousarray(R).ctypes.data_as(
        C.POINTER(C.c_double)), pmt.ctypes.data, 0, None) == 0
    want = orc.make_hits(recs, s, R)
    np.testing.assert_array_equal(pmt, want)
    assert np.any(pmt > 0)
    sel = nt.make_hits_from_photons(h, s, R)
    assert len(sel) == int(np.sum(want > 0)) and np.all(sel["pmt_id"] > 0)


def test_total_weight_and_time_residual_match_oracle(orc):
    s = cascade_small_setup(500_000)
    h = nt.propagate_photons(s, seed=23, reference_columns=False)
    nt.calc_total_weight(h, s)
    want = orc.total_weight(h.records, s, nt.p_one_pmt_acc)
    np.testing.assert_array_equal(h["area_acc"], want["area_acc"])
    np.testing.assert_allclose(h["wl_acc"], want["wl_acc"], rtol=1e-12)
    np.testing.assert_allclose(h["abs_weight"], want["abs_weight"], rtol=1e-6)
    np.testing.assert_allclose(h["total_weight"], want["total_weight"], rtol=1e-6)
    nt.calc_time_residual(h, s)
    n800 = float(np.float32(s.medium.refractive_index(np.array([800.0]))[0]))
    np.testing.assert_allclose(h["tres"], orc.time_residual(h.records, s, n800), rtol=1e-12, atol=1e-9)


def test_single_target_column_swap():
    s = iso_close_setup(50_000)
    h = nt.propagate_photons(s, seed=2)
    assert np.array_equal(h["direction"], h.records["initial_direction"])
    assert np.array_equal(h["initial_direction"], h.records["direction"])


def test_pmt_summary_matches_oracle_composition(orc):
    # per (module, PMT) FP64 sums of the oracle's per-hit PMT ids, weights and time residuals
    s = cascade_small_setup(1_000_000)
    h = nt.propagate_photons(s, seed=31, reference_columns=False)
    R = nt.utils.random_rotation(np.random.default_rng(4))
    out = nt.pmt_summary(h, s, R, n_bins=64, t_range=(-20.0, 300.0))
    recs = h.records
    pmt = orc.make_hits(recs, s, R)
    w = orc.total_weight(recs, s, nt.p_one_pmt_acc)["total_weight"]
    n800 = float(np.float32(s.medium.refractive_index(np.array([800.0]))[0]))
    tres = orc.time_residual(recs, s, n800)
    index = {t.module_id: i for i, t in enumerate(s.targets)}
    k = np.array([index[m] for m in recs["module_id"]])
    sel = pmt > 0
    want_w = np.zeros((20, 16))
    want_c = np.zeros((20, 16))
    np.add.at(want_w, (k[sel], pmt[sel] - 1), w[sel])
    np.add.at(want_c, (k[sel], pmt[sel] - 1), 1.0)
    np.testing.assert_array_equal(out["hit_count"], want_c)
    np.testing.assert_allclose(out["weight_sum"], want_w, rtol=1e-6, atol=1e-12)
    assert want_c.sum() > 10
    edges = out["bin_edges"]
    want_h = np.zeros((20, 16, 64))
    b = np.floor((tres - edges[0]) * 64 / (edges[-1] - edges[0]))
    inb = sel & (b >= 0) & (b < 64)
    np.add.at(want_h, (k[inb], pmt[inb] - 1, b[inb].astype(int)), w[inb])
    np.testing.assert_allclose(out["time_hist"], want_h, rtol=1e-6, atol=1e-12)


def test_resample_matches_oracle_and_reference_usage(orc):
    # the reference's chain (simulate_event_full_test.jl:61-65): make_hits -> weights -> resample
    s = cascade_small_setup(2_000_000)
    h = nt.propagate_photons(s, seed=41, reference_columns=False)
    R = np.eye(3)
    hits = nt.make_hits_from_photons(h, s, R)
    nt.calc_total_weight(hits, s)
    nt.calc_time_residual(hits, s)
    assert len(hits) > 30
    for seed, down in ((5, 1.0), (6, 25.0)):
        got = nt.resample_simulation(hits, s, downsample=down, seed=seed, time_col="tres")
        want = orc.resample(hits.records, hits["pmt_id"], hits["total_weight"], s, 16, down, seed, hits["tres"])
        a = sorted(zip(got["hit_index"].tolist(), (got["module_id"] * 100 + got["pmt_id"]).tolist()))
        index = {t.module_id: i for i, t in enumerate(s.targets)}
        b = sorted(zip(want["hit"].tolist(),
                       [s.targets[g // 16].module_id * 100 + g % 16 + 1 for g in want["group"].tolist()]))
        assert a == b
        np.testing.assert_array_equal(np.sort(got["tres"]), np.sort(want["time"]))
        # drawn hits are distinct and belong to their group
        assert len(set(got["hit_index"].tolist())) == len(got["hit_index"])
        assert np.all(hits["pmt_id"][got["hit_index"].astype(int)] == got["pmt_id"])
    # a large downsample factor draws (nearly) every hit with w > 0, never more
    big = nt.resample_simulation(hits, s, downsample=1e6, seed=1, time_col="tres")
    want = orc.resample(hits.records, hits["pmt_id"], hits["total_weight"], s, 16, 1e6, 1, hits["tres"])
    assert sorted(big["hit_index"].tolist()) == sorted(want["hit"].tolist())
    assert len(big["tres"]) <= int(np.sum(hits["total_weight"] > 0))
    assert len(big["tres"]) >= 0.9 * int(np.sum(hits["total_weight"] > 0))
