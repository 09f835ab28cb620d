"""The oracle and the host helpers against the reference's known-answer tests
(tests/golden/reference_kats.json, extracted from test/runtests.jl) and
Philox4x32-10's published known-answer vectors."""
import math

import numpy as np
import pytest

from neutrinotelescopes_gb300 import PointlikeTimeRangeEmitter, split_source, utils


# Random123 known-answer vectors for philox4x32 with 10 rounds
PHILOX_KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,want", PHILOX_KAT)
def test_philox_known_answers(oracle_lib, ctr, key, want):
    assert oracle_lib.philox(ctr, key) == want


def test_u01_open_interval_and_exact(oracle_lib):
    L = oracle_lib.lib()
    for w in (0, 1, 511, 512, 2 ** 31, 2 ** 32 - 1):
        u = L.ntpo_u01_f64(w)
        assert 0.0 < u < 1.0
        assert np.float32(u) == u  # exactly representable in float
        assert np.float32(1.0 - u) == 1.0 - u


def test_intersection_kats(oracle_lib, kats):
    for case in kats["intersections"]:
        hit, d = oracle_lib.check_intersection(case["center"], case["radius"], case["pos"], case["dir"], case["step"])
        assert hit == case["hit"], f"runtests.jl:{case['line']}"
        # the single-precision mirror agrees on every case
        import ctypes as C
        f3 = lambda v: (C.c_float * 3)(*v)
        df = C.c_float()
        hit32 = oracle_lib.lib().ntpo_check_intersection_f32(f3(case["center"]), case["radius"], f3(case["pos"]),
                                                             f3(case["dir"]), case["step"], C.byref(df))
        assert bool(hit32) == case["hit"], f"runtests.jl:{case['line']} (float)"


def test_intersection_distance(oracle_lib, kats):
    # case runtests.jl:73: from z=14 down to a sphere at z=12, r=0.5 -> d = 1.5
    case = next(c for c in kats["intersections"] if c["line"] == 73)
    hit, d = oracle_lib.check_intersection(case["center"], case["radius"], case["pos"], case["dir"], case["step"])
    assert hit and d == pytest.approx(1.5, abs=1e-12)


def test_sph_to_cart_kats(oracle_lib, kats):
    for case in kats["sph_to_cart"]:
        np.testing.assert_allclose(oracle_lib.sph_to_cart(case["theta"], case["phi"]), case["expected"], atol=1e-12)
        np.testing.assert_allclose(utils.sph_to_cart(case["theta"], case["phi"]), case["expected"], atol=1e-12)


def test_cart_to_sph_roundtrip(oracle_lib, kats):
    for case in kats["cart_to_sph"]:
        v = utils.sph_to_cart(case["theta"], case["phi"])
        assert oracle_lib.cart_to_sph(v) == pytest.approx((case["theta"], case["phi"]), rel=1e-12)
        assert utils.cart_to_sph(v) == pytest.approx((case["theta"], case["phi"]), rel=1e-12)


def test_rotation_kats(oracle_lib, kats):
    e_z, e_x = [0.0, 0.0, 1.0], [1.0, 0.0, 0.0]
    r0, r1, r2 = kats["rotations"]
    d = utils.sph_to_cart(r0["theta"], r0["phi"])
    np.testing.assert_allclose(oracle_lib.apply_rot(d, e_z, d), e_z, atol=1e-9)
    np.testing.assert_allclose(utils.apply_rot(d, e_z, d), e_z, atol=1e-9)
    d1 = utils.sph_to_cart(r1["θ_1"], r1["ϕ_1"])
    d2 = utils.sph_to_cart(r1["θ_2"], r1["ϕ_2"])
    want = [1 / math.sqrt(2), 1 / math.sqrt(2), 0.0]
    np.testing.assert_allclose(oracle_lib.apply_rot(d1, d2, e_x), want, atol=1e-9)
    np.testing.assert_allclose(utils.apply_rot(d1, d2, e_x), want, atol=1e-9)
    d1 = utils.sph_to_cart(r2["θ_1"], r2["ϕ_1"])
    d2 = utils.sph_to_cart(r2["θ_2"], r2["ϕ_2"])
    np.testing.assert_allclose(oracle_lib.apply_rot(d1, e_z, d2), oracle_lib.rot_to_ez_fast(d1, d2), rtol=1e-9)
    np.testing.assert_allclose(oracle_lib.apply_rot(e_z, d1, d2), oracle_lib.rot_from_ez_fast(d1, d2), rtol=1e-9)
    np.testing.assert_allclose(utils.rot_to_ez_fast(d1, d2), oracle_lib.rot_to_ez_fast(d1, d2), rtol=1e-12)
    np.testing.assert_allclose(utils.rot_from_ez_fast(d1, d2), oracle_lib.rot_from_ez_fast(d1, d2), rtol=1e-12)


def test_rot_from_ez_pole_quirk(oracle_lib):
    # utils.jl:230-232: at a = +-e_z the reference returns (v1, copysign(v2, a3), copysign(v3, a3))
    v = [0.3, -0.4, -0.866]
    np.testing.assert_array_equal(oracle_lib.rot_from_ez_fast([0, 0, 1.0], v), [0.3, 0.4, 0.866])
    np.testing.assert_array_equal(oracle_lib.rot_from_ez_fast([0, 0, -1.0], v), [0.3, -0.4, -0.866])
    # with the exact rotation flag the identity / the rotation by pi about x
    np.testing.assert_array_equal(oracle_lib.rot_from_ez_fast([0, 0, 1.0], v, True), v)
    np.testing.assert_array_equal(oracle_lib.rot_from_ez_fast([0, 0, -1.0], v, True), [0.3, 0.4, 0.866])


def test_gauss_quad_kats(kats):
    fs = {"x^3": lambda x: x ** 3, "cos": math.cos}
    for case in kats["gauss_quad"]:
        assert utils.integrate_gauss_quad(fs[case["f"]], case["a"], case["b"]) == pytest.approx(case["expected"],
                                                                                               rel=1e-12)


def test_gauss_legendre_nodes_match(oracle_lib):
    import ctypes as C
    x, w = (C.c_double * 10)(), (C.c_double * 10)()
    oracle_lib.lib().ntpo_gauss_legendre_10(x, w)
    nodes, weights = utils.GL10
    np.testing.assert_allclose(np.array(x), nodes, atol=1e-14)
    np.testing.assert_allclose(np.array(w), weights, atol=1e-14)


def test_split_source_conserves_photons(kats):
    case = kats["split_source"][0]
    src = PointlikeTimeRangeEmitter((0.0, 0.0, 0.7), (0.0, 1e6), case["photons"])
    parts = split_source(src, case["parts"])
    assert len(parts) == case["parts"]
    assert sum(p.photons for p in parts) == src.photons
    with pytest.raises(ValueError):
        split_source(PointlikeTimeRangeEmitter((0, 0, 0), (0, 1), 3), 4)


@pytest.mark.parametrize("lam", [0.3, 5.0, 29.0, 31.0, 300.0, 1e4])
def test_poisson_sampler_moments(oracle_lib, lam):
    L = oracle_lib.lib()
    x = np.array([L.ntpo_poisson(lam, 12345, g) for g in range(20000)])
    assert abs(x.mean() - lam) < 5 * np.sqrt(lam / len(x))
    assert abs(x.var() / lam - 1) < 0.1
    assert np.all(x == np.floor(x)) and np.all(x >= 0)
