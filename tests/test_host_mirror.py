"""Host-side mirror of the reference interface: records, layouts, sources."""
import numpy as np
import pytest

import neutrinotelescopes_gb300 as nt
from neutrinotelescopes_gb300 import _abi, workloads
from neutrinotelescopes_gb300.detection import pack_targets
from neutrinotelescopes_gb300.photon_prop import HitTable, pack_sources


def test_pom_layout():
    c = nt.make_pom_pmt_coordinates()
    assert c.shape == (2, 16) and c.dtype == np.float32
    axes = np.array([nt.utils.sph_to_cart(t, p) for t, p in c.T])
    np.testing.assert_allclose(np.linalg.norm(axes, axis=1), 1, atol=1e-6)
    # after the e_z -> e_x rotation the rings sit at x = cos(32.5 deg), cos(65 deg), ...
    np.testing.assert_allclose(np.sort(np.round(axes[:, 0], 4)),
                               np.sort(np.round(np.repeat(np.cos(np.deg2rad([32.5, 65, 115, 147.5])), 4), 4)),
                               atol=2e-4)
    # distinct directions, at least 25 degrees apart
    dots = axes @ axes.T - 2 * np.eye(16)
    assert dots.max() < np.cos(np.deg2rad(25)) + 1e-6


def test_pack_sources_and_targets():
    s = workloads.cascade_string_setup(3, photon_scale=1e-4)
    srcs = pack_sources(s.sources)
    assert srcs[0].kind == _abi.SRC_EXTENDED_CHERENKOV
    assert srcs[1].photons == s.sources[1].photons
    assert srcs[2].long_b == pytest.approx(0.63)
    recs, coords = pack_targets(s.targets)
    assert len(coords) == 32  # one shared 16-PMT layout
    assert recs[19].module_id == 20 and recs[19].position[2] == pytest.approx(285.0)
    assert all(recs[i].pmt_offset == 0 and recs[i].n_pmts == 16 for i in range(20))


def test_hit_table_columns_and_swap():
    rec = np.zeros(3, dtype=_abi.HIT_DTYPE)
    rec["direction"] = [[1, 0, 0]] * 3
    rec["initial_direction"] = [[0, 1, 0]] * 3
    rec["photon_index"] = [5, 1, 3]
    t = HitTable(rec)
    assert np.array_equal(t["direction"], rec["direction"])
    t._swap = True
    assert np.array_equal(t["direction"], rec["initial_direction"])
    t["w"] = np.arange(3.0)
    s = t.sorted_by_photon()
    assert list(s["photon_index"]) == [1, 3, 5] and list(s["w"]) == [1.0, 2.0, 0.0]
    with pytest.raises(ValueError):
        t["bad"] = np.zeros(2)


def test_oversample_and_emitter_records():
    e = nt.AxiconeEmitter((0, 0, 0), (0, 0, 1), 0.0, 100, 0.5)
    assert nt.oversample_source(e, 10).photons == 1000
    c = e.to_c()
    assert c.kind == _abi.SRC_AXICONE and c.angle == pytest.approx(0.5)
    m = nt.make_cascadia_medium_properties(0.99)
    p = nt.Particle((0, 0, 0), (0, 0, 1), 0.0, 1e3, nt.PEMinus)
    ext = nt.ExtendedCherenkovEmitter.from_particle(p, m, (300.0, 800.0), rng=np.random.default_rng(0))
    assert ext.photons == pytest.approx(nt.total_lightyield(p, m, (300.0, 800.0)), rel=0.01)


def test_setup_validates_options():
    s = workloads.point_cone_setup(10, hit_policy="bogus")
    with pytest.raises(ValueError):
        s.prop_opts()
