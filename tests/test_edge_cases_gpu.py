"""Empty and degenerate inputs across the C ABI: no hits to resample,
summarise or tabulate, a flow evaluation without tuples, a sampler whose
expectations are all but zero."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import neutrinotelescopes_gb300 as nt  # noqa: E402
from neutrinotelescopes_gb300 import _abi  # noqa: E402
from neutrinotelescopes_gb300.flow import RQNormFlow, RQNormFlowHParams  # noqa: E402
from neutrinotelescopes_gb300.photon_prop import HitTable, pack_sources  # noqa: E402
from neutrinotelescopes_gb300.tables import TableConfig, draw_simulations, table_setup  # noqa: E402

pytestmark = pytest.mark.gpu


def _string_setup():
    return nt.PhotonPropSetup([], nt.string_of_modules(3, 15.0), nt.make_simple_water(),
                              nt.InverseSquareSpectrum(300.0, 600.0))


def test_resample_and_summary_of_no_hits():
    setup = _string_setup()
    empty = HitTable(np.zeros(0, dtype=_abi.HIT_DTYPE))
    empty.extra["pmt_id"] = np.zeros(0, np.int32)
    empty.extra["total_weight"] = np.zeros(0)
    r = nt.resample_simulation(empty, setup, seed=1)
    assert len(r["pmt_id"]) == 0
    setup.sources = [nt.PointlikeIsotropicEmitter((0.0, 0.0, 0.0), 0.0, 0)]
    s = nt.pmt_summary(empty, setup, np.eye(3), n_bins=8)
    assert s["weight_sum"].sum() == 0 and s["hit_count"].sum() == 0 and s["time_hist"].sum() == 0
    setup.close()


def test_table_of_no_hits_has_one_count_row_per_group():
    cfg = TableConfig(n_sims=3, n_orientations=2)
    setup = table_setup(cfg)
    lib, ctx = setup.context()
    sims = draw_simulations(cfg, np.random.default_rng(0))
    srcs = pack_sources(sims["sources"])
    le = np.ascontiguousarray(sims["log10_energy"], np.float32)
    orient = np.ascontiguousarray(np.tile(np.eye(3), (6, 1, 1)).reshape(-1), np.float64)
    spec = _abi.NtpTableSpec(n_sims=3, n_orientations=2, max_rows_per_group=5, zero_rows=1, downsample=1.0,
                             n800=1.35, seed=1)
    G = 3 * 2 * 16
    outs = [torch.empty((G, 5), device="cuda"), torch.empty(G, device="cuda"), torch.empty(G, device="cuda"),
            torch.empty(G, dtype=torch.int32, device="cuda"), torch.empty(G, dtype=torch.int32, device="cuda")]
    n_rows = C.c_uint64()
    dp = C.POINTER(C.c_double)
    torch.cuda.synchronize()
    st = lib.ntp_make_table(ctx, None, 0, None, srcs, _abi.fptr(le), None, orient.ctypes.data_as(dp),
                            C.byref(spec), *[o.data_ptr() for o in outs], G, C.byref(n_rows), None, None, None,
                            None, None)
    assert st == _abi.NTP_OK and n_rows.value == G
    assert torch.all(outs[3] == 0) and torch.all(outs[2] == 0)
    assert sorted(outs[4].cpu().tolist()) == list(range(G))
    setup.close()


def test_flow_without_tuples_and_near_zero_expectations():
    with RQNormFlow(RQNormFlowHParams(batch_size=256, seed=2)) as fl:
        fl.init_output_bias(log_expec=-25.0)
        cond = np.random.default_rng(1).uniform(-1, 1, (100, 5)).astype(np.float32)
        lp, le = fl.logpdf(cond, np.zeros(0, np.int32), np.zeros(0, np.float32), log_expec=True)
        assert lp.size == 0 and np.all(le < -20)
        cnt, hc, ht = fl.sample_hits(cond, np.arange(100, dtype=np.uint64), seed=3)
        assert cnt.sum() == 0 and hc.size == 0 and ht.size == 0
        bad = fl.logpdf(cond, np.array([100, -1], np.int32), np.zeros(2, np.float32))
        assert np.all(np.isnan(bad))  # indices outside the conditions give NaN
        with pytest.raises(ValueError):
            fl.logpdf(cond, np.zeros(2, np.int32), np.zeros(1, np.float32))
