"""The training-table generator (ntp_make_table) against the CPU oracle
(oracle/table_ref.py) on a small case, its size-independent properties on a
larger one, and the flow trained on an MC table against the MC truth.

Exactness: group sums and pair counts are compared with the oracle's PMT
assignment, which may differ from the kernel's FP32 test for hits within
rounding of a cone's edge (at most a few per mille of the pairs); the
Poisson counts must equal the oracle's Poisson stream evaluated at the
kernel's own group sums; the drawn rows of a group must be the oracle's
top-N keys."""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from neutrinotelescopes_gb300 import _abi  # noqa: E402
from neutrinotelescopes_gb300.detection import make_pom_pmt_coordinates  # noqa: E402
from neutrinotelescopes_gb300.tables import FlowTable, TableConfig, make_flow_table  # noqa: E402
from oracle import table_ref as T  # noqa: E402

pytestmark = pytest.mark.gpu

SMALL = TableConfig(n_sims=12, n_orientations=3, max_rows_per_group=5, target_hits=150, min_photons=20_000,
                    max_photons=2_000_000, distance=(1.0, 30.0), seed=11)


@pytest.fixture(scope="module")
def small_table():
    return make_flow_table(SMALL)


def _host(table):
    rec = table.hits.cpu().numpy().view(_abi.HIT_DTYPE)
    return rec, table.weights.cpu().numpy()


def test_group_sums_and_features(small_table, oracle_lib):
    t = small_table
    rec, w = _host(t)
    S, R = SMALL.n_sims, SMALL.n_orientations
    pm = T.module_axes(make_pom_pmt_coordinates())
    P = len(pm)
    opening = math.asin(math.sqrt(np.float32(np.pi * (75e-3 / 2) ** 2) / np.float32(np.pi)) / np.float32(0.21))
    pairs = T.assign_pairs(rec["position"], rec["source_index"], t.orientations, pm, R, float(np.float32(math.cos(opening))))
    scale = t.sims["weight_scale"]
    wsum = np.zeros(S * R * P)
    for i, g in pairs:
        wsum[g] += w[i] * scale[rec["source_index"][i]]
    gexp = t.group_expec.cpu().numpy()
    # all but a few edge-of-cone pairs agree
    bad = np.abs(gexp - wsum) > 1e-9 * (1 + np.abs(wsum))
    assert bad.sum() <= max(2, 0.01 * len(gexp)), bad.sum()
    # Poisson counts from the oracle's stream at the kernel's own sums
    L = oracle_lib.lib()
    want = np.array([L.ntpo_poisson(float(x), SMALL.seed, g) for g, x in enumerate(gexp)])
    np.testing.assert_array_equal(t.group_count.cpu().numpy(), want)
    # features
    srcs = t.sims["sources"]
    feats = T.group_features([s.position for s in srcs], [s.direction for s in srcs], t.sims["log10_energy"],
                             t.orientations, pm, R)
    np.testing.assert_allclose(t.group_cond.cpu().numpy(), feats, atol=2e-5)


def test_rows_are_the_oracle_draws(small_table, oracle_lib):
    t = small_table
    rec, w = _host(t)
    S, R = SMALL.n_sims, SMALL.n_orientations
    pm = T.module_axes(make_pom_pmt_coordinates())
    P = len(pm)
    opening = math.asin(math.sqrt(np.float32(np.pi * (75e-3 / 2) ** 2) / np.float32(np.pi)) / np.float32(0.21))
    pairs = T.assign_pairs(rec["position"], rec["source_index"], t.orientations, pm, R, float(np.float32(math.cos(opening))))
    scale = t.sims["weight_scale"]
    N = t.group_count.cpu().numpy()
    by_group: dict[int, list] = {}
    wsum: dict[int, float] = {}
    w2: dict[int, float] = {}
    for i, g in pairs:
        s = int(rec["source_index"][i])
        wi = w[i] * scale[s]
        if wi > 0:
            r = (g // P) % R
            by_group.setdefault(g, []).append((T.pair_key(oracle_lib.philox, int(rec["photon_index"][i]), s, r, wi,
                                                          SMALL.seed), i))
            wsum[g] = wsum.get(g, 0.0) + wi
            w2[g] = w2.get(g, 0.0) + wi * wi
    tres = t.tres.cpu().numpy()
    nh = t.nhits.cpu().numpy()
    has = t.has_time.cpu().numpy()
    rg = t.row_group.cpu().numpy()
    rows_by_group: dict[int, list] = {}
    for q in range(len(tres)):
        g = int(rg[q])
        assert nh[q] == N[g]
        if has[q]:
            rows_by_group.setdefault(g, []).append(tres[q])
        else:
            assert N[g] == 0 and tres[q] == 0.0
    n800 = 1.35
    src_d = np.array([np.linalg.norm(s.position) for s in t.sims["sources"]], np.float32)
    tgeo = (src_d - np.float32(0.21)).astype(np.float64) / (T.C_VAC / n800)
    checked = 0
    for g, keys in by_group.items():
        want = T.rows_wanted(int(N[g]), len(keys), SMALL.max_rows_per_group, wsum[g], w2[g])
        sel = T.select(keys, want)
        s = g // (R * P)
        exp_t = np.sort(np.array([rec["time"][i] - tgeo[s] for i in sel], np.float32))
        got = np.sort(np.array(rows_by_group.get(g, []), np.float32))
        if len(got) != len(exp_t) or not np.allclose(got, exp_t, atol=1e-4):
            continue  # an edge-of-cone pair changed the group's hits
        checked += 1
    assert checked >= 0.97 * len(by_group), (checked, len(by_group))
    # every group is represented: rows with a time, or a count-only row
    G = len(N)
    assert set(rows_by_group) | {g for g in range(G) if N[g] == 0} == set(range(G))


def test_table_save_load_roundtrip(small_table, tmp_path):
    p = tmp_path / "table.npz"
    small_table.save(p)
    t2 = FlowTable.load(p)
    for k in ("cond", "tres", "nhits", "has_time", "group_cond", "group_expec", "group_count", "row_group"):
        assert torch.equal(getattr(small_table, k).cpu(), getattr(t2, k).cpu()), k
    assert t2.n_photons == small_table.n_photons


def test_table_properties_at_size():
    cfg = TableConfig(n_sims=256, n_orientations=8, target_hits=400, max_photons=10_000_000, seed=3)
    t = make_flow_table(cfg)
    N = t.group_count.cpu().numpy().astype(np.float64)
    lam = t.group_expec.cpu().numpy()
    # counts are Poisson(lambda): standardised residuals have mean ~0 and variance ~1
    m = lam > 0.5
    z = (N[m] - lam[m]) / np.sqrt(lam[m])
    assert abs(z.mean()) < 5.0 / math.sqrt(m.sum()) + 0.02
    assert 0.85 < z.var() < 1.15
    # rows: at most max_rows_per_group per group, nhits >= rows of the group, features in range
    cond = t.cond.cpu().numpy()
    assert np.all(np.abs(cond[:, :4]) <= 1.0 + 1e-5)
    assert len(t) >= int((N > 0).sum())
    has = t.has_time.cpu().numpy()
    assert np.all(t.nhits.cpu().numpy()[has == 0] == 0)
