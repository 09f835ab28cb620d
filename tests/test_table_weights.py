"""FlowTable.count_once_weights: 1 / (rows of the row's group), so that each
group's count term enters a training loss once."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from neutrinotelescopes_gb300.tables import FlowTable  # noqa: E402


def test_count_once_weights():
    rg = torch.tensor([2, 0, 0, 2, 0, 3], dtype=torch.int32)
    n = rg.numel()
    t = FlowTable(torch.zeros((n, 5)), torch.zeros(n), torch.zeros(n), torch.ones(n, dtype=torch.int32),
                  torch.zeros((5, 5)), torch.zeros(5, dtype=torch.float64), torch.zeros(5, dtype=torch.int64),
                  row_group=rg)
    w = t.count_once_weights().numpy()
    np.testing.assert_allclose(w, [1 / 2, 1 / 3, 1 / 3, 1 / 2, 1 / 3, 1.0], rtol=1e-7)
    # every group's weights sum to one
    np.testing.assert_allclose(np.bincount(rg.numpy(), weights=w), [1.0, 0.0, 1.0, 1.0])
    with pytest.raises(ValueError):
        FlowTable(t.cond, t.tres, t.nhits, t.has_time, t.group_cond, t.group_expec, t.group_count).count_once_weights()


def test_information_weights():
    # 2 simulations x 2 groups; simulation 0 oversampled 4x (scale 0.25), simulation 1 scale 4
    rg = torch.tensor([0, 0, 1, 2, 3, 3, 3], dtype=torch.int32)
    n = rg.numel()
    gexp = torch.tensor([8.0, 2.0, 40.0, 0.0], dtype=torch.float64)
    t = FlowTable(torch.zeros((n, 5)), torch.zeros(n), torch.zeros(n), torch.ones(n, dtype=torch.int32),
                  torch.zeros((4, 5)), gexp, torch.zeros(4, dtype=torch.int64), row_group=rg,
                  sim_scale=torch.tensor([0.25, 4.0], dtype=torch.float64))
    w, target = t.information_weights()
    c = np.array([4.0, 4.0, 0.25, 0.25])
    c /= c.mean()
    rows = np.bincount(rg.numpy(), minlength=4)
    np.testing.assert_allclose(w.numpy(), c[rg.numpy()] / rows[rg.numpy()], rtol=1e-6)
    # every group's weights sum to its c; the c average to one over the groups
    np.testing.assert_allclose(np.bincount(rg.numpy(), weights=w.numpy()), c, rtol=1e-6)
    np.testing.assert_allclose(target.numpy(), gexp.numpy()[rg.numpy()])
    # the count term's curvature at its minimum (c times the expectation) is the
    # simulated weighted hits, expectation / scale, up to the common factor
    info = np.bincount(rg.numpy(), weights=(w * target).numpy())
    np.testing.assert_allclose(info / info[0], (gexp.numpy() / np.array([0.25, 0.25, 4, 4])) / 32.0, rtol=1e-6)
    with pytest.raises(ValueError):
        FlowTable(t.cond, t.tres, t.nhits, t.has_time, t.group_cond, t.group_expec, t.group_count,
                  row_group=rg).information_weights()


def test_focus_draws():
    """TableConfig.focus_fraction: that fraction of the simulations (about)
    drawn over focus_distance and focus_cos_theta; energies, azimuths and
    the other simulations as without it (the same generator stream)."""
    from neutrinotelescopes_gb300.tables import TableConfig, draw_simulations
    cfg = TableConfig(n_sims=4000, seed=3)
    a = draw_simulations(cfg, np.random.default_rng(3))
    b = draw_simulations(TableConfig(n_sims=4000, seed=3, focus_fraction=0.5), np.random.default_rng(3))
    moved = a["distance"] != b["distance"]
    assert abs(moved.mean() - 0.5) < 0.04
    assert np.all((b["distance"][moved] >= 8.0) & (b["distance"][moved] <= 80.0))
    assert np.all((b["cos_theta"][moved] >= -0.95) & (b["cos_theta"][moved] <= -0.5))
    np.testing.assert_array_equal(a["cos_theta"][~moved], b["cos_theta"][~moved])
    np.testing.assert_array_equal(a["log10_energy"], b["log10_energy"])
    np.testing.assert_array_equal(a["phi"], b["phi"])
    # photons per simulation follow the distance: the focus simulations reach
    # the hit target up to the cap
    assert np.all(b["n_simulated"] >= cfg.min_photons) and np.all(b["n_simulated"] <= cfg.max_photons)


def test_save_load_keeps_what_training_needs(tmp_path):
    """FlowTable.save / load round trip (CPU tensors): rows, groups, row groups
    and the simulations' weight scales, so a loaded table trains with any
    count_mode."""
    rg = torch.tensor([0, 0, 1, 2, 3, 3, 3], dtype=torch.int32)
    n = rg.numel()
    t = FlowTable(torch.arange(n * 5, dtype=torch.float32).reshape(n, 5), torch.linspace(-5, 50, n),
                  torch.arange(n, dtype=torch.float32), torch.ones(n, dtype=torch.int32),
                  torch.zeros((4, 5)), torch.tensor([8.0, 2.0, 40.0, 0.0], dtype=torch.float64),
                  torch.tensor([7, 1, 45, 0]), n_photons=123, n_hits=45, row_group=rg,
                  sim_scale=torch.tensor([0.25, 4.0], dtype=torch.float64))
    t.save(tmp_path / "t.npz")
    u = FlowTable.load(tmp_path / "t.npz", device="cpu")
    for k in ("cond", "tres", "nhits", "has_time", "group_cond", "group_expec", "group_count", "row_group",
              "sim_scale"):
        assert torch.equal(getattr(u, k), getattr(t, k)), k
    assert (u.n_photons, u.n_hits) == (123, 45)
    for a, b in zip(u.information_weights(), t.information_weights()):
        assert torch.equal(a, b)
