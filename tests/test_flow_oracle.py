"""The flow oracle (oracle/flow_ref.py) pinned by the reference's own spline
tests (test/runtests.jl:14-45) and its autograd gradient by finite
differences; plus the host-side layout of the flow's parameters."""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import flow_ref as R  # noqa: E402


def _spline(num_bins, n, seed, r0=-5.0, r1=5.0):
    g = torch.Generator().manual_seed(seed)
    params = torch.randn(n, 3 * num_bins + 1, generator=g, dtype=torch.float64)
    return R.constrain_spline_params(params, r0, r1)


def test_round_trip_and_logdet_reference_case():
    # runtests.jl:15-23: 10 bins on [-5, 5], x = -10:0.1:10, one random spline per point
    x = torch.arange(-100, 101, dtype=torch.float64) / 10.0
    xp, yp, d = _spline(10, x.numel(), 1)
    y, ld = R.rqs_univariate(xp, yp, d, x)
    xrt, ld_inv = R.inv_rqs_univariate(xp, yp, d, y)
    assert torch.allclose(ld, -ld_inv, rtol=1e-9, atol=1e-12)
    assert torch.allclose(x, xrt, atol=1e-5)


@pytest.mark.parametrize("bins,r0,r1", [(10, -5.0, 5.0), (12, -20.0, 1500.0), (10, -20.0, 100.0)])
def test_round_trip_other_ranges(bins, r0, r1):
    x = torch.linspace(r0 - 0.2 * (r1 - r0), r1 + 0.2 * (r1 - r0), 4001, dtype=torch.float64)
    xp, yp, d = _spline(bins, x.numel(), 7, r0, r1)
    y, ld = R.rqs_univariate(xp, yp, d, x)
    xrt, ld_inv = R.inv_rqs_univariate(xp, yp, d, y)
    assert torch.allclose(ld, -ld_inv, rtol=1e-8, atol=1e-10)
    assert torch.allclose(x, xrt, atol=1e-5 * max(1.0, (r1 - r0) / 10.0))


def test_spline_is_monotone_and_fixes_the_range():
    xp, yp, d = _spline(12, 64, 3, -20.0, 1500.0)
    assert torch.all(torch.diff(xp, dim=-1) >= 1e-4 - 1e-9)
    assert torch.all(torch.diff(yp, dim=-1) >= 1e-4 - 1e-9)
    assert torch.all(xp[:, 0] == -20.0) and torch.all(xp[:, -1] == 1500.0)
    assert torch.all(d >= 1e-4)
    # zero raw slopes give unit slopes (the offset of _normalize_knot_slopes)
    assert float(R.normalize_knot_slopes(torch.zeros(1, dtype=torch.float64))) == pytest.approx(1.0, abs=1e-12)


def _integrate(f, a, b, r0, r1, n=400_001):
    """Trapezoid rule, dense inside the spline range [r0, r1] (steep bins make
    narrow peaks there) and coarser in the linear tails."""
    x = np.unique(np.concatenate([np.linspace(a, r0, n // 4), np.linspace(r0, r1, n), np.linspace(r1, b, n // 4)]))
    y = f(x)
    return float(np.sum((y[1:] + y[:-1]) * 0.5 * np.diff(x)))


def test_transformed_normal_integrates_to_one_reference_case():
    # runtests.jl:35-45: p = randn(3*10+1+2), p[end] = |p[end]|, integral over [-10, 10] == 1 to 1e-5
    rng = np.random.default_rng(11)
    for _ in range(3):
        p = rng.standard_normal(3 * 10 + 1 + 2)
        p[-1] = abs(p[-1])
        P = torch.as_tensor(p)

        def f(x):
            xt = torch.as_tensor(x)
            lp = R.eval_transformed_normal_logpdf(xt, P.expand(xt.numel(), -1), -5.0, 5.0)
            return np.exp(lp.numpy())

        # scale = 100 sigmoid(|p|) >= 50: most of the mass lies outside [-10, 10]
        # in the reference's test as well; the property is the total mass
        total = _integrate(f, -5000.0, 5000.0, -5.0, 5.0, 2_000_001)
        assert total == pytest.approx(1.0, abs=1e-5)


def test_stacked_layers_integrate_to_one():
    rng = np.random.default_rng(5)
    L, K = 5, 12
    raw = torch.as_tensor(rng.standard_normal(L * (3 * K + 1) + 2) * 0.7)
    raw[-2] = 300.0
    raw[-1] = -0.5

    def f(x):
        xt = torch.as_tensor(x)
        return np.exp(R.flow_logpdf(xt, raw.expand(xt.numel(), -1), L, -20.0, 1500.0).numpy())

    assert _integrate(f, -3000.0, 5000.0, -20.0, 1500.0, 2_000_001) == pytest.approx(1.0, abs=1e-5)


def test_head_gradient_matches_finite_differences():
    rng = np.random.default_rng(2)
    L, K, B = 2, 10, 6
    n_out = L * (3 * K + 1) + 3
    raw = torch.as_tensor(rng.standard_normal((B, n_out)) * 0.5, dtype=torch.float64).requires_grad_(True)
    with torch.no_grad():
        raw[:, L * (3 * K + 1)] = 30.0
    tres = torch.as_tensor(np.array([-25.0, 0.0, 10.0, 40.0, 90.0, 130.0]))
    nhits = torch.as_tensor(np.array([0.0, 1.0, 3.0, 10.0, 2.0, 5.0]))
    has = torch.as_tensor(np.array([True, True, False, True, True, True]))
    assert torch.autograd.gradcheck(lambda r: R.head_loss(r, tres, nhits, has, L, K, -20.0, 100.0), (raw,),
                                    eps=1e-6, atol=1e-6, rtol=1e-4)


def test_full_loss_gradient_matches_finite_differences():
    rng = np.random.default_rng(4)
    L, K, B, n_pad = 1, 10, 8, 64
    n_out = L * (3 * K + 1) + 3
    sizes = [256 * 64, 256, 256 * 256, 256, 256 * 256, 256, n_pad * 256, n_pad]
    theta = rng.standard_normal(sum(sizes)) * 0.05
    cond = rng.uniform(-1, 1, (B, 5))
    tres = rng.uniform(-10, 80, B)
    nhits = rng.integers(0, 6, B).astype(float)
    has = np.ones(B, bool)
    loss, g = R.full_loss(theta, cond, tres, nhits, has, L, K, -20.0, 100.0, n_pad)
    # central differences on a few parameters of every block
    off = 0
    for size in sizes:
        for j in (off, off + size // 2, off + size - 1):
            t1, t2 = theta.copy(), theta.copy()
            t1[j] += 1e-6
            t2[j] -= 1e-6
            fd = (R.full_loss(t1, cond, tres, nhits, has, L, K, -20.0, 100.0, n_pad)[0] -
                  R.full_loss(t2, cond, tres, nhits, has, L, K, -20.0, 100.0, n_pad)[0]) / 2e-6
            assert g[j] == pytest.approx(fd, rel=1e-4, abs=1e-8)
        off += size
    assert math.isfinite(loss)


def test_adam_update_bias_correction():
    th, m, v = R.adam_update(np.zeros(3), np.zeros(3), np.zeros(3), np.array([1.0, -2.0, 0.0]), 1, 1e-3, 0.9, 0.999,
                             1e-8)
    # first step: m_hat = g, v_hat = g^2 -> step = lr * sign(g)
    np.testing.assert_allclose(th, [-1e-3, 1e-3, 0.0], atol=1e-9)
