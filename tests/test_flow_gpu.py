"""The flow's CUDA kernels (ntp_flow_*) against the torch-float64 CPU oracle
(oracle/flow_ref.py).

Tolerances, and why:
* head (spline loss and its gradient by the raw outputs, FP32 on the GPU
  versus float64 on the same FP32 inputs): loss to 1e-5 relative; gradient
  rows to 2e-3 relative L2 (the inverse spline in FP32 loses a few bits in
  steep bins, where dx/dy reaches ~100, and the loss of 5 stacked layers
  chains them).
* conditioner forward (BF16 tensor cores, FP32 accumulation) versus the
  oracle with the same BF16 rounding of input, weights and activations in
  float64: |dP| <= 2e-3 (1 + |P|) (accumulation order, and an activation
  that rounds to a neighbouring BF16 value).
* full-network gradient: the GPU backward also rounds dP, dZ and the
  transposed weights to BF16; per parameter block relative L2 error <= 3e-2
  and cosine similarity >= 0.999 against the float64 autograd gradient.
* Adam: the update itself is FP32 elementwise: 1e-6 relative.
The parity tests run without the per-sample gradient clip (the oracle has
none); a separate test checks the clip.
"""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from neutrinotelescopes_gb300 import _abi  # noqa: E402
from neutrinotelescopes_gb300.flow import RQNormFlow, RQNormFlowHParams, log_likelihood_with_poisson  # noqa: E402
from oracle import flow_ref as R  # noqa: E402

pytestmark = pytest.mark.gpu

CASES = [  # (n_layers, K, range): the reference's default model and the 5-layer benchmark model
    (1, 10, -20.0, 100.0),
    (5, 12, -20.0, 1500.0),
]


def make(L, K, r0, r1, cap=2048, seed=1, clip=0.0):
    """A flow without the per-sample gradient clip unless asked for: the
    oracle computes the unclipped gradient."""
    return RQNormFlow(RQNormFlowHParams(K=K, n_layers=L, range_min=r0, range_max=r1, batch_size=cap, seed=seed,
                                        grad_clip=clip))


def batch(rng, B, r0, r1, frac_count_only=0.1):
    R_ = r1 - r0
    tres = rng.uniform(r0 - 0.1 * R_, r0 + 0.6 * R_, B).astype(np.float32)
    nhits = rng.poisson(3.0, B).astype(np.float32)
    has = (rng.uniform(size=B) > frac_count_only).astype(np.int32)
    cond = rng.uniform(-1, 1, (B, 5)).astype(np.float32)
    return cond, tres, nhits, has


@pytest.mark.parametrize("L,K,r0,r1", CASES)
def test_head_loss_and_gradient(L, K, r0, r1):
    rng = np.random.default_rng(10 + L)
    B = 1024
    with make(L, K, r0, r1) as fl:
        n_out = fl.n_outputs
        raw = (rng.standard_normal((B, n_out)) * 0.8).astype(np.float32)
        NP = 3 * K + 1
        raw[:, L * NP] = rng.uniform(r0, r0 + 0.5 * (r1 - r0), B)     # shift
        raw[:, L * NP + 2] = rng.standard_normal(B) * 2.0               # log expectation
        _, tres, nhits, has = batch(rng, B, r0, r1)
        loss, grad = fl.head(raw, tres, nhits, has)
    t = torch.as_tensor(raw.astype(np.float64)).requires_grad_(True)
    ref = R.head_loss(t, torch.as_tensor(tres.astype(np.float64)), torch.as_tensor(nhits.astype(np.float64)),
                      torch.as_tensor(has.astype(bool)), L, K, r0, r1)
    ref.backward()
    g_ref = t.grad.numpy()
    assert loss == pytest.approx(ref.item(), rel=1e-5)
    err = np.linalg.norm(grad - g_ref, axis=1) / (np.linalg.norm(g_ref, axis=1) + 1e-12)
    assert np.quantile(err, 0.99) < 2e-3, np.sort(err)[-5:]
    assert np.linalg.norm(grad - g_ref) / np.linalg.norm(g_ref) < 2e-3


def test_head_with_per_row_count_weights():
    """Per-row factors of the Poisson term (0 on most rows, fractional on the
    rest, as the expected-count tables give) against the oracle."""
    L, K, r0, r1 = 5, 12, -20.0, 1500.0
    rng = np.random.default_rng(15)
    B = 1024
    with make(L, K, r0, r1) as fl:
        raw = (rng.standard_normal((B, fl.n_outputs)) * 0.8).astype(np.float32)
        NP = 3 * K + 1
        raw[:, L * NP] = rng.uniform(r0, r0 + 0.5 * (r1 - r0), B)
        raw[:, L * NP + 2] = rng.standard_normal(B) * 2.0
        _, tres, nhits, has = batch(rng, B, r0, r1)
        nhits = (nhits * rng.uniform(0.5, 1.5, B)).astype(np.float32)  # expectations, not integers
        cw = np.where(rng.uniform(size=B) < 0.3, rng.uniform(0.05, 1.0, B), 0.0).astype(np.float32)
        loss, grad = fl.head(raw, tres, nhits, has, count_weight=cw)
        loss1, _ = fl.head(raw, tres, nhits, has)
    t = torch.as_tensor(raw.astype(np.float64)).requires_grad_(True)
    ref = R.head_loss(t, torch.as_tensor(tres.astype(np.float64)), torch.as_tensor(nhits.astype(np.float64)),
                      torch.as_tensor(has.astype(bool)), L, K, r0, r1, torch.as_tensor(cw.astype(np.float64)))
    ref.backward()
    g_ref = t.grad.numpy()
    assert loss == pytest.approx(ref.item(), rel=1e-5)
    assert loss != pytest.approx(loss1, rel=1e-3)
    assert np.linalg.norm(grad - g_ref) / np.linalg.norm(g_ref) < 2e-3


def test_full_gradient_with_count_weights():
    L, K, r0, r1 = 5, 12, -20.0, 1500.0
    rng = np.random.default_rng(25)
    B = 1024
    with make(L, K, r0, r1) as fl:
        cond, tres, nhits, has = batch(rng, B, r0, r1)
        cw = np.where(rng.uniform(size=B) < 0.2, rng.uniform(0.1, 1.0, B), 0.0).astype(np.float32)
        dev = lambda x: torch.as_tensor(x, device="cuda")  # noqa: E731
        loss = fl.train_steps(dev(cond), dev(tres), dev(nhits), dev(has), B, 1, count_weight=dev(cw),
                              update=False)[0]
        g = fl.gradient()
        theta = fl.get_params()
        n_pad = fl.n_outputs_padded
    ref_loss, g_ref = R.full_loss(theta, cond, tres, nhits, has.astype(bool), L, K, r0, r1, n_pad, bf16=True,
                                  count_weight=cw)
    assert loss == pytest.approx(ref_loss, rel=1e-3)
    assert np.linalg.norm(g - g_ref) <= 3e-2 * np.linalg.norm(g_ref)


def test_head_gradient_clip():
    """With grad_clip = c every row of dL/dP has an L2 norm of at most c / B and
    points along the unclipped row; rows below the bound are unchanged."""
    L, K, r0, r1 = 5, 12, -20.0, 1500.0
    rng = np.random.default_rng(15)
    B, c = 1024, 50.0
    NP = 3 * K + 1
    with make(L, K, r0, r1) as fl0, make(L, K, r0, r1, clip=c) as fl1:
        raw = (rng.standard_normal((B, fl0.n_outputs)) * 0.8).astype(np.float32)
        raw[:, L * NP] = rng.uniform(r0, r0 + 0.5 * (r1 - r0), B)
        raw[:, L * NP + 2] = rng.standard_normal(B) * 2.0
        _, tres, nhits, has = batch(rng, B, r0, r1)
        l0, g0 = fl0.head(raw, tres, nhits, has)
        l1, g1 = fl1.head(raw, tres, nhits, has)
    assert l0 == l1
    n0 = np.linalg.norm(g0.astype(np.float64), axis=1)
    n1 = np.linalg.norm(g1.astype(np.float64), axis=1)
    assert np.all(n1 <= c / B * (1 + 1e-5))
    big = n0 > c / B
    assert big.any() and (~big).any()
    np.testing.assert_array_equal(g1[~big], g0[~big])
    cos = np.sum(g0[big] * g1[big], axis=1) / (n0[big] * n1[big])
    assert np.all(cos > 1 - 1e-5)


def test_degenerate_knots_stay_finite():
    """Raw widths that put all the range in the first bin leave the other
    bins at the minimum width; their FP32 running sum passes the pinned last
    knot unless the knots are kept strictly increasing."""
    L, K, r0, r1 = 5, 12, -20.0, 1500.0
    NP = 3 * K + 1
    B = 256
    raw = np.zeros((B, L * NP + 3), np.float32)
    for li in range(L):
        raw[:, li * NP] = 60.0             # bin 0 takes the whole width ...
        raw[:, li * NP + K] = 60.0         # ... and the whole height
        raw[:, li * NP + 2 * K:(li + 1) * NP] = -12.0   # slopes near the minimum
    raw[:, L * NP] = 1400.0
    tres = np.linspace(1495.0, 1500.5, B).astype(np.float32)
    with make(L, K, r0, r1) as fl:
        loss, grad = fl.head(raw, tres, np.ones(B, np.float32), np.ones(B, np.int32))
    assert np.isfinite(loss) and np.all(np.isfinite(grad))


@pytest.mark.parametrize("L,K,r0,r1", CASES)
def test_conditioner_forward(L, K, r0, r1):
    rng = np.random.default_rng(3)
    with make(L, K, r0, r1) as fl:
        cond = rng.uniform(-1, 1, (1000, 5)).astype(np.float32)   # not a multiple of 128: padded pass
        P = fl.forward_params(cond)
        theta = fl.get_params()
        n_pad = fl.n_outputs_padded
    ref = R.conditioner(R.unpack(theta, n_pad), torch.as_tensor(cond.astype(np.float64)), bf16=True).numpy()
    ref = ref[:, :P.shape[1]]
    assert np.all(np.abs(P - ref) <= 2e-3 * (1 + np.abs(ref))), np.abs(P - ref).max()


@pytest.mark.parametrize("L,K,r0,r1", CASES)
def test_full_gradient(L, K, r0, r1):
    rng = np.random.default_rng(20 + L)
    B = 1024
    with make(L, K, r0, r1) as fl:
        cond, tres, nhits, has = batch(rng, B, r0, r1)
        loss = fl.train_step(cond, tres, nhits, has, update=False)
        g = fl.gradient()
        theta = fl.get_params()
        layout = fl.layout()
        n_pad, n_out = fl.n_outputs_padded, fl.n_outputs
    ref_loss, g_ref = R.full_loss(theta, cond, tres, nhits, has.astype(bool), L, K, r0, r1, n_pad, bf16=True)
    assert loss == pytest.approx(ref_loss, rel=1e-3)
    for name, shape, off in layout:
        size = int(np.prod(shape))
        a, b = g[off:off + size].astype(np.float64), g_ref[off:off + size]
        if name == "W1":  # padding input columns carry no gradient
            assert np.all(a.reshape(shape)[:, 5:] == 0.0)
        if name in ("W4", "b4"):
            rows = a.reshape(shape[0], -1)
            assert np.all(rows[n_out:] == 0.0)
        nb = np.linalg.norm(b)
        assert np.linalg.norm(a - b) <= 3e-2 * nb + 1e-7, (name, np.linalg.norm(a - b) / nb)
        assert np.dot(a, b) >= 0.999 * np.linalg.norm(a) * nb, name


def test_adam_steps_and_weight_copies():
    L, K, r0, r1 = 5, 12, -20.0, 1500.0
    rng = np.random.default_rng(30)
    hp = RQNormFlowHParams(K=K, n_layers=L, range_min=r0, range_max=r1, batch_size=512, seed=9, lr=1e-3,
                           grad_clip=0.0)
    with RQNormFlow(hp) as fl:
        th = fl.get_params().astype(np.float64)
        m = np.zeros_like(th)
        v = np.zeros_like(th)
        for step in (1, 2):
            cond, tres, nhits, has = batch(rng, 512, r0, r1)
            fl.train_step(cond, tres, nhits, has)
            g = fl.gradient().astype(np.float64)
            # the hyperparameters as the FP32 values the kernel uses (1 - 0.999f differs from 1e-3 by 1.3e-5)
            f32 = lambda x: float(np.float32(x))  # noqa: E731
            th, m, v = R.adam_update(th, m, v, g, step, f32(hp.lr), f32(hp.beta1), f32(hp.beta2), f32(hp.eps))
            # FP32 elementwise: relative to each array's scale where b1 m + (1 - b1) g cancels
            np.testing.assert_allclose(fl.get_params(2), m, rtol=1e-5, atol=1e-6 * np.abs(m).max())
            np.testing.assert_allclose(fl.get_params(3), v, rtol=1e-5, atol=1e-6 * np.abs(v).max())
            np.testing.assert_allclose(fl.get_params(0), th, rtol=1e-6, atol=1e-7)
        # the BF16 copies follow the updated master weights
        cond = rng.uniform(-1, 1, (256, 5)).astype(np.float32)
        P = fl.forward_params(cond)
        ref = R.conditioner(R.unpack(fl.get_params(), fl.n_outputs_padded),
                            torch.as_tensor(cond.astype(np.float64)), bf16=True).numpy()[:, :P.shape[1]]
        assert np.all(np.abs(P - ref) <= 2e-3 * (1 + np.abs(ref)))


def test_multi_step_call_follows_single_steps():
    """ntp_flow_train_steps over n consecutive batches gives the losses and
    parameters of n single train_step calls (the split-K weight gradients add
    in FP32 atomics, so equal up to rounding)."""
    L, K, r0, r1 = 5, 12, -20.0, 1500.0
    rng = np.random.default_rng(31)
    B, n = 512, 6
    cond, tres, nhits, has = batch(rng, B * n, r0, r1)
    hp = RQNormFlowHParams(K=K, n_layers=L, range_min=r0, range_max=r1, batch_size=B, seed=4, lr=1e-3)
    with RQNormFlow(hp) as a, RQNormFlow(hp) as b:
        la = [a.train_step(cond[i * B:(i + 1) * B], tres[i * B:(i + 1) * B], nhits[i * B:(i + 1) * B],
                           has[i * B:(i + 1) * B]) for i in range(n)]
        dev = lambda x: torch.as_tensor(x, device="cuda")  # noqa: E731
        lb = b.train_steps(dev(cond), dev(tres), dev(nhits), dev(has), B, n)
        assert len(lb) == n and np.all(np.isfinite(lb))
        np.testing.assert_allclose(lb, la, rtol=1e-4)
        np.testing.assert_allclose(b.get_params(), a.get_params(), rtol=1e-3, atol=1e-5)


@pytest.mark.parametrize("L,K,r0,r1", CASES)
def test_evaluate_matches_oracle_on_the_same_parameters(L, K, r0, r1):
    rng = np.random.default_rng(40)
    with make(L, K, r0, r1) as fl:
        n_cond = 300
        cond = rng.uniform(-1, 1, (n_cond, 5)).astype(np.float32)
        P = fl.forward_params(cond)
        idx = rng.integers(0, n_cond, 20000).astype(np.int32)
        t = rng.uniform(r0 - 0.2 * (r1 - r0), r1 + 0.2 * (r1 - r0), idx.size).astype(np.float32)
        lp, le = fl.logpdf(cond, idx, t, log_expec=True)
        bad = fl.logpdf(cond, np.array([-1, n_cond], np.int32), np.zeros(2, np.float32))
        # the reference-style call and loss
        x = {"tres": t[:1000], "label": cond[idx[:1000]], "nhits": rng.poisson(2.0, 1000).astype(np.float32)}
        ll = log_likelihood_with_poisson(x, fl)
    Pt = torch.as_tensor(P[idx].astype(np.float64))
    ref = R.flow_logpdf(torch.as_tensor(t.astype(np.float64)), Pt, L, r0, r1, K).numpy()
    np.testing.assert_allclose(lp, ref, rtol=1e-4, atol=2e-4)
    np.testing.assert_allclose(le, P[:, -1], rtol=0, atol=0)
    assert np.all(np.isnan(bad))
    P1 = torch.as_tensor(P[idx[:1000]].astype(np.float64))
    lp1 = R.flow_logpdf(torch.as_tensor(t[:1000].astype(np.float64)), P1, L, r0, r1, K).numpy()
    le1 = P[idx[:1000], -1].astype(np.float64)
    n = x["nhits"].astype(np.float64)
    want = -(lp1.sum() + (n * le1 - np.exp(le1) - np.array([math.lgamma(a + 1) for a in n])).sum()) / 1000
    assert ll == pytest.approx(want, rel=1e-4)


@pytest.mark.parametrize("L,K,r0,r1", CASES)
def test_mixture_cdf_matches_oracle(L, K, r0, r1):
    """The pooled CDF of 70 conditions with offsets, weighted by their
    expected counts and by given weights, against the oracle's CDFs (float64)
    of the same raw parameters; monotone in time, 0 and 1 far out."""
    rng = np.random.default_rng(41)
    n_cond, n_t = 70, 3000
    cond = rng.uniform(-1, 1, (n_cond, 5)).astype(np.float32)
    off = rng.uniform(0.0, 400.0, n_cond).astype(np.float32)
    t = np.sort(rng.uniform(r0 - 50.0, r1 + 500.0, n_t)).astype(np.float32)
    w = rng.uniform(0.1, 3.0, n_cond).astype(np.float32)
    with make(L, K, r0, r1) as fl:
        P = fl.forward_params(cond)
        F_le = fl.mixture_cdf(cond, t, off)
        F_w = fl.mixture_cdf(cond, t, off, w)
        dev = fl.mixture_cdf(torch.as_tensor(cond, device="cuda"), torch.as_tensor(t, device="cuda"),
                             torch.as_tensor(off, device="cuda")).cpu().numpy()
        ends = fl.mixture_cdf(cond, np.array([-1e6, 1e7], np.float32))
    Pt = torch.as_tensor(np.repeat(P.astype(np.float64), n_t, axis=0))
    y = torch.as_tensor((t[None, :].astype(np.float64) - off[:, None].astype(np.float64)).reshape(-1))
    Fi = R.flow_cdf(y, Pt, L, r0, r1, K).numpy().reshape(n_cond, n_t)
    lam = np.exp(P[:, -1].astype(np.float64))
    np.testing.assert_allclose(F_le, (lam[:, None] * Fi).sum(0) / lam.sum(), atol=2e-4)
    np.testing.assert_allclose(F_w, (w[:, None] * Fi).sum(0) / w.sum(), atol=2e-4)
    np.testing.assert_array_equal(dev, F_le)
    assert np.all(np.diff(F_le) >= -1e-6)
    np.testing.assert_allclose(ends, [0.0, 1.0], atol=1e-6)


def test_grid_evaluation_equals_tuples():
    L, K, r0, r1 = 5, 12, -20.0, 1500.0
    rng = np.random.default_rng(70)
    with make(L, K, r0, r1, seed=6) as fl:
        cond = rng.uniform(-1, 1, (37, 5)).astype(np.float32)
        times = np.concatenate([rng.uniform(-60, 1700, 200), [-20.0, 1500.0]]).astype(np.float32)
        g, le = fl.logpdf_grid(cond, times, log_expec=True)
        idx = np.repeat(np.arange(37, dtype=np.int32), times.size)
        t = np.tile(times, 37)
        lp, le2 = fl.logpdf(cond, idx, t, log_expec=True)
        gd = fl.logpdf_grid(torch.as_tensor(cond, device="cuda"), torch.as_tensor(times, device="cuda")).cpu().numpy()
    np.testing.assert_allclose(g.ravel(), lp, rtol=2e-6, atol=2e-6)
    np.testing.assert_array_equal(le, le2)
    np.testing.assert_array_equal(gd, g)


def test_density_integrates_to_one_on_device():
    # a size-independent property at a full-size evaluation (16.8 M tuples)
    L, K, r0, r1 = 5, 12, -20.0, 1500.0
    rng = np.random.default_rng(50)
    with make(L, K, r0, r1, seed=4) as fl:
        n_cond = 64
        cond = torch.as_tensor(rng.uniform(-1, 1, (n_cond, 5)).astype(np.float32), device="cuda")
        grid = np.unique(np.concatenate([np.linspace(-3000.0, r0, 20000), np.linspace(r0, r1, 222144),
                                         np.linspace(r1, 6000.0, 20000)]))
        n_t = grid.size
        t = torch.as_tensor(np.tile(grid, n_cond).astype(np.float32), device="cuda")
        idx = torch.arange(n_cond, device="cuda", dtype=torch.int32).repeat_interleave(n_t)
        lp = fl.logpdf(cond, idx, t).view(n_cond, n_t).double().cpu().numpy()
    p = np.exp(lp)
    mass = np.sum((p[:, 1:] + p[:, :-1]) * 0.5 * np.diff(grid)[None, :], axis=1)
    np.testing.assert_allclose(mass, 1.0, atol=2e-3)


def test_training_learns_a_conditional_density():
    """Loss falls and the fitted density matches held-out samples (KS) and
    the expected counts on a synthetic conditional distribution."""
    L, K, r0, r1 = 5, 12, -20.0, 1500.0
    rng = np.random.default_rng(60)

    def sample(cond):
        mu = 50.0 + 40.0 * cond[:, 0]
        return (mu + rng.gamma(2.0, 15.0 * (1.5 + cond[:, 1]))).astype(np.float32)

    def lam(cond):
        return np.exp(1.0 + 0.8 * cond[:, 2])

    n = 1 << 19
    cond = rng.uniform(-1, 1, (n, 5)).astype(np.float32)
    tres = sample(cond)
    nhits = rng.poisson(lam(cond)).astype(np.float32)
    hp = RQNormFlowHParams(K=K, n_layers=L, range_min=r0, range_max=r1, batch_size=4096, lr=2e-3, seed=3)
    with RQNormFlow(hp) as fl:
        losses = fl.fit(cond, tres, nhits, epochs=24)
        assert np.mean(losses[-20:]) < np.mean(losses[:5]) - 1.0, (losses[:5], losses[-20:])
        test_c = np.array([[-0.5, 0.0, 0.5, 0.0, 0.0], [0.5, -0.5, -0.5, 0.3, 0.2]], np.float32)
        grid = np.linspace(r0, 600.0, 20001).astype(np.float32)
        for c in test_c:
            lp, le = fl.logpdf(c[None], np.zeros(grid.size, np.int32), grid, log_expec=True)
            pdf = np.exp(lp.astype(np.float64))
            cdf = np.concatenate([[0.0], np.cumsum((pdf[1:] + pdf[:-1]) * 0.5 * np.diff(grid))])
            s = np.sort(sample(np.repeat(c[None], 4000, axis=0)))
            F = np.interp(s, grid, cdf)
            ks = np.max(np.maximum(np.arange(1, s.size + 1) / s.size - F, F - np.arange(s.size) / s.size))
            assert ks < 0.05, ks
            assert abs(float(le[0]) - math.log(lam(c[None])[0])) < 0.1


def test_invalid_arguments():
    lib = _abi.load_library()
    import ctypes as C
    bad = _abi.NtpFlowConfig(batch_capacity=1024, n_layers=1, n_bins=11, t_min=-20, t_max=100, lr=1e-3, beta1=0.9,
                             beta2=0.999, eps=1e-8, grad_clip=0.0, count_weight=1.0, seed=0)
    h = C.c_void_p()
    assert lib.ntp_flow_create(0, C.byref(bad), C.byref(h)) == _abi.NTP_ERR_INVALID
    assert not h.value
    with make(1, 10, -20.0, 100.0, cap=256) as fl:
        cond, tres, nhits, has = batch(np.random.default_rng(0), 200, -20.0, 100.0)
        with pytest.raises(_abi.NtpError) as e:
            fl.train_step(cond, tres, nhits, has)  # not a multiple of 128
        assert e.value.status == _abi.NTP_ERR_INVALID
        with pytest.raises(ValueError):
            fl.set_params(np.zeros(3, np.float32))


def make_derived(L=1, K=10, r0=-20.0, r1=100.0, cap=2048, seed=2):
    return RQNormFlow(RQNormFlowHParams(K=K, n_layers=L, range_min=r0, range_max=r1, batch_size=cap, seed=seed,
                                        grad_clip=0.0, input_columns="derived"))


def test_derived_columns_forward():
    """The count model's conditioner reads four derived input columns
    computed on the device; the oracle computes them in float32 from the
    same features.  Same bound as the plain forward; a derived column whose
    float32 value lies at a BF16 rounding boundary may round the other way
    on one side (rare: at most 0.5 % of the rows may exceed the bound, by at
    most 5x)."""
    rng = np.random.default_rng(4)
    cond = rng.uniform(-1, 1, (1000, 5)).astype(np.float32)
    with make_derived() as fl:
        P = fl.forward_params(cond)
        theta = fl.get_params()
        n_pad = fl.n_outputs_padded
        W1 = theta[:256 * 64].reshape(256, 64)
        assert np.all(W1[:, 9:] == 0.0) and np.all(W1[:, 5:9] != 0.0)
    x = torch.as_tensor(R.derived_columns(cond).astype(np.float64))
    ref = R.conditioner(R.unpack(theta, n_pad), x, bf16=True).numpy()[:, :P.shape[1]]
    bound = 2e-3 * (1 + np.abs(ref))
    over = np.any(np.abs(P - ref) > bound, axis=1)
    assert np.mean(over) <= 0.005, np.mean(over)
    assert np.all(np.abs(P - ref) <= 5 * bound)


def test_derived_columns_count_only_gradient():
    """A count-only batch (no time rows, expectations as targets, per-row
    information weights) through the derived-column model: the full
    gradient against the float64 oracle, as test_full_gradient."""
    rng = np.random.default_rng(26)
    B = 1024
    L, K, r0, r1 = 1, 10, -20.0, 100.0
    cond = rng.uniform(-1, 1, (B, 5)).astype(np.float32)
    nhits = (rng.gamma(0.5, 20.0, B)).astype(np.float32)
    tres = np.zeros(B, np.float32)
    has = np.zeros(B, np.int32)
    cw = rng.uniform(0.2, 2.0, B).astype(np.float32)
    with make_derived() as fl:
        dev = lambda x: torch.as_tensor(x, device="cuda")  # noqa: E731
        loss = fl.train_steps(dev(cond), dev(tres), dev(nhits), dev(has), B, 1, count_weight=dev(cw),
                              update=False)[0]
        g = fl.gradient()
        theta = fl.get_params()
        layout = fl.layout()
        n_pad = fl.n_outputs_padded
    ref_loss, g_ref = R.full_loss(theta, cond, tres, nhits, has.astype(bool), L, K, r0, r1, n_pad, bf16=True,
                                  count_weight=cw, derived=True)
    assert loss == pytest.approx(ref_loss, rel=1e-3)
    for name, shape, off in layout:
        size = int(np.prod(shape))
        a, b = g[off:off + size].astype(np.float64), g_ref[off:off + size]
        if name == "W1":
            assert np.all(a.reshape(shape)[:, 9:] == 0.0)
        nb = np.linalg.norm(b)
        if nb == 0.0:
            assert np.all(a == 0.0), name
            continue
        assert np.linalg.norm(a - b) <= 3e-2 * nb + 1e-7, (name, np.linalg.norm(a - b) / nb)
        assert np.dot(a, b) >= 0.999 * np.linalg.norm(a) * nb, name


def test_sampling_with_external_expectations():
    """Counts drawn from given log expectations: the same keys and
    expectations give the same hits whichever flow supplies the times'
    knots' own count head, and the counts follow the given expectations."""
    rng = np.random.default_rng(41)
    n = 4000
    cond = torch.as_tensor(rng.uniform(-1, 1, (n, 5)).astype(np.float32), device="cuda")
    keys = torch.as_tensor(np.arange(n, dtype=np.int64) * 7919 + 11, device="cuda")
    le = torch.as_tensor(rng.uniform(-1.0, 2.5, n).astype(np.float32), device="cuda")
    with make(5, 12, -20.0, 1500.0) as fl:
        own_le = fl.log_expectation(cond)
        cnt, hc, ht = fl.sample_hits(cond, keys, seed=5, log_expec=le)
        cnt2, hc2, ht2 = fl.sample_hits(cond, keys, seed=5, log_expec=le)
        cnt0, _, _ = fl.sample_hits(cond, keys, seed=5)
        cnt_h, hc_h, ht_h = fl.sample_hits(cond.cpu().numpy(), keys.cpu().numpy(), seed=5,
                                           log_expec=le.cpu().numpy())
    assert torch.equal(cnt, cnt2) and torch.equal(hc, hc2) and torch.equal(ht, ht2)
    np.testing.assert_array_equal(cnt.cpu().numpy().astype(np.uint64), cnt_h)
    np.testing.assert_array_equal(ht.cpu().numpy(), ht_h)
    lam = np.exp(le.double().cpu().numpy())
    c = cnt.double().cpu().numpy()
    assert abs(c.sum() - lam.sum()) < 4 * np.sqrt(lam.sum())
    lam0 = np.exp(own_le.double().cpu().numpy())
    assert abs(cnt0.double().sum().item() - lam0.sum()) < 4 * np.sqrt(lam0.sum())
    assert not np.allclose(lam0, lam)


def test_log_expectation_query_matches_evaluate():
    """The knot-free count query gives the log expectations of the full
    model call, bit for bit, across chunks of the batch capacity, with host
    and device buffers."""
    rng = np.random.default_rng(42)
    n = 5000  # more than the capacity below: three chunks
    cond = rng.uniform(-1, 1, (n, 5)).astype(np.float32)
    with RQNormFlow(RQNormFlowHParams(K=12, n_layers=5, batch_size=2048, seed=3), batch_capacity=2048) as fl:
        le_h = fl.log_expectation(cond)
        le_d = fl.log_expectation(torch.as_tensor(cond, device="cuda")).cpu().numpy()
        ref = np.empty(n, np.float32)
        fl._check(fl.lib.ntp_flow_evaluate(fl._h, cond.ctypes.data, n, None, None, 0, None, ref.ctypes.data, 0))
    np.testing.assert_array_equal(le_h, ref)
    np.testing.assert_array_equal(le_d, ref)


def _flow_with_chain(monkeypatch, chain, L, K, r0, r1, cap=2048, seed=1):
    monkeypatch.setenv("NTP_FLOW_CHAIN", "1" if chain else "0")
    return make(L, K, r0, r1, cap=cap, seed=seed)


@pytest.mark.parametrize("L,K,r0,r1", CASES)
def test_layer_chain_matches_per_layer_gemms(monkeypatch, L, K, r0, r1):
    """The fused layer chain (forward X -> H1 -> H2 -> H3 -> P and backward
    dP -> dZ3 -> dZ2 -> dZ1 in one kernel per 128-row tile) against one
    tensor-core GEMM per layer on the same weights and batch.  Both
    accumulate every output over K in the same slice order in FP32 and round
    the same activations to BF16, so P, the loss and the gradient agree to
    the last bits (atomic column sums and split-K weight gradients add in
    varying order: 1e-5 relative per parameter block)."""
    rng = np.random.default_rng(50 + L)
    B = 1024
    cond, tres, nhits, has = batch(rng, B, r0, r1)
    out = {}
    for chain in (True, False):
        with _flow_with_chain(monkeypatch, chain, L, K, r0, r1) as fl:
            P = fl.forward_params(cond[:1000])  # not a multiple of 128: the last tile is partly padding
            loss = fl.train_step(cond, tres, nhits, has, update=False)
            out[chain] = (P, loss, fl.gradient().astype(np.float64), fl.layout())
    (P1, l1, g1, layout), (P0, l0, g0, _) = out[True], out[False]
    np.testing.assert_array_equal(P1, P0)
    assert l1 == pytest.approx(l0, rel=1e-6)
    for name, shape, off in layout:
        size = int(np.prod(shape))
        a, b = g1[off:off + size], g0[off:off + size]
        assert np.linalg.norm(a - b) <= 1e-5 * np.linalg.norm(b) + 1e-9, (name, np.abs(a - b).max())


def test_layer_chain_wait_runs_out(monkeypatch):
    """Failure detection of the fused chain: with its input tile withheld the
    first barrier is a flag that nothing completes; the bounded wait gives up
    after 1 ms, the call returns NTP_ERR_TIMEOUT and the context stays usable
    (the same forward pass succeeds afterwards)."""
    import time

    lib = _abi.load_library()
    rng = np.random.default_rng(5)
    cond = rng.uniform(-1, 1, (256, 5)).astype(np.float32)
    with _flow_with_chain(monkeypatch, True, 5, 12, -20.0, 1500.0) as fl:
        ref = fl.forward_params(cond)
        assert lib.ntp_gemm_set_wait_limit(1_000_000, 1) == _abi.NTP_OK
        try:
            t0 = time.perf_counter()
            with pytest.raises(_abi.NtpError) as ei:
                fl.forward_params(cond)
            elapsed = time.perf_counter() - t0
        finally:
            assert lib.ntp_gemm_set_wait_limit(0, 0) == _abi.NTP_OK
        assert ei.value.status == _abi.NTP_ERR_TIMEOUT
        assert elapsed < 1.0
        np.testing.assert_array_equal(fl.forward_params(cond), ref)
