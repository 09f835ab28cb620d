"""CPU oracle of the arrival-time flow in torch float64.

TEST INFRASTRUCTURE ONLY: imported by tests/ to verify the flow's
CUDA kernels (forward, head gradient, full-network gradient, Adam), never by
the product path.

Restates src/surrogate_models/rq_spline_flow.jl of chrhck/NeutrinoTelescopes
(``_normalize_bin_sizes`` :127-136, ``_normalize_knot_slopes`` :146-154,
``constrain_spline_params`` :170-206, ``safe_quadratic_root`` :215-244,
``rqs_univariate`` :262-324, ``inv_rqs_univariate`` :334-389,
``eval_transformed_normal_logpdf`` :396-418) and the model and loss of
extended_cascade_model.jl (``RQNormFlow`` call :110-125,
``log_likelihood_with_poisson`` :132-139), batch-first: spline parameters
are rows [n x (3K+1)] where the reference uses columns.  Gradients come from
torch autograd.  Pinned by the reference's own spline tests
(test/runtests.jl:14-45: forward/inverse round trip to 1e-5, logdet equal to
minus the inverse logdet, the transformed-normal density integrating to 1),
restated in tests/test_flow_oracle.py.

Stacked layers (n_layers > 1) compose inverse splines: the time residual
passes layer L-1 first, layer 0 last, then the shifted and scaled normal.
"""
from __future__ import annotations

import math

import numpy as np
import torch

F = torch.nn.functional
DT = torch.float64
# the kernels' FP32 range guards: log expectation within [-30, 30], raw scale
# within [-20, 20], standardised residual within +-1e6 (held, zero gradient
# outside); inactive for ordinary values
LE_CLAMP = 30.0
SCALE_CLAMP = 20.0
MAX_U = 1e6


def normalize_bin_sizes(u: torch.Tensor, total: float, min_bin: float = 1e-4) -> torch.Tensor:
    K = u.shape[-1]
    return torch.softmax(u, dim=-1) * (total - K * min_bin) + min_bin


def normalize_knot_slopes(u: torch.Tensor, min_slope: float = 1e-4) -> torch.Tensor:
    offset = math.log(math.exp(1.0 - min_slope) - 1.0)
    return F.softplus(u + offset) + min_slope


def constrain_spline_params(p: torch.Tensor, r0: float, r1: float):
    """p [n x (3K+1)] -> x_pos, y_pos, slopes [n x (K+1)]."""
    K = (p.shape[-1] - 1) // 3
    w = normalize_bin_sizes(p[:, :K], r1 - r0)
    h = normalize_bin_sizes(p[:, K:2 * K], r1 - r0)
    d = normalize_knot_slopes(p[:, 2 * K:])
    lo = torch.full_like(p[:, :1], r0)
    hi = torch.full_like(p[:, :1], r1)
    x_pos = torch.cat([lo, r0 + torch.cumsum(w[:, :-1], dim=-1), hi], dim=-1)
    y_pos = torch.cat([lo, r0 + torch.cumsum(h[:, :-1], dim=-1), hi], dim=-1)
    return x_pos, y_pos, d


def safe_quadratic_root(a, b, c):
    disc = b * b - 4.0 * a * c
    sq = torch.where(disc > 0, torch.sqrt(torch.clamp(disc, min=1e-300)), torch.zeros_like(disc))
    return torch.where(b >= 0, (2.0 * c) / (-b - sq), (-b + sq) / (2.0 * a))


def _bin(pos: torch.Tensor, v: torch.Tensor) -> torch.Tensor:
    K = pos.shape[-1] - 1
    return (v[:, None] >= pos[:, 1:K]).sum(dim=-1, keepdim=True)


def _take(t: torch.Tensor, k: torch.Tensor) -> torch.Tensor:
    return t.gather(1, k).squeeze(1)


def rqs_univariate(x_pos, y_pos, d, x):
    """Forward spline: y and log|dy/dx| (rq_spline_flow.jl:262-324)."""
    k = _bin(x_pos, x)
    x0, x1 = _take(x_pos, k), _take(x_pos, k + 1)
    y0, y1 = _take(y_pos, k), _take(y_pos, k + 1)
    d0, d1 = _take(d, k), _take(d, k + 1)
    w, h = x1 - x0, y1 - y0
    s = h / w
    z = torch.clamp((x - x0) / w, 0.0, 1.0)
    sq_z, z1mz, sq_1mz = z * z, z - z * z, (1.0 - z) ** 2
    st = d1 + d0 - 2.0 * s
    num = h * (s * sq_z + d0 * z1mz)
    den = s + st * z1mz
    y = y0 + num / den
    logdet = 2.0 * torch.log(s) + torch.log(d1 * sq_z + 2.0 * s * z1mz + d0 * sq_1mz) - 2.0 * torch.log(den)
    below, above = x <= x_pos[:, 0], x >= x_pos[:, -1]
    y = torch.where(below, (x - x_pos[:, 0]) * d[:, 0] + y_pos[:, 0], y)
    y = torch.where(above, (x - x_pos[:, -1]) * d[:, -1] + y_pos[:, -1], y)
    logdet = torch.where(below, torch.log(d[:, 0]), logdet)
    logdet = torch.where(above, torch.log(d[:, -1]), logdet)
    return y, logdet


def inv_rqs_univariate(x_pos, y_pos, d, y):
    """Inverse spline: x and log|dx/dy| (rq_spline_flow.jl:334-389)."""
    k = _bin(y_pos, y)
    x0, x1 = _take(x_pos, k), _take(x_pos, k + 1)
    y0, y1 = _take(y_pos, k), _take(y_pos, k + 1)
    d0, d1 = _take(d, k), _take(d, k + 1)
    w, h = x1 - x0, y1 - y0
    s = h / w
    ww = torch.clamp((y - y0) / h, 0.0, 1.0)
    st = d1 + d0 - 2.0 * s
    c = -s * ww
    b = d0 - st * ww
    a = s - b
    z = torch.clamp(safe_quadratic_root(a, b, c), 0.0, 1.0)
    x = w * z + x0
    sq_z, z1mz, sq_1mz = z * z, z - z * z, (1.0 - z) ** 2
    den = s + st * z1mz
    logdet = -2.0 * torch.log(s) - torch.log(d1 * sq_z + 2.0 * s * z1mz + d0 * sq_1mz) + 2.0 * torch.log(den)
    below, above = y <= y_pos[:, 0], y >= y_pos[:, -1]
    x = torch.where(below, (y - y_pos[:, 0]) / d[:, 0] + x_pos[:, 0], x)
    x = torch.where(above, (y - y_pos[:, -1]) / d[:, -1] + x_pos[:, -1], x)
    logdet = torch.where(below, -torch.log(d[:, 0]), logdet)
    logdet = torch.where(above, -torch.log(d[:, -1]), logdet)
    return x, logdet


def eval_transformed_normal_logpdf(y, params, r0, r1):
    """One spline + shifted/scaled normal (rq_spline_flow.jl:396-418);
    params [n x (3K+3)]: spline parameters, shift, raw scale."""
    return flow_logpdf(y, params, 1, r0, r1)


def flow_logpdf(y, raw, n_layers: int, r0: float, r1: float, K: int | None = None):
    """log p(y) for raw outputs [n x (n_layers (3K+1) + 2)]: n_layers spline
    blocks, then shift and raw scale (further columns are ignored when K is
    given)."""
    L = n_layers
    if K is None:
        K = ((raw.shape[-1] - 2) // L - 1) // 3
    NP = 3 * K + 1
    cur, ldsum = y, torch.zeros_like(y)
    for li in range(L - 1, -1, -1):
        xp, yp, d = constrain_spline_params(raw[:, li * NP:(li + 1) * NP], r0, r1)
        cur, ld = inv_rqs_univariate(xp, yp, d, cur)
        ldsum = ldsum + ld
    shift = raw[:, L * NP]
    scale = torch.sigmoid(torch.clamp(raw[:, L * NP + 1], -SCALE_CLAMP, SCALE_CLAMP)) * 100.0
    u = torch.clamp((cur - shift) / scale, -MAX_U, MAX_U)
    normal = -torch.log(scale) - 0.5 * (math.log(2 * math.pi) + u ** 2)
    return normal + ldsum


def flow_cdf(y, raw, n_layers: int, r0: float, r1: float, K: int):
    """P(T <= y) for raw outputs: the base normal's CDF of the standardised
    inverse-transformed time (every layer and the affine map increase)."""
    L = n_layers
    NP = 3 * K + 1
    cur = y
    for li in range(L - 1, -1, -1):
        xp, yp, d = constrain_spline_params(raw[:, li * NP:(li + 1) * NP], r0, r1)
        cur, _ = inv_rqs_univariate(xp, yp, d, cur)
    shift = raw[:, L * NP]
    scale = torch.sigmoid(torch.clamp(raw[:, L * NP + 1], -SCALE_CLAMP, SCALE_CLAMP)) * 100.0
    return 0.5 * torch.erfc(-((cur - shift) / scale) / math.sqrt(2.0))


def head_loss(raw, tres, nhits, has_time, L: int, K: int, r0: float, r1: float, count_weight=None):
    """Batch-mean loss of raw outputs [B x (L(3K+1)+3)] (log expectation last);
    count_weight multiplies each row's Poisson term (None = 1)."""
    NP = 3 * K + 1
    le = torch.clamp(raw[:, L * NP + 2], -LE_CLAMP, LE_CLAMP)
    n = nhits
    poiss = n * le - torch.exp(le) - torch.lgamma(n + 1.0)
    if count_weight is not None:
        poiss = poiss * count_weight
    lp = flow_logpdf(tres, raw, L, r0, r1, K)
    lp = torch.where(has_time, lp, torch.zeros_like(lp))
    return -(lp.sum() + poiss.sum()) / raw.shape[0]


def bf16_round(t: torch.Tensor) -> torch.Tensor:
    """Round to the nearest bfloat16 (ties to even), kept in float64."""
    return t.to(torch.float32).to(torch.bfloat16).to(DT)


def unpack(theta: np.ndarray, n_pad: int):
    """Flat parameter vector -> [(W, b)] of the four layers (float64 tensors)."""
    dims = [(256, 64), (256, 256), (256, 256), (n_pad, 256)]
    out, off = [], 0
    th = torch.as_tensor(np.asarray(theta, np.float64))
    for r, c in dims:
        W = th[off:off + r * c].reshape(r, c)
        off += r * c
        b = th[off:off + r]
        off += r
        out.append((W, b))
    assert off == th.numel()
    return out


def derived_columns(cond) -> np.ndarray:
    """The conditioner inputs of the derived-column mode: the 5 features
    followed by the distance / 100 m, the source direction's cosine minus
    1/1.35 and its square, and sin(theta_pmt) cos(phi), computed in float32
    from the float32 features (features: log distance over 1-200 m mapped to
    [-1, 1], cos theta_src, cos theta_pmt, azimuth over [0, 2 pi) mapped to
    [-1, 1], log10 E)."""
    f = np.asarray(cond, np.float32)
    one = np.float32(1.0)
    d100 = np.exp((f[:, 0] + one) * np.float32(math.log(200.0) / 2)) * np.float32(0.01)
    c = f[:, 1] + np.float32(1.0 / 1.35)
    s = np.sqrt(np.maximum(one - f[:, 2] * f[:, 2], np.float32(0.0))) * np.cos(np.float32(math.pi) * (f[:, 3] + one))
    return np.concatenate([f, np.stack([d100, c, c * c, s], axis=1)], axis=1).astype(np.float32)


def conditioner(layers, cond: torch.Tensor, bf16: bool = False) -> torch.Tensor:
    """The MLP: cond [n x c] (the c input columns, c <= 64) -> raw outputs
    [n x n_pad].  With bf16 the input, weights and hidden activations are
    rounded to bfloat16 as in the tensor-core path (accumulation stays
    float64)."""
    x = torch.zeros(cond.shape[0], 64, dtype=DT)
    x[:, :cond.shape[1]] = cond
    r = bf16_round if bf16 else (lambda t: t)
    h = r(x)
    for i, (W, b) in enumerate(layers):
        z = h @ r(W).T + b
        if i < 3:
            h = r(torch.relu(z))
        else:
            h = z
    return h


def full_loss(theta: np.ndarray, cond, tres, nhits, has_time, L: int, K: int, r0: float, r1: float,
              n_pad: int, bf16: bool = False, count_weight=None, derived: bool = False):
    """Loss and its gradient by the flat parameters (float64 numpy);
    derived: the conditioner reads derived_columns(cond)."""
    layers = [(W.clone().requires_grad_(True), b.clone().requires_grad_(True)) for W, b in unpack(theta, n_pad)]
    c = torch.as_tensor(np.asarray(derived_columns(cond) if derived else cond, np.float64))
    raw = conditioner(layers, c, bf16=bf16)
    n_out = L * (3 * K + 1) + 3
    loss = head_loss(raw[:, :n_out], torch.as_tensor(np.asarray(tres, np.float64)),
                     torch.as_tensor(np.asarray(nhits, np.float64)),
                     torch.as_tensor(np.asarray(has_time, bool)), L, K, r0, r1,
                     None if count_weight is None else torch.as_tensor(np.asarray(count_weight, np.float64)))
    loss.backward()
    g = np.concatenate([np.concatenate([W.grad.numpy().ravel(), b.grad.numpy().ravel()]) for W, b in layers])
    return float(loss.item()), g


def adam_update(theta, m, v, g, step: int, lr: float, b1: float, b2: float, eps: float):
    """Flux's Adam with bias correction: returns (theta, m, v) after one step."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return theta - lr * mh / (np.sqrt(vh) + eps), m, v
