"""The arrival-time surrogate: RQNormFlow on the GPU (include/ntp.h, ntp_flow_*).

Mirrors src/surrogate_models/extended_cascade_model.jl of
chrhck/NeutrinoTelescopes: ``RQNormFlow`` (:53-101) with its call
``model(x, cond, pred_log_expec)`` (:110-125), ``log_likelihood_with_poisson``
(:132-139), ``RQNormFlowHParams`` (:153-164) and a ``train_model!``-style loop
(:237-295).  The conditioner's GEMMs run on the tensor cores (BF16 weights,
FP32 accumulation), the spline head and Adam in FP32, all in libntp.so.

Conditions are 5 features; ``flow_features`` maps (distance, cos theta of the
source direction, cos theta of the PMT axis, azimuth, energy) to them.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import _abi

N_FEATURES = 5
INPUT_MODES = {"features": _abi.FLOW_INPUT_FEATURES, "derived": _abi.FLOW_INPUT_DERIVED}


def flow_features(distance, cos_theta_src, cos_theta_pmt, phi, log10_energy) -> np.ndarray:
    """Normalised condition features [n x 5] (float32): log-distance over
    1-200 m and log10 E over 2-6 mapped to [-1, 1], the cosines as they are,
    the azimuth over [0, 2 pi) mapped to [-1, 1]."""
    d = np.asarray(distance, np.float64)
    f = np.stack([
        2.0 * (np.log(d) - math.log(1.0)) / (math.log(200.0) - math.log(1.0)) - 1.0,
        np.asarray(cos_theta_src, np.float64),
        np.asarray(cos_theta_pmt, np.float64),
        np.asarray(phi, np.float64) / math.pi - 1.0,
        (np.asarray(log10_energy, np.float64) - 4.0) / 2.0,
    ], axis=-1)
    return np.ascontiguousarray(f, dtype=np.float32)


@dataclass
class RQNormFlowHParams:
    """RQNormFlowHParams (extended_cascade_model.jl:153-164) for this model:
    the MLP is fixed at 3 x 256 and dropout is not applied."""
    K: int = 12
    n_layers: int = 5
    range_min: float = -20.0
    range_max: float = 1500.0
    batch_size: int = 8192
    lr: float = 1e-3
    beta1: float = 0.9
    beta2: float = 0.999
    eps: float = 1e-8
    grad_clip: float = 1e3   # per-sample bound on |dL/draw outputs| x batch size; 0 = none
    count_weight: float = 1.0  # weight of the Poisson count term (1 = log_likelihood_with_poisson)
    seed: int = 31338
    # conditioner inputs: "features" (the 5 condition features) or "derived"
    # (the features plus the distance / 100 m, the source direction's offset
    # from the Cherenkov cosine and its square, sin theta_pmt cos phi; for a
    # count-only model)
    input_columns: str = "features"


def _f32(a, n=None) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    if n is not None and a.shape[0] != n:
        raise ValueError(f"expected {n} rows, got {a.shape[0]}")
    return a


class RQNormFlow:
    """Conditional RQ-spline flow with a log-expectation head on one GPU."""

    def __init__(self, hparams: RQNormFlowHParams | None = None, *, device: int = 0, batch_capacity: int | None = None):
        self.hparams = hp = hparams or RQNormFlowHParams()
        self.lib = _abi.load_library()
        cap = int(batch_capacity or max(hp.batch_size, 128))
        cap = (cap + 127) // 128 * 128
        cfg = _abi.NtpFlowConfig(batch_capacity=cap, n_layers=int(hp.n_layers), n_bins=int(hp.K),
                                 t_min=float(hp.range_min), t_max=float(hp.range_max), lr=float(hp.lr),
                                 beta1=float(hp.beta1), beta2=float(hp.beta2), eps=float(hp.eps),
                                 grad_clip=float(hp.grad_clip), count_weight=float(hp.count_weight),
                                 seed=int(hp.seed) & (2 ** 64 - 1),
                                 input_columns=INPUT_MODES[hp.input_columns])
        h = C.c_void_p()
        st = self.lib.ntp_flow_create(int(device), C.byref(cfg), C.byref(h))
        if st != 0:
            raise _abi.NtpError(st, "ntp_flow_create failed (invalid configuration or CUDA error)")
        self._h = h
        self.batch_capacity = cap
        self._hits_per_cond = 1.0  # sampled hits per condition of the last sample_hits call
        n_params, n_out, n_pad = C.c_uint64(), C.c_int32(), C.c_int32()
        self._check(self.lib.ntp_flow_get_layout(h, C.byref(n_params), C.byref(n_out), C.byref(n_pad)))
        self.n_params, self.n_outputs, self.n_outputs_padded = n_params.value, n_out.value, n_pad.value
        self.K, self.n_layers = hp.K, hp.n_layers
        self.range_min, self.range_max = hp.range_min, hp.range_max

    # ----------------------------------------------------------------- plumbing
    def _check(self, status: int) -> None:
        if status != 0:
            msg = self.lib.ntp_flow_last_error(self._h) if getattr(self, "_h", None) else b""
            raise _abi.NtpError(status, (msg or b"").decode())

    def close(self) -> None:
        if getattr(self, "_h", None):
            self.lib.ntp_flow_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def layout(self) -> list[tuple[str, tuple[int, int], int]]:
        """(name, shape, offset) of each block of the flat parameter vector."""
        dims = [("W1", (256, 64)), ("b1", (256,)), ("W2", (256, 256)), ("b2", (256,)), ("W3", (256, 256)),
                ("b3", (256,)), ("W4", (self.n_outputs_padded, 256)), ("b4", (self.n_outputs_padded,))]
        out, off = [], 0
        for name, shape in dims:
            out.append((name, shape, off))
            off += int(np.prod(shape))
        assert off == self.n_params
        return out

    # -------------------------------------------------------------- parameters
    def get_params(self, which: int = 0) -> np.ndarray:
        """which: 0 weights, 1 gradient of the last step, 2 / 3 Adam moments."""
        out = np.empty(self.n_params, np.float32)
        self._check(self.lib.ntp_flow_get_params(self._h, out.ctypes.data, self.n_params, int(which)))
        return out

    def set_params(self, theta) -> None:
        theta = _f32(theta)
        if theta.size != self.n_params:
            raise ValueError(f"expected {self.n_params} parameters, got {theta.size}")
        self._check(self.lib.ntp_flow_set_params(self._h, theta.ctypes.data, self.n_params))

    def gradient(self) -> np.ndarray:
        return self.get_params(1)

    def set_lr(self, lr: float) -> None:
        """The Adam step size of the following steps (for schedules)."""
        self._check(self.lib.ntp_flow_set_lr(self._h, float(lr)))

    # ---------------------------------------------------------------- training
    def train_step(self, cond, tres, nhits, has_time=None, *, update: bool = True) -> float:
        """One Adam step on a batch (rows a multiple of 128); returns the loss
        of log_likelihood_with_poisson before the step.  Inputs may be numpy
        arrays (host) or CUDA torch tensors (device)."""
        dev = _is_device(cond)
        if dev:
            B = int(cond.shape[0])
            ptrs = [cond.data_ptr(), tres.data_ptr(), nhits.data_ptr(), has_time.data_ptr()]
            keep = None
        else:
            cond = _f32(cond)
            B = cond.shape[0]
            tres, nhits = _f32(tres, B), _f32(nhits, B)
            has_time = np.ones(B, np.int32) if has_time is None else np.ascontiguousarray(has_time, np.int32)
            keep = (cond, tres, nhits, has_time)
            ptrs = [a.ctypes.data for a in keep]
        loss = C.c_double()
        self._check(self.lib.ntp_flow_train_step(self._h, *ptrs, B, int(dev), int(bool(update)), C.byref(loss)))
        del keep
        return loss.value

    def fit(self, cond, tres, nhits, has_time=None, *, epochs: int = 1, batch_size: int | None = None,
            seed: int = 0, max_steps: int | None = None) -> list[float]:
        """train_model! (extended_cascade_model.jl:237-295) without the test
        split and early stopping: shuffled mini-batches over the table, one
        Adam step each; returns the per-step losses.  A ragged last batch is
        dropped (batches are multiples of 128)."""
        cond = _f32(cond)
        n = cond.shape[0]
        tres, nhits = _f32(tres, n), _f32(nhits, n)
        has_time = np.ones(n, np.int32) if has_time is None else np.ascontiguousarray(has_time, np.int32)
        bs = int(batch_size or self.hparams.batch_size)
        bs = max(128, min(bs, self.batch_capacity) // 128 * 128)
        rng = np.random.default_rng(seed)
        losses: list[float] = []
        for _ in range(epochs):
            perm = rng.permutation(n)
            for s in range(0, n - bs + 1, bs):
                idx = perm[s:s + bs]
                losses.append(self.train_step(cond[idx], tres[idx], nhits[idx], has_time[idx]))
                if max_steps is not None and len(losses) >= max_steps:
                    return losses
        return losses

    def init_output_bias(self, *, shift: float | None = None, log_expec: float | None = None) -> None:
        """Sets the output-layer biases of the shift and of the log
        expectation (a start near the data's scale; Adam at lr 1e-3 moves a
        bias by about lr per step)."""
        th = self.get_params()
        off = dict((name, o) for name, _, o in self.layout())["b4"]
        base = self.n_layers * (3 * self.K + 1)
        if shift is not None:
            th[off + base] = shift
        if log_expec is not None:
            th[off + base + 2] = log_expec
        self.set_params(th)

    def init_from_table(self, table) -> None:
        """init_output_bias from a FlowTable: the median time residual of
        its timed rows and the mean of log(N + 1) over its groups (a typical
        count; the counts span many decades)."""
        import torch
        t = table.tres[table.has_time.bool()]
        shift = float(torch.median(t).item()) if t.numel() else 0.0
        log_n = float(torch.log1p(table.group_expec.double()).mean().item())
        self.init_output_bias(shift=shift, log_expec=log_n)

    def fit_table(self, table, *, epochs: int = 1, batch_size: int | None = None, seed: int = 0,
                  max_steps: int | None = None, count_once: bool = False,
                  count_mode: str | None = None) -> list[float]:
        """Trains on a FlowTable held in device memory: the rows are shuffled
        on the device once per epoch and fed to the training step batch by
        batch without leaving the GPU; returns the per-step losses.

        count_mode selects the count term:
          "rows" (the default): the reference's tables, every row carries
            its PMT's drawn count, which weights a PMT by its number of
            rows; for small counts the rows grow with the count itself.
          "once" (or count_once=True): every row's count term weighted by
            1 / (rows of its PMT), so that each PMT's count enters once.
          "information": each PMT once, weighted by the hits simulated for
            it, with its MC expectation as the target
            (FlowTable.information_weights)."""
        import torch
        mode = count_mode or ("once" if count_once else "rows")
        if mode not in ("rows", "once", "information"):
            raise ValueError(f"unknown count_mode {mode!r}")
        n = len(table)
        bs = int(batch_size or self.hparams.batch_size)
        bs = max(128, min(bs, self.batch_capacity) // 128 * 128)
        gen = torch.Generator(device=table.tres.device)
        gen.manual_seed(int(seed))
        cw_all, nh_all = None, table.nhits
        if mode == "once":
            cw_all = table.count_once_weights()
        elif mode == "information":
            cw_all, nh_all = table.information_weights()
        losses: list[float] = []
        for _ in range(epochs):
            perm = torch.randperm(n, device=table.tres.device, generator=gen)
            cond = table.cond[perm].contiguous()
            tres = table.tres[perm].contiguous()
            nh = nh_all[perm].contiguous()
            has = table.has_time[perm].contiguous()
            cw = cw_all[perm].contiguous() if cw_all is not None else None
            torch.cuda.synchronize()
            steps = n // bs
            if max_steps is not None:
                steps = min(steps, max_steps - len(losses))
            if steps > 0:
                losses.extend(self.train_steps(cond, tres, nh, has, bs, steps, count_weight=cw))
            if max_steps is not None and len(losses) >= max_steps:
                return losses
        return losses

    def fit_counts(self, table, *, steps: int, batch_size: int | None = None, seed: int = 0,
                   lr_schedule=None) -> list[float]:
        """Trains the count head alone on a FlowTable's groups (one
        (module orientation, PMT) of one simulation each): the condition, the
        MC expectation as the target and the information weight of the
        group (the hits simulated for it, FlowTable.information_weights), no
        time rows.  For a count-only model next to a shape model; each epoch
        reshuffles the groups on the device.  lr_schedule(step) -> lr, or
        None for the configured rate."""
        import torch
        if table.sim_scale is None:
            raise ValueError("the table needs sim_scale")
        dev = table.group_cond.device
        G = int(table.group_cond.shape[0])
        S = int(table.sim_scale.shape[0])
        c = (1.0 / torch.as_tensor(table.sim_scale, dtype=torch.float64, device=dev)).repeat_interleave(G // S)
        c = (c / c.mean()).to(torch.float32)
        target = table.group_expec.to(torch.float32)
        bs = int(batch_size or self.hparams.batch_size)
        bs = max(128, min(bs, self.batch_capacity) // 128 * 128)
        tres = torch.zeros(G, dtype=torch.float32, device=dev)
        no_time = torch.zeros(G, dtype=torch.int32, device=dev)
        gen = torch.Generator(device=dev)
        gen.manual_seed(int(seed))
        losses: list[float] = []
        per_epoch = G // bs
        chunk = 50
        while len(losses) < steps:
            perm = torch.randperm(G, device=dev, generator=gen)
            cond = table.group_cond[perm].contiguous()
            nh, cw = target[perm].contiguous(), c[perm].contiguous()
            torch.cuda.synchronize()
            done = 0
            while done < per_epoch and len(losses) < steps:
                k = min(chunk, per_epoch - done, steps - len(losses))
                if lr_schedule is not None:
                    self.set_lr(float(lr_schedule(len(losses))))
                r = done * bs
                losses.extend(self.train_steps(cond[r:], tres[r:], nh[r:], no_time[r:], bs, k,
                                               count_weight=cw[r:]))
                done += k
        return losses

    def log_expectation(self, cond):
        """Per condition the log expected hit count of the count head
        (float32; a CUDA tensor for a CUDA input, else numpy)."""
        if _is_device(cond):
            import torch
            n = int(cond.shape[0])
            le = torch.empty(n, dtype=torch.float32, device=cond.device)
            c = cond.to(torch.float32).contiguous()
            self._check(self.lib.ntp_flow_log_expectation(self._h, c.data_ptr(), n, le.data_ptr(), 1))
            return le
        c = _f32(cond)
        le = np.empty(c.shape[0], np.float32)
        self._check(self.lib.ntp_flow_log_expectation(self._h, c.ctypes.data, c.shape[0], le.ctypes.data, 0))
        return le

    def train_steps(self, cond, tres, nhits, has_time, batch: int, steps: int, *, count_weight=None,
                    update: bool = True) -> list[float]:
        """`steps` Adam steps on consecutive batches of `batch` rows of CUDA
        tensors, one synchronisation for all; returns the losses.
        count_weight: per-row factors of the count term (None = 1); update
        False computes loss and gradient only."""
        out = np.empty(steps, np.float64)
        self._check(self.lib.ntp_flow_train_steps(self._h, cond.data_ptr(), tres.data_ptr(), nhits.data_ptr(),
                                                  has_time.data_ptr(),
                                                  count_weight.data_ptr() if count_weight is not None else None,
                                                  int(batch), int(steps), 1, int(bool(update)), out.ctypes.data))
        return out.tolist()

    # --------------------------------------------------------------- inference
    def forward_params(self, cond) -> np.ndarray:
        """The conditioner's raw outputs [n x n_outputs] (spline parameters,
        shift, raw scale, log expectation)."""
        cond = _f32(cond)
        out = np.empty((cond.shape[0], self.n_outputs), np.float32)
        self._check(self.lib.ntp_flow_forward(self._h, cond.ctypes.data, cond.shape[0], out.ctypes.data))
        return out

    def head(self, params, tres, nhits, has_time=None, count_weight=None) -> tuple[float, np.ndarray]:
        """Loss and its gradient by the raw outputs for given raw outputs
        (count_weight: per-row factors of the count term, None = 1)."""
        params = _f32(params)
        B = params.shape[0]
        tres, nhits = _f32(tres, B), _f32(nhits, B)
        has_time = np.ones(B, np.int32) if has_time is None else np.ascontiguousarray(has_time, np.int32)
        cw = None if count_weight is None else _f32(count_weight, B)
        grad = np.empty_like(params)
        loss = C.c_double()
        self._check(self.lib.ntp_flow_head(self._h, params.ctypes.data, tres.ctypes.data, nhits.ctypes.data,
                                           has_time.ctypes.data, cw.ctypes.data if cw is not None else None, B,
                                           C.byref(loss), grad.ctypes.data))
        return loss.value, grad

    def logpdf(self, cond, cond_index, times, *, log_expec: bool = False):
        """log p(t | cond[cond_index]) for each (cond_index, time) pair, and
        optionally the log expectation of every condition."""
        dev = _is_device(cond)
        n_cond = int(cond.shape[0])
        if dev:
            import torch
            n = int(times.numel())
            out = torch.empty(n, dtype=torch.float32, device=times.device)
            le = torch.empty(n_cond, dtype=torch.float32, device=times.device) if log_expec else None
            self._check(self.lib.ntp_flow_evaluate(self._h, cond.data_ptr(), n_cond, cond_index.data_ptr(),
                                                   times.data_ptr(), n, out.data_ptr(),
                                                   le.data_ptr() if le is not None else None, 1))
        else:
            cond = _f32(cond)
            cond_index = np.ascontiguousarray(cond_index, np.int32)
            times = _f32(times)
            n = times.size
            if cond_index.size != n:
                raise ValueError("cond_index and times differ in length")
            out = np.empty(n, np.float32)
            le = np.empty(n_cond, np.float32) if log_expec else None
            self._check(self.lib.ntp_flow_evaluate(self._h, cond.ctypes.data, n_cond, cond_index.ctypes.data,
                                                   times.ctypes.data, n, out.ctypes.data,
                                                   le.ctypes.data if le is not None else None, 0))
        return (out, le) if log_expec else out

    def mixture_cdf(self, cond, times, offsets=None, weights=None):
        """The pooled CDF sum_c w_c F(t - offset_c | cond_c) / sum_c w_c at
        each time (w = the conditions' expected counts unless given): an
        event's predicted hit-time distribution from its PMTs' conditions and
        geometric times.  CUDA tensors in, a float64 CUDA tensor out; or
        numpy in and out."""
        dev = _is_device(cond)
        n_cond = int(cond.shape[0])
        if dev:
            import torch
            n = int(times.numel())
            out = torch.empty(n, dtype=torch.float64, device=times.device)
            ptr = (lambda a: a.data_ptr() if a is not None else None)
            self._check(self.lib.ntp_flow_mixture_cdf(self._h, cond.data_ptr(), n_cond, ptr(weights), ptr(offsets),
                                                      times.data_ptr(), n, out.data_ptr(), 1))
            return out
        cond = _f32(cond)
        times = _f32(times)
        w = None if weights is None else _f32(weights, n_cond)
        o = None if offsets is None else _f32(offsets, n_cond)
        out = np.empty(times.size, np.float64)
        self._check(self.lib.ntp_flow_mixture_cdf(self._h, cond.ctypes.data, n_cond,
                                                  w.ctypes.data if w is not None else None,
                                                  o.ctypes.data if o is not None else None, times.ctypes.data,
                                                  times.size, out.ctypes.data, 0))
        return out

    def logpdf_grid(self, cond, times, *, log_expec: bool = False):
        """log p(times[j] | cond[c]) as an [n_cond x n_times] array (the
        reference's per-module evaluation on a time grid)."""
        dev = _is_device(cond)
        n_cond, n_t = int(cond.shape[0]), int(times.shape[0])
        if dev:
            import torch
            out = torch.empty((n_cond, n_t), dtype=torch.float32, device=cond.device)
            le = torch.empty(n_cond, dtype=torch.float32, device=cond.device) if log_expec else None
            self._check(self.lib.ntp_flow_evaluate_grid(self._h, cond.data_ptr(), n_cond, times.data_ptr(), n_t,
                                                        out.data_ptr(), le.data_ptr() if le is not None else None,
                                                        1))
        else:
            cond, times = _f32(cond), _f32(times)
            out = np.empty((n_cond, n_t), np.float32)
            le = np.empty(n_cond, np.float32) if log_expec else None
            self._check(self.lib.ntp_flow_evaluate_grid(self._h, cond.ctypes.data, n_cond, times.ctypes.data, n_t,
                                                        out.ctypes.data, le.ctypes.data if le is not None else None,
                                                        0))
        return (out, le) if log_expec else out

    MAX_SAMPLE_CONDITIONS = 1 << 20

    def sample_hits(self, cond, keys, seed: int = 0, capacity: int | None = None, log_expec=None):
        """Hits the surrogate predicts: per condition a Poisson count of its
        expectation and that many times drawn from its density.  keys:
        64-bit stream key per condition; log_expec: per condition the log
        expectation to draw the counts from (None = this flow's count head;
        e.g. a separate count model's ``log_expectation``).  Returns
        (counts, hit condition index, hit time) -- numpy arrays, or CUDA
        tensors for CUDA inputs.  More than 2^20 conditions are sampled in
        pieces (the draws are keyed by condition, so the result is the
        same)."""
        n = int(cond.shape[0])
        step = self.MAX_SAMPLE_CONDITIONS
        if n > step:
            parts = [self.sample_hits(cond[s:s + step], keys[s:s + step], seed, capacity,
                                      None if log_expec is None else log_expec[s:s + step])
                     for s in range(0, n, step)]
            if _is_device(cond):
                import torch
                offs = [s for s in range(0, n, step)]
                return (torch.cat([p[0] for p in parts]), torch.cat([p[1] + o for p, o in zip(parts, offs)]),
                        torch.cat([p[2] for p in parts]))
            offs = [s for s in range(0, n, step)]
            return (np.concatenate([p[0] for p in parts]),
                    np.concatenate([p[1] + np.int32(o) for p, o in zip(parts, offs)]),
                    np.concatenate([p[2] for p in parts]))
        dev = _is_device(cond)
        n_hits = C.c_uint64()
        # first buffer: from the hits per condition of the previous call; on
        # an overflow the pending sample is drawn into an exact-size buffer
        # (ntp_flow_sample_resume: no second conditioner pass)
        guess = int(capacity if capacity is not None else max(1 << 16, 1.25 * self._hits_per_cond * n + 4096))
        if dev:
            import torch
            cnt = torch.empty(n, dtype=torch.int64, device=cond.device)
            hc = torch.empty(max(guess, 1), dtype=torch.int32, device=cond.device)
            ht = torch.empty(max(guess, 1), dtype=torch.float32, device=cond.device)
            le = None if log_expec is None else log_expec.to(torch.float32).contiguous()
            torch.cuda.synchronize()
            st = self.lib.ntp_flow_sample_expec(self._h, cond.data_ptr(), n, keys.data_ptr(),
                                                int(seed) & (2 ** 64 - 1), le.data_ptr() if le is not None else None,
                                                cnt.data_ptr(), hc.data_ptr(), ht.data_ptr(), guess, C.byref(n_hits),
                                                1)
            if st == _abi.NTP_ERR_OVERFLOW and capacity is None:
                m = int(n_hits.value)
                hc = torch.empty(m, dtype=torch.int32, device=cond.device)
                ht = torch.empty(m, dtype=torch.float32, device=cond.device)
                torch.cuda.synchronize()
                st = self.lib.ntp_flow_sample_resume(self._h, hc.data_ptr(), ht.data_ptr(), m, C.byref(n_hits), 1)
            self._check(st)
            m = int(n_hits.value)
            self._hits_per_cond = m / max(n, 1)
            return cnt, hc[:m], ht[:m]
        cond = _f32(cond)
        keys = np.ascontiguousarray(keys, np.uint64)
        cnt = np.empty(n, np.uint64)
        hc = np.empty(max(guess, 1), np.int32)
        ht = np.empty(max(guess, 1), np.float32)
        le = None if log_expec is None else _f32(log_expec, n)
        st = self.lib.ntp_flow_sample_expec(self._h, cond.ctypes.data, n, keys.ctypes.data, int(seed) & (2 ** 64 - 1),
                                            le.ctypes.data if le is not None else None, cnt.ctypes.data,
                                            hc.ctypes.data, ht.ctypes.data, guess, C.byref(n_hits), 0)
        if st == _abi.NTP_ERR_OVERFLOW and capacity is None:
            m = int(n_hits.value)
            hc = np.empty(max(m, 1), np.int32)
            ht = np.empty(max(m, 1), np.float32)
            st = self.lib.ntp_flow_sample_resume(self._h, hc.ctypes.data, ht.ctypes.data, m, C.byref(n_hits), 0)
        self._check(st)
        m = int(n_hits.value)
        self._hits_per_cond = m / max(n, 1)
        return cnt, hc[:m], ht[:m]

    def __call__(self, x, cond, pred_log_expec: bool = False):
        """The reference's model call (extended_cascade_model.jl:110-125):
        per sample i the log-pdf of x[i] under cond[i], and with
        pred_log_expec the per-sample log expectation."""
        cond = _f32(cond)
        n = cond.shape[0]
        idx = np.arange(n, dtype=np.int32)
        if pred_log_expec:
            return self.logpdf(cond, idx, _f32(x, n), log_expec=True)
        return self.logpdf(cond, idx, _f32(x, n))


class CountEnsemble:
    """Count models (RQNormFlow, usually trained on the counts alone with
    derived input columns) averaged: the log expectation of a condition is
    the mean of the members' log expectations.  Members trained from
    different initialisations and shuffles err on different conditions, so
    the mean errs less than one member (measured on the hybrid detector:
    1.6 % median per-module error against 1.8-2.1 % for single members)."""

    def __init__(self, members):
        self.members = list(members)
        if not self.members:
            raise ValueError("an ensemble needs at least one member")

    def log_expectation(self, cond):
        les = [m.log_expectation(cond) for m in self.members]
        if _is_device(cond):
            import torch
            return torch.stack(les).mean(0).contiguous()
        return np.mean(np.stack(les), axis=0).astype(np.float32)

    def close(self) -> None:
        for m in self.members:
            m.close()


def log_likelihood_with_poisson(x: dict, model: RQNormFlow) -> float:
    """log_likelihood_with_poisson (extended_cascade_model.jl:132-139):
    -(sum(logpdf(tres)) + sum(Poisson log-likelihood of nhits)) / n."""
    lp, le = model(x["tres"], x["label"], True)
    n = np.asarray(x["nhits"], np.float64)
    le = le.astype(np.float64)
    poiss = n * le - np.exp(le) - np.array([math.lgamma(v + 1.0) for v in n])
    return float(-(lp.astype(np.float64).sum() + poiss.sum()) / len(lp))


def _is_device(a) -> bool:
    return hasattr(a, "is_cuda") and bool(a.is_cuda)
