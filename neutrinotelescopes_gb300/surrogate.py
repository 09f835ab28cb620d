"""Hybrid event simulation: the flow surrogate for the modules it covers, plain
MC where it does not.

For each event (a cascade), ``ntp_event_conditions`` lists every (module,
PMT) within [d_min, d_max] of the vertex with its flow condition; the flow
draws each PMT's hit count (Poisson of its expectation) and arrival-time
residuals (``ntp_flow_sample``), and the geometric time turns them into hit
times.  Events with a module closer than d_min, or energies outside the
training range, go to plain MC (``propagate_photons`` + ``calc_total_weight``
+ ``resample_simulation`` on the device): plain MC is the fallback outside
the surrogate's training domain.  Modules beyond d_max get no light from the surrogate (200 m is about
7 absorption lengths at 400 nm).

``mc_truth`` runs plain MC for one event and returns per-(module, PMT)
expected hits and the resampled times, the reference point of the error
measures in ``compare``.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math
from dataclasses import dataclass

import numpy as np

from . import _abi
from .flow import RQNormFlow
from .photon_prop import (PhotonPropSetup, _check, calc_total_weight, make_hits_from_photons, pack_sources,
                          propagate_photons, resample_simulation)


def ks_noise_bound(n: int, confidence: float) -> float:
    """eps(n) with P(sup |F_n - F| > eps) <= 1 - confidence for the
    empirical CDF F_n of n samples of F: the Dvoretzky-Kiefer-Wolfowitz
    inequality with Massart's constant, eps = sqrt(ln(2 / (1 - confidence))
    / (2 n)); 0 for confidence 0, infinite without samples."""
    if not 0.0 <= confidence < 1.0:
        raise ValueError(f"confidence must be in [0, 1), got {confidence}")
    if confidence == 0.0:
        return 0.0
    if n <= 0:
        return math.inf
    return math.sqrt(math.log(2.0 / (1.0 - confidence)) / (2.0 * n))


@dataclass
class EventHits:
    event_id: int
    method: str            # "flow" or "mc"
    n_hits: int
    target: object = None  # per hit: target index
    pmt: object = None     # per hit: 1-based PMT
    time: object = None    # per hit: time (ns)


class HybridSimulator:
    """Flow surrogate with an MC fallback on the detector of ``setup``."""

    def __init__(self, setup: PhotonPropSetup, flow: RQNormFlow, *, count_flow=None,
                 d_range=(1.0, 200.0), log10_energy_range=(2.0, 6.0), seed: int = 0, ks_check_every: int = 0,
                 ks_threshold: float = 0.02, ks_min_hits: int = 40_000, ks_max_photons: float = 2e10,
                 ks_confidence: float = 0.95):
        """count_flow: a separate count model (an RQNormFlow trained on the
        counts alone, usually with derived input columns, or a CountEnsemble
        of them; anything with log_expectation(cond)) that supplies every
        PMT's expected hits; the flow then supplies only the arrival times.
        None: the flow's own count head.

        ks_check_every > 0: every that many flow-served events one is also
        simulated with plain MC (``ks_check``): the one-sample
        Kolmogorov-Smirnov distance D of the MC hit times from the flow's
        predicted hit-time distribution of the event.  The MC run is
        oversampled towards ks_min_hits hits (at most ks_max_photons photons)
        so that its own noise stays small next to the threshold.

        D measures the surrogate's distance from the MC's true hit-time
        distribution plus the MC sample's own deviation from it, which the
        Dvoretzky-Kiefer-Wolfowitz inequality bounds by
        eps(n) = sqrt(ln(2 / (1 - ks_confidence)) / (2 n)) with probability
        ks_confidence (0.0068 at 40 000 hits and 95 %).  A check fails when
        D - eps(n) > ks_threshold, i.e. when the surrogate's own distance is
        above the threshold at that confidence, and hands every later event
        to plain MC.  ks_confidence = 0 compares D itself with the
        threshold."""
        self.setup = setup
        self.flow = flow
        self.count_flow = count_flow
        self.d_range = (float(d_range[0]), float(d_range[1]))
        self.e_range = log10_energy_range
        self.seed = int(seed)
        self.ks_check_every = int(ks_check_every)
        self.ks_threshold = float(ks_threshold)
        self.ks_min_hits = int(ks_min_hits)
        self.ks_max_photons = float(ks_max_photons)
        self.ks_confidence = float(ks_confidence)
        if not 0.0 <= self.ks_confidence < 1.0:
            raise ValueError(f"ks_confidence must be in [0, 1), got {ks_confidence}")
        self.fallback = False
        self.checks: list[tuple[int, float, int]] = []   # (event id, KS distance, MC hits)
        self._served = 0
        self.lib, self.ctx = setup.context()
        self.n800 = float(np.float32(np.asarray(setup.medium.refractive_index(np.array([800.0])))[0]))

    def conditions(self, sources, log10_energy, event_ids):
        """Device tensors of the (event, module, PMT) rows, and the per-event
        offsets and close-module counts (host)."""
        import torch
        n = len(sources)
        srcs = pack_sources(sources)
        le = np.ascontiguousarray(log10_energy, np.float32)
        ids = np.ascontiguousarray(event_ids, np.uint32)
        first = np.zeros(n + 1, np.uint64)
        close = np.zeros(n, np.int32)
        n_cond = C.c_uint64()
        dev = f"cuda:{self.setup.device}"
        st = self.lib.ntp_event_conditions(self.ctx, srcs, _abi.fptr(le), ids.ctypes.data, n, self.d_range[0],
                                           self.d_range[1], self.n800, None, None, None, None, None, None, 0,
                                           C.byref(n_cond), first.ctypes.data, close.ctypes.data, None)
        if st not in (_abi.NTP_OK, _abi.NTP_ERR_OVERFLOW):
            _check(self.lib, self.ctx, st)
        m = int(n_cond.value)
        cond = torch.empty((max(m, 1), 5), dtype=torch.float32, device=dev)
        key = torch.empty(max(m, 1), dtype=torch.int64, device=dev)
        tgeo = torch.empty(max(m, 1), dtype=torch.float32, device=dev)
        tgt = torch.empty(max(m, 1), dtype=torch.int32, device=dev)
        pmt = torch.empty(max(m, 1), dtype=torch.int32, device=dev)
        torch.cuda.synchronize()
        if m:
            _check(self.lib, self.ctx, self.lib.ntp_event_conditions(
                self.ctx, srcs, _abi.fptr(le), ids.ctypes.data, n, self.d_range[0], self.d_range[1], self.n800,
                cond.data_ptr(), key.data_ptr(), tgeo.data_ptr(), None, tgt.data_ptr(), pmt.data_ptr(), m,
                C.byref(n_cond), first.ctypes.data, close.ctypes.data, None))
        return cond[:m], key[:m], tgeo[:m], tgt[:m], pmt[:m], first, close

    def log_expectation(self, cond):
        """Per condition (device tensor) the log expected hit count: the
        count model's, or the flow's own count head."""
        return (self.count_flow or self.flow).log_expectation(cond)

    def simulate(self, events) -> list[EventHits]:
        """events: (event_id, source, log10 E) triples, one batch.  Hits stay
        on the device (torch tensors)."""
        import torch
        ids = [int(e[0]) for e in events]
        srcs = [e[1] for e in events]
        le = np.array([float(e[2]) for e in events])
        cond, key, tgeo, tgt, pmt, first, close = self.conditions(srcs, le, ids)
        out: list[EventHits | None] = [None] * len(events)
        in_domain = (close == 0) & (le >= self.e_range[0]) & (le <= self.e_range[1]) & (not self.fallback)
        if cond.shape[0] and in_domain.any():
            le_c = self.count_flow.log_expectation(cond) if self.count_flow is not None else None
            cnt, hc, ht = self.flow.sample_hits(cond, key, seed=self.seed, log_expec=le_c)
            hc64 = hc.long()
            dev = hc.device
            # per hit, once for the batch: target, PMT and time (residual +
            # geometric time + the event's time); each event then takes views
            rows_per_event = torch.as_tensor(np.diff(first.astype(np.int64)), device=dev)
            ev_of_row = torch.repeat_interleave(torch.arange(len(events), device=dev), rows_per_event,
                                                output_size=int(first[-1]))
            ev_time = torch.as_tensor(np.array([s.time for s in srcs], np.float32), device=dev)
            times = ht + tgeo[hc64] + ev_time[ev_of_row[hc64]]
            tgt_h, pmt_h = tgt[hc64], pmt[hc64]
            # hits are grouped by condition, conditions by event
            bounds = torch.searchsorted(hc.contiguous(), torch.as_tensor(first.astype(np.int64), device=dev,
                                                                         dtype=torch.int32))
            b = bounds.cpu().numpy()
            for i in range(len(events)):
                if not in_domain[i]:
                    continue
                sl = slice(int(b[i]), int(b[i + 1]))
                out[i] = EventHits(ids[i], "flow", int(b[i + 1] - b[i]), tgt_h[sl], pmt_h[sl], times[sl])
        for i in range(len(events)):
            if out[i] is None:
                out[i] = self.mc_event(ids[i], srcs[i])
            elif self.ks_check_every > 0:
                self._served += 1
                if self._served % self.ks_check_every == 0:
                    ks, n_mc = self.ks_check(ids[i], srcs[i], float(le[i]))
                    self.checks.append((ids[i], ks, n_mc))
                    if self.ks_fails(ks, n_mc):
                        self.fallback = True
        return out

    def ks_noise_bound(self, n_mc: int) -> float:
        """ks_noise_bound(n_mc, ks_confidence)."""
        return ks_noise_bound(n_mc, self.ks_confidence)

    def ks_fails(self, ks: float, n_mc: int) -> bool:
        """True when a check of distance ks from n_mc MC hits shows the
        surrogate above ks_threshold.  An event without MC hits (n_mc == 0)
        decides nothing; with MC hits, a distance that is not finite (a
        diverged or degenerate flow CDF) is a failure."""
        if n_mc <= 0:
            return False
        return bool(not math.isfinite(ks) or ks - self.ks_noise_bound(n_mc) > self.ks_threshold)

    def ks_check(self, event_id: int, source, log10_energy: float) -> tuple[float, int]:
        """One-sample KS distance of plain-MC hit times (modules in the
        surrogate's domain only) from the flow's predicted hit-time CDF of
        the event (``RQNormFlow.mixture_cdf`` over its PMTs, weighted by
        their expected counts, offset by geometric and event time), and the
        number of MC hits.  The MC run takes k times the source's photons, k
        chosen from the flow's expected hits to reach ks_min_hits, and once
        more from the hits that run gave when it fell short (at most
        ks_max_photons photons)."""
        import torch
        cond, _, tgeo, tgt, _, _, _ = self.conditions([source], [log10_energy], [event_id])
        if cond.shape[0] == 0:
            return float("nan"), 0
        le = self.log_expectation(cond)
        expected = float(torch.exp(le.double()).sum().item())
        k_max = max(1, int(self.ks_max_photons // max(int(source.photons), 1)))
        k = min(max(1, math.ceil(self.ks_min_hits / max(expected, 1e-9))), k_max)
        domain = np.unique(tgt.cpu().numpy())
        for attempt in range(2):
            truth = mc_truth(self.setup, dataclasses.replace(source, photons=int(source.photons) * k),
                             seed=self.seed + 0x4B53 + int(event_id) + attempt)
            keep = np.isin(truth["target"], domain)
            n_got = int(keep.sum())
            k_next = min(max(1, math.ceil(k * self.ks_min_hits / max(n_got, 1))), k_max)
            if n_got >= self.ks_min_hits or k_next <= k:
                break
            k = k_next
        t = np.sort(truth["time"][keep])
        if t.size == 0:
            return float("nan"), 0
        off = tgeo + float(source.time)
        w = torch.exp(le.double()).to(torch.float32) if self.count_flow is not None else None
        F = self.flow.mixture_cdf(cond, torch.as_tensor(t.astype(np.float32), device=cond.device), off, weights=w)
        return ks_distance(F.cpu().numpy()), int(t.size)

    def serve(self, arrivals, *, max_batch: int = 64) -> list[tuple[int, str, float]]:
        """Real-time replay: events (arrival time in s, event_id, source,
        log10 E) are served in arrival order, each batch holding the events
        arrived so far (at most max_batch); returns (event_id, method,
        latency in s) per event."""
        import time as _t

        import torch
        t0 = _t.perf_counter()
        i, out = 0, []
        while i < len(arrivals):
            now = _t.perf_counter() - t0
            if arrivals[i][0] > now:
                _t.sleep(min(arrivals[i][0] - now, 1e-3))
                continue
            j = i
            while j < len(arrivals) and j - i < max_batch and arrivals[j][0] <= now:
                j += 1
            res = self.simulate([(a[1], a[2], a[3]) for a in arrivals[i:j]])
            torch.cuda.synchronize()
            done = _t.perf_counter() - t0
            out.extend((r.event_id, r.method, done - a[0]) for r, a in zip(res, arrivals[i:j]))
            i = j
        return out

    def mc_event(self, event_id: int, source) -> EventHits:
        """Plain MC for one event: propagation, weights and resampling."""
        r = mc_truth(self.setup, source, seed=self.seed + event_id)
        return EventHits(event_id, "mc", len(r["time"]), r["target"], r["pmt"], r["time"])


def ks_distance(cdf_at_sorted: np.ndarray) -> float:
    """One-sample KS distance sup |F_n - F| from the model CDF evaluated at
    the sorted sample; NaN when any CDF value is not finite (a diverged or
    degenerate model), so that the check cannot pass on it."""
    F = np.asarray(cdf_at_sorted, dtype=np.float64)
    n = F.size
    if n == 0 or not np.all(np.isfinite(F)):
        return float("nan")
    i = np.arange(1, n + 1)
    return float(max(np.max(i / n - F), np.max(F - (i - 1) / n)))


def mc_truth(setup: PhotonPropSetup, source, *, seed: int = 0) -> dict:
    """Plain MC of one event on the detector of ``setup``: expected hits per
    (target, PMT) (sum of weights) and the resampled hits (target index, PMT,
    time, time residual)."""
    from .photon_prop import calc_time_residual, pmt_summary
    old = setup.sources
    setup.sources = [source]
    try:
        all_hits = propagate_photons(setup, seed=seed)
        summ = pmt_summary(all_hits, setup, np.eye(3))
        hits = make_hits_from_photons(all_hits, setup, np.eye(3))
        calc_total_weight(hits, setup)
        calc_time_residual(hits, setup)
        r = resample_simulation(hits, setup, seed=seed, time_col="tres")
        t_idx = {int(t.module_id): k for k, t in enumerate(setup.targets)}
        tg = np.array([t_idx[int(m)] for m in r["module_id"]], np.int32)
        rows = hits.records[r["hit_index"].astype(np.int64)] if len(r["hit_index"]) else hits.records[:0]
        return {"expected": summ["weight_sum"], "raw_hits": summ["hit_count"], "target": tg, "pmt": r["pmt_id"],
                "tres": r["tres"], "time": rows["time"].astype(np.float64) if len(rows) else np.zeros(0)}
    finally:
        setup.sources = old


def ks_statistic(a: np.ndarray, b: np.ndarray) -> float:
    """Two-sample Kolmogorov-Smirnov distance."""
    a = np.sort(np.asarray(a, np.float64))
    b = np.sort(np.asarray(b, np.float64))
    if a.size == 0 or b.size == 0:
        return float("nan")
    x = np.concatenate([a, b])
    fa = np.searchsorted(a, x, side="right") / a.size
    fb = np.searchsorted(b, x, side="right") / b.size
    return float(np.max(np.abs(fa - fb)))


def compare(sim: HybridSimulator, source, log10_energy: float, event_id: int, *, seed: int = 0,
            min_hits: int = 100, oversample: int = 1) -> dict:
    """Surrogate against plain MC for one event: per-module expected hits
    (flow count head vs sum of MC weights, from an MC run of `oversample`
    times the event's photons divided by it) and arrival times (two-sample
    KS per module with at least min_hits hits in both, and pooled over the
    event), plus the one-sample KS of an oversampled MC run against the
    flow's predicted hit-time distribution (``HybridSimulator.ks_check``,
    free of the flow sample's noise)."""
    import torch
    k = max(1, int(oversample))
    truth = mc_truth(sim.setup, dataclasses.replace(source, photons=int(source.photons) * k), seed=seed)
    truth["expected"] = truth["expected"] / k
    cond, key, tgeo, tgt, pmt, first, close = sim.conditions([source], [log10_energy], [event_id])
    if cond.shape[0] == 0:
        return {"modules": 0}
    lam = np.exp(sim.log_expectation(cond).double().cpu().numpy())
    tg = tgt.cpu().numpy()
    mod_flow: dict[int, float] = {}
    for k, v in zip(tg, lam):
        mod_flow[int(k)] = mod_flow.get(int(k), 0.0) + float(v)
    exp_mc = truth["expected"].sum(axis=1)
    rel = []
    for k, v in mod_flow.items():
        if exp_mc[k] >= min_hits:
            rel.append(v / exp_mc[k] - 1.0)
    ev = sim.simulate([(event_id, source, log10_energy)])[0]
    ft, fk = ev.time.cpu().numpy(), ev.target.cpu().numpy()
    ks_mod = []
    for k in np.unique(truth["target"]):
        a = truth["time"][truth["target"] == k]
        b = ft[fk == k]
        if a.size >= min_hits and b.size >= min_hits:
            ks_mod.append(ks_statistic(a, b))
    ks_pred, n_pred = sim.ks_check(event_id, source, log10_energy)
    return {"modules": len(rel), "expected_rel_err": np.array(rel), "ks_modules": np.array(ks_mod),
            "ks_pooled": ks_statistic(truth["time"], ft), "mc_hits": int(truth["time"].size),
            "flow_hits": int(ft.size), "method": ev.method,
            "ks_predicted": ks_pred, "ks_predicted_mc_hits": n_pred,
            "ks_predicted_bound": sim.ks_noise_bound(n_pred)}


def mc_reference(sim: HybridSimulator, source, log10_energy: float, event_id: int, *, seed: int = 0,
                 max_photons: float = 1e10, min_raw_hits: int = 400_000) -> dict:
    """Plain-MC reference of one event for judging the surrogate: one MC run
    of f times the event's photons, f chosen (from the surrogate's expected
    hits) for about min_raw_hits simulated hits and at most max_photons
    photons (f < 1 for the brightest events: the expectations are divided by
    f, so they stay unbiased).  Returns the per-(target, PMT) expectations of
    the event and raw simulated hits, and the resampled MC hit times of the
    modules in the surrogate's domain (the sample of the one-sample KS test
    against the surrogate's predicted hit-time CDF).  Independent of the
    surrogate's parameters: one reference serves every trained model."""
    import torch
    cond, _, tgeo, tgt, _, _, _ = sim.conditions([source], [log10_energy], [event_id])
    photons = max(int(source.photons), 1)
    expected = float(torch.exp(sim.log_expectation(cond).double()).sum().item()) if cond.shape[0] else 0.0
    # raw hits per expected hit: the weights (acceptance x absorption) average about 0.1
    f = min(max_photons / photons, max(1.0, min_raw_hits / max(10.0 * expected, 1.0)))
    n_mc = max(1, int(round(photons * f)))
    truth = mc_truth(sim.setup, dataclasses.replace(source, photons=n_mc), seed=seed)
    scale = photons / n_mc
    domain = np.unique(tgt.cpu().numpy()) if cond.shape[0] else np.zeros(0, np.int32)
    keep = np.isin(truth["target"], domain)
    return {"event_id": int(event_id), "log10_energy": float(log10_energy), "photons": photons, "mc_photons": n_mc,
            "expected": truth["expected"] * scale, "raw_hits": truth["raw_hits"],
            "ks_times": np.sort(truth["time"][keep]), "cond": cond, "tgeo": tgeo, "tgt": tgt,
            "time_offset": float(source.time)}


def evaluate_against(sim: HybridSimulator, ref: dict, *, min_raw_hits: int = 10_000) -> dict:
    """The surrogate of `sim` against an MC reference (mc_reference):
    per module in the surrogate's domain (1-200 m from the vertex) the
    relative error of the expected hits (the PMTs' expected counts summed
    over the module) where the MC's module estimate rests on at least
    min_raw_hits simulated hits (relative MC noise about 1 %), the share of
    the event's MC light on modules outside the domain, the share of its
    in-domain MC light on its brightest module, and
    the one-sample KS distance of the MC hit times from the surrogate's
    predicted hit-time CDF of the event with its 95 % DKW noise bound."""
    import torch
    cond = ref["cond"]
    if cond.shape[0] == 0:
        return {"modules": 0, "rel_err": np.zeros(0), "ks": float("nan"), "mc_hits": 0}
    le = sim.log_expectation(cond)
    lam = np.exp(le.double().cpu().numpy())
    tg = ref["tgt"].cpu().numpy()
    flow_mod = np.bincount(tg, weights=lam, minlength=ref["expected"].shape[0])
    mc_mod = ref["expected"].sum(axis=1)
    raw_mod = ref["raw_hits"].sum(axis=1)
    in_domain = np.zeros(mc_mod.shape[0], bool)
    in_domain[np.unique(tg)] = True
    sel = np.flatnonzero(in_domain & (raw_mod >= min_raw_hits) & (mc_mod > 0))
    rel = flow_mod[sel] / mc_mod[sel] - 1.0
    t = ref["ks_times"]
    ks = float("nan")
    if t.size:
        w = torch.exp(le.double()).to(torch.float32)
        F = sim.flow.mixture_cdf(cond, torch.as_tensor(t.astype(np.float32), device=cond.device),
                                 ref["tgeo"] + ref["time_offset"], weights=w)
        ks = ks_distance(F.cpu().numpy())
    return {"modules": int(sel.size), "rel_err": rel, "ks": ks, "mc_hits": int(t.size),
            "ks_noise_bound": ks_noise_bound(int(t.size), 0.95) if t.size else float("inf"),
            "event_expected_rel_err": float(flow_mod.sum() / max(mc_mod[in_domain].sum(), 1e-30) - 1.0),
            "mc_light_outside_domain": float(mc_mod[~in_domain].sum() / max(mc_mod.sum(), 1e-30)),
            "top_module_share": float(mc_mod[in_domain].max() / max(mc_mod[in_domain].sum(), 1e-30))}


def hybrid_events(n: int, setup: PhotonPropSetup, *, seed: int = 4, log10_energy=(2.0, 6.0),
                  photons_per_gev: float = 1.3e5):
    """The hybrid workload: n cascades, E log-uniform, vertex uniform inside
    the detector's bounding box, isotropic direction; (event_id, source,
    log10 E) triples."""
    from .lightyield import ExtendedCherenkovEmitter, LongitudinalParameterisation
    rng = np.random.default_rng(seed)
    pos = np.array([t.position for t in setup.targets], np.float64)
    lo, hi = pos.min(axis=0), pos.max(axis=0)
    out = []
    for i in range(n):
        le = rng.uniform(*log10_energy)
        e = 10 ** le
        ct = rng.uniform(-1, 1)
        ph = rng.uniform(0, 2 * math.pi)
        st = math.sqrt(1 - ct * ct)
        d = (st * math.cos(ph), st * math.sin(ph), ct)
        v = tuple(rng.uniform(lo, hi))
        lp = LongitudinalParameterisation(a=float(np.float32(2.0 + 0.6 * math.log(e))), b=0.63, lrad=0.36)
        out.append((i, ExtendedCherenkovEmitter(v, d, 0.0, int(photons_per_gev * e), lp), le))
    return out
