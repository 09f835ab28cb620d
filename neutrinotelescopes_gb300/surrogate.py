"""Hybrid event simulation: the flow surrogate for the modules it covers, plain
MC where it does not.

For each event (a cascade), ``ntp_event_conditions`` lists every (module,
PMT) within [d_min, d_max] of the vertex with its flow condition; the flow
draws each PMT's hit count (Poisson of its expectation) and arrival-time
residuals (``ntp_flow_sample``), and the geometric time turns them into hit
times.  Events with a module closer than d_min, or energies outside the
training range, go to plain MC (``propagate_photons`` + ``calc_total_weight``
+ ``resample_simulation`` on the device), as the benchmark spec's hybrid mode
asks.  Modules beyond d_max get no light from the surrogate (200 m is about
7 absorption lengths at 400 nm).

``mc_truth`` runs plain MC for one event and returns per-(module, PMT)
expected hits and the resampled times, the reference point of the error
measures in ``compare``.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import _abi
from .flow import RQNormFlow
from .photon_prop import (PhotonPropSetup, _check, calc_total_weight, make_hits_from_photons, pack_sources,
                          propagate_photons, resample_simulation)


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

    def __init__(self, setup: PhotonPropSetup, flow: RQNormFlow, *, d_range=(1.0, 200.0),
                 log10_energy_range=(2.0, 6.0), seed: int = 0, ks_check_every: int = 0,
                 ks_threshold: float = 0.02):
        """ks_check_every > 0: every that many flow-served events one is also
        simulated with plain MC and the two hit-time samples compared (KS,
        pooled over the event); a KS above ks_threshold hands every later
        event to plain MC."""
        self.setup = setup
        self.flow = flow
        self.d_range = (float(d_range[0]), float(d_range[1]))
        self.e_range = log10_energy_range
        self.seed = int(seed)
        self.ks_check_every = int(ks_check_every)
        self.ks_threshold = float(ks_threshold)
        self.fallback = False
        self.checks: list[tuple[int, float]] = []
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
            cnt, hc, ht = self.flow.sample_hits(cond, key, seed=self.seed)
            hc64 = hc.long()
            times = ht + tgeo[hc64]
            ev_time = torch.as_tensor(np.array([s.time for s in srcs], np.float32), device=times.device)
            # hits are grouped by condition, conditions by event
            bounds = torch.searchsorted(hc.contiguous(), torch.as_tensor(first.astype(np.int64), device=hc.device,
                                                                         dtype=torch.int32))
            b = bounds.cpu().numpy()
            for i in range(len(events)):
                if not in_domain[i]:
                    continue
                sl = slice(int(b[i]), int(b[i + 1]))
                out[i] = EventHits(ids[i], "flow", int(b[i + 1] - b[i]), tgt[hc64[sl]], pmt[hc64[sl]],
                                   times[sl] + ev_time[i])
        for i in range(len(events)):
            if out[i] is None:
                out[i] = self.mc_event(ids[i], srcs[i])
            elif self.ks_check_every > 0:
                self._served += 1
                if self._served % self.ks_check_every == 0:
                    mc = self.mc_event(ids[i], srcs[i])
                    ks = ks_statistic(mc.time, out[i].time.cpu().numpy())
                    self.checks.append((ids[i], ks))
                    if not (ks <= self.ks_threshold):
                        self.fallback = True
        return out

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
        return {"expected": summ["weight_sum"], "target": tg, "pmt": r["pmt_id"], "tres": r["tres"],
                "time": rows["time"].astype(np.float64) if len(rows) else np.zeros(0)}
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
            min_hits: int = 100) -> dict:
    """Surrogate against plain MC for one event: per-module expected hits
    (flow count head vs sum of MC weights) and arrival times (KS per module
    with at least min_hits hits in both, and pooled over the event)."""
    import torch
    truth = mc_truth(sim.setup, source, seed=seed)
    cond, key, tgeo, tgt, pmt, first, close = sim.conditions([source], [log10_energy], [event_id])
    if cond.shape[0] == 0:
        return {"modules": 0}
    idx = torch.zeros(1, dtype=torch.int32, device=cond.device)
    _, le = sim.flow.logpdf(cond, idx, torch.zeros(1, dtype=torch.float32, device=cond.device), log_expec=True)
    lam = np.exp(le.double().cpu().numpy())
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
    return {"modules": len(rel), "expected_rel_err": np.array(rel), "ks_modules": np.array(ks_mod),
            "ks_pooled": ks_statistic(truth["time"], ft), "mc_hits": int(truth["time"].size),
            "flow_hits": int(ft.size), "method": ev.method}


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
