"""Benchmark of the photon-propagation hot path on one GB300 (or N replicas).

Workload (one step): the cascade_string workload of
neutrinotelescopes_gb300.workloads -- 4 electromagnetic cascades with
energies log-uniform in 1e3-1e5 GeV (fixed by seed, 7.5e9 photons in total),
1.3e5 photons/GeV, gamma longitudinal profile, on a string of 20 POM modules
15 m apart, in water with n = 1.35, group index 1.39, absorption 30 m at
400 nm, scattering 50 m, 0.85 HG(0.97) + 0.15 Rayleigh.  Every step draws a
new Philox key, so each step simulates different photons.

Metric: photons/s (whole job).  Timed on the device with CUDA events per
step; the L2 is flushed (a 512 MB write) between steps, outside the events.
e2e: the same metric through the public call propagate_photons(), host
buffers and all copies included, timed on the host.
"""
from __future__ import annotations

import argparse
import ctypes as C
import gc
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_CASCADES = 4
WORKLOAD_SEED = 1
METRIC = "photons/s"
# Algorithmic lane-operations per photon-step (one scatter segment): one
# Philox4x32-10 block (10 rounds x 6 integer ops + 10 for counter / uniform
# conversion), about 50 FP32 operations for the step length, phase function,
# rotation and position / time update, 5 special-function operations (log,
# sin, cos, sqrt, reciprocal), and 12 FP32 operations for the one geometric
# test a step needs on this detector (the closest approach of the segment to
# the single string; a sphere test only follows when the segment passes within
# a module radius, which is rare enough not to count).
OPS_BASE = 70 + 50 + 5
OPS_PER_GEOMETRY_TEST = 12
# Algorithmic lane-operations of one extended-cascade photon's start (once per
# photon): two Philox4x32-10 blocks (initial uniforms, track smearing) and one
# per gamma attempt (~1 on average), 140 + 70; wavelength and medium-table
# lookup 15; the gamma variate (Box-Muller, Marsaglia-Tsang test) 20; the
# Cherenkov cone 10; the track smearing (log, power, sine, cosine) 15; two
# rotations 40; the position and time along the shower axis 10.
OPS_PHOTON_INIT = 140 + 70 + 15 + 20 + 10 + 15 + 40 + 10


# DRAM traffic of one full-size launch of this workload, from an ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum, one pass, the timed step of
# `bench.py --legs propagation --steps 1 --warmup 1`): 1.20 MB read (the
# medium, spectrum and target tables) and 341.95 MB written for 6092214 hits
# (the 64-byte hit records that leave the L2).  A step's traffic is scaled
# by its hits.
TRAFFIC_READ_BYTES = 1_195_264
TRAFFIC_WRITE_BYTES_PER_HIT = 341_950_720 / 6_092_214


def algo_ops_per_step(n_strings: int) -> int:
    return OPS_BASE + OPS_PER_GEOMETRY_TEST * n_strings


def step_seed(rank: int, i: int) -> int:
    """Philox key of step i on a rank: distinct across ranks and steps, so
    replicas never simulate the same photons."""
    return 0x5EED0000 + 1 + rank * 1_000_003 + i


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="target length of the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--serving-requests", type=int, default=4096,
                    help="requests of the serving measurement (0 = skip)")
    ap.add_argument("--flow", type=int, default=1, help="1: include the flow surrogate measurement")
    ap.add_argument("--legs", default="propagation,serving,flow,hybrid",
                    help="comma list of the measurements to run: propagation (the headline line), serving, flow, "
                         "hybrid; compat (the bench cascades in the reference's own water) and grid (propagation "
                         "on the 10 x 10 string grid), not in the default list, run when propagation is not among "
                         "them")
    ap.add_argument("--details", default=None, help="also write the full per-leg results (JSON) to this path")
    ap.add_argument("--small", action="store_true",
                    help="profiling case: one cascade at 1% of its photons, 64 MB hit buffer, 256 MB L2 flush")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                try:
                    rows.append((float(f[1]), float(f[2]), float(f[3]), f[5], f[6], f[7], f[8]))
                except ValueError:
                    pass
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        pmax = max(r[2] for r in rows)
        loaded = [r for r in rows if r[2] >= 0.5 * pmax] or rows
        reasons = set()
        for r in loaded:
            for name, v in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"), r[3:]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(r[0] for r in loaded), "sm_max_mhz": max(r[1] for r in rows),
                "power_w_max": pmax, "samples": len(loaded), "reasons": sorted(reasons)}


def serving_bench(n_requests: int, budget_bytes: int = 120 * 10 ** 9) -> dict:
    """Serving workload: n_requests cascade events (1e4-1e8 photons, Poisson
    arrivals at 200/s) on the 10 x 10 string detector, through the
    continuous-batching server with a 120 GB hit arena, batches of at most
    2e7 photons and events split into chunks of at most 1e7 photons (so an
    arriving event waits for a short batch, not for a large event).  Two
    passes: all requests at once (throughput, events/s), then the arrivals
    replayed in real time (latency p50 / p99 at 200/s)."""
    import numpy as np
    from neutrinotelescopes_gb300 import workloads
    from neutrinotelescopes_gb300.serving import EventServer
    reqs = workloads.serving_requests(n_requests)
    setup = workloads.serving_setup()
    photons = sum(r[2].photons for r in reqs)
    out = {"workload": f"{n_requests} cascade events, photons log-uniform 1e4-1e8 ({photons:.3g} in total), vertex "
                       "uniform in a 100 m cube, 10 x 10 strings x 20 modules, hits kept on the device",
           "hbm_budget_bytes": budget_bytes}
    # saturated: every request queued at t = 0
    kw = dict(hbm_budget_bytes=budget_bytes, seed=workloads.SEED_BASE + 2, reserve_hits_per_photon=5e-3,
              min_reserve_hits=4096, max_batch_photons=20_000_000, chunk_photons=10_000_000)
    out["server"] = {k: v for k, v in kw.items() if k != "seed"}
    srv = EventServer(setup, **kw)
    for _, eid, src in reqs:
        srv.submit(eid, src)
    t0 = srv.stats().clock
    res = srv.run_all()
    t1 = max(r.t_done for r in res)
    st = srv.stats()
    out["saturated"] = {"events_per_s": len(res) / (t1 - t0), "photons_per_s": photons / (t1 - t0),
                        "batches": st.batches, "reruns": int(sum(r.reruns for r in res)),
                        "hits": int(sum(r.n_hits for r in res)), "seconds": t1 - t0}
    srv.close()
    # real time: arrivals replayed on the server clock, results released on completion
    srv = EventServer(setup, **kw)
    start = srv.stats().clock
    i, lat, done = 0, [], 0
    while done < len(reqs):
        now = srv.stats().clock - start
        while i < len(reqs) and reqs[i][0] <= now:
            srv.submit(reqs[i][1], reqs[i][2])
            i += 1
        wait_us = int(max(0.0, min(1e-3, (reqs[i][0] - now) if i < len(reqs) else 1e-3)) * 1e6)
        for r in srv.poll(wait_us):
            lat.append(r.t_done - r.t_submit)
            srv.release(r.event_id)
            done += 1
    span = srv.stats().clock - start
    lat = np.array(lat)
    out["realtime"] = {"arrival_rate_hz": 200.0, "events_per_s": len(lat) / span,
                       "latency_p50_ms": float(np.percentile(lat, 50) * 1e3),
                       "latency_p99_ms": float(np.percentile(lat, 99) * 1e3),
                       "latency_max_ms": float(lat.max() * 1e3), "batches": srv.stats().batches,
                       "largest_event_ms_at_saturated_rate": 1e3 * max(r[2].photons for r in reqs)
                       / out["saturated"]["photons_per_s"]}
    srv.close()
    setup.close()
    return out


def flow_bench(train_steps: int = 300, n_tuples: int = 100_000_000) -> dict:
    """Flow surrogate workload (5 spline layers of 12 bins on [-20, 1500] ns,
    3 x 256 conditioner, count head, batch 8192, Adam 1e-3):
      table      -- the MC kernel generates a training table of about 2e7
                    rows (65536 simulations, distance 1-200 m log-uniform,
                    direction isotropic, log10 E 2-6, 16 module orientations
                    each) on the device;
      training   -- Adam steps on rows of that table already in HBM, run
                    back to back by one multi-step call;
                    samples/s and the conditioner GEMMs' tensor throughput
                    (algorithmic FLOPs: 3 x forward, forward = 2 x (5 x 256 +
                    2 x 256 x 256 + 256 x 188) per sample);
      inference  -- 1e8 (condition, time) log-pdf tuples over 128000 PMT
                    conditions (8000 modules x 16 PMTs), inputs in HBM; and
                    the same through host buffers (e2e)."""
    import numpy as np
    import torch

    from neutrinotelescopes_gb300.flow import RQNormFlow, RQNormFlowHParams
    from neutrinotelescopes_gb300.tables import TableConfig, make_flow_table

    out = {"model": "5 x RQ spline (12 bins, [-20, 1500] ns) + affine normal + count head, 3 x 256 ReLU "
                    "conditioner on 5 features, BF16 weights / FP32 accumulate and master weights"}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    n_sims = 65536
    tab = make_flow_table(TableConfig(n_sims=n_sims, n_orientations=16, target_hits=300, max_photons=10_000_000,
                                      seed=1))
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    out["table"] = {"simulations": n_sims, "orientations": 16, "rows": len(tab), "photons": tab.n_photons,
                    "seconds": dt, "rows_per_s": len(tab) / dt, "photons_per_s": tab.n_photons / dt}
    bs = 8192
    fl = RQNormFlow(RQNormFlowHParams(batch_size=bs), batch_capacity=131072)
    fl.init_from_table(tab)
    perm = torch.randperm(len(tab), device="cuda")
    cond, tres = tab.cond[perm].contiguous(), tab.tres[perm].contiguous()
    nh, has = tab.nhits[perm].contiguous(), tab.has_time[perm].contiguous()
    torch.cuda.synchronize()
    nb = len(tab) // bs

    def tsteps(first, n):
        # consecutive batches of the shuffled table, one host synchronisation per pass
        done = []
        while len(done) < n:
            b0 = (first + len(done)) % nb
            k = min(n - len(done), nb - b0)
            s = b0 * bs
            done += fl.train_steps(cond[s:], tres[s:], nh[s:], has[s:], bs, k)
        return done

    tsteps(0, 20)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    losses = tsteps(20, train_steps)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    fwd_flops = 2 * (5 * 256 + 2 * 256 * 256 + 256 * 188)
    step_flops = 3 * fwd_flops * bs
    peak = _measured_peak("bf16_tflops_sustained", 1700.0)
    ach = step_flops * train_steps / dt / 1e12
    out["training"] = {"batch": bs, "steps": train_steps, "ms_per_step": dt / train_steps * 1e3,
                       "samples_per_s": bs * train_steps / dt,
                       "loss_first_last": [float(losses[0]), float(np.nanmean(losses[-20:]))],
                       "roofline": {"bound": "tensor", "achieved": ach, "peak": peak[0], "unit": "TFLOP/s",
                                    "frac": ach / peak[0], "peak_source": peak[1],
                                    "flops_per_step": step_flops}}
    # inference: 1e8 (condition, time) log-pdf tuples over 128000 conditions:
    # (a) as a 781-point time grid per condition (the reference's per-module
    # evaluation), (b) as arbitrary (condition index, time) pairs
    n_cond = 8000 * 16
    n_t = n_tuples // n_cond
    g = torch.Generator(device="cuda").manual_seed(5)
    c = (torch.rand((n_cond, 5), device="cuda", generator=g) * 2 - 1).contiguous()
    times = torch.linspace(-20.0, 280.0, n_t, device="cuda")
    fl.logpdf_grid(c[:128], times)
    torch.cuda.synchronize()
    reps = 3
    t0 = time.perf_counter()
    for _ in range(reps):
        lpg = fl.logpdf_grid(c, times)
    torch.cuda.synchronize()
    dt_g = (time.perf_counter() - t0) / reps
    idx = torch.randint(0, n_cond, (n_tuples,), device="cuda", dtype=torch.int32, generator=g)
    idx, _ = torch.sort(idx)
    tt = (torch.rand(n_tuples, device="cuda", generator=g) * 300.0 - 20.0).contiguous()
    fl.logpdf(c, idx[:1000], tt[:1000])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        lp = fl.logpdf(c, idx, tt)
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / reps
    out["inference"] = {"tuples": n_cond * n_t, "conditions": n_cond, "times_per_condition": n_t,
                        "grid_seconds": dt_g, "tuples_per_s": n_cond * n_t / dt_g,
                        "finite": bool(torch.isfinite(lpg).all().item() and torch.isfinite(lp).all().item()),
                        "pairs": {"tuples": n_tuples, "seconds": dt, "tuples_per_s": n_tuples / dt},
                        "note": "times include the conditioner pass over the 128000 conditions"}
    hc, ht = c.cpu().numpy(), times.cpu().numpy()
    t0 = time.perf_counter()
    fl.logpdf_grid(hc, ht)
    dt = time.perf_counter() - t0
    out["inference"]["e2e"] = {"tuples_per_s": n_cond * n_t / dt, "seconds": dt,
                               "h2d_bytes": int(hc.nbytes + ht.nbytes), "d2h_bytes": 4 * n_cond * n_t}
    fl.close()
    del tab, cond, tres, nh, has, c, idx, tt, lp, lpg
    torch.cuda.empty_cache()
    return out


def compat_bench(steps: int = 3, photon_scale: float = 0.25) -> dict:
    """The bench workload's cascades (at photon_scale of their photons) on
    the same 20-module string in the reference's own water: Cascadia Basin
    optics (Quan-Fry dispersion with the reference's coefficients, Kopper
    scattering, STRAW absorption as a per-hit weight, pure Henyey-Greenstein
    with g = 0.99) and its Frank-Tamm spectrum on 300-800 nm as a 30-knot
    texture table.  Device photons/s (CUDA events, L2 flushed between
    steps)."""
    import numpy as np
    import torch

    from neutrinotelescopes_gb300 import _abi, workloads
    from neutrinotelescopes_gb300.detection import string_of_modules
    from neutrinotelescopes_gb300.medium import make_cascadia_medium_properties
    from neutrinotelescopes_gb300.photon_prop import PhotonPropSetup, pack_sources
    from neutrinotelescopes_gb300.spectrum import CherenkovSpectrum

    medium = make_cascadia_medium_properties(0.99)
    srcs = workloads.cascade_sources(N_CASCADES, np.random.default_rng(WORKLOAD_SEED), photon_scale=photon_scale)
    setup = PhotonPropSetup(srcs, string_of_modules(20, 15.0, pmt_area=workloads.PMT_AREA), medium,
                            CherenkovSpectrum((300.0, 800.0), 30, medium))
    lib, ctx = setup.context()
    psrc = pack_sources(setup.sources)
    photons = sum(int(s.photons) for s in setup.sources)
    cap = 1 << 24
    hits = torch.empty((cap, 64), dtype=torch.uint8, device="cuda")
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    opts = setup.prop_opts(stream=stream.cuda_stream)
    nh, ns = C.c_uint64(), C.c_uint64()
    stats = _abi.NtpRunStats()

    def run(seed: int) -> None:
        st = lib.ntp_propagate(ctx, psrc, len(setup.sources), seed, C.byref(opts), hits.data_ptr(), cap, 1,
                               C.byref(nh), C.byref(ns))
        if st != _abi.NTP_OK:
            raise _abi.NtpError(st, lib.ntp_last_error(ctx).decode())

    run(20_000)
    torch.cuda.synchronize()
    ms, photon_steps, n_hits = [], 0, 0
    for i in range(steps):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        run(20_001 + i)
        b.record(stream)
        torch.cuda.synchronize()
        ms.append(a.elapsed_time(b))
        lib.ntp_get_run_stats(ctx, C.byref(stats))
        photon_steps += int(stats.photon_steps)
        n_hits += int(stats.hits)
    setup.close()
    t = sum(ms) / 1e3
    return {"workload": f"{N_CASCADES} EM cascades 1e3-1e5 GeV at {photon_scale} of their photons, 20 POM "
                        "modules; Cascadia Basin water (reference optics, HG g = 0.99), Frank-Tamm spectrum "
                        "300-800 nm (30-knot texture table)",
            "photons_per_step": photons, "steps": steps, "photons_per_s": photons * steps / t,
            "photon_steps_per_photon": photon_steps / (photons * steps), "hits_per_step": n_hits / steps,
            "ms_per_step": 1e3 * t / steps}


def _cosine(lr_max: float, lr_min: float, steps: int):
    return lambda k: lr_min + 0.5 * (lr_max - lr_min) * (1 + math.cos(math.pi * min(k, steps) / steps))


def train_hybrid_models(tab, seed: int, shape_steps: int, count_steps: int, count_members: int = 3):
    """The hybrid simulator's models, trained on one MC table: the
    arrival-time flow (5 spline layers of 12 bins, joint count head with the
    information-weighted count term, the 5 features) and the count model, an
    ensemble of count_members conditioners with derived input columns, each
    trained on the table's (simulation, orientation, PMT) groups alone,
    information-weighted, from its own initialisation and shuffle.  Cosine
    learning-rate schedules from 1e-3 to 1e-5.  The arrival-time flow starts
    from two initialisations and keeps, after ten epochs, the one with the
    lower NLL on held-out rows of the table."""
    from neutrinotelescopes_gb300.flow import CountEnsemble, RQNormFlow, RQNormFlowHParams
    t0 = time.perf_counter()
    per = len(tab) // 8192
    sched = _cosine(1e-3, 1e-5, shape_steps)
    # the time density's NLL on a fixed sample of timed rows (count term
    # off) after every epoch; the parameters of the best epoch are kept, so
    # that a run that degrades late does not end in its degraded state (the
    # training is not bit-reproducible: the weight gradients are summed with
    # floating-point atomics)
    import numpy as np
    import torch
    gen = torch.Generator(device=tab.tres.device)
    gen.manual_seed(97 + seed)
    timed = torch.nonzero(tab.has_time, as_tuple=True)[0]
    vi = timed[torch.randperm(timed.numel(), device=timed.device, generator=gen)[:32768]]
    vc, vt, vh = tab.cond[vi].contiguous(), tab.tres[vi].contiguous(), tab.has_time[vi].contiguous()
    vn, vw = torch.zeros_like(vt), torch.zeros_like(vt)

    def val_nll(f):
        return float(np.mean(f.train_steps(vc, vt, vn, vh, 8192, 4, count_weight=vw, update=False)))

    def train_epoch(f, done, ep):
        f.set_lr(sched(done))
        return done + len(f.fit_table(tab, epochs=1, seed=1000 * seed + ep, max_steps=min(per, shape_steps - done),
                                      count_mode="information"))

    # two initialisations for the first probe_epochs epochs; the one with the
    # lower validation NLL goes on (the quality of a run is mostly set by its
    # start: a run that ends 0.15 nats worse is already behind after ten
    # epochs)
    probe_epochs = 10
    cands = []
    for c in range(2):
        # the batch capacity also sets the chunk of conditions an inference
        # pass takes at once: the hybrid evaluates millions of PMT conditions
        # per batch
        f = RQNormFlow(RQNormFlowHParams(batch_size=8192, seed=31338 + 101 * seed + 7919 * c), batch_capacity=131072)
        f.init_from_table(tab)
        done, hist = 0, []
        for ep in range(probe_epochs):
            if done >= shape_steps:
                break
            done = train_epoch(f, done, ep)
            hist.append(val_nll(f))
        cands.append((min(hist), f, done, hist))
    cands.sort(key=lambda x: x[0])
    for _, f, _, _ in cands[1:]:
        f.close()
    _, fl, done, nll_per_epoch = cands[0]
    probe_nll = [round(min(c[3]), 5) for c in cands]
    best_nll, best_theta = nll_per_epoch[-1], fl.get_params()
    ep = best_ep = len(nll_per_epoch)
    while done < shape_steps:
        done = train_epoch(fl, done, ep)
        ep += 1
        nll = val_nll(fl)
        nll_per_epoch.append(nll)
        if nll < best_nll:
            best_nll, best_theta, best_ep = nll, fl.get_params(), ep
    if best_nll < nll_per_epoch[-1]:
        fl.set_params(best_theta)
    t_shape = time.perf_counter() - t0
    t0 = time.perf_counter()
    import torch
    members = []
    for j in range(count_members):
        cf = RQNormFlow(RQNormFlowHParams(K=10, n_layers=1, range_min=-20.0, range_max=100.0, batch_size=8192,
                                          seed=777 + 101 * seed + 13 * j, input_columns="derived"),
                        batch_capacity=131072)
        cf.init_output_bias(log_expec=float(torch.log1p(tab.group_expec.double()).mean().item()))
        cf.fit_counts(tab, steps=count_steps, seed=100 * seed + j, lr_schedule=_cosine(1e-3, 1e-5, count_steps))
        members.append(cf)
    return fl, CountEnsemble(members), {"seed": seed, "shape_steps": shape_steps, "shape_seconds": t_shape,
                                        "probe_epochs": probe_epochs, "probe_best_nll": probe_nll,
                                        "time_nll_last": nll_per_epoch[-1], "time_nll_best": best_nll,
                                        "best_epoch": best_ep, "epochs": ep,
                                        "time_nll_per_epoch": [round(x, 5) for x in nll_per_epoch],
                                        "count_members": count_members, "count_steps_per_member": count_steps,
                                        "count_seconds": time.perf_counter() - t0}


def grid_bench(steps: int = 3, photon_scale: float = 0.01) -> dict:
    """Propagation on the serving detector's geometry: three EM cascades
    (1e3-1e5 GeV at photon_scale of their photons) 8 m from the centre of a
    10 x 10 grid of strings (50 m apart, 20 POM modules each), simple water;
    hits kept on the device.  Device photons/s (CUDA events, two warm-up
    launches)."""
    import numpy as np
    import torch

    from neutrinotelescopes_gb300 import _abi, workloads
    from neutrinotelescopes_gb300.medium import make_simple_water
    from neutrinotelescopes_gb300.photon_prop import PhotonPropSetup, pack_sources
    from neutrinotelescopes_gb300.spectrum import InverseSquareSpectrum

    srcs = workloads.cascade_sources(3, np.random.default_rng(5), photon_scale=photon_scale, string_z=(0.0, 285.0),
                                     distance=8.0)
    setup = PhotonPropSetup(srcs, workloads.string_grid(10, 10, 50.0, 20, 15.0), make_simple_water(),
                            InverseSquareSpectrum(300.0, 600.0))
    lib, ctx = setup.context()
    psrc = pack_sources(setup.sources)
    photons = sum(int(s.photons) for s in setup.sources)
    cap = 1 << 22
    hits = torch.empty((cap, 64), dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    opts = setup.prop_opts(stream=stream.cuda_stream)
    nh, ns = C.c_uint64(), C.c_uint64()
    ms = []
    for i in range(2 + steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        st = lib.ntp_propagate(ctx, psrc, len(setup.sources), 100 + i, C.byref(opts), hits.data_ptr(), cap, 1,
                               C.byref(nh), C.byref(ns))
        b.record(stream)
        torch.cuda.synchronize()
        if st != _abi.NTP_OK:
            raise _abi.NtpError(st, lib.ntp_last_error(ctx).decode())
        if i >= 2:
            ms.append(a.elapsed_time(b))
    setup.close()
    t = sum(ms) / 1e3
    return {"workload": f"3 EM cascades at {photon_scale} of their photons, 10 x 10 strings x 20 POM modules "
                        "(50 m, 15 m), simple water", "photons_per_step": photons, "steps": steps,
            "photons_per_s": photons * steps / t, "ms_per_step": 1e3 * t / steps, "hits_last_step": int(nh.value)}


def hybrid_bench(n_events: int = 10_000, batch: int = 256, shape_steps: int = 48_000, count_steps: int = 24_000,
                 seeds=(0, 1, 2), eval_per_decade: int = 3, mc_per_decade: int = 2) -> dict:
    """Hybrid serving workload: 10 x 10 strings x 80 POM modules x 16 PMTs
    (50 m, 15 m spacing), n_events cascades with E log-uniform 1e2-1e6 GeV,
    vertex uniform in the detector's bounding box, isotropic direction.  The
    surrogate (an arrival-time flow and a count model, trained here on an MC
    table of 8192 simulations, half of them drawn 8-80 m from the module
    near the Cherenkov angle) supplies every PMT within 1-200 m of the
    vertex; events with a module closer than 1 m go to plain MC.
    Reported: events/s and per-event latency of the saturated stream
    (batches of `batch` events) and of Poisson arrivals at 1000/s; plain
    MC's events/s on the same stream, measured on an energy-stratified sample
    of its events through the MC event server; the error against MC on an
    energy-stratified sample (per-module expected hits, event hit-time KS
    against the surrogate's predicted CDF), for models trained from
    `seeds` (mean and spread over the seeds); the hybrid mode's KS check."""
    import numpy as np
    import torch

    from neutrinotelescopes_gb300 import workloads
    from neutrinotelescopes_gb300.serving import EventServer
    from neutrinotelescopes_gb300.surrogate import (HybridSimulator, evaluate_against, hybrid_events,
                                                    mc_reference)
    from neutrinotelescopes_gb300.tables import TableConfig, make_flow_table

    out = {"workload": f"{n_events} cascades 1e2-1e6 GeV, 10 x 10 strings x 80 modules x 16 PMTs (50 m, 15 m), "
                       "simple water; surrogate for PMTs 1-200 m from the vertex, MC for events with a module "
                       "< 1 m"}
    tcfg = TableConfig(n_sims=8192, n_orientations=16, target_hits=1000, max_photons=100_000_000, seed=2,
                       focus_fraction=0.5)
    t0 = time.perf_counter()
    tab = make_flow_table(tcfg)
    torch.cuda.synchronize()
    out["table"] = {"simulations": tcfg.n_sims, "photons": int(tab.n_photons), "rows": len(tab),
                    "seconds": time.perf_counter() - t0}
    models = [train_hybrid_models(tab, sd, shape_steps, count_steps) for sd in seeds]
    out["training"] = [m[2] for m in models]
    del tab
    torch.cuda.empty_cache()
    setup = workloads.hybrid_setup()
    events = hybrid_events(n_events, setup)
    fl, cf = models[0][0], models[0][1]
    sim = HybridSimulator(setup, fl, count_flow=cf, seed=workloads.SEED_BASE + 4)
    sim.simulate(events[:8])  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lat, n_flow, n_mc, n_hits = [], 0, 0, 0
    for s0 in range(0, n_events, batch):
        res = sim.simulate(events[s0:s0 + batch])
        torch.cuda.synchronize()
        t = time.perf_counter() - t0
        for r in res:
            lat.append(t)
            n_flow += r.method == "flow"
            n_mc += r.method == "mc"
            n_hits += r.n_hits
    dt = time.perf_counter() - t0
    lat = np.array(lat)
    out["saturated"] = {"events_per_s": n_events / dt, "seconds": dt, "events_flow": n_flow, "events_mc": n_mc,
                        "hits": n_hits, "latency_p50_ms": float(np.percentile(lat, 50) * 1e3),
                        "latency_p99_ms": float(np.percentile(lat, 99) * 1e3),
                        "note": "all events queued at t = 0 and served in batches; latency = completion time"}
    # real time: Poisson arrivals at 1000 events/s, each batch the events arrived so far
    rng = np.random.default_rng(9)
    n_rt = min(n_events, 4000)
    arr = np.cumsum(rng.exponential(1e-3, n_rt))
    sim.serve([(float(arr[i]), *events[n_events - 1 - i]) for i in range(200)], max_batch=64)
    gc.collect()
    res_rt = sim.serve([(float(arr[i]), *events[i]) for i in range(n_rt)], max_batch=64)
    lat_rt = np.array([r[2] for r in res_rt])
    out["realtime"] = {"arrival_rate_hz": 1000.0, "events": n_rt,
                       "events_per_s": n_rt / (float(arr[-1]) + lat_rt[-1]),
                       "latency_p50_ms": float(np.percentile(lat_rt, 50) * 1e3),
                       "latency_p99_ms": float(np.percentile(lat_rt, 99) * 1e3),
                       "latency_max_ms": float(lat_rt.max() * 1e3),
                       "events_mc": int(sum(r[1] == "mc" for r in res_rt))}
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    sim.simulate(events[:1])
    torch.cuda.synchronize()
    out["single_event_latency_ms"] = (time.perf_counter() - t1) * 1e3

    # energy strata of the stream (decades of E)
    le_all = np.array([e[2] for e in events])
    edges = [2.0, 3.0, 4.0, 5.0, 6.0 + 1e-9]
    frac = [float(np.mean((le_all >= a) & (le_all < b))) for a, b in zip(edges[:-1], edges[1:])]

    def stratum(k, count, skip=0):
        a, b = edges[k], edges[k + 1]
        return [e for e in events if a <= e[2] < b][skip:skip + count]

    # plain MC serving on the same GPU and detector: per decade the MC event
    # server's time for a few of the stream's events; events/s of the stream
    # = 1 / sum_d (share of decade d) x (mean time of an event of decade d)
    mc_rows, t_mean = [], 0.0
    for k in range(4):
        sample = stratum(k, mc_per_decade)
        srv = EventServer(setup, hbm_budget_bytes=120 * 10 ** 9, seed=workloads.SEED_BASE + 5,
                          reserve_hits_per_photon=2e-3, min_reserve_hits=4096, max_batch_photons=2_000_000_000)
        for e in sample:
            srv.submit(e[0], e[1])
        t_a = srv.stats().clock
        res_mc = srv.run_all()
        mc_dt = max(r.t_done for r in res_mc) - t_a
        srv.close()
        ph = sum(e[1].photons for e in sample)
        per_event = mc_dt / len(sample)
        t_mean += frac[k] * per_event
        mc_rows.append({"log10_energy": [edges[k], round(edges[k + 1], 3)], "events": len(sample),
                        "photons": ph, "seconds_per_event": per_event, "photons_per_s": ph / mc_dt,
                        "stream_share": frac[k]})
    out["plain_mc"] = {"events_per_s": 1.0 / t_mean, "strata": mc_rows,
                       "note": "events/s of the stream from the per-decade mean MC time of its events (MC event "
                               "server, hits kept on the device)"}
    out["speedup_vs_plain_mc"] = out["saturated"]["events_per_s"] / out["plain_mc"]["events_per_s"]

    # error against MC: energy-stratified events, one MC reference each,
    # every trained model judged against the same references
    t1 = time.perf_counter()
    refs = []
    for k in range(4):
        for e in stratum(k, eval_per_decade, skip=mc_per_decade):
            refs.append(mc_reference(sim, e[1], e[2], e[0], seed=workloads.SEED_BASE + 77 + e[0]))
    per_seed = []
    for fl_s, cf_s, _ in models:
        sim_s = HybridSimulator(setup, fl_s, count_flow=cf_s, seed=workloads.SEED_BASE + 4)
        ev = [evaluate_against(sim_s, r) for r in refs]
        errs = np.abs(np.concatenate([v["rel_err"] for v in ev]))
        ks = np.array([v["ks"] for v in ev if v["mc_hits"] > 0])
        eps = np.array([v["ks_noise_bound"] for v in ev if v["mc_hits"] > 0])
        share = np.array([v["top_module_share"] for v in ev if v["mc_hits"] > 0])
        spread = share <= 0.5
        dec = []
        for k in range(4):
            idx = [i for i, r in enumerate(refs) if edges[k] <= r["log10_energy"] < edges[k + 1]]
            e_k = np.abs(np.concatenate([ev[i]["rel_err"] for i in idx])) if idx else np.zeros(0)
            dec.append({"log10_energy": [edges[k], round(edges[k + 1], 3)], "modules": int(e_k.size),
                        "rel_err_median": float(np.median(e_k)) if e_k.size else None,
                        "ks_max": float(np.nanmax([ev[i]["ks"] for i in idx])) if idx else None})
        per_seed.append({"rel_err_median": float(np.median(errs)), "rel_err_p90": float(np.quantile(errs, 0.9)),
                         "modules": int(errs.size),
                         "event_total_rel_err_max": float(np.max(np.abs([v["event_expected_rel_err"] for v in ev]))),
                         "mc_light_outside_domain_max": float(np.max([v["mc_light_outside_domain"] for v in ev])),
                         "ks_median": float(np.median(ks)), "ks_max": float(np.max(ks)),
                         "ks_minus_noise_max": float(np.max(ks - eps)),
                         "ks_max_spread_events": float(np.max(ks[spread])) if spread.any() else None,
                         "ks_max_single_module_events": float(np.max(ks[~spread])) if (~spread).any() else None,
                         "single_module_events": int((~spread).sum()), "decades": dec})
    agg = lambda key: {"mean": float(np.mean([p[key] for p in per_seed])),  # noqa: E731
                       "sd": float(np.std([p[key] for p in per_seed], ddof=1)) if len(per_seed) > 1 else 0.0}
    out["error_vs_mc"] = {
        "events": len(refs), "per_decade": eval_per_decade, "seeds": len(per_seed),
        "rel_err_median": agg("rel_err_median"), "rel_err_p90": agg("rel_err_p90"),
        "ks_median": agg("ks_median"), "ks_max": agg("ks_max"), "ks_minus_noise_max": agg("ks_minus_noise_max"),
        "ks_max_spread_events": agg("ks_max_spread_events") if all(p["ks_max_spread_events"] is not None
                                                                    for p in per_seed) else None,
        "single_module_events": per_seed[0]["single_module_events"],
        "per_seed": per_seed, "seconds": time.perf_counter() - t1,
        "note": "per-module expected hits (count model) against MC where the MC module estimate rests on >= 1e4 "
                "simulated hits (MC noise ~1 %); ks: one-sample KS of the event's MC hit times against the "
                "predicted hit-time CDF (raw distance; ks_minus_noise subtracts the MC sample's 95 % DKW bound); "
                "single-module events: one module holds more than half of the event's MC light, so the event's "
                "KS is that module's"}
    # the hybrid mode's KS check: every 25th flow event also through
    # oversampled MC; plain MC from the first check whose distance, less the
    # MC sample's own 95 % noise bound, is above 0.02
    chk = HybridSimulator(setup, fl, count_flow=cf, seed=workloads.SEED_BASE + 6, ks_check_every=25,
                          ks_threshold=0.02)
    chk_events = [e for e in events if e[2] <= 4.0][:100]
    t1 = time.perf_counter()
    res_chk = []
    for s0 in range(0, len(chk_events), 25):
        res_chk += chk.simulate(chk_events[s0:s0 + 25])
    raw = [float(b) for _, b, _ in chk.checks]
    out["ks_check"] = {"threshold": 0.02, "every": 25, "events": len(chk_events), "confidence": chk.ks_confidence,
                       "checks": len(chk.checks), "ks_raw_max": max(raw) if raw else None,
                       "raw_at_most_threshold": int(sum(r <= 0.02 for r in raw)),
                       "fails_after_noise_bound": int(sum(chk.ks_fails(b, c) for _, b, c in chk.checks)),
                       "fell_back_to_mc": chk.fallback, "events_mc": int(sum(r.method == "mc" for r in res_chk)),
                       "seconds": time.perf_counter() - t1,
                       "note": "a check fails when its raw distance minus the MC sample's 95 % noise bound is above "
                               "the threshold; raw_at_most_threshold counts checks with the raw distance itself "
                               "<= 0.02"}
    setup.close()
    for a, b, _ in models:
        a.close()
        b.close()
    return out


def legs_summary(out: dict) -> dict:
    """The headline numbers of every leg in a few keys, printed last on the
    JSON line so that a tail of the line keeps them."""
    s = {}
    sv = out.get("serving")
    if sv:
        s["serving"] = {"events_per_s": sv["saturated"]["events_per_s"],
                        "p50_ms_at_200hz": sv["realtime"]["latency_p50_ms"],
                        "p99_ms_at_200hz": sv["realtime"]["latency_p99_ms"]}
    fl = out.get("flow")
    if fl:
        s["flow"] = {"table_rows": fl["table"]["rows"], "train_samples_per_s": fl["training"]["samples_per_s"],
                     "train_tflops": fl["training"]["roofline"]["achieved"],
                     "train_frac_of_bf16_sustained": fl["training"]["roofline"]["frac"],
                     "infer_tuples_per_s": fl["inference"]["tuples_per_s"],
                     "infer_e2e_tuples_per_s": fl["inference"]["e2e"]["tuples_per_s"]}
    hy = out.get("hybrid")
    if hy:
        err = hy["error_vs_mc"]
        s["hybrid"] = {"events_per_s": hy["saturated"]["events_per_s"],
                       "p50_ms_at_1000hz": hy["realtime"]["latency_p50_ms"],
                       "p99_ms_at_1000hz": hy["realtime"]["latency_p99_ms"],
                       "plain_mc_events_per_s": hy["plain_mc"]["events_per_s"],
                       "speedup_vs_plain_mc": hy["speedup_vs_plain_mc"],
                       "count_err_median": [err["rel_err_median"]["mean"], err["rel_err_median"]["sd"]],
                       "count_err_p90": [err["rel_err_p90"]["mean"], err["rel_err_p90"]["sd"]],
                       "ks_median": [err["ks_median"]["mean"], err["ks_median"]["sd"]],
                       "ks_max": [err["ks_max"]["mean"], err["ks_max"]["sd"]],
                       "ks_max_spread_events": ([err["ks_max_spread_events"]["mean"],
                                                 err["ks_max_spread_events"]["sd"]]
                                                if err.get("ks_max_spread_events") else None),
                       "seeds": err["seeds"], "events_judged": err["events"],
                       "ks_checks_raw_le_0.02": [hy["ks_check"]["raw_at_most_threshold"], hy["ks_check"]["checks"]]}
    return s


def _measured_peak(key: str, fallback: float):
    try:
        v = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())[key]
        return float(v), f"MEASURED_PEAKS.json {key} (measured)"
    except Exception:
        return fallback, "fallback"


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        import torch
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend)
    return world, rank, local


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if torch.cuda.is_available() and dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def sample_ranges(setup, n: int) -> list[tuple[int, int]]:
    """Photon-index ranges of a bounded sample of n photons spread over every
    source in proportion to its photons (the first photons of each source),
    so that the sample has the workload's mix of cascades."""
    counts = [int(s.photons) for s in setup.sources]
    total = sum(counts)
    out, first = [], 0
    for c in counts:
        k = min(c, int(round(n * c / total))) if total else 0
        if k > 0:
            out.append((first, first + k))
        first += c
    return out


def run_ranges(oracle, setup, seed: int, ranges, threads: int) -> int:
    """The oracle's single-precision port over the ranges; photons simulated."""
    for b, e in ranges:
        oracle.propagate_f32(setup, seed=seed, gid_begin=b, gid_end=e, threads=threads)
    return sum(e - b for b, e in ranges)


def cpu_baseline(setup, seconds: float, threads: int) -> dict:
    """The oracle's single-precision port on the host cores, on a bounded
    sample spread over all of the step's sources."""
    import oracle
    oracle.build()
    total = sum(int(s.photons) for s in setup.sources)
    n = 40_000
    t0 = time.perf_counter()
    n = run_ranges(oracle, setup, 7, sample_ranges(setup, n), threads)
    dt = time.perf_counter() - t0
    n = int(min(total, max(n, n * seconds / max(dt, 1e-6))))
    t0 = time.perf_counter()
    n = run_ranges(oracle, setup, 8, sample_ranges(setup, n), threads)
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"{n} photons of the step's {len(setup.sources)} cascades in proportion to their photons "
                      f"(of {total}), {dt:.1f} s, single-precision oracle port, OpenMP"}


def run_reference(args, world, rank):
    """--impl reference: the reference's step law on the host cores (the
    reference itself is Julia + CUDA.jl and has no CPU path; its restatement in
    oracle/ runs instead), on a bounded sample per step."""
    if rank != 0:
        return
    from neutrinotelescopes_gb300 import workloads
    import oracle
    oracle.build()
    setup = workloads.cascade_string_setup(N_CASCADES, WORKLOAD_SEED)
    threads = os.cpu_count() or 1
    total = sum(int(s.photons) for s in setup.sources)
    t0 = time.perf_counter()
    n = run_ranges(oracle, setup, 1, sample_ranges(setup, 40_000), threads)
    per = (time.perf_counter() - t0) / n
    ranges = sample_ranges(setup, int(min(total, max(n, 5.0 / per))))
    n = sum(e - b for b, e in ranges)
    for i in range(args.warmup):
        run_ranges(oracle, setup, 100 + i, sample_ranges(setup, 40_000), threads)
    times = []
    for i in range(args.steps):
        t0 = time.perf_counter()
        run_ranges(oracle, setup, 1000 + i, ranges, threads)
        times.append(time.perf_counter() - t0)
    value = n * len(times) / sum(times)
    out = {"metric": METRIC, "value": value, "unit": METRIC, "impl": "reference", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic",
           "config": {"workload": "cascade_string: 4 EM cascades 1e3-1e5 GeV, 20 POM modules, simple water",
                      "photons_per_step": n, "sample_of": total},
           "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port",
                            "sample": f"{n} photons per step over the workload's {len(setup.sources)} cascades "
                                      f"in proportion to their photons"},
           "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    args = parse()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    import numpy as np
    import torch

    import neutrinotelescopes_gb300 as nt
    from neutrinotelescopes_gb300 import _abi, workloads
    from neutrinotelescopes_gb300.photon_prop import pack_sources

    torch.cuda.set_device(local)
    legs = set(args.legs.split(","))
    if "propagation" not in legs:
        out = {"metric": METRIC, "value": None, "unit": METRIC, "n_gpus": world, "legs": sorted(legs)}
        if "serving" in legs and args.serving_requests > 0:
            out["serving"] = serving_bench(args.serving_requests)
        if "flow" in legs and args.flow and rank == 0:
            out["flow"] = flow_bench()
        if "hybrid" in legs and rank == 0:
            out["hybrid"] = hybrid_bench()
        if "compat" in legs and rank == 0:
            out["compat_medium"] = compat_bench()
        if "grid" in legs and rank == 0:
            out["string_grid"] = grid_bench()
        if rank == 0:
            if args.details:
                Path(args.details).write_text(json.dumps(out, indent=1))
            out["legs"] = legs_summary(out)
            print(json.dumps(out))
        return
    if args.small:
        setup = workloads.cascade_string_setup(1, WORKLOAD_SEED, photon_scale=0.01, device=local)
    else:
        setup = workloads.cascade_string_setup(N_CASCADES, WORKLOAD_SEED, device=local)
    lib, ctx = setup.context()
    srcs = pack_sources(setup.sources)
    n_src = len(setup.sources)
    photons = sum(int(s.photons) for s in setup.sources)
    cap = 1 << (20 if args.small else 24)
    hits = torch.empty((cap, 64), dtype=torch.uint8, device=f"cuda:{local}")
    flush = torch.empty((256 if args.small else 512) << 20, dtype=torch.uint8, device=f"cuda:{local}")
    stream = torch.cuda.current_stream()
    opts = setup.prop_opts(stream=stream.cuda_stream)
    nh, ns = C.c_uint64(), C.c_uint64()
    stats = _abi.NtpRunStats()

    def step(i: int) -> None:
        seed = step_seed(rank, i)
        st = lib.ntp_propagate(ctx, srcs, n_src, seed, C.byref(opts), hits.data_ptr(), cap, 1, C.byref(nh),
                               C.byref(ns))
        if st != _abi.NTP_OK:
            raise _abi.NtpError(st, lib.ntp_last_error(ctx).decode())

    for i in range(args.warmup):
        step(10_000 + i)
    barrier(world)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    steps_taken, hit_counts = [], []
    with ClockSampler(local) as clk:
        for i in range(args.steps):
            flush.zero_()
            ev[i][0].record(stream)
            step(i)
            ev[i][1].record(stream)
            lib.ntp_get_run_stats(ctx, C.byref(stats))
            steps_taken.append(stats.photon_steps)
            hit_counts.append(stats.hits)
        torch.cuda.synchronize()
    barrier(world)
    ms = [a.elapsed_time(b) for a, b in ev]
    t_dev = max_over_ranks(sum(ms) / 1e3, world)
    value = photons * args.steps * world / t_dev
    clocks = clk.summary()

    # roofline of the propagation kernel: algorithmic lane-ops / kernel time
    n_strings = len({(float(t.position[0]), float(t.position[1])) for t in setup.targets})
    ops_step = algo_ops_per_step(n_strings)
    achieved = (sum(steps_taken) * ops_step + photons * args.steps * OPS_PHOTON_INIT) / (sum(ms) / 1e3) / 1e9
    sm_mhz = clocks.get("sm_mhz") or 2070.0
    peak = 152 * 4 * 32 * sm_mhz * 1e6 / 1e9  # lane-instructions issued per second at the sampled clock
    roofline = {"bound": "issue", "achieved": achieved, "peak": peak, "unit": "Gop/s",
                "frac": achieved / peak,
                "peak_source": f"nominal issue rate 152 SM x 4 schedulers x 32 lanes at the sampled {sm_mhz:.0f} MHz",
                "ops_per_photon_step": ops_step, "ops_per_photon_init": OPS_PHOTON_INIT,
                "photon_steps_per_step": int(statistics.mean(steps_taken)),
                "traffic": None if args.small else
                TRAFFIC_READ_BYTES + TRAFFIC_WRITE_BYTES_PER_HIT * statistics.mean(hit_counts),
                "traffic_unit": "bytes per launch (ncu capture of this workload, scaled by the launch's hits)"}

    # e2e through the public call with host buffers
    e2e_t, e2e_hits = [], []
    for i in range(args.e2e_steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        h = nt.propagate_photons(setup, seed=workloads.SEED_BASE + 500 + i, capacity=cap)
        e2e_t.append(time.perf_counter() - t0)
        e2e_hits.append(len(h))
    e2e_val = photons * len(e2e_t) * world / max_over_ranks(sum(e2e_t), world) if e2e_t else None
    h2d = C.sizeof(_abi.NtpSource) * n_src + 8 * (n_src + 1)
    d2h = int(statistics.mean(e2e_hits)) * 64 + 32 if e2e_hits else 0

    out = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": statistics.mean(ms), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": ("cascade_string (small profiling case: 1 cascade at 1% of its photons)" if args.small
                                   else "cascade_string: 4 EM cascades 1e3-1e5 GeV (7.5e9 photons), 20 POM modules "
                                        "x 16 PMTs on one string, simple water"), "photons_per_step": photons,
                      "hits_per_step": int(statistics.mean(hit_counts)), "l2": "flushed between steps (512 MB write)",
                      "parallelism": f"replicas x{world}"},
           "roofline": roofline, "clocks": clocks,
           "e2e": {"value": e2e_val, "unit": METRIC, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
           "gpu_launches": args.steps}
    setup.close()
    del hits, flush
    torch.cuda.empty_cache()
    if args.serving_requests > 0 and not args.small and "serving" in legs:
        out["serving"] = serving_bench(args.serving_requests)
    if args.flow and not args.small and rank == 0 and "flow" in legs:
        out["flow"] = flow_bench()
    if not args.small and rank == 0 and "hybrid" in legs:
        out["hybrid"] = hybrid_bench()
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(workloads.cascade_string_setup(N_CASCADES, WORKLOAD_SEED),
                                           args.cpu_seconds, os.cpu_count() or 1)
    if rank == 0:
        if args.details:
            Path(args.details).write_text(json.dumps(out, indent=1))
        hy = out.get("hybrid")
        if hy:  # the per-seed breakdowns stay in the details file
            hy["error_vs_mc"] = {k: v for k, v in hy["error_vs_mc"].items() if k != "per_seed"}
            hy["training"] = [{k: v for k, v in t.items() if k != "time_nll_per_epoch"} for t in hy["training"]]
        out["legs"] = legs_summary(out)
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
