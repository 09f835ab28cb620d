"""The surrogate path: flow conditions of (event, module, PMT) triples
(ntp_event_conditions) against a numpy computation, the sampler
(ntp_flow_sample) against the flow's own density and count head, sampling
keyed by condition (independent of the batch), and the hybrid simulator's
domain split (flow inside, MC outside)."""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from neutrinotelescopes_gb300 import workloads  # noqa: E402
from neutrinotelescopes_gb300.detection import MultiPMTDetector, make_pom_pmt_coordinates  # noqa: E402
from neutrinotelescopes_gb300.flow import RQNormFlow, RQNormFlowHParams, flow_features  # noqa: E402
from neutrinotelescopes_gb300.lightyield import ExtendedCherenkovEmitter, LongitudinalParameterisation  # noqa: E402
from neutrinotelescopes_gb300.medium import make_simple_water  # noqa: E402
from neutrinotelescopes_gb300.photon_prop import PhotonPropSetup  # noqa: E402
from neutrinotelescopes_gb300.spectrum import InverseSquareSpectrum  # noqa: E402
from neutrinotelescopes_gb300.surrogate import HybridSimulator  # noqa: E402

pytestmark = pytest.mark.gpu


def _cascade(pos, d, e=1e3):
    lp = LongitudinalParameterisation(a=float(np.float32(2.0 + 0.6 * math.log(e))), b=0.63, lrad=0.36)
    return ExtendedCherenkovEmitter(pos, d, 0.0, int(1.3e5 * e), lp)


def _setup():
    coords = make_pom_pmt_coordinates()
    targets = [MultiPMTDetector((x, 0.0, z), 0.21, workloads.PMT_AREA, coords, 1 + i)
               for i, (x, z) in enumerate([(0.0, 0.0), (0.0, 15.0), (0.0, 30.0), (40.0, 0.0), (40.0, 15.0)])]
    return PhotonPropSetup([], targets, make_simple_water(), InverseSquareSpectrum(300.0, 600.0))


def _flow(log_expec: float):
    fl = RQNormFlow(RQNormFlowHParams(batch_size=4096, seed=3))
    fl.init_output_bias(shift=20.0, log_expec=log_expec)
    return fl


def test_event_conditions_match_numpy():
    setup = _setup()
    d = np.array([0.3, -0.5, 0.81])
    d /= np.linalg.norm(d)
    events = [_cascade((5.0, 3.0, 10.0), tuple(d)), _cascade((0.0, 0.2, 15.5), (0.0, 0.0, 1.0)),
              _cascade((300.0, 0.0, 0.0), (1.0, 0.0, 0.0))]
    le = [3.0, 4.5, 2.5]
    with _flow(1.0) as fl:
        sim = HybridSimulator(setup, fl, d_range=(1.0, 200.0))
        cond, key, tgeo, tgt, pmt, first, close = sim.conditions(events, le, [7, 8, 9])
    cond, key, tgeo = cond.cpu().numpy(), key.cpu().numpy(), tgeo.cpu().numpy()
    tgt, pmt = tgt.cpu().numpy(), pmt.cpu().numpy()
    # event 0 sees all 5 modules, event 1 is 0.55 m from module 2 (outside the domain), event 2 is beyond 200 m
    assert list(first) == [0, 80, 144, 144] and list(close) == [0, 1, 0]
    coords = make_pom_pmt_coordinates().astype(np.float32)
    th, ph = coords[0], coords[1]
    axes = np.stack([np.cos(ph) * np.sin(th), np.sin(ph) * np.sin(th), np.cos(th)], -1).astype(np.float64)
    for r in range(len(key)):
        e = 0 if r < 80 else 1
        src = events[e]
        k, j = int(tgt[r]), int(pmt[r]) - 1
        assert key[r] == ((7 + e) << 32) | (k << 8) | j
        u = np.asarray(src.position, np.float64) - np.asarray(setup.targets[k].position)
        dist = np.linalg.norm(u)
        u /= dist
        v = np.asarray(src.direction, np.float64)
        a = axes[j]
        e1, e2 = v - (v @ u) * u, a - (a @ u) * u
        phi = math.atan2(np.cross(e1, e2) @ u, e1 @ e2) % (2 * math.pi)
        want = flow_features([dist], [v @ u], [a @ u], [phi], [le[e]])[0]
        if abs(phi - 2 * math.pi) < 1e-4 or phi < 1e-4:
            want[3] = cond[r, 3]  # the azimuth wraps at 0 / 2 pi
        np.testing.assert_allclose(cond[r], want, atol=2e-5)
        assert tgeo[r] == pytest.approx((dist - 0.21) * 1.35 / 0.299792458, rel=1e-5)


def test_sampler_follows_the_density_and_counts():
    with _flow(math.log(40.0)) as fl:
        n = 2000
        c = np.repeat(np.array([[0.1, -0.3, 0.6, 0.2, -0.1]], np.float32), n, axis=0)
        keys = np.arange(n, dtype=np.uint64) + (np.uint64(5) << np.uint64(32))
        cnt, hc, ht = fl.sample_hits(c, keys, seed=11)
        _, le = fl.logpdf(c[:1], np.zeros(1, np.int32), np.zeros(1, np.float32), log_expec=True)
        lam = math.exp(float(le[0]))
        grid = np.linspace(-200.0, 1700.0, 380001).astype(np.float32)
        lp = fl.logpdf(c[:1], np.zeros(grid.size, np.int32), grid).astype(np.float64)
    cnt = cnt.astype(np.float64)
    assert abs(cnt.mean() - lam) < 5 * math.sqrt(lam / n)
    assert abs(cnt.var() / lam - 1) < 0.15
    assert hc.size == cnt.sum() and np.all(np.diff(hc) >= 0)
    pdf = np.exp(lp)
    cdf = np.concatenate([[0.0], np.cumsum((pdf[1:] + pdf[:-1]) * 0.5 * np.diff(grid))])
    s = np.sort(ht.astype(np.float64))
    F = np.interp(s, grid, cdf / cdf[-1])
    ks = np.max(np.maximum(np.arange(1, s.size + 1) / s.size - F, F - np.arange(s.size) / s.size))
    assert ks < 1.63 / math.sqrt(s.size) + 2e-3, ks   # 1 % level plus grid error


def test_sampling_is_keyed_by_condition():
    with _flow(math.log(8.0)) as fl:
        rng = np.random.default_rng(2)
        c = rng.uniform(-1, 1, (300, 5)).astype(np.float32)
        keys = rng.integers(0, 2 ** 62, 300).astype(np.uint64)
        cnt1, hc1, ht1 = fl.sample_hits(c, keys, seed=4)
        sel = np.arange(100, 200)
        cnt2, hc2, ht2 = fl.sample_hits(c[sel][::-1].copy(), keys[sel][::-1].copy(), seed=4)
    for i_new, i_old in enumerate(sel[::-1]):
        a = ht1[hc1 == i_old]
        b = ht2[hc2 == i_new]
        assert cnt1[i_old] == cnt2[i_new]
        np.testing.assert_array_equal(a, b)


def test_hybrid_domain_split():
    setup = _setup()
    events = [(0, _cascade((5.0, 3.0, 10.0), (0.0, 0.0, 1.0), e=200.0), 2.3),
              (1, _cascade((0.0, 0.3, 15.0), (0.0, 0.0, 1.0), e=200.0), 2.3)]
    with _flow(math.log(3.0)) as fl:
        sim = HybridSimulator(setup, fl)
        out = sim.simulate(events)
    assert [o.method for o in out] == ["flow", "mc"]
    assert out[0].n_hits == int(out[0].time.numel())
    assert np.all(out[0].target.cpu().numpy() < 5) and np.all((out[0].pmt.cpu().numpy() >= 1))


def test_sampled_hits_follow_the_predicted_cdf():
    """The flow's sampled hit times of an event against its own predicted
    hit-time CDF (mixture_cdf over the event's PMTs, weighted by their
    expected counts, offset by the geometric times): one-sample KS at the
    noise level of the sample (99 % bound 1.63 / sqrt(n))."""
    setup = _setup()
    ev = (5, _cascade((5.0, 3.0, 10.0), (0.0, 0.6, 0.8), e=300.0), 2.5)
    with _flow(math.log(40.0)) as fl:
        sim = HybridSimulator(setup, fl, seed=17)
        out = sim.simulate([ev])[0]
        cond, _, tgeo, _, _, _, _ = sim.conditions([ev[1]], [ev[2]], [ev[0]])
        t = torch.sort(out.time.float())[0]
        F = fl.mixture_cdf(cond, t.contiguous(), tgeo + float(ev[1].time)).cpu().numpy()
    n = F.size
    assert out.method == "flow" and n > 2000
    i = np.arange(1, n + 1)
    ks = max(np.max(i / n - F), np.max(F - (i - 1) / n))
    assert ks < 1.63 / math.sqrt(n), (ks, n)


def test_ks_check_hands_later_events_to_mc():
    """A surrogate far from the MC (an untrained flow) fails its first
    check: the check's MC run is oversampled towards ks_min_hits (here up
    to the photon cap, rescaled from the hits of a first run), its distance
    less the MC sample's 95 % noise bound is above the threshold, and every
    later event goes to plain MC."""
    setup = _setup()
    events = [(i, _cascade((5.0, 3.0, 10.0 + i), (0.0, 0.0, 1.0), e=200.0), 2.3) for i in range(3)]
    with _flow(math.log(3.0)) as fl:
        sim = HybridSimulator(setup, fl, ks_check_every=1, ks_threshold=0.1, ks_min_hits=100_000,
                              ks_max_photons=1e10)
        first = sim.simulate(events[:1])
        assert first[0].method == "flow" and len(sim.checks) == 1
        _, ks, n_mc = sim.checks[0]
        assert n_mc >= (1.36 / 0.1) ** 2 and ks - sim.ks_noise_bound(n_mc) > 0.1 and sim.fallback
        later = sim.simulate(events[1:])
    assert [o.method for o in later] == ["mc", "mc"]


def test_sample_resume_after_overflow():
    """A sample whose hits overflow the buffer is drawn by
    ntp_flow_sample_resume into a larger one: the same counts and hits as one
    call with room enough; a resume without a pending sample is refused."""
    import ctypes as C

    from neutrinotelescopes_gb300 import _abi
    rng = np.random.default_rng(8)
    n = 3000
    cond = torch.as_tensor(rng.uniform(-1, 1, (n, 5)).astype(np.float32), device="cuda")
    keys = torch.as_tensor(rng.integers(0, 2 ** 62, n), dtype=torch.int64, device="cuda")
    with _flow(math.log(4.0)) as fl:
        cnt, hc, ht = fl.sample_hits(cond, keys, seed=5, capacity=1 << 20)
        total = int(hc.numel())
        assert total > 1000
        lib, h = fl.lib, fl._h
        n_hits = C.c_uint64()
        cnt2 = torch.empty(n, dtype=torch.int64, device="cuda")
        small = torch.empty(16, dtype=torch.int32, device="cuda"), torch.empty(16, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        st = lib.ntp_flow_sample(h, cond.data_ptr(), n, keys.data_ptr(), 5, cnt2.data_ptr(), small[0].data_ptr(),
                                 small[1].data_ptr(), 16, C.byref(n_hits), 1)
        assert st == _abi.NTP_ERR_OVERFLOW and n_hits.value == total
        assert torch.equal(cnt2, cnt)
        hc2 = torch.empty(total, dtype=torch.int32, device="cuda")
        ht2 = torch.empty(total, dtype=torch.float32, device="cuda")
        st = lib.ntp_flow_sample_resume(h, hc2.data_ptr(), ht2.data_ptr(), total, C.byref(n_hits), 1)
        assert st == _abi.NTP_OK and n_hits.value == total
        assert torch.equal(hc2, hc) and torch.equal(ht2, ht)
        # consumed: a second resume has nothing pending
        st = lib.ntp_flow_sample_resume(h, hc2.data_ptr(), ht2.data_ptr(), total, C.byref(n_hits), 1)
        assert st == _abi.NTP_ERR_NOT_READY
