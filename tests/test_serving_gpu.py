"""The continuous-batching event server: every event's hits are the same alone
and in any mix (bit-exact: its photons draw from the Philox stream of its
event id), admission respects the HBM budget, reservation overflows re-run
with exact sizes, impossible events are refused."""
import time

import numpy as np
import pytest

import neutrinotelescopes_gb300 as nt
from neutrinotelescopes_gb300 import _abi, workloads
from neutrinotelescopes_gb300.serving import EventServer

pytestmark = pytest.mark.gpu


def detector_setup():
    targets = workloads.string_grid(3, 3, 30.0, 10, 15.0)
    return nt.PhotonPropSetup([], targets, nt.make_simple_water(), nt.InverseSquareSpectrum(300.0, 600.0))


def events(n, seed=0, lo=1e4, hi=4e5):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        photons = int(10 ** rng.uniform(np.log10(lo), np.log10(hi)))
        src = workloads.cascade_sources(1, rng, photon_scale=1.0, distance=6.0, string_z=(0.0, 135.0))[0]
        src.photons = photons
        out.append((1000 + i, src))
    return out


def sorted_hits(h):
    return h[np.lexsort((h["photon_index"], h["source_index"]))]


def run(server, evs):
    for eid, src in evs:
        server.submit(eid, src)
    res = {r.event_id: r for r in server.run_all()}
    hits = {eid: sorted_hits(server.hits(eid)) for eid in res if res[eid].status == _abi.NTP_OK}
    return res, hits


def test_event_hits_same_alone_and_in_mix():
    setup = detector_setup()
    evs = events(24, seed=1)
    mix = EventServer(setup, hbm_budget_bytes=1 << 28, seed=77, max_events_per_batch=8)
    res, hits = run(mix, evs)
    assert len(res) == 24 and all(r.status == _abi.NTP_OK for r in res.values())
    assert sum(len(h) for h in hits.values()) > 200
    assert max(r.batch_events for r in res.values()) > 1
    for eid in (1000, 1007, 1023):
        alone = EventServer(setup, hbm_budget_bytes=1 << 26, seed=77, max_events_per_batch=1)
        r1, h1 = run(alone, [e for e in evs if e[0] == eid])
        assert r1[eid].batch_events == 1
        assert np.array_equal(h1[eid], hits[eid])
        assert np.all(h1[eid]["source_index"] == eid)
        alone.close()
    mix.close()
    setup.close()


def test_admission_within_budget_and_release():
    setup = detector_setup()
    evs = events(40, seed=2)
    # room for about 3 reservations of the largest events at a time
    server = EventServer(setup, hbm_budget_bytes=64 * 3 * 1024, seed=5, max_events_per_batch=16,
                         reserve_hits_per_photon=0.0, min_reserve_hits=1024)
    for eid, src in evs:
        server.submit(eid, src)
    done = {}
    peak = 0
    while len(done) < len(evs):
        for r in server.poll(2000):
            assert r.status == _abi.NTP_OK
            done[r.event_id] = r
            server.release(r.event_id)
        st = server.stats()
        peak = max(peak, st.arena_reserved_hits)
        assert st.arena_reserved_hits <= st.arena_hits
    assert peak <= 3 * 1024
    st = server.stats()
    assert st.released == 40 and st.arena_reserved_hits == 0 and st.batches >= 13
    server.close()
    setup.close()


def test_overflow_reruns_with_exact_size():
    setup = detector_setup()
    evs = events(6, seed=3, lo=1e5, hi=3e5)
    tight = EventServer(setup, hbm_budget_bytes=1 << 26, seed=9, reserve_hits_per_photon=0.0, min_reserve_hits=1)
    r_t, h_t = run(tight, evs)
    ample = EventServer(setup, hbm_budget_bytes=1 << 26, seed=9)
    r_a, h_a = run(ample, evs)
    assert any(r.reruns > 0 for r in r_t.values())
    for eid, _ in evs:
        assert np.array_equal(h_t[eid], h_a[eid])
    tight.close()
    ample.close()
    setup.close()


def test_refuses_impossible_and_duplicate_events():
    setup = detector_setup()
    server = EventServer(setup, hbm_budget_bytes=64 * 100, seed=1, min_reserve_hits=1000)
    (eid, src), = events(1, seed=4)
    server.submit(eid, src)
    with pytest.raises(_abi.NtpError):
        server.submit(eid, src)
    res = server.run_all()
    assert len(res) == 1 and res[0].status == _abi.NTP_ERR_NOMEM
    server.close()
    setup.close()


@pytest.mark.parametrize("chunk,reserve", [(0, 5e-3), (60_000, 5e-3), (60_000, 0.0)])
def test_events_submitted_while_others_run(chunk, reserve):
    """Continuous batching: events arrive while earlier ones are on the GPU
    (submitted between polls whenever the server has events running), with
    large events split into chunks of `chunk` photons (one chunk per batch)
    and, in the last case, reservations so small that every event with hits
    overflows and re-runs.  Each event's hits equal those of the event
    simulated alone, whole and unchunked (bit-exact)."""
    setup = detector_setup()
    evs = events(30, seed=5, lo=3e4, hi=1.5e6)
    srv = EventServer(setup, hbm_budget_bytes=1 << 28, seed=77, max_events_per_batch=8, chunk_photons=chunk,
                      max_batch_photons=1_000_000, reserve_hits_per_photon=reserve, min_reserve_hits=16)
    pending = list(evs)
    got, batch_mix, submitted_while_running = {}, 0, 0
    for _ in range(2):
        srv.submit(*pending.pop(0))
    while len(got) < len(evs):
        # poll without waiting: it launches what it can and returns, so the
        # next submission usually finds a batch on the GPU
        done = srv.poll(0)
        st = srv.stats()
        if pending and (st.running > 0 or st.queued == 0):
            submitted_while_running += st.running > 0
            srv.submit(*pending.pop(0))
        if not done:
            time.sleep(50e-6)
        for r in done:
            assert r.status == _abi.NTP_OK
            got[r.event_id] = (r, sorted_hits(srv.hits(r.event_id)))
            batch_mix = max(batch_mix, r.batch_events)
            srv.release(r.event_id)
    assert submitted_while_running >= 10 and batch_mix > 1
    if reserve == 0.0:
        assert sum(r.reruns > 0 for r, _ in got.values()) >= 10
    assert sum(len(h) for _, h in got.values()) > 500
    alone = EventServer(setup, hbm_budget_bytes=1 << 28, seed=77, max_events_per_batch=1)
    for eid, src in evs:
        r1, h1 = run(alone, [(eid, src)])
        assert r1[eid].batch_events == 1
        assert np.array_equal(h1[eid], got[eid][1]), eid
        alone.release(eid)
    alone.close()
    srv.close()
    setup.close()
