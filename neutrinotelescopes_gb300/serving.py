"""Continuous-batching event server (include/ntp.h, ntp_server_*).

Requests are single-source events; their hits stay on the device in an arena
of ``hbm_budget_bytes`` until released.  See the header for the admission,
batching and determinism rules.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _abi
from .photon_prop import PhotonPropSetup, _check


@dataclass
class EventResult:
    event_id: int
    status: int
    n_hits: int
    n_photons: int
    hits_ptr: int          # device address of the event's hits (valid until release)
    t_submit: float
    t_launch: float
    t_done: float
    reruns: int
    batch_events: int

    @property
    def latency(self) -> float:
        return self.t_done - self.t_submit


class EventServer:
    """Serving loop over the medium, spectrum and targets of ``setup``.
    chunk_photons > 0 splits events into chunks of at most that many
    photons, one chunk per batch (see ntp_server_config)."""

    def __init__(self, setup: PhotonPropSetup, *, hbm_budget_bytes: int = 1 << 30, seed: int = 0,
                 max_events_per_batch: int = 1024, reserve_hits_per_photon: float = 2e-3,
                 min_reserve_hits: int = 1024, max_batch_photons: int = 4_000_000_000, chunk_photons: int = 0):
        self.lib, ctx = setup.context()
        self.setup = setup
        cfg = _abi.NtpServerConfig(
            hbm_budget_bytes=int(hbm_budget_bytes), seed=int(seed) & (2 ** 64 - 1),
            max_events_per_batch=int(max_events_per_batch), max_steps=setup.max_steps,
            hit_policy=setup.prop_opts().hit_policy, flags=setup.prop_opts().flags,
            reserve_hits_per_photon=float(reserve_hits_per_photon), min_reserve_hits=int(min_reserve_hits),
            max_batch_photons=int(max_batch_photons), chunk_photons=int(chunk_photons))
        self._ctx = ctx
        srv = C.c_void_p()
        _check(self.lib, ctx, self.lib.ntp_server_create(ctx, C.byref(cfg), C.byref(srv)))
        self._srv = srv
        self._buf = (_abi.NtpEventResult * 512)()

    def submit(self, event_id: int, source) -> None:
        rec = source.to_c()
        _check(self.lib, self._ctx, self.lib.ntp_server_submit(self._srv, int(event_id), C.byref(rec)))

    def poll(self, timeout_us: int = 1000, max_results: int = 512) -> list[EventResult]:
        n = self.lib.ntp_server_poll(self._srv, self._buf, min(max_results, len(self._buf)), int(timeout_us))
        if n < 0:
            raise _abi.NtpError(_abi.NTP_ERR_CUDA, self.lib.ntp_last_error(self._ctx).decode())
        return [EventResult(r.event_id, r.status, r.n_hits, r.n_photons, r.hits or 0, r.t_submit, r.t_launch,
                            r.t_done, r.reruns, r.batch_events) for r in self._buf[:n]]

    def hits(self, event_id: int) -> np.ndarray:
        """Host copy of a finished event's hits."""
        n = C.c_uint64()
        _check(self.lib, self._ctx, self.lib.ntp_server_copy_hits(self._srv, int(event_id), None, 0, C.byref(n)))
        out = np.zeros(n.value, dtype=_abi.HIT_DTYPE)
        _check(self.lib, self._ctx, self.lib.ntp_server_copy_hits(self._srv, int(event_id), out.ctypes.data,
                                                                  n.value, C.byref(n)))
        return out

    def release(self, event_id: int) -> None:
        _check(self.lib, self._ctx, self.lib.ntp_server_release(self._srv, int(event_id)))

    def stats(self) -> _abi.NtpServerStats:
        st = _abi.NtpServerStats()
        _check(self.lib, self._ctx, self.lib.ntp_server_get_stats(self._srv, C.byref(st)))
        return st

    def run_all(self, timeout_us: int = 2000) -> list[EventResult]:
        """Polls until every submitted event has finished."""
        out = []
        while True:
            got = self.poll(timeout_us)
            out += got
            st = self.stats()
            if not got and st.queued == 0 and st.running == 0:
                return out

    def close(self) -> None:
        if self._srv is not None:
            self.lib.ntp_server_destroy(self._srv)
            self._srv = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
