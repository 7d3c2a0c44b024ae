"""Serving: continuous batching of DOS.median requests over resident nodes.

``Server`` wraps ``poyalgn_server_*``: requests of 1..N pairs of store nodes
are queued, batched as execution slots free up, and completed with their
costs and medians. ``poisson_trace`` builds the open-loop request traces that
``Server.replay`` submits at their arrival times.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from .align import CostMatrix, _ptr, check
from .tree import Store


@dataclass
class Reply:
    cost: np.ndarray
    status: np.ndarray
    medians: list        # one array per pair
    latency_s: float


@dataclass
class Trace:
    arrival_s: np.ndarray      # per request, ascending
    npairs: np.ndarray         # per request
    node_a: np.ndarray         # per pair, requests in order
    node_b: np.ndarray

    @property
    def nreq(self) -> int:
        return len(self.arrival_s)


@dataclass
class ReplayResult:
    cost: np.ndarray           # per pair
    status: np.ndarray         # per pair; 1 = request refused by admission control
    latency_s: np.ndarray      # per request; -1 = refused
    wall_s: float

    def served(self) -> np.ndarray:
        return self.latency_s >= 0


def poisson_trace(rng: np.random.Generator, rate: float, nreq: int, pool_a, pool_b,
                  max_pairs: int = 64) -> Trace:
    """Poisson arrivals at `rate` requests/s, U{1..max_pairs} pairs per
    request drawn uniformly from the pool of node pairs (pool_a[i], pool_b[i])."""
    gaps = rng.exponential(1.0 / rate, nreq)
    arrival = np.cumsum(gaps) - gaps[0]
    npairs = rng.integers(1, max_pairs + 1, nreq).astype(np.int32)
    pick = rng.integers(0, len(pool_a), int(npairs.sum()))
    return Trace(arrival, npairs, np.asarray(pool_a, np.int32)[pick],
                 np.asarray(pool_b, np.int32)[pick])


MEDIAN, DISTANCE = 0, 1   # POYALGN_SERVE_*


class Server:
    """kind MEDIAN serves DOS.median (cost and median per pair), DISTANCE
    serves DOS.distance (cost only; missing_distance for all-gap pairs)."""

    def __init__(self, store: Store, cm: CostMatrix, nslots: int = 3,
                 max_batch_pairs: int = 4096, max_waiting_pairs: int = 65536,
                 hbm_budget: int = 16 << 30, kind: int = MEDIAN, missing_distance: int = 0):
        self.store = store
        self.cm = cm
        self.kind = kind
        h = C.c_void_p()
        check(_lib.load().poyalgn_server_create(store.handle, cm.handle, int(kind),
                                                int(missing_distance), nslots,
                                                max_batch_pairs, max_waiting_pairs,
                                                int(hbm_budget), C.byref(h)))
        self._h = h
        self._pending = {}

    def submit(self, node_a, node_b) -> int:
        na = np.ascontiguousarray(node_a, np.int32)
        nb = np.ascontiguousarray(node_b, np.int32)
        t = C.c_int64()
        check(_lib.load().poyalgn_server_submit(self._h, len(na), _ptr(na), _ptr(nb),
                                                C.byref(t)))
        lib = _lib.load()
        cap = sum(lib.poyalgn_store_length(self.store.handle, int(x)) +
                  lib.poyalgn_store_length(self.store.handle, int(y)) + 2
                  for x, y in zip(na, nb))
        self._pending[t.value] = (len(na), cap)
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1) -> Reply:
        npairs, cap = self._pending[ticket]
        cost, status, mlen = (np.zeros(npairs, np.int32) for _ in range(3))
        med = np.zeros(cap, np.uint8)
        lat = C.c_double()
        check(_lib.load().poyalgn_server_wait(self._h, ticket, timeout_ms, _ptr(cost),
                                              _ptr(status), _ptr(mlen), _ptr(med), cap,
                                              C.byref(lat)))
        del self._pending[ticket]
        ends = np.cumsum(mlen)
        meds = [med[e - n:e].copy() for e, n in zip(ends, mlen)]
        return Reply(cost, status, meds, lat.value)

    def replay(self, trace: Trace) -> ReplayResult:
        n = len(trace.node_a)
        cost = np.zeros(n, np.int32)
        status = np.zeros(n, np.int32)
        lat = np.zeros(trace.nreq, np.float64)
        wall = C.c_double()
        arr = np.ascontiguousarray(trace.arrival_s, np.float64)
        check(_lib.load().poyalgn_server_replay(
            self._h, trace.nreq, _ptr(arr), _ptr(trace.npairs), _ptr(trace.node_a),
            _ptr(trace.node_b), _ptr(cost), _ptr(status), _ptr(lat), C.byref(wall)))
        return ReplayResult(cost, status, lat, wall.value)

    def stats(self) -> dict:
        b, p, r = C.c_int64(), C.c_int64(), C.c_int64()
        check(_lib.load().poyalgn_server_stats(self._h, C.byref(b), C.byref(p), C.byref(r)))
        return {"batches": b.value, "pairs": p.value, "refused": r.value}

    def close(self):
        if self._h:
            _lib.load().poyalgn_server_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
