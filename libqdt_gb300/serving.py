"""Serving: the request loop of the GB300 library (qdtg_server_* in
qdt_gpu.h) and an open-loop driver that measures it.

The scheduler itself is native (csrc/server.cu): worker threads that own
resident GPU engines, a batching thread that coalesces small requests into
one many-set call, admission under an HBM budget. This module binds it and
adds `run_open_loop`, which submits a request stream at its arrival times
(a Poisson process) from a separate thread, waits for every result and
reports latency percentiles, throughput and the rejected/queued counts.
Latency is counted from each request's scheduled arrival, so a submitter
that falls behind adds to it (the open-loop convention).
"""
from __future__ import annotations

import ctypes
import threading
import time

import numpy as np

from . import load
from .qdt_api import QDT_OK

SERVER_SYMBOLS = ("qdtg_server_default_config", "qdtg_server_create", "qdtg_server_destroy", "qdtg_server_submit",
                  "qdtg_server_wait", "qdtg_server_result", "qdtg_server_timing", "qdtg_server_release",
                  "qdtg_server_get_stats")


class ServerConfig(ctypes.Structure):
    _fields_ = [
        ("hbm_budget_bytes", ctypes.c_size_t),
        ("large_workers", ctypes.c_int),
        ("small_threshold", ctypes.c_size_t),
        ("batch_max_points", ctypes.c_size_t),
        ("batch_max_sets", ctypes.c_size_t),
        ("max_queue", ctypes.c_size_t),
        ("cell_points", ctypes.c_int),
        ("batch_cell_points", ctypes.c_int),
    ]


class ServerStats(ctypes.Structure):
    _fields_ = [
        ("submitted", ctypes.c_ulonglong), ("completed", ctypes.c_ulonglong), ("rejected", ctypes.c_ulonglong),
        ("queued", ctypes.c_ulonglong), ("batches", ctypes.c_ulonglong), ("batched_requests", ctypes.c_ulonglong),
        ("pool_releases", ctypes.c_ulonglong),
        ("resident_bytes", ctypes.c_size_t), ("peak_resident_bytes", ctypes.c_size_t),
        ("hbm_budget_bytes", ctypes.c_size_t), ("waiting", ctypes.c_size_t),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


def bind(lib: ctypes.CDLL) -> ctypes.CDLL:
    P = ctypes.c_void_p
    S = ctypes.c_size_t
    U64 = ctypes.c_uint64
    D = ctypes.c_double
    for name, args, res in (
            ("qdtg_server_default_config", [ctypes.POINTER(ServerConfig)], None),
            ("qdtg_server_create", [ctypes.POINTER(ServerConfig)], P),
            ("qdtg_server_destroy", [P], None),
            ("qdtg_server_submit", [P, P, S, ctypes.POINTER(U64)], ctypes.c_int),
            ("qdtg_server_wait", [P, U64, D], ctypes.c_int),
            ("qdtg_server_result", [P, U64, ctypes.POINTER(P), ctypes.POINTER(S), ctypes.POINTER(P),
                                    ctypes.POINTER(S)], ctypes.c_int),
            ("qdtg_server_timing", [P, U64, ctypes.POINTER(D), ctypes.POINTER(D), ctypes.POINTER(D),
                                    ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
            ("qdtg_server_release", [P, U64], ctypes.c_int),
            ("qdtg_server_get_stats", [P, ctypes.POINTER(ServerStats)], None)):
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    return lib


def default_config(lib=None) -> ServerConfig:
    lib = bind(lib or load())
    c = ServerConfig()
    lib.qdtg_server_default_config(ctypes.byref(c))
    return c


class Server:
    """A qdtg_server. submit() keeps the points array alive until the
    request's result has been taken (result()) or released."""

    def __init__(self, lib: ctypes.CDLL | None = None, **config):
        self.lib = bind(lib or load())
        c = default_config(self.lib)
        for k, v in config.items():
            setattr(c, k, v)
        self.config = c
        self.ptr = self.lib.qdtg_server_create(ctypes.byref(c))
        if not self.ptr:
            raise RuntimeError("qdtg_server_create failed")
        self._keep = {}
        self._lock = threading.Lock()

    def close(self):
        if self.ptr:
            self.lib.qdtg_server_destroy(self.ptr)
            self.ptr = None
            self._keep.clear()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def submit(self, pts) -> tuple[int, int]:
        """Returns (status, ticket)."""
        p = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 2)
        t = ctypes.c_uint64(0)
        st = self.lib.qdtg_server_submit(self.ptr, p.ctypes.data if p.size else None, p.shape[0], ctypes.byref(t))
        if t.value:
            with self._lock:
                self._keep[t.value] = p
        return st, t.value

    def wait(self, ticket: int, timeout: float = -1.0) -> bool:
        return self.lib.qdtg_server_wait(self.ptr, ticket, timeout) == 1

    def result(self, ticket: int, release: bool = True):
        """(status, triangles (k, 3) uint32, rep (n,) uint32, distinct count)."""
        tp, rp = ctypes.c_void_p(0), ctypes.c_void_p(0)
        nt, nu = ctypes.c_size_t(0), ctypes.c_size_t(0)
        st = self.lib.qdtg_server_result(self.ptr, ticket, ctypes.byref(tp), ctypes.byref(nt), ctypes.byref(rp),
                                         ctypes.byref(nu))
        with self._lock:
            n = self._keep[ticket].shape[0] if ticket in self._keep else 0
        tris = np.zeros((0, 3), np.uint32)
        rep = np.zeros(0, np.uint32)
        if st == QDT_OK:
            if nt.value and tp.value:
                tris = np.ctypeslib.as_array((ctypes.c_uint32 * (3 * nt.value)).from_address(tp.value)).reshape(
                    -1, 3).copy()
            if n and rp.value:
                rep = np.ctypeslib.as_array((ctypes.c_uint32 * n).from_address(rp.value)).copy()
        if release:
            self.release(ticket)
        return st, tris, rep, nu.value

    def timing(self, ticket: int):
        q, r, t, path = ctypes.c_double(), ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
        ok = self.lib.qdtg_server_timing(self.ptr, ticket, ctypes.byref(q), ctypes.byref(r), ctypes.byref(t),
                                         ctypes.byref(path))
        return (q.value, r.value, t.value, path.value) if ok else None

    def release(self, ticket: int):
        self.lib.qdtg_server_release(self.ptr, ticket)
        with self._lock:
            self._keep.pop(ticket, None)

    def stats(self) -> dict:
        s = ServerStats()
        self.lib.qdtg_server_get_stats(self.ptr, ctypes.byref(s))
        return s.as_dict()


def run_open_loop(server: Server, requests, keep_results: bool = False) -> dict:
    """Submits `requests` ([(arrival_s, points), ...], arrival times from 0)
    at their arrival times and waits for all of them. Returns latency
    percentiles (ms, from scheduled arrival to result), throughput and the
    server's counters; with keep_results, also every result by index."""
    n = len(requests)
    tickets = [0] * n
    statuses = [0] * n
    submit_lag = [0.0] * n
    t0 = time.perf_counter() + 0.05

    def submitter():
        for i, (at, pts) in enumerate(requests):
            now = time.perf_counter() - t0
            if at > now:
                time.sleep(at - now)
            submit_lag[i] = max(0.0, (time.perf_counter() - t0) - at)
            statuses[i], tickets[i] = server.submit(pts)

    th = threading.Thread(target=submitter)
    th.start()
    th.join()
    lat, qms, paths, pts_done = [], [], [], 0
    results = {}
    t_last = 0.0
    for i, (at, pts) in enumerate(requests):
        tk = tickets[i]
        if not tk:
            continue
        server.wait(tk)
        tm = server.timing(tk)
        st, tris, rep, uniq = server.result(tk)
        if keep_results:
            results[i] = (st, tris, rep, uniq)
        if statuses[i] != QDT_OK:
            continue
        q, r, total, path = tm
        lat.append(submit_lag[i] * 1e3 + total)
        qms.append(q)
        paths.append(path)
        pts_done += pts.shape[0]
        t_last = max(t_last, at + (submit_lag[i] * 1e3 + total) / 1e3)
    lat = np.asarray(lat)
    span = max(t_last, 1e-9)
    out = {
        "requests": n,
        "completed": int(lat.size),
        "p50_ms": float(np.percentile(lat, 50)) if lat.size else None,
        "p99_ms": float(np.percentile(lat, 99)) if lat.size else None,
        "mean_ms": float(lat.mean()) if lat.size else None,
        "max_queue_wait_ms": float(max(qms)) if qms else None,
        "mpts_per_s": pts_done / span / 1e6,
        "points": int(pts_done),
        "span_s": span,
        "coalesced": int(sum(paths)),
        "stats": server.stats(),
    }
    if keep_results:
        out["results"] = results
    return out
