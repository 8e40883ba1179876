"""Request loop with continuous batching (include/pfdtd_server.h).

``Server`` wraps the native scheduler: requests are queued in arrival order
and admitted while a slot is free and their estimated device bytes fit the
HBM budget beside the running requests; each admitted request runs on its
own domain and stream, so admitted requests overlap on the GPU.
``Request.from_room`` builds a request from a procedural room, and
``serving_trace`` / ``run_trace`` generate and replay the seeded serving
workload (Poisson arrivals of rooms with per-axis sizes U(64, 512), SRL or
IWB, frequency-independent or 3rd-order frequency-dependent boundaries,
500-8000 steps, 1-16 sources) with queue and service latencies.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import time
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import _lib as L
from .domain import arith_dtype, default_params, precision_code, scheme_code

QUEUED, RUNNING, DONE, FAILED = 0, 1, 2, 3


class _Stats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("admitted", C.c_int64), ("completed", C.c_int64),
                ("failed", C.c_int64), ("queued", C.c_int64), ("running", C.c_int64),
                ("bytes_in_use", C.c_uint64), ("bytes_peak", C.c_uint64),
                ("max_running", C.c_int), ("node_updates", C.c_double),
                ("setup_seconds", C.c_double), ("retire_seconds", C.c_double)]


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t)) if a is not None else None


class Request:
    """One room solve: geometry, materials, sources, receivers, step count."""

    def __init__(self, dims: Sequence[int], steps: int, fields: int = 1, precision="f32",
                 scheme="forward"):
        L.load()
        self.dims = tuple(int(v) for v in dims)
        self.steps = int(steps)
        self.fields = int(fields)
        self.precision = precision_code(precision)
        self.scheme = scheme_code(scheme)
        self.n_rec = 0
        self.source_fields = self.fields
        h = C.c_void_p()
        L.call("pfdtd_request_create", *self.dims, self.fields, self.precision, self.scheme,
               self.steps, C.byref(h))
        self._h = h

    @property
    def handle(self):
        if self._h is None:
            raise RuntimeError("request already submitted or destroyed")
        return self._h

    def set_voxels(self, bid: np.ndarray, mat: np.ndarray) -> "Request":
        b = np.ascontiguousarray(bid, dtype=np.uint8).reshape(-1)
        m = np.ascontiguousarray(mat, dtype=np.uint8).reshape(-1)
        L.call("pfdtd_request_set_voxels", self.handle, b.ctypes.data, m.ctypes.data)
        return self

    def set_materials(self, table: np.ndarray) -> "Request":
        t = np.ascontiguousarray(table, dtype=np.float64)
        t2 = t.reshape(t.shape[0], -1) if t.ndim > 1 else t.reshape(-1, 20)
        L.call("pfdtd_request_set_materials", self.handle, _p(t2, C.c_double), t2.shape[0],
               t2.shape[1])
        return self

    def set_dif_filters(self, flags: Sequence[int], coefs: np.ndarray) -> "Request":
        f = np.ascontiguousarray(flags, dtype=np.int32)
        c = np.ascontiguousarray(coefs, dtype=np.float64).reshape(-1, 7)
        L.call("pfdtd_request_set_dif_filters", self.handle, f.size, _p(f, C.c_int32),
               _p(c, C.c_double))
        return self

    def set_params(self, params: Sequence[float]) -> "Request":
        p = np.ascontiguousarray(params, dtype=np.float64)
        L.call("pfdtd_request_set_params", self.handle, _p(p, C.c_double))
        return self

    def set_sources(self, xyz, types, samples, fields=None) -> "Request":
        x = np.ascontiguousarray(xyz, dtype=np.int64).reshape(-1, 3)
        n = x.shape[0]
        ty = np.ascontiguousarray(types, dtype=np.int32).reshape(-1)
        f = None if fields is None else np.ascontiguousarray(fields, dtype=np.int32)
        s = np.ascontiguousarray(samples, dtype=np.float64).reshape(n, -1)
        L.call("pfdtd_request_set_sources", self.handle, n, _p(x, C.c_int64), _p(f, C.c_int32),
               _p(ty, C.c_int32), _p(s, C.c_double), s.shape[1])
        if n > 0:
            used = {0} if f is None else {int(v) for v in f if 0 <= int(v) < self.fields}
            self.source_fields = len(used) or self.fields
        return self

    def set_receivers(self, xyz, fields=None) -> "Request":
        x = np.ascontiguousarray(xyz, dtype=np.int64).reshape(-1, 3)
        f = None if fields is None else np.ascontiguousarray(fields, dtype=np.int32)
        L.call("pfdtd_request_set_receivers", self.handle, x.shape[0], _p(x, C.c_int64),
               _p(f, C.c_int32))
        self.n_rec = x.shape[0]
        return self

    def set_temporal_block(self, depth: int) -> "Request":
        L.call("pfdtd_request_set_temporal_block", self.handle, int(depth))
        return self

    def bytes(self) -> int:
        b = C.c_uint64()
        L.call("pfdtd_request_bytes", self.handle, C.byref(b))
        return int(b.value)

    def node_updates(self) -> float:
        """Updates of the fields that carry a source: a request whose source
        count was rounded up to a power of two is not credited for the
        padding fields it also computes."""
        X, Y, Z = self.dims
        return float(X) * Y * (Z - 2) * self.steps * self.source_fields

    def computed_updates(self) -> float:
        """Every field the request computes.  The server runs the fields that
        carry a source one after another on a single-field domain whenever
        some field has none (and for IWB, or a field count the batched kernel
        does not take), so it computes exactly the source fields."""
        X, Y, Z = self.dims
        return float(X) * Y * (Z - 2) * self.steps * self.source_fields

    def close(self) -> None:
        if self._h is not None:
            L.load().pfdtd_request_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @classmethod
    def from_room(cls, room, steps: int, sources, receivers, samples, precision="f32",
                  scheme="forward", fields: int = 1, src_fields=None, rec_fields=None,
                  dif=None, src_types=None, tb: int = 0) -> "Request":
        r = cls(room.dims, steps, fields, precision, scheme)
        r.set_voxels(room.bid, room.mat)
        r.set_materials(room.admittance)
        if dif is not None:
            r.set_dif_filters(*dif)
        r.set_params(default_params(scheme=scheme))
        types = [1] * len(sources) if src_types is None else src_types
        r.set_sources(sources, types, samples, src_fields)
        r.set_receivers(receivers, rec_fields)
        if tb:
            r.set_temporal_block(tb)
        return r


class Server:
    """Native request loop on one GPU."""

    def __init__(self, device: int = 0, hbm_budget: int = 160 << 30, max_active: int = 8):
        L.load()
        h = C.c_void_p()
        L.call("pfdtd_server_create", int(device), int(hbm_budget), int(max_active), C.byref(h))
        self._h = h
        self._meta: Dict[int, tuple] = {}

    def submit(self, req: Request) -> int:
        t = C.c_int64()
        meta = (req.n_rec, req.steps, arith_dtype(req.precision), req.node_updates())
        h = req.handle
        req._h = None  # the server owns it now
        rc = L.load().pfdtd_server_submit(self._h, h, C.byref(t))
        self._meta[t.value] = meta
        L.check(rc, "pfdtd_server_submit")
        return t.value

    def wait(self, ticket: int, timeout: float = -1.0) -> int:
        st = C.c_int()
        L.call("pfdtd_server_wait", self._h, int(ticket), float(timeout), C.byref(st))
        return st.value

    def result(self, ticket: int):
        """(receivers [n_rec, steps], (queued s, service s, total s))."""
        n_rec, steps, dt, _ = self._meta[ticket]
        out = np.zeros((n_rec, steps), dtype=dt)
        times = (C.c_double * 3)()
        L.call("pfdtd_server_result", self._h, int(ticket), out.ctypes.data, times)
        return out, (times[0], times[1], times[2])

    def error(self, ticket: int) -> str:
        return L.load().pfdtd_server_request_error(self._h, int(ticket)).decode()

    def release(self, ticket: int) -> None:
        L.call("pfdtd_server_release", self._h, int(ticket))
        self._meta.pop(ticket, None)

    def stats(self) -> dict:
        s = _Stats()
        L.call("pfdtd_server_stats_get", self._h, C.byref(s))
        return {k: getattr(s, k) for k, _ in _Stats._fields_}

    def drain(self, timeout: float = -1.0) -> None:
        L.call("pfdtd_server_drain", self._h, float(timeout))

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            L.load().pfdtd_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


# ---------------------------------------------------------------------------
# seeded serving workload

@dataclasses.dataclass
class TraceItem:
    arrival: float          # seconds after the start
    dims: tuple
    scheme: str             # "forward" (SRL) or "iwb"
    dif: bool
    steps: int
    n_src: int
    seed: int


def serving_trace(n: int, seed: int = 0, rate: float = 20.0, axis=(64, 512),
                  steps=(500, 8000), sources=(1, 16)) -> List[TraceItem]:
    """n requests with Poisson arrivals at `rate` per second; per-axis sizes
    U(axis) (rounded to multiples of 4), SRL forward or IWB with equal odds,
    frequency-independent or 3rd-order frequency-dependent boundaries with
    equal odds, steps U(steps), sources U(sources)."""
    g = np.random.default_rng(seed)
    t = 0.0
    items = []
    for i in range(n):
        t += float(g.exponential(1.0 / rate))
        dims = tuple(int(v) // 4 * 4 for v in g.integers(axis[0], axis[1] + 1, size=3))
        items.append(TraceItem(t, dims, "forward" if g.random() < 0.5 else "iwb",
                               bool(g.random() < 0.5), int(g.integers(steps[0], steps[1] + 1)),
                               int(g.integers(sources[0], sources[1] + 1)), seed * 100003 + i))
    return items


def build_request(item: TraceItem, precision="f32") -> Request:
    """Procedural room of the trace item: solid shell, seeded boxes, 8
    materials; one field per source (the power of two at or above the source
    count), 4 air receivers per source, a soft impulse per source."""
    from . import materials, rooms
    X, Y, Z = item.dims
    n_boxes = max(1, X * Y * Z // (128 ** 3))
    room = rooms.boxes_room(item.dims, n_boxes=n_boxes, edge=(4, max(6, min(item.dims) // 4)),
                            n_materials=8, admittance_range=(0.01, 0.9), seed=item.seed)
    fields = 1
    while fields < item.n_src:
        fields *= 2
    pts = room.random_air_nodes(5 * item.n_src, seed=item.seed + 1)
    srcs = [tuple(p) for p in pts[:item.n_src]]
    recs = [tuple(p) for p in pts[item.n_src:]]
    dif = None
    if item.dif:
        filt = materials.positive_real_filters(8, 3, seed=item.seed + 2)
        dif = (np.ones(8, np.int32), materials.dif_table(filt, 3))
    samples = np.zeros((item.n_src, item.steps))
    samples[:, 1] = 1.0
    return Request.from_room(room, item.steps, srcs, recs, samples, precision=precision,
                             scheme=item.scheme, fields=fields,
                             src_fields=list(range(item.n_src)),
                             rec_fields=[i // 4 for i in range(4 * item.n_src)], dif=dif)


def run_trace(server: Server, requests: Sequence[Request], arrivals: Sequence[float],
              timeout: float = 3600.0) -> dict:
    """Submit each request at its arrival time (seconds after the start),
    wait for all; returns per-request times and the aggregate figures."""
    updates = [r.node_updates() for r in requests]
    computed = [r.computed_updates() for r in requests]
    t0 = time.perf_counter()
    tickets = []
    for req, at in zip(requests, arrivals):
        delay = at - (time.perf_counter() - t0)
        if delay > 0:
            time.sleep(delay)
        tickets.append(server.submit(req))
    states = [server.wait(t, timeout) for t in tickets]
    wall = time.perf_counter() - t0
    times = []
    for t, st in zip(tickets, states):
        if st != DONE:
            raise RuntimeError(f"request {t} failed: {server.error(t)}")
        _, tm = server.result(t)
        times.append(tm)
        server.release(t)
    q = np.array([t[0] for t in times])
    s = np.array([t[1] for t in times])
    tot = np.array([t[2] for t in times])
    pct = lambda a, p: float(np.percentile(a, p))
    return {"wall_s": wall, "node_updates": float(sum(updates)),
            "computed_updates": float(sum(computed)), "requests": len(requests),
            "throughput": float(sum(updates)) / wall,
            "latency_p50_s": pct(tot, 50), "latency_p99_s": pct(tot, 99),
            "queue_p50_s": pct(q, 50), "queue_p99_s": pct(q, 99),
            "service_p50_s": pct(s, 50), "service_p99_s": pct(s, 99),
            "stats": server.stats()}
