"""Domain: Python handle over the C ABI's pfdtd_domain (include/pfdtd.h).

A Domain is one whole grid on one GPU.  Arrays cross the boundary as numpy
arrays (host memory); every call goes straight to libpfdtd.so.
"""
from __future__ import annotations

import ctypes as C
import math
from typing import Callable, Optional, Sequence, Tuple

import numpy as np

from . import _lib as L

_PREC = {"f32": L.F32, "f64": L.F64, "f16": L.F16, "bf16": L.BF16}
_SCHEME = {"forward": L.SRL_FORWARD, "srl_forward": L.SRL_FORWARD, "shared": L.SHARED,
           "centred": L.SRL, "centered": L.SRL, "srl": L.SRL, "iwb": L.IWB}
_STORE_DTYPE = {L.F32: np.float32, L.F64: np.float64, L.F16: np.float16, L.BF16: np.uint16}


def precision_code(p) -> int:
    return _PREC[p] if isinstance(p, str) else int(p)


def scheme_code(s) -> int:
    return _SCHEME[s] if isinstance(s, str) else int(s)


def arith_dtype(precision: int):
    """numpy dtype of the arithmetic type (samples, receiver outputs)."""
    return np.float64 if precision == L.F64 else np.float32


def default_params(octave: int = 0, scheme="forward", lam: Optional[float] = None) -> np.ndarray:
    """[lambda, lambda^2, 1/3, octave] as the reference's
    SimulationParameters::getParameterPtrDouble (SimulationParameters.cpp:389-396)
    after setUpdateType, which every reference entry point calls and which sets
    lambda = sqrt(1/3) (SimulationParameters.cpp:123-137; one ulp below the
    constructor's 1/sqrt(3) in double); lambda = 1 (its stability limit) for
    the IWB scheme unless `lam` is given."""
    if lam is None:
        lam = 1.0 if scheme_code(scheme) == L.IWB else math.sqrt(1.0 / 3.0)
    return np.array([lam, lam * lam, 1.0 / 3.0, float(octave)], dtype=np.float64)


def transparent_source(samples: np.ndarray, grid_ir: np.ndarray, device: int = 0) -> np.ndarray:
    """Transparent source vector computed on the device:
    out[n] = s[n] - sum_{i<n} h[n-i] s[i] in float, in the reference's order
    (SimulationParameters.cpp:300-310)."""
    s = np.ascontiguousarray(samples, dtype=np.float32).reshape(-1)
    h = np.ascontiguousarray(grid_ir, dtype=np.float32).reshape(-1)
    out = np.empty_like(s)
    L.call("pfdtd_transparent_source", s.ctypes.data, s.size, h.ctypes.data if h.size else None,
           h.size, out.ctypes.data, int(device))
    return out


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


class Domain:
    """One FDTD grid on one GPU (pfdtd_create ... pfdtd_destroy)."""

    def __init__(self, dims: Sequence[int], precision="f32", device: int = 0, fields: int = 1):
        self._lib = L.load()
        X, Y, Z = (int(v) for v in dims)
        self.dims = (X, Y, Z)
        self.n = X * Y * Z
        self.fields = int(fields)
        self.precision = precision_code(precision)
        h = C.c_void_p()
        L.call("pfdtd_create_batched", X, Y, Z, self.fields, self.precision, int(device),
               C.byref(h))
        self._h = h
        self.n_rec = 0
        self.n_src = 0

    # -- lifecycle -------------------------------------------------------
    @property
    def handle(self) -> C.c_void_p:
        if self._h is None:
            raise RuntimeError("domain closed")
        return self._h

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            self._lib.pfdtd_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- set-up ----------------------------------------------------------
    def set_quirks(self, quirks: int) -> None:
        L.call("pfdtd_set_quirks", self.handle, int(quirks))

    def set_scheme(self, scheme) -> None:
        L.call("pfdtd_set_scheme", self.handle, scheme_code(scheme))

    def set_update_form(self, form) -> None:
        """"reference" (the reference's expression, bit for bit) or
        "difference" (the same forward update with less float roundoff)."""
        code = {"reference": 0, "difference": 1}[form] if isinstance(form, str) else int(form)
        L.call("pfdtd_set_update_form", self.handle, code)

    def set_nodes(self, pos: np.ndarray, mat: np.ndarray) -> None:
        pos = np.ascontiguousarray(pos, dtype=np.uint8).reshape(-1)
        mat = np.ascontiguousarray(mat, dtype=np.uint8).reshape(-1)
        if pos.size != self.n or mat.size != self.n:
            raise ValueError("node arrays must hold X*Y*Z bytes")
        L.call("pfdtd_set_nodes", self.handle, _ptr(pos), _ptr(mat), 0)

    def set_voxels(self, bid: np.ndarray, mat: np.ndarray, centred: bool) -> None:
        """Upload voxelizer ids 0..27 and translate them on the device
        (toBilbao / toKowalczyk)."""
        self.set_nodes(bid, mat)
        p, m = C.c_void_p(), C.c_void_p()
        L.call("pfdtd_get_node_ptrs", self.handle, C.byref(p), C.byref(m))
        L.call("pfdtd_encode_nodes", 1 if centred else 0, p, m, self.n, self.device_index)
        L.call("pfdtd_nodes_changed", self.handle)

    @property
    def device_index(self) -> int:
        return 0

    def get_nodes(self) -> Tuple[np.ndarray, np.ndarray]:
        pos = np.empty(self.n, dtype=np.uint8)
        mat = np.empty(self.n, dtype=np.uint8)
        L.call("pfdtd_get_nodes", self.handle, _ptr(pos), _ptr(mat))
        return pos, mat

    def count_boundaries(self, air_value: int, outside_value: int = 0) -> Tuple[int, int]:
        p, m = C.c_void_p(), C.c_void_p()
        L.call("pfdtd_get_node_ptrs", self.handle, C.byref(p), C.byref(m))
        a, b = C.c_uint32(), C.c_uint32()
        L.call("pfdtd_count_boundaries", p, self.n, air_value, outside_value, self.device_index,
               C.byref(a), C.byref(b))
        return int(a.value), int(b.value)

    def set_materials(self, table: np.ndarray) -> None:
        t = np.ascontiguousarray(table, dtype=np.float64)
        if t.ndim == 1:
            t = t.reshape(-1, 20)
        L.call("pfdtd_set_materials", self.handle,
               t.ctypes.data_as(C.POINTER(C.c_double)), t.shape[0], t.shape[1])

    def set_dif_filters(self, flags: Sequence[int], coefs: np.ndarray) -> None:
        """Per-material frequency-dependent admittance filters: flags [n_mat],
        coefs [n_mat, 7] = b0..b3, a1..a3 (see materials.dif_table)."""
        f = np.ascontiguousarray(flags, dtype=np.int32).reshape(-1)
        c = np.ascontiguousarray(coefs, dtype=np.float64).reshape(-1, 7)
        L.call("pfdtd_set_dif_filters", self.handle, f.size,
               f.ctypes.data_as(C.POINTER(C.c_int32)), c.ctypes.data_as(C.POINTER(C.c_double)))

    def dif_count(self) -> int:
        n = C.c_int64()
        L.call("pfdtd_get_dif_count", self.handle, C.byref(n))
        return int(n.value)

    def set_params(self, params: Optional[Sequence[float]] = None) -> None:
        p = np.ascontiguousarray(default_params() if params is None else params, dtype=np.float64)
        L.call("pfdtd_set_params", self.handle, p.ctypes.data_as(C.POINTER(C.c_double)))

    def set_sources(self, xyz: np.ndarray, types: Sequence[int], samples: np.ndarray,
                    fields: Optional[Sequence[int]] = None) -> None:
        """Sources at element coordinates; `fields` picks the field each one
        drives (batched domains; default field 0)."""
        xyz = np.ascontiguousarray(np.asarray(xyz, dtype=np.int64).reshape(-1, 3))
        types = np.ascontiguousarray(np.asarray(types, dtype=np.int32).reshape(-1))
        f = np.ascontiguousarray(np.zeros(xyz.shape[0], np.int32) if fields is None
                                 else np.asarray(fields, dtype=np.int32).reshape(-1))
        dt = arith_dtype(self.precision)
        smp = np.ascontiguousarray(np.asarray(samples, dtype=dt).reshape(xyz.shape[0], -1))
        self.n_src = xyz.shape[0]
        L.call("pfdtd_set_sources_batched", self.handle, xyz.shape[0],
               xyz.ctypes.data_as(C.POINTER(C.c_int64)), f.ctypes.data_as(C.POINTER(C.c_int32)),
               types.ctypes.data_as(C.POINTER(C.c_int32)), _ptr(smp), smp.shape[1])
        self._src_keep = (xyz, types, smp, f)

    def set_receivers(self, xyz: np.ndarray, fields: Optional[Sequence[int]] = None) -> None:
        xyz = np.ascontiguousarray(np.asarray(xyz, dtype=np.int64).reshape(-1, 3))
        f = np.ascontiguousarray(np.zeros(xyz.shape[0], np.int32) if fields is None
                                 else np.asarray(fields, dtype=np.int32).reshape(-1))
        self.n_rec = xyz.shape[0]
        L.call("pfdtd_set_receivers_batched", self.handle, xyz.shape[0],
               xyz.ctypes.data_as(C.POINTER(C.c_int64)), f.ctypes.data_as(C.POINTER(C.c_int32)))

    # -- running ---------------------------------------------------------
    def run(self, steps: int, interrupt: Optional[Callable[[], bool]] = None,
            progress: Optional[Callable[[int, int, float], None]] = None,
            out: Optional[np.ndarray] = None) -> Tuple[np.ndarray, float, int]:
        """Run `steps` steps from step 0; returns (receivers [n_rec, steps],
        seconds per step, status)."""
        dt = arith_dtype(self.precision)
        if out is None:
            out = np.zeros((max(self.n_rec, 0), steps), dtype=dt)
        icb = L.INTERRUPT_FN(lambda: 1 if interrupt() else 0) if interrupt else L.INTERRUPT_FN()
        pcb = L.PROGRESS_FN(progress) if progress else L.PROGRESS_FN()
        sec = C.c_double()
        st = L.call("pfdtd_run", self.handle, int(steps), _ptr(out) if out.size else None,
                    icb, pcb, C.byref(sec))
        return out, float(sec.value), st

    def step(self, step: int, direction: int = 1, out: Optional[np.ndarray] = None,
             num_steps: int = 0) -> None:
        L.call("pfdtd_step", self.handle, int(step), int(direction),
               _ptr(out) if out is not None else None, int(num_steps))

    # -- field access ----------------------------------------------------
    def set_sample(self, x, y, z, v) -> None:
        L.call("pfdtd_set_sample", self.handle, x, y, z, float(v))

    def add_sample(self, x, y, z, v) -> None:
        L.call("pfdtd_add_sample", self.handle, x, y, z, float(v))

    def get_sample(self, x, y, z) -> float:
        v = C.c_double()
        L.call("pfdtd_get_sample", self.handle, x, y, z, C.byref(v))
        return float(v.value)

    def flip(self) -> None:
        L.call("pfdtd_flip", self.handle)

    def reset_fields(self) -> None:
        L.call("pfdtd_reset_fields", self.handle)

    def download_field(self, which: int = L.FIELD_CURRENT) -> np.ndarray:
        """The whole field, N * fields elements (node-major)."""
        a = np.empty(self.n * self.fields, dtype=_STORE_DTYPE[self.precision])
        L.call("pfdtd_download_field", self.handle, int(which), _ptr(a))
        return a

    def upload_field(self, which: int, data: np.ndarray) -> None:
        a = np.ascontiguousarray(data, dtype=_STORE_DTYPE[self.precision]).reshape(-1)
        if a.size != self.n * self.fields:
            raise ValueError("field must hold X*Y*Z*fields values")
        L.call("pfdtd_upload_field", self.handle, int(which), _ptr(a))

    def capture_slice(self, orientation: int, slice_idx: int) -> Tuple[np.ndarray, np.ndarray]:
        X, Y, Z = self.dims
        w, h = {0: (X, Y), 1: (X, Z), 2: (Y, Z)}[orientation]
        p = np.empty((h, w), dtype=np.float32)
        q = np.empty((h, w), dtype=np.uint8)
        L.call("pfdtd_capture_slice", self.handle, int(orientation), int(slice_idx), _ptr(p), _ptr(q))
        return p, q

    def capture_slice_noalloc(self, orientation: int, slice_idx: int) -> Tuple[np.ndarray, np.ndarray]:
        """capture_slice without any device allocation: the slice is gathered
        into the library's fixed scratch (at most 1,048,576 nodes per slice),
        for callers that must not allocate device memory while running."""
        X, Y, Z = self.dims
        w, h = {0: (X, Y), 1: (X, Z), 2: (Y, Z)}[orientation]
        p = np.empty((h, w), dtype=np.float32)
        q = np.empty((h, w), dtype=np.uint8)
        L.call("pfdtd_capture_slice_noalloc", self.handle, int(orientation), int(slice_idx),
               _ptr(p), _ptr(q))
        return p, q

    def set_kernel(self, variant) -> None:
        v = {"auto": L.KERNEL_AUTO, "zmarch": L.KERNEL_ZMARCH, "tma": L.KERNEL_TMA}.get(variant, variant)
        L.call("pfdtd_set_kernel", self.handle, int(v))

    def kernel(self) -> str:
        v = C.c_int()
        L.call("pfdtd_get_kernel", self.handle, C.byref(v))
        return {L.KERNEL_ZMARCH: "zmarch", L.KERNEL_TMA: "tma", L.KERNEL_TB: "tb"}[v.value]

    def run_captures(self, steps: int, captures: Sequence[Tuple[int, int, int]]):
        """Run `steps` steps from step 0 capturing slices on the way:
        captures = [(step, orientation, slice), ...]; returns (receivers
        [n_rec, steps], [(pressure [h, w] float32, node bytes [h, w]), ...]),
        each capture the field after its step.  The copies go to pinned host
        buffers, asynchronously on the domain's stream."""
        n = len(captures)
        X, Y, Z = self.dims
        shape = lambda o: (Y, X) if o == 0 else ((Z, X) if o == 1 else (Z, Y))
        st = np.array([c[0] for c in captures], np.int64)
        ori = np.array([c[1] for c in captures], np.int32)
        sl = np.array([c[2] for c in captures], np.int64)
        sizes = [int(np.prod(shape(int(o)))) for o in ori]
        ptrs = []
        try:
            pp = (C.c_void_p * max(n, 1))()
            qq = (C.c_void_p * max(n, 1))()
            for i, sz in enumerate(sizes):
                a, b = C.c_void_p(), C.c_void_p()
                L.call("pfdtd_host_alloc", C.c_size_t(4 * sz), C.byref(a))
                ptrs.append(a)
                L.call("pfdtd_host_alloc", C.c_size_t(sz), C.byref(b))
                ptrs.append(b)
                pp[i], qq[i] = a, b
            out = np.zeros((max(self.n_rec, 0), steps), dtype=arith_dtype(self.precision))
            L.call("pfdtd_run_captures", self.handle, int(steps), out.ctypes.data, n,
                   st.ctypes.data_as(C.POINTER(C.c_int64)),
                   ori.ctypes.data_as(C.POINTER(C.c_int32)),
                   sl.ctypes.data_as(C.POINTER(C.c_int64)), pp, qq)
            caps = []
            for i, o in enumerate(ori):
                h, w = shape(int(o))
                p = np.ctypeslib.as_array((C.c_float * sizes[i]).from_address(pp[i])).copy()
                q = np.ctypeslib.as_array((C.c_uint8 * sizes[i]).from_address(qq[i])).copy()
                caps.append((p.reshape(h, w), q.reshape(h, w)))
            return out, caps
        finally:
            for a in ptrs:
                L.load().pfdtd_host_free(a)

    def set_temporal_block(self, depth: int) -> None:
        """Steps per update kernel: 0 (one kernel per step) or 2, 3, 4."""
        L.call("pfdtd_set_temporal_block", self.handle, int(depth))

    def set_tb_shape(self, shape: int) -> None:
        """Tile shape of the blocked kernel (-1 default, 0..3; 2 and 3 are the
        packed two-field kernels for batched fields)."""
        L.call("pfdtd_set_tb_shape", self.handle, int(shape))

    def autotune(self, max_depth: int = 4, iters: int = 10):
        """Time the per-step and blocked configurations on this domain, keep the
        fastest; returns (depth, shape, ms per step)."""
        depth, shape, ms = C.c_int(), C.c_int(), C.c_double()
        L.call("pfdtd_autotune", self.handle, int(max_depth), int(iters), C.byref(depth),
               C.byref(shape), C.byref(ms))
        return depth.value, shape.value, ms.value

    def temporal_block(self):
        """(depth, active, reason): whether the next run uses the blocked kernel."""
        depth, active = C.c_int(), C.c_int()
        why = C.create_string_buffer(256)
        L.call("pfdtd_get_temporal_block", self.handle, C.byref(depth), C.byref(active), why, 256)
        return depth.value, bool(active.value), why.value.decode()

    def synchronize(self) -> None:
        L.call("pfdtd_synchronize", self.handle)

    def stream_ptr(self) -> int:
        s = C.c_void_p()
        L.call("pfdtd_get_stream", self.handle, C.byref(s))
        return s.value or 0


def autotune_fields(dims: Sequence[int], setup: Callable[["Domain"], None], precision="f32",
                    candidates: Sequence[int] = (1, 4, 8, 16, 32), max_depth: int = 3,
                    iters: int = 10, device: int = 0, memory_fraction: float = 0.8):
    """Pick the number of batched fields K for many sources in one room.

    Sources in the same room can run as K fields of one domain sharing the
    geometry, the class ids and the coefficient table (one run per K sources).
    For every candidate K whose fields fit in `memory_fraction` of the
    device's free memory, a K-field domain is created and prepared by
    `setup(domain)` (geometry, materials, parameters, scheme), and
    Domain.autotune times its per-step kernel and every blocked (depth <=
    max_depth, tile shape) configuration and keeps the fastest.  The rate is
    field-updates per second, X*Y*(Z-2)*K per step.

    Returns (K, depth, shape, rates): the K with the highest rate, its kernel
    configuration (depth 0 = per step), and {K: (rate, depth, shape)} for
    every candidate timed.  No counterpart in the reference, which runs one
    source set per simulation.
    """
    X, Y, Z = (int(v) for v in dims)
    esize = {L.F32: 4, L.F64: 8, L.F16: 2, L.BF16: 2}[precision_code(precision)]
    free = None
    try:
        import torch
        if torch.cuda.is_available():
            free = torch.cuda.mem_get_info(device)[0]
    except Exception:
        free = None
    rates = {}
    for K in candidates:
        K = int(K)
        if K != 1 and (K % 4 != 0 or K & (K - 1)):
            raise ValueError("candidate field counts are 1 or powers of two from 4")
        need = (4 if max_depth >= 2 else 2) * X * Y * Z * K * esize + 2 * X * Y * Z
        if free is not None and need > memory_fraction * free:
            continue
        with Domain((X, Y, Z), precision, device=device, fields=K) as d:
            setup(d)
            depth, shape, ms = d.autotune(max_depth=max_depth, iters=iters)
        rates[K] = (X * Y * (Z - 2) * K / (ms * 1e-3), depth, shape)
    if not rates:
        raise RuntimeError("no candidate field count fits in device memory")
    best = max(rates, key=lambda k: rates[k][0])
    return best, rates[best][1], rates[best][2], rates
