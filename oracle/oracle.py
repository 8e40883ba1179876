"""Python access to the CPU oracle (test infrastructure only).

Loads oracle/_build/liboracle.so, built from oracle/fdtd_oracle.cpp by
oracle/build.py, and exposes numpy-level calls.  Only the tests, the smoke
check and the CPU-baseline leg of the benchmark use this module; the product
never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Sequence, Tuple

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None


def load(build_if_missing: bool = True) -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    import importlib.util
    spec = importlib.util.spec_from_file_location("oracle_build", os.path.join(_HERE, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    path = mod.LIB
    if build_if_missing:
        path = mod.build()
    lib = C.CDLL(path)
    vp, i64, i32 = C.c_void_p, C.c_int64, C.c_int
    lib.oracle_encode_nodes.argtypes = [i32, vp, vp, i64]
    lib.oracle_encode_nodes.restype = None
    lib.oracle_count_boundaries.argtypes = [vp, i64, C.c_uint8, C.c_uint8,
                                            C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
    lib.oracle_count_boundaries.restype = None
    lib.oracle_pad.argtypes = [vp, i64, C.POINTER(C.c_uint32), C.c_uint32, C.c_uint32,
                               C.c_uint32, vp, C.POINTER(C.c_uint32)]
    lib.oracle_pad.restype = None
    lib.oracle_source_sample_f32.argtypes = [i32, i32, C.c_uint32, C.c_uint32, vp, C.c_uint32,
                                             vp, C.c_uint32]
    lib.oracle_source_sample_f32.restype = C.c_float
    lib.oracle_source_sample_f64.argtypes = [i32, i32, C.c_uint32, C.c_uint32, vp, C.c_uint32,
                                             vp, C.c_uint32]
    lib.oracle_source_sample_f64.restype = C.c_double
    lib.oracle_run.argtypes = [i32, i32, i32, i64, i64, i64, vp, vp, vp, i32, vp, i32, vp, vp,
                               vp, i32, vp, i64, vp, vp, vp, i32, vp, vp]
    lib.oracle_run.restype = i32
    lib.oracle_max_threads.argtypes = []
    lib.oracle_max_threads.restype = i32
    _lib = lib
    return lib


def _p(a: Optional[np.ndarray]):
    return None if a is None else C.c_void_p(a.ctypes.data)


def encode_nodes(bid: np.ndarray, mat: np.ndarray, centred: bool) -> Tuple[np.ndarray, np.ndarray]:
    """toBilbao / toKowalczyk on copies of (bid, mat)."""
    pos = np.array(bid, dtype=np.uint8, copy=True).reshape(-1)
    m = np.array(mat, dtype=np.uint8, copy=True).reshape(-1)
    load().oracle_encode_nodes(1 if centred else 0, _p(pos), _p(m), pos.size)
    return pos, m


def count_boundaries(pos: np.ndarray, air_value: int, outside_value: int = 0) -> Tuple[int, int]:
    a, b = C.c_uint32(), C.c_uint32()
    p = np.ascontiguousarray(pos, dtype=np.uint8).reshape(-1)
    load().oracle_count_boundaries(_p(p), p.size, air_value, outside_value, C.byref(a), C.byref(b))
    return int(a.value), int(b.value)


def pad(mesh: np.ndarray, dims: Sequence[int], block: Sequence[int]) -> Tuple[np.ndarray, Tuple[int, int, int]]:
    m = np.ascontiguousarray(mesh, dtype=np.uint8).reshape(-1)
    d = (C.c_uint32 * 3)(*dims)
    od = (C.c_uint32 * 3)()
    load().oracle_pad(None, 0, d, block[0], block[1], block[2], None, od)
    out = np.zeros(int(od[0]) * int(od[1]) * int(od[2]), dtype=np.uint8)
    load().oracle_pad(_p(m), m.size, d, block[0], block[1], block[2], _p(out), od)
    return out, (int(od[0]), int(od[1]), int(od[2]))


def source_vector(src_type: int, input_type: int, steps: int, fs: int = 7000,
                  data: Optional[np.ndarray] = None, grid_ir: Optional[np.ndarray] = None,
                  double: bool = False) -> np.ndarray:
    lib = load()
    dd = None if data is None else np.ascontiguousarray(data, dtype=np.float64 if double else np.float32)
    ir = None if grid_ir is None else np.ascontiguousarray(grid_ir, dtype=np.float32)
    f = lib.oracle_source_sample_f64 if double else lib.oracle_source_sample_f32
    out = np.empty(steps, dtype=np.float64 if double else np.float32)
    for s in range(steps):
        out[s] = f(src_type, input_type, s, fs, _p(dd), 0 if dd is None else dd.size,
                   _p(ir), 0 if ir is None else ir.size)
    return out


def run(pos: np.ndarray, mat: np.ndarray, dims: Sequence[int], table: np.ndarray,
        params: Sequence[float], src_idx: Sequence[int], src_type: Sequence[int],
        samples: np.ndarray, rec_idx: Sequence[int], steps: int, scheme: int = 0,
        quirks: int = 0, double: bool = False, threads: int = 0,
        P0: Optional[np.ndarray] = None, Pp0: Optional[np.ndarray] = None,
        storage: Optional[str] = None, dif: Optional[Tuple[np.ndarray, np.ndarray]] = None,
        form: str = "reference"):
    """Oracle step loop.  Returns (receivers [n_rec, steps], P, P_past).
    storage: None (FP32, or FP64 with double=True), "f16" or "bf16" (16-bit
    fields with float arithmetic; fields returned as float16 / uint16).
    dif: (flags [n_mat] int, coefs [n_mat, 7] b0..b3, a1..a3) for materials
    with frequency-dependent admittance.  form: "reference" or "difference"
    (the library's PFDTD_FORM_DIFFERENCE forward update)."""
    lib = load()
    dt = np.float64 if double else np.float32
    prec = 1 if double else {None: 0, "f32": 0, "f16": 2, "bf16": 3}[storage]
    st_dt = {0: np.float32, 1: np.float64, 2: np.float16, 3: np.uint16}[prec]
    X, Y, Z = (int(v) for v in dims)
    N = X * Y * Z
    pos = np.ascontiguousarray(pos, dtype=np.uint8).reshape(-1)
    mat = np.ascontiguousarray(mat, dtype=np.uint8).reshape(-1)
    tab = np.ascontiguousarray(table, dtype=dt).reshape(-1)
    n_mat = tab.size // 20
    prm = np.ascontiguousarray(params, dtype=dt)
    si = np.ascontiguousarray(src_idx, dtype=np.int64).reshape(-1)
    st = np.ascontiguousarray(src_type, dtype=np.int32).reshape(-1)
    sm = np.ascontiguousarray(samples, dtype=dt).reshape(si.size, -1) if si.size else np.zeros((0, steps), dt)
    ri = np.ascontiguousarray(rec_idx, dtype=np.int64).reshape(-1)
    P = np.zeros(N, dtype=st_dt) if P0 is None else np.array(P0, dtype=st_dt, copy=True)
    Pp = np.zeros(N, dtype=st_dt) if Pp0 is None else np.array(Pp0, dtype=st_dt, copy=True)
    out = np.zeros((ri.size, steps), dtype=dt)
    if threads <= 0:
        threads = lib.oracle_max_threads()
    dflag = dcoef = None
    if dif is not None:
        dflag = np.ascontiguousarray(dif[0], dtype=np.int32).reshape(-1)
        dcoef = np.ascontiguousarray(dif[1], dtype=dt).reshape(-1, 7)
        if dflag.size != n_mat or dcoef.shape[0] != n_mat:
            raise ValueError("dif tables must have one row per material")
    if form not in ("reference", "difference"):
        raise ValueError("form must be 'reference' or 'difference'")
    if form == "difference":
        quirks = quirks | 0x100
    rc = lib.oracle_run(prec, scheme, quirks, X, Y, Z, _p(pos), _p(mat), _p(tab),
                        n_mat, _p(prm), si.size, _p(si), _p(st), _p(sm), ri.size, _p(ri),
                        steps, _p(P), _p(Pp), _p(out), threads, _p(dflag), _p(dcoef))
    if rc != 0:
        raise RuntimeError(f"oracle_run failed with {rc}")
    return out, P, Pp


def max_threads() -> int:
    return int(load().oracle_max_threads())
