"""The reference's own code, run for parity checks — test infrastructure only.

Two ways in, both built by oracle/build_ref.py from the reference's unchanged
sources:

* CPU (this container only, where the sources are mounted): libref_cpu.so
  holds the reference's SimulationParameters / MaterialHandler / SrcRec classes
  and its update, padding and node-translation kernels compiled for the host.
  `run_cpu` drives them with the step order of launchFDTD3d
  (src/kernels/kernels3d.cu:86-175).  tests/golden/make_ref_golden.py uses it
  to write golden vectors.
* GPU: the reference's kernels3d.cu / cudaMesh.cu compiled unchanged for
  sm_103a (with and without floating-point contraction) and launched by
  oracle/ref_gpu_runner.cpp (`run_gpu`).

Only the tests, the smoke check and the benchmark's reference-kernel figure
use this module; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import tempfile
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
CPU_LIB = os.path.join(REF_DIR, "libref_cpu.so")
CUBIN_KERNELS = os.path.join(REF_DIR, "kernels3d_sm103a.cubin")
CUBIN_KERNELS_NOFMA = os.path.join(REF_DIR, "kernels3d_sm103a_nofma.cubin")
CUBIN_MESH = os.path.join(REF_DIR, "cudaMesh_sm103a.cubin")
GPU_LIB = os.path.join(HERE, "_build", "libref_gpu.so")

# SrcType / InputType / UpdateType of the reference (SrcRec.h, SimulationParameters.h:39)
SRC_HARD, SRC_SOFT, SRC_TRANSPARENT = 0, 1, 2
IMPULSE, GAUSSIAN, SINE, DATA = 0, 1, 2, 3
SRL_FORWARD, SHARED, SRL = 0, 1, 2
BLOCK = (32, 4)  # App.cpp:193, the block every reference mesh is set up with

_cpu = None
_gpu = None
_gpu_cubin = None


def cpu_available() -> bool:
    return os.path.exists(CPU_LIB)


def gpu_available() -> bool:
    return all(os.path.exists(p) for p in (CUBIN_KERNELS, CUBIN_KERNELS_NOFMA, CUBIN_MESH))


def _vp(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def cpu() -> C.CDLL:
    global _cpu
    if _cpu is None:
        if not cpu_available():
            raise FileNotFoundError("oracle/_ref/libref_cpu.so is missing (oracle/build_ref.py "
                                    "needs the reference sources)")
        lib = C.CDLL(CPU_LIB)
        vp, u, f, d, i = C.c_void_p, C.c_uint, C.c_float, C.c_double, C.c_int
        lib.refh_sp_new.restype = vp
        lib.refh_sp_free.argtypes = [vp]
        lib.refh_sp_config.argtypes = [vp, i, d, u, u, u, f]
        lib.refh_sp_lambda.argtypes = [vp]
        lib.refh_sp_lambda.restype = d
        lib.refh_sp_dx.argtypes = [vp]
        lib.refh_sp_dx.restype = f
        lib.refh_sp_add_source.argtypes = [vp, f, f, f, i, i, u]
        lib.refh_sp_add_receiver.argtypes = [vp, f, f, f]
        lib.refh_sp_add_input_f32.argtypes = [vp, vp, u]
        lib.refh_sp_add_input_f64.argtypes = [vp, vp, u]
        lib.refh_sp_read_grid_ir.argtypes = [vp, C.c_char_p]
        lib.refh_sp_source_coords.argtypes = [vp, u, vp]
        lib.refh_sp_receiver_coords.argtypes = [vp, u, vp]
        lib.refh_sp_source_vector_f32.argtypes = [vp, u, u, vp]
        lib.refh_sp_source_vector_f64.argtypes = [vp, u, u, vp]
        lib.refh_sp_params_f32.argtypes = [vp, vp]
        lib.refh_sp_params_f64.argtypes = [vp, vp]
        lib.refh_mh_new.argtypes = [i]
        lib.refh_mh_new.restype = vp
        lib.refh_mh_free.argtypes = [vp]
        lib.refh_mh_add_materials.argtypes = [vp, vp, u, u]
        lib.refh_mh_unique.argtypes = [vp]
        lib.refh_mh_unique.restype = u
        lib.refh_mh_table_f32.argtypes = [vp, vp]
        lib.refh_mh_table_f64.argtypes = [vp, vp]
        lib.refh_mh_indices.argtypes = [vp, vp]
        lib.refcpu_pad.argtypes = [vp, u, u, u, u, u, u, vp, vp]
        lib.refcpu_encode.argtypes = [i, vp, vp, u]
        lib.refcpu_count.argtypes = [vp, u, C.c_uint8, C.c_uint8, vp, vp]
        lib.refcpu_update_f32.argtypes = [i, vp, vp, vp, vp, vp, vp, u, u, u, u, u]
        lib.refcpu_update_f64.argtypes = [i, vp, vp, vp, vp, vp, vp, u, u, u, u, u]
        _cpu = lib
    return _cpu


class _InScratch:
    """Runs reference host code from a scratch directory: its logger appends
    to solver_log.txt in the working directory."""

    def __enter__(self):
        self.old = os.getcwd()
        self.tmp = tempfile.TemporaryDirectory()
        os.chdir(self.tmp.name)
        return self.tmp.name

    def __exit__(self, *exc):
        os.chdir(self.old)
        self.tmp.cleanup()


# -- reference host classes ---------------------------------------------------
def host_setup(scheme: str, octave: int, steps: int, admittance_rows: np.ndarray,
               sources: Sequence[tuple], receivers: Sequence[tuple],
               data: Sequence[np.ndarray] = (), fs: int = 7000, double: bool = False,
               grid_ir=None):
    """Builds the reference's SimulationParameters and MaterialHandler.

    grid_ir: None, an array, or the path of a text file for readGridIr.

    sources: (x, y, z, src_type, input_type, data_idx) element coordinates
    (placed at (idx - 1) * dx metres, which the reference maps back to idx);
    receivers: (x, y, z).  Returns dict with params (4), table (n_mat*20),
    source samples [n_src, steps], source/receiver element coords, material
    indices and dx — every value computed by the reference's own classes."""
    lib = cpu()
    dt = np.float64 if double else np.float32
    out = {}
    with _InScratch() as tmp:
        sp = lib.refh_sp_new()
        try:
            ut = SRL_FORWARD if scheme == "forward" else SRL
            if lib.refh_sp_config(sp, ut, -1.0, octave, steps, fs, 344.0) != 0:
                raise RuntimeError("SimulationParameters rejected the configuration")
            dx = float(np.float32(lib.refh_sp_dx(sp)))
            for vec in data:
                v = np.ascontiguousarray(vec, dtype=dt)
                (lib.refh_sp_add_input_f64 if double else lib.refh_sp_add_input_f32)(sp, _vp(v), v.size)
            if grid_ir is not None:
                if isinstance(grid_ir, str):
                    path = grid_ir
                else:
                    path = os.path.join(tmp, "grid_ir.txt")
                    np.savetxt(path, np.asarray(grid_ir, dtype=np.float64))
                if lib.refh_sp_read_grid_ir(sp, path.encode()) != 0:
                    raise RuntimeError("readGridIr failed")
            for (x, y, z, st, it, di) in sources:
                lib.refh_sp_add_source(sp, np.float32((x - 1) * dx), np.float32((y - 1) * dx),
                                       np.float32((z - 1) * dx), st, it, di)
            for (x, y, z) in receivers:
                lib.refh_sp_add_receiver(sp, np.float32((x - 1) * dx), np.float32((y - 1) * dx),
                                         np.float32((z - 1) * dx))
            xyz = np.zeros(3, np.int32)
            sc, rc = [], []
            for i in range(len(sources)):
                if lib.refh_sp_source_coords(sp, i, _vp(xyz)) != 0:
                    raise RuntimeError("getSourceElementCoordinates failed")
                sc.append(tuple(int(v) for v in xyz))
            for i in range(len(receivers)):
                if lib.refh_sp_receiver_coords(sp, i, _vp(xyz)) != 0:
                    raise RuntimeError("getReceiverElementCoordinates failed")
                rc.append(tuple(int(v) for v in xyz))
            smp = np.zeros((len(sources), steps), dt)
            for i in range(len(sources)):
                row = np.zeros(steps, dt)
                f = lib.refh_sp_source_vector_f64 if double else lib.refh_sp_source_vector_f32
                if f(sp, i, steps, _vp(row)) != 0:
                    raise RuntimeError("getSourceSample failed")
                smp[i] = row
            prm = np.zeros(4, dt)
            (lib.refh_sp_params_f64 if double else lib.refh_sp_params_f32)(sp, _vp(prm))
            out.update(params=prm, samples=smp, source_coords=sc, receiver_coords=rc, dx=dx,
                       lam=float(lib.refh_sp_lambda(sp)))
        finally:
            lib.refh_sp_free(sp)
        mh = lib.refh_mh_new(0)
        try:
            rows = np.ascontiguousarray(admittance_rows, dtype=np.float32)
            if lib.refh_mh_add_materials(mh, _vp(rows), rows.shape[0], rows.shape[1]) != 0:
                raise RuntimeError("addMaterials failed")
            nu = lib.refh_mh_unique(mh)
            tab = np.zeros(nu * 20, dt)
            (lib.refh_mh_table_f64 if double else lib.refh_mh_table_f32)(mh, _vp(tab))
            idx = np.zeros(rows.shape[0], np.uint8)
            lib.refh_mh_indices(mh, _vp(idx))
            out.update(table=tab, material_indices=idx)
        finally:
            lib.refh_mh_free(mh)
    return out


# -- reference kernels on the CPU ---------------------------------------------
def encode_cpu(bid: np.ndarray, mat: np.ndarray, centred: bool):
    """toBilbaoKernel / toKowalczykKernel alone on copies of (bid, mat)."""
    pos = np.array(bid, np.uint8, copy=True).reshape(-1)
    m = np.array(mat, np.uint8, copy=True).reshape(-1)
    cpu().refcpu_encode(1 if centred else 0, _vp(pos), _vp(m), pos.size)
    return pos, m


def setup_mesh_cpu(bid: np.ndarray, mat: np.ndarray, dims: Sequence[int], centred: bool,
                   block=BLOCK):
    """padWithZeros + toBilbao/toKowalczyk + calcBoundaries, the reference's
    kernels run on the host.  Returns (pos, mat, padded dims, (air, boundary))."""
    lib = cpu()
    X, Y, Z = (int(v) for v in dims)
    slack = X * Y + X + 1
    od = np.zeros(3, np.uint32)
    lib.refcpu_pad(None, X, Y, Z, block[0], block[1], 1, None, _vp(od))
    n = int(od[0]) * int(od[1]) * int(od[2])
    outs = []
    for src in (bid, mat):
        old = np.zeros(X * Y * Z + slack, np.uint8)
        old[:X * Y * Z] = np.asarray(src, np.uint8).reshape(-1)
        new = np.zeros(n, np.uint8)
        lib.refcpu_pad(_vp(old), X, Y, Z, block[0], block[1], 1, _vp(new), _vp(od))
        outs.append(new)
    pos, m = outs
    lib.refcpu_encode(1 if centred else 0, _vp(pos), _vp(m), n)
    air, bnd = C.c_uint(), C.c_uint()
    lib.refcpu_count(_vp(pos), n, 0x80 if centred else 0x86, 0, C.byref(air), C.byref(bnd))
    return pos, m, tuple(int(v) for v in od), (int(air.value), int(bnd.value))


def run_cpu(bid, mat, dims, scheme: str, table, params, src_idx, samples, rec_idx, steps: int,
            double: bool = False, block=BLOCK):
    """The reference's update kernels on the host with launchFDTD3d's step
    order (kernels3d.cu:86-175): each source sample written into the current
    field (setSample; addSample as run also writes the sample alone), one
    update launch over z = 1..Z-2, swap, receivers read from the new field.
    Returns (receivers [n_rec, steps], P, P_past) on the padded mesh."""
    lib = cpu()
    dt = np.float64 if double else np.float32
    pos, m, pd, _ = setup_mesh_cpu(bid, mat, dims, scheme != "forward", block)
    X, Y, Z = pd
    n = X * Y * Z
    P = np.zeros(n + 1 + X, dt)  # size + 1 + X elements (cudaMesh.h:683, :717)
    Pp = np.zeros(n + 1 + X, dt)
    tab = np.ascontiguousarray(table, dtype=dt)
    prm = np.ascontiguousarray(params, dtype=dt)
    smp = np.asarray(samples, dtype=dt).reshape(len(src_idx), -1)
    rec = np.zeros((len(rec_idx), steps), dt)
    upd = lib.refcpu_update_f64 if double else lib.refcpu_update_f32
    sch = 0 if scheme == "forward" else 1
    for step in range(steps):
        for i, e in enumerate(src_idx):
            P[e] = smp[i, step]
        upd(sch, _vp(pos), _vp(m), _vp(P), _vp(Pp), _vp(prm), _vp(tab), X, Y, Z, block[0], block[1])
        P, Pp = Pp, P
        for r, e in enumerate(rec_idx):
            rec[r, step] = P[e]
    return rec, P[:n].copy(), Pp[:n].copy()


# -- reference kernels on the GPU ---------------------------------------------
def gpu(nofma: bool = False) -> C.CDLL:
    """The driver-API runner with the reference's cubins loaded (default
    contraction, or -fmad=false with nofma=True)."""
    global _gpu, _gpu_cubin
    if _gpu is None:
        if not os.path.exists(GPU_LIB):
            from oracle import build as ob
            ob.build_ref_gpu()
        lib = C.CDLL(GPU_LIB)
        vp, i, u = C.c_void_p, C.c_int, C.c_uint
        lib.refgpu_error.restype = C.c_char_p
        lib.refgpu_load.argtypes = [C.c_char_p, C.c_char_p]
        lib.refgpu_run.argtypes = [i, i, vp, vp, u, u, u, u, u, vp, vp, u, i, vp, vp, vp, i, vp,
                                   i, vp, vp, vp, vp, vp]
        _gpu = lib
    want = CUBIN_KERNELS_NOFMA if nofma else CUBIN_KERNELS
    if _gpu_cubin != want:
        if not gpu_available():
            raise FileNotFoundError("reference cubins missing from oracle/_ref")
        if _gpu.refgpu_load(want.encode(), CUBIN_MESH.encode()) != 0:
            raise RuntimeError("refgpu_load: " + _gpu.refgpu_error().decode())
        _gpu_cubin = want
    return _gpu


def run_gpu(bid, mat, dims, scheme: str, table, params, src_idx, samples, rec_idx, steps: int,
            double: bool = False, nofma: bool = False, block=BLOCK, fields: bool = True):
    """The reference's kernels, compiled unchanged for sm_103a, run on GPU 0
    with launchFDTD3d's host sequence.  Returns (receivers, P, P_past,
    (air, boundary), summed update-kernel ms); P and P_past on the padded mesh
    (None if fields=False)."""
    lib = gpu(nofma)
    dt = np.float64 if double else np.float32
    X, Y, Z = (int(v) for v in dims)
    PX = X + (-X) % block[0]
    PY = Y + (-Y) % block[1]
    n = PX * PY * Z
    b = np.ascontiguousarray(bid, np.uint8).reshape(-1)
    m = np.ascontiguousarray(mat, np.uint8).reshape(-1)
    tab = np.ascontiguousarray(table, dtype=dt).reshape(-1)
    prm = np.ascontiguousarray(params, dtype=dt).reshape(-1)
    si = np.ascontiguousarray(src_idx, np.int64).reshape(-1)
    sh = np.ones(si.size, np.int32)
    smp = np.ascontiguousarray(np.asarray(samples, dtype=dt).reshape(si.size, -1)[:, :steps])
    if smp.shape[1] < steps:
        smp = np.ascontiguousarray(np.pad(smp, ((0, 0), (0, steps - smp.shape[1]))))
    ri = np.ascontiguousarray(rec_idx, np.int64).reshape(-1)
    rec = np.zeros((ri.size, steps), dt)
    P = np.zeros(n, dt) if fields else None
    Pp = np.zeros(n, dt) if fields else None
    counts = np.zeros(2, np.uint32)
    ms = C.c_float()
    rc = lib.refgpu_run(1 if double else 0, 0 if scheme == "forward" else 1, _vp(b), _vp(m), X, Y,
                        Z, block[0], block[1], _vp(prm), _vp(tab), tab.size // 20, si.size,
                        _vp(si), _vp(sh), _vp(smp), ri.size, _vp(ri), steps, _vp(rec), _vp(P),
                        _vp(Pp), _vp(counts), C.byref(ms))
    if rc != 0:
        raise RuntimeError("refgpu_run: " + lib.refgpu_error().decode())
    return rec, P, Pp, (int(counts[0]), int(counts[1])), float(ms.value)
