"""Benchmark of the FDTD time-stepping hot path (one JSON line on rank 0).

Workload (one "step" of this benchmark = one whole simulation): the
512 x 384 x 256 room (50.3M nodes) with a 1-voxel solid shell and 40 seeded
axis-aligned solid boxes (edges 8..64), 20 materials with admittance
U(0.01, 0.9), a soft impulse source, 8 seeded air-node receivers, 2000 leapfrog
steps of the SRL forward scheme in FP32.  Metric: node-updates/s, counting the
X*Y*(Z-2) nodes each leapfrog step updates.

  value  — device-resident: geometry and source table already in HBM, the
           2000-step run timed with CUDA events on the domain's stream.
  e2e    — through the C ABI with host buffers: node bytes and source table
           copied host->device, run, receiver traces copied back, every step.
  roofline — the update kernel alone, timed with CUDA events on the same
           stream: 14 algorithmic bytes per node-update (1 class byte is read
           in place of the reference's 2 node bytes, so actual traffic is 13 B).
  cpu_baseline — the C++ oracle (a restatement of the reference's update rule)
           on all host cores over a bounded sample of the same room.

Multi-GPU: the path is replicas only; each rank runs its own copy of the
workload on its own GPU (no collective in the data path), timing is the max
over ranks after a barrier.

--impl reference times the CPU restatement of the reference's own update rule
(the reference itself cannot be built here: it needs Boost, OpenGL and an
external voxelizer, and its gencodes predate nvcc 13).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "node-updates/s"
DIMS = (512, 384, 256)
FDTD_STEPS = 2000
N_REC = 8


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--precision", default="f32", choices=["f32", "f64", "f16", "bf16"])
    p.add_argument("--fdtd-steps", type=int, default=FDTD_STEPS)
    p.add_argument("--dims", type=str, default=None, help="X,Y,Z override (testing)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--cpu-seconds", type=float, default=12.0)
    p.add_argument("--serve", type=int, default=0,
                   help="serving workload: replay N requests of the seeded trace (Poisson "
                        "arrivals at 20/s, rooms U(64,512) per axis, SRL/IWB, FI/DIF, "
                        "500-8000 steps, 1-16 sources) through the request loop")
    p.add_argument("--serve-seed", type=int, default=0)
    p.add_argument("--serve-slots", type=int, default=8)
    p.add_argument("--serve-budget-gb", type=float, default=160.0)
    p.add_argument("--scheme", default="forward", choices=["forward", "centred", "iwb"],
                   help="update scheme (iwb: the 27-point compact scheme at lambda = 1)")
    p.add_argument("--dif", action="store_true",
                   help="3rd-order frequency-dependent admittance on every material (seeded "
                        "stable poles |p| < 0.95, positive real)")
    p.add_argument("--iwb-lambda", type=float, default=1.0,
                   help="Courant number of the IWB scheme (1 = its stability limit)")
    p.add_argument("--vs-f64", action="store_true",
                   help="also run the same workload with FP64 fields and report each "
                        "receiver's relative L2 error against it")
    p.add_argument("--form", choices=["reference", "difference"], default="reference",
                   help="arithmetic form of the forward update (difference: the same update "
                        "with less float roundoff; see pfdtd_set_update_form)")
    p.add_argument("--tb", type=int, default=0,
                   help="temporal block depth (0 = one update kernel per step; 2, 3, 4)")
    p.add_argument("--fields", type=int, default=1,
                   help="batched: K source fields sharing the room (the 384x320x256 multi-source "
                        "room, 4 receivers per field, when --dims is not given)")
    return p.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(value: float, world: int, device: str) -> float:
    """The largest of every rank's value (replicas are timed by the slowest
    rank); the value itself on one rank.  Needs an initialised process group
    when world > 1 (NCCL with a CUDA device, gloo with "cpu")."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(units_per_rank: float, world: int, seconds: float) -> float:
    """Whole-job rate of independent replicas: every rank's units over the
    slowest rank's time."""
    return units_per_rank * world / seconds


C4_DIMS = (384, 320, 256)
C4_STEPS = 4000


def make_room(dims, fields=1):
    """The benchmark room; for fields > 1 one seeded air source per field and
    4 receivers per field (the multi-source workload)."""
    from parallelfdtd_gb300 import rooms
    room = rooms.boxes_room(dims, n_boxes=40, edge=(8, 64), n_materials=20,
                            admittance_range=(0.01, 0.9), seed=2)
    if fields == 1:
        src = [room.random_air_nodes(1, seed=8)[0]]
        rec = room.random_air_nodes(N_REC, seed=9)
        return room, src, rec, [0], [0] * N_REC
    src = room.random_air_nodes(fields, seed=8)
    rec = room.random_air_nodes(4 * fields, seed=9)
    return room, src, rec, list(range(fields)), [i // 4 for i in range(4 * fields)]


def bytes_per_update(prec, fields):
    """Algorithmic bytes per node-update: 2 geometry bytes per node shared by
    the fields, read P^n and P^{n-1}, write P^{n+1} per field."""
    s = {"f32": 4, "f64": 8, "f16": 2, "bf16": 2}[prec]
    return (2 + 3 * s * fields) / fields


class ClockSampler:
    """nvidia-smi clock/throttle sampling while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.samples = []
        self._stop = threading.Event()
        self._proc = None

    def __enter__(self):
        try:
            self._proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self._proc = None
        return self

    def _read(self):
        for line in self._proc.stdout:
            parts = [s.strip() for s in line.split(",")]
            if len(parts) >= 9:
                self.samples.append(parts)

    def __exit__(self, *exc):
        if self._proc is not None:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except Exception:
                self._proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if s[5 + i].lower() == "active"})
        loaded = [v for v in sm if mx and v > 0.5 * max(mx)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


def peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_per_launch(prec, fields=1, scheme="forward"):
    """DRAM bytes per update-kernel launch from the committed ncu summaries
    (profiles/traffic.json); None where no capture of that kernel exists."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            t = json.load(f)
        if scheme == "iwb":
            return t.get(f"update_iwb_{prec}_bytes_per_launch") if fields == 1 else None
        if scheme != "forward":
            return None
        return t.get(f"update_{prec}_bytes_per_launch" if fields == 1 else
                     f"update_{prec}_k{fields}_bytes_per_launch")
    except Exception:
        return None


def cpu_baseline(room, src, rec, budget_s: float, fields=1):
    """Oracle on all host cores over a bounded number of steps of the room."""
    import numpy as np
    from oracle import oracle as O
    from parallelfdtd_gb300 import rooms
    from parallelfdtd_gb300.domain import default_params
    pos, mat = O.encode_nodes(room.bid, room.mat, centred=False)
    X, Y, Z = room.dims
    threads = O.max_threads()
    args = (pos, mat, room.dims, room.admittance, default_params(),
            [room.flat(*src[0])], [1])
    rec_idx = [room.flat(*r) for r in rec[:N_REC]]
    probe = 2
    t0 = time.perf_counter()
    O.run(*args, rooms.impulse(probe)[None], rec_idx, probe, threads=threads)
    per = (time.perf_counter() - t0) / probe
    n = max(2, min(200, int(budget_s / max(per, 1e-6))))
    t0 = time.perf_counter()
    O.run(*args, rooms.impulse(n)[None], rec_idx, n, threads=threads)
    dt = time.perf_counter() - t0
    # the same rule on one thread, a short sample
    n1 = 2
    t0 = time.perf_counter()
    O.run(*args, rooms.impulse(n1)[None], rec_idx, n1, threads=1)
    dt1 = time.perf_counter() - t0
    # the 64^3 shoebox of the contract (6 wall materials, soft Gaussian at the
    # centre, receiver (16, 40, 24)), all 500 steps
    box = rooms.shoebox((64, 64, 64), n_materials=6, seed=1)
    bpos, bmat = O.encode_nodes(box.bid, box.mat, centred=False)
    c1_steps = 500
    t0 = time.perf_counter()
    O.run(bpos, bmat, box.dims, box.admittance, default_params(), [box.flat(32, 32, 32)], [1],
          rooms.gaussian_pulse(c1_steps, 5.0)[None], [box.flat(16, 40, 24)], c1_steps,
          threads=threads)
    dtc1 = time.perf_counter() - t0
    return {"value": X * Y * (Z - 2) * n / dt, "unit": METRIC, "cores": threads,
            "kind": "port",
            "sample": f"{X}x{Y}x{Z} room, {n} leapfrog steps of one field, FP32 "
                      f"SRL forward, {threads} OpenMP threads",
            "one_thread": {"value": X * Y * (Z - 2) * n1 / dt1, "sample": f"{n1} steps"},
            "c1_shoebox": {"value": 64 * 64 * 62 * c1_steps / dtc1,
                           "sample": "64^3 shoebox, all 500 steps, FP32 SRL forward, "
                                     f"{threads} OpenMP threads"},
            "cpu_model": cpu_model()}


def cpu_model() -> str:
    """The host CPU's model name (lscpu), else the machine type."""
    import platform
    import subprocess
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return platform.processor() or platform.machine()


def run_reference_arm(a, world, rank):
    """--impl reference: the CPU restatement of the reference's update rule."""
    if rank != 0:
        return 0
    dims = tuple(int(v) for v in a.dims.split(",")) if a.dims else (C4_DIMS if a.fields > 1 else DIMS)
    room, src, rec, _, _ = make_room(dims)
    src = src[0]
    import numpy as np
    from oracle import oracle as O
    from parallelfdtd_gb300 import rooms
    from parallelfdtd_gb300.domain import default_params
    pos, mat = O.encode_nodes(room.bid, room.mat, centred=False)
    X, Y, Z = dims
    threads = O.max_threads()
    sample_steps = 10
    args = (pos, mat, dims, room.admittance, default_params(), [room.flat(*src)], [1],
            rooms.impulse(sample_steps)[None], [room.flat(*r) for r in rec], sample_steps)
    for _ in range(a.warmup):
        O.run(*args, threads=threads, double=(a.precision == "f64"))
    t0 = time.perf_counter()
    for _ in range(a.steps):
        O.run(*args, threads=threads, double=(a.precision == "f64"))
    dt = (time.perf_counter() - t0) / a.steps
    value = X * Y * (Z - 2) * sample_steps / dt
    sample = (f"{X}x{Y}x{Z} room, {sample_steps} leapfrog steps per benchmark step, "
              f"{a.precision.upper()} SRL forward, {threads} OpenMP threads")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": METRIC,
        "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup, "ms_per_step": dt * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": a.precision, "data": "synthetic",
        "config": {"workload": f"boxes room {X}x{Y}x{Z}, 40 boxes, 20 materials, soft impulse, "
                               f"{N_REC} receivers, SRL forward (CPU sample of {sample_steps} steps)",
                   "parallelism": "host threads", "l2": "inputs larger than L2"},
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_serving(a, world, rank, local):
    """Replay the seeded serving trace through the native request loop."""
    import concurrent.futures as cf
    import __graft_entry__ as g
    g.build()
    import torch
    from parallelfdtd_gb300.serving import Server, build_request, run_trace, serving_trace
    torch.cuda.set_device(local)
    trace = serving_trace(a.serve, seed=a.serve_seed + 1000 * rank)
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        reqs = list(ex.map(lambda it: build_request(it, a.precision), trace))
    budget = int(a.serve_budget_gb * (1 << 30))
    with ClockSampler(local) as clk:
        with Server(local, hbm_budget=budget, max_active=a.serve_slots) as srv:
            res = run_trace(srv, reqs, [it.arrival for it in trace])
    wall = res["wall_s"]
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        wall = max_over_ranks(wall, world, f"cuda:{local}")
        dist.destroy_process_group()
    st = res["stats"]
    if rank == 0:
        line = {
            "metric": METRIC, "value": replica_rate(res["node_updates"], world, wall),
            "unit": METRIC,
            "n_gpus": world, "steps": len(trace), "warmup": 0,
            "ms_per_step": wall * 1e3 / len(trace), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": a.precision,
            "data": "synthetic",
            "config": {"workload": f"serving trace of {len(trace)} requests (seed "
                                   f"{a.serve_seed}): Poisson arrivals 20/s, per-axis sizes "
                                   "U(64,512), SRL forward / IWB 50/50, FI / 3rd-order DIF "
                                   "50/50, steps U(500,8000), 1-16 sources (one field each, "
                                   "4 receivers per source)",
                       "hbm_budget_gb": a.serve_budget_gb, "slots": a.serve_slots,
                       "parallelism": f"replicas x{world}"},
            "latency": {k: res[k] for k in ("latency_p50_s", "latency_p99_s", "queue_p50_s",
                                            "queue_p99_s", "service_p50_s", "service_p99_s")},
            "e2e": {"value": res["node_updates"] * world / wall, "unit": METRIC,
                    "h2d_bytes_per_step": None, "d2h_bytes_per_step": None},
            "server": {k: st[k] for k in ("completed", "failed", "max_running", "bytes_peak",
                                             "setup_seconds", "retire_seconds")},
            "work": {"requests": res["requests"],
                     "node_updates": res["node_updates"],
                     "computed_node_updates": res["computed_updates"],
                     "note": "value counts the fields that carry a source; a request's field "
                             "count is rounded up to a power of two, and a request with "
                             "fields without a source (or IWB, or 2 fields) runs its source "
                             "fields one after another on a single-field domain"},
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    return 0


def main():
    a = parse()
    world, rank, local = dist_env()
    if a.impl == "reference":
        return run_reference_arm(a, world, rank)
    if a.serve:
        return run_serving(a, world, rank, local)

    import numpy as np
    import torch
    import __graft_entry__ as g
    g.build()
    from parallelfdtd_gb300 import _lib as L
    from parallelfdtd_gb300 import rooms
    from parallelfdtd_gb300.domain import Domain, default_params

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    K = a.fields
    dims = tuple(int(v) for v in a.dims.split(",")) if a.dims else (C4_DIMS if K > 1 else DIMS)
    S = a.fdtd_steps if (a.fdtd_steps != FDTD_STEPS or K == 1) else C4_STEPS
    room, src, rec, src_f, rec_f = make_room(dims, K)
    n_rec = len(rec)
    X, Y, Z = dims
    updates_per_run = X * Y * (Z - 2) * S * K
    prec = a.precision
    samples = np.repeat(rooms.impulse(S)[None], len(src), axis=0).astype(
        np.float64 if prec == "f64" else np.float32)
    esize = {"f32": 4, "f64": 8, "f16": 2, "bf16": 2}[prec]
    dif = None
    if a.dif:
        from parallelfdtd_gb300 import materials
        n_mat = room.admittance.shape[0]
        dif = (np.ones(n_mat, np.int32),
               materials.dif_table(materials.positive_real_filters(n_mat, 3, seed=77), 3))

    def setup(dom, float_params=False):
        # float_params: the material, filter and scheme parameters rounded to
        # float first, as every FP32-arithmetic run holds them
        rnd = (lambda v: np.asarray(v, np.float64).astype(np.float32).astype(np.float64)) \
            if float_params else (lambda v: v)
        dom.set_voxels(room.bid, room.mat, centred=(a.scheme != "forward"))
        dom.set_materials(rnd(room.admittance))
        if dif is not None:
            dom.set_dif_filters(dif[0], rnd(dif[1]))
        dom.set_params(rnd(default_params(scheme=a.scheme,
                                          lam=a.iwb_lambda if a.scheme == "iwb" else None)))
        dom.set_scheme(a.scheme)
        if a.form != "reference" and dom.precision != 1:  # the FP64 comparison run keeps
            dom.set_update_form(a.form)                    # the reference form

    d = Domain(dims, prec, device=local, fields=K)
    setup(d)
    pos_host, mat_host = d.get_nodes()
    d.set_sources(src, [1] * len(src), samples, fields=src_f)
    d.set_receivers(rec, fields=rec_f)
    d.set_temporal_block(a.tb)
    tb_info = d.temporal_block()
    if a.tb and not tb_info[1]:
        raise SystemExit(f"temporal blocking requested but inactive: {tb_info[2]}")
    stream = torch.cuda.ExternalStream(d.stream_ptr())
    d_out = torch.zeros(n_rec * S, dtype=torch.float64 if prec == "f64" else torch.float32,
                        device=f"cuda:{local}")

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    def run_device():
        L.call("pfdtd_run_device", d.handle, S, d_out.data_ptr())

    # ---- device-resident timing ------------------------------------------
    for _ in range(a.warmup):
        run_device()
    barrier()
    l0 = L.load().pfdtd_kernel_launches()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        with torch.cuda.stream(stream):
            ev0.record(stream)
        for _ in range(a.steps):
            run_device()
        with torch.cuda.stream(stream):
            ev1.record(stream)
        barrier()
    launches = L.load().pfdtd_kernel_launches() - l0
    ms = ev0.elapsed_time(ev1) / a.steps
    ms = max_over_ranks(ms, world, f"cuda:{local}")
    value = replica_rate(updates_per_run, world, ms * 1e-3)

    # ---- dominant kernel alone (same stream, same arguments) ---------------
    prof_iters = 50
    k0, k1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        k0.record(stream)
    import ctypes as C
    L.call("pfdtd_profile_update", d.handle, prof_iters)
    with torch.cuda.stream(stream):
        k1.record(stream)
    torch.cuda.synchronize()
    kms = k0.elapsed_time(k1) / prof_iters
    nodes = X * Y * (Z - 2)
    bpu = bytes_per_update(prec, K)
    T = a.tb if a.tb else 1
    n_dif = d.dif_count() if a.dif else 0
    if T > 1:
        # a blocked launch advances T steps; its compulsory traffic is one
        # read of P^n, P^{n-1} and the class ids and one write of the two
        # output levels (4 field passes + 1 byte per node)
        algo_bytes = (4 * esize * K + 1) * nodes
    else:
        algo_bytes = bpu * nodes * K
    achieved = algo_bytes / (kms * 1e-3) / 1e9
    effective = bpu * nodes * K * T / (kms * 1e-3) / 1e9
    peak, peak_kind = peak_hbm()
    traffic = traffic_per_launch(prec, K, a.scheme)
    kernel_name = "k_update_" + d.kernel()
    in_kernel_closure = os.environ.get("PFDTD_TMA_TILE", "-1").strip() in ("0", "1", "2", "3", "4", "5")
    if a.scheme == "iwb" and d.kernel() == "tma" and not in_kernel_closure:
        kernel_name += " + k_iwb_closure"  # the update of a step: both kernels, timed together

    # ---- end to end through the C ABI with host buffers ------------------------
    out_host = np.zeros((n_rec, S), dtype=np.float64 if prec == "f64" else np.float32)
    for _ in range(max(1, a.warmup)):
        d.set_nodes(pos_host, mat_host)
        d.set_sources(src, [1] * len(src), samples, fields=src_f)
        d.reset_fields()
        d.run(S, out=out_host)
    barrier()
    t0 = time.perf_counter()
    for _ in range(a.steps):
        d.set_nodes(pos_host, mat_host)
        d.set_sources(src, [1] * len(src), samples, fields=src_f)
        d.reset_fields()
        d.run(S, out=out_host)
    barrier()
    e2e_s = (time.perf_counter() - t0) / a.steps
    e2e_s = max_over_ranks(e2e_s, world, f"cuda:{local}")
    e2e = {"value": replica_rate(updates_per_run, world, e2e_s), "unit": METRIC,
           "h2d_bytes_per_step": int(2 * room.n_nodes + samples.nbytes),
           "d2h_bytes_per_step": int(n_rec * S * (8 if prec == "f64" else 4))}

    err64 = None
    if a.vs_f64 and prec != "f64":
        ref = np.zeros((n_rec, S), dtype=np.float64)
        with Domain(dims, "f64", device=local, fields=K) as d64:
            setup(d64)
            d64.set_sources(src, [1] * len(src), samples.astype(np.float64), fields=src_f)
            d64.set_receivers(rec, fields=rec_f)
            d64.run(S, out=ref)
        num = np.linalg.norm(out_host.astype(np.float64) - ref, axis=1)
        den = np.maximum(np.linalg.norm(ref, axis=1), 1e-300)
        e = num / den
        err64 = {"max_rel_l2": float(e.max()), "median_rel_l2": float(np.median(e)),
                 "per_receiver": [float(v) for v in e]}
        # The same FP64 run with the parameters rounded to float (lambda,
        # lambda^2, admittances, filters), as this run holds them: what is
        # left is the arithmetic and storage rounding alone.
        ref2 = np.zeros((n_rec, S), dtype=np.float64)
        with Domain(dims, "f64", device=local, fields=K) as d64:
            setup(d64, float_params=True)
            d64.set_sources(src, [1] * len(src), samples.astype(np.float64), fields=src_f)
            d64.set_receivers(rec, fields=rec_f)
            d64.run(S, out=ref2)
        e2 = np.linalg.norm(out_host.astype(np.float64) - ref2, axis=1) / \
            np.maximum(np.linalg.norm(ref2, axis=1), 1e-300)
        err64["same_float_parameters"] = {"max_rel_l2": float(e2.max()),
                                          "median_rel_l2": float(np.median(e2))}

    if rank == 0:
        base = None
        if not a.no_cpu_baseline and world == 1 and a.scheme == "forward" and not a.dif:
            base = cpu_baseline(room, src, rec, a.cpu_seconds)
        src_txt = (f"soft impulse, {N_REC} air receivers" if K == 1 else
                   f"{K} fields (one soft impulse each), 4 receivers per field")
        line = {
            "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": prec, "data": "synthetic",
            "config": {"workload": f"boxes room {X}x{Y}x{Z}, 40 boxes (edges 8-64), 20 materials "
                                   f"U(0.01,0.9){', 3rd-order DIF admittance' if a.dif else ''}"
                                   f", {src_txt}, {S} leapfrog steps, "
                                   f"{ {'forward': 'SRL forward', 'centred': 'SRL centred', 'iwb': 'IWB 27-point'}[a.scheme]}, "
                                   f"{prec}",
                       "scheme": a.scheme, "dif_nodes": int(n_dif),
                       "courant": float(default_params(scheme=a.scheme, lam=a.iwb_lambda
                                                       if a.scheme == "iwb" else None)[0]),
                       "fdtd_steps_per_step": S, "nodes": X * Y * Z, "fields": K,
                       "temporal_block": a.tb, "update_form": a.form,
                       "bytes_per_update": bpu,
                       "parallelism": f"replicas x{world}",
                       "l2": f"inputs larger than L2 (fields 2 x {X * Y * Z * K * esize / 1e6:.0f} MB "
                             f"+ {X * Y * Z / 1e6:.0f} MB class ids)"},
            "e2e": e2e,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": kernel_name, "kernel_ms": kms,
                         "algorithmic_bytes_per_launch": algo_bytes,
                         "steps_per_launch": T,
                         "effective_gbs": effective,
                         "peak_kind": f"of {peak_kind}"},
            "clocks": clk.summary(),
            "gpu_launches": int(launches),
            "cpu_baseline": base,
        }
        if err64 is not None:
            line["error_vs_f64"] = err64
        print(json.dumps(line), flush=True)
    d.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
