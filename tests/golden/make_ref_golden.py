"""Golden vectors made by the reference's own code (ParallelFDTD), run here.

Needs the reference sources (PFDTD_REFERENCE_DIR, or where this container
mounts them): oracle/build_ref.py compiles its SimulationParameters /
MaterialHandler / SrcRec classes and its update, padding and node-translation
kernels, unchanged, for the host (oracle/_ref/libref_cpu.so), and
oracle/ref.py drives them with launchFDTD3d's step order
(src/kernels/kernels3d.cu:86-175).

Writes:
* ref_fields.npz — per case: the room recipe, the reference's source samples,
  parameter vector and material table, the receiver traces, the air/boundary
  counts and SHA-256 digests of both final fields (bit-exact checks of the
  whole mesh without storing it).
* ref_host_golden.txt — source samples of every source and input type in
  float and double, parameter vectors and a material table with repeated
  materials, as the reference's host classes give them; read by
  tests/cpp/golden_host_test.cpp and tests/test_ref_golden_cpu.py.

Run: python tests/golden/make_ref_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build_ref, ref  # noqa: E402
from parallelfdtd_gb300 import rooms  # noqa: E402

# Each field case: room recipe, scheme, precision, octave, the product quirk
# bits that reproduce the reference as it runs (PFDTD_QUIRK_MATIDX = 1 for the
# forward kernel's m*20*octave index at octave 0, PFDTD_QUIRK_SOFTSRC = 2 for a
# soft source that overwrites), sources (x, y, z, src_type, input_type,
# data index) and receivers.
FIELD_CASES = [
    dict(name="c1_forward_f32_asrun", room=("shoebox", (64, 64, 64), 6, 1), scheme="forward",
         double=False, octave=0, quirks=3, steps=500,
         sources=[(32, 32, 32, ref.SRC_SOFT, ref.DATA, 0)], receivers=[(16, 40, 24)],
         data="gauss5"),
    dict(name="c1_forward_f64_asrun", room=("shoebox", (64, 64, 64), 6, 1), scheme="forward",
         double=True, octave=0, quirks=3, steps=500,
         sources=[(32, 32, 32, ref.SRC_SOFT, ref.DATA, 0)], receivers=[(16, 40, 24)],
         data="gauss5"),
    dict(name="c1_forward_f32_octave1_hard", room=("shoebox", (64, 64, 64), 6, 1),
         scheme="forward", double=False, octave=1, quirks=0, steps=500,
         sources=[(32, 32, 32, ref.SRC_HARD, ref.DATA, 0)], receivers=[(16, 40, 24)],
         data="gauss5"),
    dict(name="boxes_forward_f32", room=("boxes", (128, 96, 64), 12, 5), scheme="forward",
         double=False, octave=1, quirks=0, steps=300,
         sources=[(40, 30, 20, ref.SRC_HARD, ref.IMPULSE, 0),
                  (90, 70, 44, ref.SRC_HARD, ref.GAUSSIAN, 0)],
         receivers="air4", data=None),
    dict(name="boxes_forward_f64", room=("boxes", (128, 96, 64), 12, 5), scheme="forward",
         double=True, octave=1, quirks=0, steps=300,
         sources=[(40, 30, 20, ref.SRC_HARD, ref.IMPULSE, 0),
                  (90, 70, 44, ref.SRC_HARD, ref.GAUSSIAN, 0)],
         receivers="air4", data=None),
    dict(name="boxes_forward_f32_asrun_soft", room=("boxes", (128, 96, 64), 12, 5),
         scheme="forward", double=False, octave=0, quirks=3, steps=300,
         sources=[(40, 30, 20, ref.SRC_SOFT, ref.GAUSSIAN, 0),
                  (90, 70, 44, ref.SRC_SOFT, ref.SINE, 0)],
         receivers="air4", data=None),
    dict(name="boxes_centred_f32", room=("boxes", (128, 96, 64), 12, 5), scheme="centred",
         double=False, octave=0, quirks=0, steps=300,
         sources=[(40, 30, 20, ref.SRC_HARD, ref.IMPULSE, 0),
                  (90, 70, 44, ref.SRC_HARD, ref.GAUSSIAN, 0)],
         receivers="air4", data=None),
    dict(name="boxes_centred_f64", room=("boxes", (128, 96, 64), 12, 5), scheme="centred",
         double=True, octave=0, quirks=0, steps=300,
         sources=[(40, 30, 20, ref.SRC_HARD, ref.IMPULSE, 0),
                  (90, 70, 44, ref.SRC_HARD, ref.GAUSSIAN, 0)],
         receivers="air4", data=None),
    dict(name="boxes_centred_f32_soft_sine", room=("boxes", (128, 96, 64), 12, 5),
         scheme="centred", double=False, octave=0, quirks=2, steps=300,
         sources=[(40, 30, 20, ref.SRC_SOFT, ref.SINE, 0)], receivers="air4", data=None),
]


def make_room(recipe):
    kind, dims, n, seed = recipe
    if kind == "shoebox":
        return rooms.shoebox(dims, n_materials=n, seed=seed)
    return rooms.boxes_room(dims, n_boxes=n, edge=(6, 24), n_materials=8, seed=seed)


def receivers_for(room, spec):
    if spec == "air4":
        return [tuple(int(v) for v in c) for c in room.random_air_nodes(4, seed=11)]
    return [tuple(c) for c in spec]


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def field_case(case):
    room = make_room(case["room"])
    recs = receivers_for(room, case["receivers"])
    dt = np.float64 if case["double"] else np.float32
    data = []
    if case["data"] == "gauss5":
        data = [rooms.gaussian_pulse(case["steps"], 5.0).astype(dt)]
    h = ref.host_setup(case["scheme"], case["octave"], case["steps"], room.admittance,
                       case["sources"], recs, data=data, double=case["double"])
    X, Y, _ = room.dims
    assert h["source_coords"] == [tuple(s[:3]) for s in case["sources"]], h["source_coords"]
    assert h["receiver_coords"] == recs, (h["receiver_coords"], recs)
    assert list(h["material_indices"]) == list(range(room.admittance.shape[0]))
    flat = [c[2] * X * Y + c[1] * X + c[0] for c in h["source_coords"]]
    rflat = [c[2] * X * Y + c[1] * X + c[0] for c in recs]
    rec, P, Pp = ref.run_cpu(room.bid, room.mat, room.dims, case["scheme"], h["table"],
                             h["params"], flat, h["samples"], rflat, case["steps"],
                             double=case["double"])
    _, _, pd, counts = ref.setup_mesh_cpu(room.bid, room.mat, room.dims, case["scheme"] != "forward")
    assert pd == tuple(room.dims)
    meta = {k: case[k] for k in ("name", "room", "scheme", "double", "octave", "quirks", "steps")}
    meta["sources"] = [list(s) for s in case["sources"]]
    meta["receivers"] = [list(r) for r in recs]
    meta["P_sha"] = sha(P)
    meta["Pp_sha"] = sha(Pp)
    meta["counts"] = list(counts)
    arrays = {"rec": rec, "samples": h["samples"], "params": h["params"], "table": h["table"]}
    return meta, arrays


def encode_case():
    room = rooms.boxes_room((37, 21, 19), n_boxes=4, edge=(3, 8), n_materials=5, seed=9)
    out = {}
    for centred in (False, True):
        pos, mat, pd, counts = ref.setup_mesh_cpu(room.bid, room.mat, room.dims, centred)
        key = "centred" if centred else "forward"
        out[key] = dict(dims=list(pd), pos_sha=sha(pos), mat_sha=sha(mat), counts=list(counts))
    ids = np.arange(28, dtype=np.uint8)
    tab = {}
    for centred in (False, True):
        pos, mat = ref.encode_cpu(ids, np.full(28, 7, np.uint8), centred)
        tab["centred" if centred else "forward"] = [int(v) for v in pos] + [int(v) for v in mat]
    out["tables"] = tab
    return out


def host_golden_lines():
    """Text lines: `data <prec> <n> v...` (the DATA input vector),
    `samples <prec> <src_type> <input_type> <fs> <n> v0 v1 ...` (transparent
    sources read tests/golden/grid_ir_kat.txt with readGridIr),
    `params <prec> <scheme> <octave> v0..v3`, `table <prec> <n_unique> <n_surf>
    idx... coefs...`.  Values printed with 17 significant digits."""
    lines = []
    steps = 200
    ir = os.path.abspath(os.path.join(HERE, "grid_ir_kat.txt"))
    data = (np.sin(np.arange(150) * 0.1) * np.linspace(1, 0, 150))
    for double in (False, True):
        prec = "f64" if double else "f32"
        dd = data.astype(np.float64 if double else np.float32)
        lines.append(f"data {prec} {dd.size} " + " ".join(repr(float(v)) for v in dd))
        for st in (ref.SRC_HARD, ref.SRC_SOFT, ref.SRC_TRANSPARENT):
            for it in (ref.IMPULSE, ref.GAUSSIAN, ref.SINE, ref.DATA):
                for fs in (7000, 10000):
                    h = ref.host_setup("forward", 0, steps, np.full((1, 20), 0.5),
                                       [(5, 5, 5, st, it, 0)], [],
                                       data=[data.astype(np.float64 if double else np.float32)],
                                       fs=fs, double=double,
                                       grid_ir=ir if st == ref.SRC_TRANSPARENT else None)
                    vals = " ".join(repr(float(v)) for v in h["samples"][0])
                    lines.append(f"samples {prec} {st} {it} {fs} {steps} {vals}")
        for scheme in ("forward", "centred"):
            for octave in (0, 3):
                h = ref.host_setup(scheme, octave, 4, np.full((1, 20), 0.5), [], [], double=double)
                vals = " ".join(repr(float(v)) for v in h["params"])
                lines.append(f"params {prec} {scheme} {octave} {vals}")
        rng = np.random.default_rng(4)
        uniq = rng.uniform(0.01, 0.9, size=(5, 20))
        surf = uniq[[0, 1, 2, 1, 3, 0, 4, 4, 2]]
        h = ref.host_setup("forward", 0, 4, surf, [], [], double=double)
        idx = " ".join(str(int(v)) for v in h["material_indices"])
        vals = " ".join(repr(float(v)) for v in h["table"])
        lines.append(f"table {prec} {h['table'].size // 20} {surf.shape[0]} {idx} {vals}")
        lines.append(f"surfaces {prec} {surf.shape[0]} "
                     + " ".join(repr(float(np.float32(v))) for v in surf.reshape(-1)))
    return lines


def main():
    if not build_ref.build():
        raise SystemExit("reference sources not found (set PFDTD_REFERENCE_DIR)")
    metas, arrays = [], {}
    for case in FIELD_CASES:
        meta, arr = field_case(case)
        metas.append(meta)
        for k, v in arr.items():
            arrays[f"{meta['name']}__{k}"] = v
        print(meta["name"], "peak", float(np.abs(arr["rec"]).max()))
    enc = encode_case()
    np.savez_compressed(os.path.join(HERE, "ref_fields.npz"),
                        meta=np.array(json.dumps({"cases": metas, "encode": enc})), **arrays)
    with open(os.path.join(HERE, "ref_host_golden.txt"), "w") as f:
        f.write("# Made by tests/golden/make_ref_golden.py from the reference's own host classes.\n")
        for line in host_golden_lines():
            f.write(line + "\n")
    print("wrote ref_fields.npz and ref_host_golden.txt")


if __name__ == "__main__":
    main()
