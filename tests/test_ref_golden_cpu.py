"""The oracle pinned to the reference's own code.  CPU only.

tests/golden/ref_fields.npz and ref_host_golden.txt were made by
tests/golden/make_ref_golden.py, which runs ParallelFDTD's own update,
padding and node-translation kernels (src/kernels/kernels3d.cu:485-529 and
:608-665, src/kernels/cudaMesh.cu:328-528) and host classes
(src/base/SimulationParameters.cpp, MaterialHandler.cpp, SrcRec.cpp),
compiled unchanged, with launchFDTD3d's step order.  Here the CPU oracle must
reproduce every one of those values bit for bit.  Where the reference sources
are mounted, a second set of seeded rooms is run through both on the spot.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from parallelfdtd_gb300 import rooms

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


@pytest.fixture(scope="module")
def O(built):
    from oracle import oracle
    return oracle


@pytest.fixture(scope="module")
def gold():
    z = np.load(os.path.join(GOLD, "ref_fields.npz"))
    meta = json.loads(str(z["meta"]))
    return meta, z


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def make_room(recipe):
    kind, dims, n, seed = recipe
    if kind == "shoebox":
        return rooms.shoebox(tuple(dims), n_materials=n, seed=seed)
    return rooms.boxes_room(tuple(dims), n_boxes=n, edge=(6, 24), n_materials=8, seed=seed)


def case_ids():
    z = np.load(os.path.join(GOLD, "ref_fields.npz"))
    return [c["name"] for c in json.loads(str(z["meta"]))["cases"]]


@pytest.mark.parametrize("name", case_ids())
def test_oracle_equals_reference_fields(O, gold, name):
    meta, z = gold
    case = next(c for c in meta["cases"] if c["name"] == name)
    room = make_room(case["room"])
    X, Y, _ = room.dims
    flat = lambda c: c[2] * X * Y + c[1] * X + c[0]  # noqa: E731
    centred = case["scheme"] == "centred"
    pos, mat = O.encode_nodes(room.bid, room.mat, centred)
    # the reference's addSample as run writes the sample alone; setSample too
    types = [1 if (s[3] == 1 and case["quirks"] & 2) else 0 for s in case["sources"]]
    rec, P, Pp = O.run(pos, mat, room.dims, z[f"{name}__table"], z[f"{name}__params"],
                       [flat(s[:3]) for s in case["sources"]], types, z[f"{name}__samples"],
                       [flat(r) for r in case["receivers"]], case["steps"],
                       scheme=2 if centred else 0, quirks=case["quirks"], double=case["double"])
    gold_rec = z[f"{name}__rec"]
    assert np.abs(gold_rec).max() > 1e-4
    assert np.array_equal(rec, gold_rec), f"receivers differ: max {np.abs(rec - gold_rec).max()}"
    assert sha(P) == case["P_sha"] and sha(Pp) == case["Pp_sha"]
    air, bnd = O.count_boundaries(pos, 0x80 if centred else 0x86)
    assert [air, bnd] == case["counts"]


def test_oracle_equals_reference_padding_and_encoding(O, gold):
    meta, _ = gold
    enc = meta["encode"]
    room = rooms.boxes_room((37, 21, 19), n_boxes=4, edge=(3, 8), n_materials=5, seed=9)
    for key, centred in (("forward", False), ("centred", True)):
        ppos, dims = O.pad(room.bid, room.dims, (32, 4, 1))
        pmat, _ = O.pad(room.mat, room.dims, (32, 4, 1))
        assert list(dims) == enc[key]["dims"]
        pos, mat = O.encode_nodes(ppos, pmat, centred)
        assert sha(pos) == enc[key]["pos_sha"] and sha(mat) == enc[key]["mat_sha"]
        assert list(O.count_boundaries(pos, 0x80 if centred else 0x86)) == enc[key]["counts"]
        ids = np.arange(28, dtype=np.uint8)
        p, m = O.encode_nodes(ids, np.full(28, 7, np.uint8), centred)
        assert [int(v) for v in p] + [int(v) for v in m] == enc["tables"][key]


def _host_lines():
    with open(os.path.join(GOLD, "ref_host_golden.txt")) as f:
        return [ln.split() for ln in f if ln.strip() and not ln.startswith("#")]


def test_oracle_source_samples_equal_reference(O):
    ir = np.loadtxt(os.path.join(GOLD, "grid_ir_kat.txt")).astype(np.float32)
    data = np.sin(np.arange(150) * 0.1) * np.linspace(1, 0, 150)
    n = 0
    for t in _host_lines():
        if t[0] != "samples":
            continue
        double = t[1] == "f64"
        st, it, fs, steps = (int(v) for v in t[2:6])
        want = np.array([float(v) for v in t[6:]], np.float64 if double else np.float32)
        got = O.source_vector(st, it, steps, fs=fs,
                              data=data.astype(np.float64 if double else np.float32),
                              grid_ir=ir if st == 2 else None, double=double)
        assert np.array_equal(got, want), (t[:6], np.abs(got - want).max())
        n += 1
    assert n == 48


def test_parameter_vectors_equal_reference():
    from parallelfdtd_gb300.domain import default_params
    seen = 0
    lines = _host_lines()
    for t in lines:
        if t[0] == "params":
            double = t[1] == "f64"
            want = np.array([float(v) for v in t[4:8]])
            got = default_params(octave=int(t[3]), scheme=t[2])
            if not double:
                got = got.astype(np.float32).astype(np.float64)
            assert np.array_equal(got, want), (t[:4], got, want)
            seen += 1
    assert seen == 8


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(HERE), "oracle", "_ref",
                                                    "libref_cpu.so")),
                    reason="the reference's own code is built only where its sources are mounted")
@pytest.mark.parametrize("seed", [21, 22, 23])
def test_oracle_equals_reference_random_rooms(O, seed):
    """Seeded rooms with odd sizes: the reference's own kernels (compiled for
    the host) and the oracle give the same receivers and fields bit for bit."""
    from oracle import ref
    from parallelfdtd_gb300.domain import default_params
    rng = np.random.default_rng(seed)
    dims = (32 * int(rng.integers(1, 3)), 4 * int(rng.integers(5, 12)), int(rng.integers(12, 30)))
    room = rooms.boxes_room(dims, n_boxes=5, edge=(3, 10), n_materials=4, seed=seed)
    X, Y, _ = room.dims
    steps = 80
    srcs = room.random_air_nodes(2, seed=seed + 1)
    recs = room.random_air_nodes(3, seed=seed + 2)
    flat = lambda c: c[2] * X * Y + c[1] * X + c[0]  # noqa: E731
    for scheme in ("forward", "centred"):
        for double in (False, True):
            dt = np.float64 if double else np.float32
            smp = np.stack([rooms.gaussian_pulse(steps, 3.0), rooms.impulse(steps)]).astype(dt)
            prm = default_params(octave=1).astype(dt)
            tab = room.admittance.astype(np.float32).astype(dt).reshape(-1)
            rr, rP, rPp = ref.run_cpu(room.bid, room.mat, room.dims, scheme, tab, prm,
                                      [flat(s) for s in srcs], smp, [flat(r) for r in recs],
                                      steps, double=double)
            pos, mat = O.encode_nodes(room.bid, room.mat, scheme == "centred")
            orr, oP, oPp = O.run(pos, mat, room.dims, tab, prm, [flat(s) for s in srcs], [0, 0],
                                 smp, [flat(r) for r in recs], steps,
                                 scheme=2 if scheme == "centred" else 0, double=double)
            assert np.array_equal(rr, orr), (scheme, double)
            assert np.array_equal(rP, oP) and np.array_equal(rPp, oPp), (scheme, double)
