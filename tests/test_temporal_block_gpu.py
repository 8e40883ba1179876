"""GPU: the temporally blocked update (T steps per kernel) against the
per-step path and the oracle.

Blocking changes only the schedule: every node update keeps its arithmetic
and rounding, intermediate steps are rounded to the storage type, and the
sources and receivers of the intermediate steps are handled inside the
kernel.  Receiver traces and both fields must therefore be equal in value to
the per-step run (a zero on an x/y face node may differ in sign only).
"""
import numpy as np
import pytest

from parallelfdtd_gb300 import rooms
from parallelfdtd_gb300 import _lib as L
from parallelfdtd_gb300.domain import Domain, default_params

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def O(built):
    from oracle import oracle
    return oracle


def values(a, prec):
    """Field elements as float64 values (bf16 fields come back as raw bits)."""
    a = np.asarray(a)
    if prec == "bf16":
        return (a.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
    return a.astype(np.float64)


def run(room, prec, scheme, depth, srcs, recs, samples, steps, fields=1, src_fields=None,
        rec_fields=None, nodes=None, shape=-1):
    with Domain(room.dims, prec, fields=fields) as d:
        d.set_voxels(room.bid, room.mat, centred=(scheme != "forward"))
        if nodes is not None:
            d.set_nodes(*nodes)
        d.set_materials(room.admittance)
        d.set_params(default_params())
        d.set_scheme(scheme)
        d.set_sources([s[0] for s in srcs], [s[1] for s in srcs], samples, fields=src_fields)
        d.set_receivers(recs, fields=rec_fields)
        d.set_temporal_block(depth)
        d.set_tb_shape(shape)
        info = d.temporal_block()
        g, _, st = d.run(steps)
        assert st == 0
        P = d.download_field(L.FIELD_CURRENT)
        Pp = d.download_field(L.FIELD_PAST)
    return g, values(P, prec), values(Pp, prec), info


def room_a():
    # 136 x 100 x 70: several x/y tiles of the blocked kernel and z chunks
    return rooms.boxes_room((136, 100, 70), n_boxes=8, edge=(6, 20), n_materials=7,
                            admittance_range=(0.01, 0.9), seed=31)


# Sources and receivers on and next to the core boundaries of the blocked
# tiles (56 nodes x 28 rows for depth 2 unbatched), two sources on one node
# (order matters: hard then soft), one hard source.
def io_a(room):
    air = set(map(tuple, room.random_air_nodes(4000, seed=3)))
    want = [(56, 28, 30), (55, 27, 31), (57, 29, 29), (112, 56, 35), (60, 24, 1), (20, 30, 68),
            (3, 3, 5), (132, 96, 64)]
    pts = [p for p in want if p in air]
    extra = room.random_air_nodes(6, seed=4)
    pts = pts + [tuple(p) for p in extra]
    srcs = [(pts[0], 0), (pts[0], 1), (pts[1], 1), (pts[2], 1)]
    recs = pts[:] + [pts[0]]
    return srcs, recs


@pytest.mark.parametrize("prec", ["f32", "f16", "bf16"])
@pytest.mark.parametrize("scheme", ["forward", "centred"])
@pytest.mark.parametrize("depth", [2, 3, 4])
def test_blocked_equals_per_step(gpu, prec, scheme, depth):
    room = room_a()
    srcs, recs = io_a(room)
    steps = 131  # chunks of 48, blocked remainder, per-step remainder
    pulse = rooms.gaussian_pulse(steps, 3.0)
    samples = np.stack([pulse, -0.5 * pulse, pulse, 0.25 * pulse])
    g0, P0, Pp0, info0 = run(room, prec, scheme, 0, srcs, recs, samples, steps)
    g1, P1, Pp1, info1 = run(room, prec, scheme, depth, srcs, recs, samples, steps)
    assert info1[1], info1[2]
    assert np.abs(g0).max() > 1e-3
    assert np.array_equal(g1, g0), f"receivers differ, max |d| {np.abs(g1 - g0).max():.3e}"
    assert np.array_equal(P1, P0) and np.array_equal(Pp1, Pp0)


def test_blocked_matches_oracle(gpu, O):
    room = room_a()
    srcs, recs = io_a(room)
    steps = 97
    pulse = rooms.gaussian_pulse(steps, 3.0)
    samples = np.stack([pulse, -0.5 * pulse, pulse, 0.25 * pulse])
    g, P, Pp, info = run(room, "f32", "forward", 3, srcs, recs, samples, steps)
    assert info[1]
    pos, mat = O.encode_nodes(room.bid, room.mat, False)
    ref, rP, rPp = O.run(pos, mat, room.dims, room.admittance, default_params(),
                         [room.flat(*s[0]) for s in srcs], [s[1] for s in srcs], samples,
                         [room.flat(*r) for r in recs], steps)
    assert np.array_equal(g, ref)
    assert np.array_equal(P, rP) and np.array_equal(Pp, rPp)


@pytest.mark.parametrize("fields,prec,depth", [(4, "f32", 2), (8, "f16", 3), (16, "f32", 2),
                                               (16, "bf16", 4), (4, "f32", 4)])
def test_blocked_batched(gpu, fields, prec, depth):
    room = rooms.boxes_room((72, 60, 44), n_boxes=5, edge=(5, 14), n_materials=6, seed=22)
    steps = 103
    pulse = rooms.gaussian_pulse(steps, 3.0)
    pts = room.random_air_nodes(fields + 2 * fields, seed=7)
    srcs = [(tuple(p), 1) for p in pts[:fields]]
    recs = [tuple(p) for p in pts[fields:]]
    src_f = list(range(fields))
    rec_f = [i // 2 for i in range(2 * fields)]
    samples = np.stack([pulse * (1 + 0.1 * f) for f in range(fields)])
    g0, P0, Pp0, _ = run(room, prec, "forward", 0, srcs, recs, samples, steps, fields, src_f, rec_f)
    g1, P1, Pp1, info = run(room, prec, "forward", depth, srcs, recs, samples, steps, fields,
                            src_f, rec_f)
    assert info[1], info[2]
    assert np.array_equal(g1, g0)
    assert np.array_equal(P1, P0) and np.array_equal(Pp1, Pp0)


def test_blocked_falls_back(gpu):
    """An inside node on an x face (the reference's flat wrap reaches it) or a
    source on plane 0 keep the per-step path, with the reason reported."""
    room = rooms.boxes_room((64, 48, 40), n_boxes=3, edge=(5, 10), n_materials=4, seed=23)
    steps = 60
    pulse = rooms.gaussian_pulse(steps, 3.0)
    src = [(tuple(room.random_air_nodes(1, seed=1)[0]), 1)]
    rec = [tuple(room.random_air_nodes(1, seed=2)[0])]
    with Domain(room.dims, "f32") as d:
        d.set_voxels(room.bid, room.mat, centred=False)
        pos, mat = d.get_nodes()
    pos[room.flat(0, 20, 20)] = 0x86
    g0, *_ = run(room, "f32", "forward", 0, src, rec, pulse[None], steps, nodes=(pos, mat))
    g1, _, _, info = run(room, "f32", "forward", 2, src, rec, pulse[None], steps,
                         nodes=(pos, mat))
    assert not info[1] and "face" in info[2]
    assert np.array_equal(g0, g1)
    _, _, _, info = run(room, "f32", "forward", 2, [((10, 10, 0), 1)], rec, pulse[None], steps)
    assert not info[1] and "plane 0" in info[2]
    _, _, _, info = run(room, "f64", "forward", 2, src, rec, pulse[None], steps)
    assert not info[1] and "FP64" in info[2]


def test_blocked_depth_validation(gpu):
    with Domain((16, 16, 16), "f32") as d:
        for bad in (1, 5, -1):
            with pytest.raises(L.PfdtdError):
                d.set_temporal_block(bad)
        d.set_temporal_block(0)


@pytest.mark.parametrize("fields,depth,shape", [(1, 2, 1), (1, 2, 2), (1, 3, 1), (1, 3, 2),
                                                (1, 4, 1), (4, 2, 1), (8, 3, 1), (4, 4, 1)])
def test_blocked_shapes(gpu, fields, depth, shape):
    room = rooms.boxes_room((136, 100, 70), n_boxes=8, edge=(6, 20), n_materials=7, seed=31)
    steps = 77
    pulse = rooms.gaussian_pulse(steps, 3.0)
    pts = room.random_air_nodes(3 * fields, seed=8)
    srcs = [(tuple(p), 1) for p in pts[:fields]]
    recs = [tuple(p) for p in pts[fields:]]
    src_f = list(range(fields)) if fields > 1 else None
    rec_f = [i // 2 for i in range(2 * fields)] if fields > 1 else None
    samples = np.stack([pulse * (1 + 0.1 * f) for f in range(fields)])
    g0, P0, Pp0, _ = run(room, "f32", "forward", 0, srcs, recs, samples, steps, fields, src_f,
                         rec_f)
    g1, P1, Pp1, info = run(room, "f32", "forward", depth, srcs, recs, samples, steps, fields,
                            src_f, rec_f, shape=shape)
    assert info[1], info[2]
    assert np.array_equal(g1, g0)
    assert np.array_equal(P1, P0) and np.array_equal(Pp1, Pp0)


def test_blocked_missing_shape_fails(gpu):
    room = rooms.boxes_room((64, 48, 40), n_boxes=3, edge=(5, 10), n_materials=4, seed=23)
    with Domain(room.dims, "f32") as d:
        d.set_voxels(room.bid, room.mat, centred=False)
        d.set_materials(room.admittance)
        d.set_params(default_params())
        d.set_sources([tuple(room.random_air_nodes(1, seed=1)[0])], [1], np.ones((1, 60)))
        d.set_receivers([tuple(room.random_air_nodes(1, seed=2)[0])])
        d.set_temporal_block(4)
        d.set_tb_shape(0)  # depth 4 exists in shape 1 only
        with pytest.raises(L.PfdtdError):
            d.run(60)


def test_autotune_restores_fields_and_keeps_results(gpu):
    """The autotuner times configurations on the domain's own fields, puts the
    fields back, and the configuration it keeps gives the per-step results."""
    room = room_a()
    srcs, recs = io_a(room)
    steps = 90
    pulse = rooms.gaussian_pulse(steps, 3.0)
    samples = np.stack([pulse, -0.5 * pulse, pulse, 0.25 * pulse])
    g0, P0, Pp0, _ = run(room, "f32", "forward", 0, srcs, recs, samples, steps)
    with Domain(room.dims, "f32") as d:
        d.set_voxels(room.bid, room.mat, centred=False)
        d.set_materials(room.admittance)
        d.set_params(default_params())
        d.set_sources([s[0] for s in srcs], [s[1] for s in srcs], samples)
        d.set_receivers(recs)
        rnd = np.random.default_rng(0).standard_normal(d.n).astype(np.float32)
        d.upload_field(L.FIELD_CURRENT, rnd)
        depth, shape, ms = d.autotune(max_depth=4, iters=3)
        assert depth in (0, 2, 3, 4) and ms > 0
        assert np.array_equal(d.download_field(L.FIELD_CURRENT), rnd)
        d.reset_fields()
        g1, _, st = d.run(steps)
        assert st == 0
        assert np.array_equal(g1, g0)
        assert np.array_equal(values(d.download_field(L.FIELD_CURRENT), "f32"), P0)


def test_autotune_fields(gpu):
    """The field-count autotuner times every candidate K on the same room
    (each with its own best kernel configuration) and returns the K with the
    highest field-update rate."""
    from parallelfdtd_gb300.domain import autotune_fields
    room = rooms.boxes_room((128, 96, 64), n_boxes=5, edge=(6, 16), n_materials=6, seed=35)

    def setup(d):
        d.set_voxels(room.bid, room.mat, centred=False)
        d.set_materials(room.admittance)
        d.set_params(default_params())
        d.set_scheme("forward")

    K, depth, shape, rates = autotune_fields(room.dims, setup, "f32", candidates=(1, 4, 16),
                                             max_depth=3, iters=3)
    assert set(rates) == {1, 4, 16}
    assert K in rates and rates[K][0] == max(r[0] for r in rates.values())
    assert (depth, shape) == rates[K][1:]
    assert all(r[0] > 0 and r[1] in (0, 2, 3) for r in rates.values())
    print("field-update rates (G/s):", {k: round(v[0] / 1e9, 1) for k, v in rates.items()})


@pytest.mark.parametrize("prec", ["f32", "f16"])
def test_blocked_then_per_step_on_the_other_buffer_pair(gpu, prec):
    """A run whose blocked launches end on the second buffer pair and then
    takes per-step TMA updates there (X a multiple of 16 selects TMA)."""
    room = rooms.boxes_room((128, 96, 60), n_boxes=6, edge=(6, 16), n_materials=6, seed=33)
    pts = room.random_air_nodes(6, seed=9)
    srcs = [(tuple(pts[0]), 1), (tuple(pts[1]), 0)]
    recs = [tuple(p) for p in pts[2:]]
    steps = 48 + 3  # one chunk, one blocked launch (odd), one per-step update
    pulse = rooms.gaussian_pulse(steps, 3.0)
    samples = np.stack([pulse, 0.5 * pulse])
    g0, P0, Pp0, _ = run(room, prec, "forward", 0, srcs, recs, samples, steps)
    g1, P1, Pp1, info = run(room, prec, "forward", 2, srcs, recs, samples, steps)
    assert info[1], info[2]
    assert np.array_equal(g1, g0)
    assert np.array_equal(P1, P0) and np.array_equal(Pp1, Pp0)


# The packed-pair kernel for batched fields (tile shapes 2 and 3, two rows
# or one row per thread): 32 x 32 node
# tiles with cores of 32 - 2T, so this room (not a multiple of the core in x
# or y) has partial tiles on both far edges; sources and receivers sit on
# and next to core boundaries.
@pytest.mark.parametrize("fields,prec,depth,shape", [
    (4, "f32", 2, 2), (4, "f32", 3, 2), (16, "f32", 3, 2), (8, "f16", 3, 2), (16, "bf16", 2, 2),
    (4, "f32", 2, 3), (4, "f32", 3, 3), (16, "f32", 3, 3), (8, "f16", 3, 3), (16, "f16", 2, 3),
    (8, "bf16", 3, 3), (16, "bf16", 2, 3)])
def test_blocked_batched_packed(gpu, fields, prec, depth, shape):
    room = rooms.boxes_room((100, 76, 46), n_boxes=6, edge=(5, 14), n_materials=7, seed=41)
    steps = 101
    pulse = rooms.gaussian_pulse(steps, 3.0)
    air = set(map(tuple, room.random_air_nodes(6000, seed=5)))
    core = 32 - 2 * depth
    want = [(core - 1 + depth, core + depth, 20), (core + depth, core - 1 + depth, 21),
            (2 * core + depth, core + depth, 3), (30, 40, 44), (97, 73, 30)]
    edge = [p for p in want if p in air]
    pts = edge + [tuple(p) for p in room.random_air_nodes(3 * fields, seed=8)]
    srcs = [(pts[i], 1) for i in range(fields)]
    recs = pts[:3 * fields]
    src_f = list(range(fields))
    rec_f = [i % fields for i in range(3 * fields)]
    samples = np.stack([pulse * (1 + 0.1 * f) for f in range(fields)])
    g0, P0, Pp0, _ = run(room, prec, "forward", 0, srcs, recs, samples, steps, fields, src_f, rec_f)
    g1, P1, Pp1, info = run(room, prec, "forward", depth, srcs, recs, samples, steps, fields,
                            src_f, rec_f, shape=shape)
    assert info[1], info[2]
    assert np.abs(g0).max() > 1e-3
    assert np.array_equal(g1, g0), f"receivers differ, max |d| {np.abs(g1 - g0).max():.3e}"
    assert np.array_equal(P1, P0) and np.array_equal(Pp1, Pp0)
