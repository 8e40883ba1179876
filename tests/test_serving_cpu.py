"""CPU: request construction, footprint estimate and the serving trace."""
import numpy as np
import pytest

from parallelfdtd_gb300 import _lib as L
from parallelfdtd_gb300.serving import Request, serving_trace


def test_request_bytes_estimate(built):
    r = Request((64, 48, 40), 100, fields=4, precision="f32")
    r.set_voxels(np.zeros(64 * 48 * 40, np.uint8), np.zeros(64 * 48 * 40, np.uint8))
    r.set_receivers([(5, 5, 5)] * 8, fields=[0] * 8)
    b = r.bytes()
    n = 64 * 48 * 40
    assert b >= 2 * n * 4 * 4 + 3 * n + 8 * 100 * 4
    assert b < 2 * n * 4 * 4 + 3 * n + 8 * 100 * 4 + (8 << 20)
    r.set_temporal_block(2)
    assert r.bytes() > b + 2 * n * 4 * 4 - 1


def test_request_bytes_iwb(built):
    """IWB requests also hold the closed-neighbour masks and geometry codes
    (5 B per node) and, with one field, the closure-node records."""
    from parallelfdtd_gb300 import rooms
    room = rooms.boxes_room((64, 48, 40), n_boxes=3, edge=(5, 10), n_materials=4, seed=3)
    n = 64 * 48 * 40
    f = Request(room.dims, 100, precision="f32", scheme="forward").set_voxels(room.bid, room.mat)
    i = Request(room.dims, 100, precision="f32", scheme="iwb").set_voxels(room.bid, room.mat)
    assert i.bytes() >= f.bytes() + 5 * n


def test_request_bytes_split(built):
    """A request that runs field by field on one single-field domain (IWB
    with several fields, or fields without a source) needs the footprint of
    that domain; a forward request whose 4 fields all carry a source runs
    batched and holds all 4 fields."""
    from parallelfdtd_gb300 import rooms
    room = rooms.boxes_room((64, 48, 40), n_boxes=3, edge=(5, 10), n_materials=4, seed=3)
    n = 64 * 48 * 40
    pulse = np.zeros((4, 100))
    src = [(10 + 3 * i, 20, 20) for i in range(4)]

    def req(scheme, fields, n_src):
        r = Request(room.dims, 100, fields=fields, precision="f32", scheme=scheme)
        r.set_voxels(room.bid, room.mat)
        r.set_sources(src[:n_src], [1] * n_src, pulse[:n_src], fields=list(range(n_src)))
        r.set_receivers(src[:n_src], fields=list(range(n_src)))
        return r

    one = req("iwb", 1, 1).bytes()
    assert abs(req("iwb", 4, 4).bytes() - one) < 64 * 1024      # one single-field domain
    fwd1 = req("forward", 1, 1).bytes()
    assert abs(req("forward", 4, 3).bytes() - fwd1) < 64 * 1024  # a field without a source
    assert req("forward", 4, 4).bytes() > fwd1 + 6 * n * 4        # batched: 4 fields


def test_request_validation(built):
    with pytest.raises(L.PfdtdError):
        Request((64, 48, 2), 100)
    with pytest.raises(L.PfdtdError):
        Request((64, 48, 40), 100, fields=3)
    r = Request((16, 16, 16), 10)
    with pytest.raises(L.PfdtdError):
        r.set_temporal_block(5)
    r4 = Request((16, 16, 16), 10, fields=4)
    with pytest.raises(L.PfdtdError):  # a field the request does not have
        r4.set_sources([(5, 5, 5)], [1], np.zeros((1, 10)), fields=[4])
    with pytest.raises(L.PfdtdError):
        r4.set_receivers([(5, 5, 5)], fields=[-1])
    r4.set_sources([(5, 5, 5)], [1], np.zeros((1, 10)), fields=[3])


def test_serving_trace_is_seeded_and_bounded():
    a = serving_trace(200, seed=1)
    b = serving_trace(200, seed=1)
    assert a == b
    arr = np.array([t.arrival for t in a])
    assert np.all(np.diff(arr) > 0)
    rate = len(a) / arr[-1]
    assert 14 < rate < 27  # Poisson, mean 20 per second
    dims = np.array([t.dims for t in a])
    assert dims.min() >= 64 and dims.max() <= 512 and np.all(dims % 4 == 0)
    assert {t.scheme for t in a} == {"forward", "iwb"}
    steps = np.array([t.steps for t in a])
    assert steps.min() >= 500 and steps.max() <= 8000
    srcs = np.array([t.n_src for t in a])
    assert srcs.min() >= 1 and srcs.max() <= 16



def test_node_updates_count_source_fields(built):
    """A request's field count is rounded up to a power of two; only the
    fields that carry a source count as node-updates, and a request with
    fields without a source runs only the others (computed_updates), while a
    request whose every field carries a source runs them batched."""
    dims, steps = (32, 24, 20), 50
    r = Request(dims, steps, fields=16, precision="f32")
    r.set_voxels(np.zeros(32 * 24 * 20, np.uint8), np.zeros(32 * 24 * 20, np.uint8))
    pulse = np.zeros((9, steps))
    r.set_sources([(5, 5, 5)] * 9, [1] * 9, pulse, fields=list(range(9)))
    per_field = 32 * 24 * 18 * steps
    assert r.node_updates() == 9 * per_field
    assert r.computed_updates() == 9 * per_field
    full = Request(dims, steps, fields=4, precision="f32")
    full.set_sources([(5, 5, 5)] * 4, [1] * 4, pulse[:4], fields=list(range(4)))
    assert full.computed_updates() == full.node_updates() == 4 * per_field
    one = Request(dims, steps, fields=1)
    one.set_sources([(5, 5, 5)], [1], pulse[:1])
    assert one.node_updates() == per_field


def test_padded_rows_in_footprint(built):
    """A room whose field rows are not 16-byte aligned (FP16, X = 60) and whose
    x = X-1 face is closed runs on rows padded to 16 nodes: the footprint
    grows with them.  FP32 rows of 60 nodes are aligned: no padding, only the
    copy of the class ids with 16-byte rows."""
    from parallelfdtd_gb300 import rooms
    room = rooms.shoebox((60, 32, 24), seed=2)  # solid shell: x = X-1 face closed
    r = Request(room.dims, 40, precision="f16").set_voxels(room.bid, room.mat)
    r.set_receivers([(10, 10, 10)])
    b60 = r.bytes()
    room64 = rooms.shoebox((64, 32, 24), seed=2)
    r64 = Request(room64.dims, 40, precision="f16").set_voxels(room64.bid, room64.mat)
    r64.set_receivers([(10, 10, 10)])
    assert abs(b60 - r64.bytes()) < 64 * 32 * 24  # the padded domain holds 64-wide rows
    # a receiver past X keeps the room unpadded
    r.set_receivers([(61, 10, 10)])
    assert r.bytes() < b60
    f32 = Request(room.dims, 40, precision="f32").set_voxels(room.bid, room.mat)
    f32_64 = Request(room64.dims, 40, precision="f32").set_voxels(room64.bid, room64.mat)
    n60 = 60 * 32 * 24
    assert f32.bytes() - 2 * n60 < f32_64.bytes()  # unpadded, plus the class-id copy
