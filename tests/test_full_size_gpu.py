"""GPU parity at the benchmark configurations' own sizes and lengths.

The rooms, sources and receivers are those bench.py measures:
* 512 x 384 x 256 room with 40 boxes (edges 8-64) and 20 materials, soft
  impulse, 8 air receivers: SRL forward FP32 for the full 2000 steps and
  FP64 for 1000 steps; receivers and both final fields bit for bit against
  the oracle.
* the same grid, IWB at lambda = 1 with 3rd-order frequency-dependent walls
  on every material, FP32, 200 steps.
* 384 x 320 x 256 with K = 16 batched fields (one soft impulse each, 4
  receivers per field), 200 steps; two fields each against an independent
  oracle run of that field alone.
The oracle is run with every host thread.
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


def bench_room(dims, fields=1):
    room = rooms.boxes_room(dims, n_boxes=40, edge=(8, 64), n_materials=20,
                            admittance_range=(0.01, 0.9), seed=2)
    if fields == 1:
        return room, [room.random_air_nodes(1, seed=8)[0]], room.random_air_nodes(8, seed=9)
    return room, room.random_air_nodes(fields, seed=8), room.random_air_nodes(4 * fields, seed=9)


@pytest.mark.parametrize("prec,steps", [("f32", 2000), ("f64", 1000)])
def test_benchmark_room_full_length(gpu, O, prec, steps):
    room, src, rec = bench_room((512, 384, 256))
    dbl = prec == "f64"
    samples = rooms.impulse(steps)[None]
    with Domain(room.dims, prec) as d:
        d.set_voxels(room.bid, room.mat, centred=False)
        d.set_materials(room.admittance)
        d.set_params(default_params())
        d.set_scheme("forward")
        d.set_sources(src, [1], samples)
        d.set_receivers(rec)
        g, _, st = d.run(steps)
        assert st == 0
        P = d.download_field(L.FIELD_CURRENT)
        Pp = d.download_field(L.FIELD_PAST)
    pos, mat = O.encode_nodes(room.bid, room.mat, False)
    r, rP, rPp = O.run(pos, mat, room.dims, room.admittance, default_params(),
                       [room.flat(*src[0])], [1], samples, [room.flat(*x) for x in rec], steps,
                       double=dbl)
    assert np.abs(r).max() > 1e-6
    assert np.array_equal(g, r)
    assert np.array_equal(P, rP) and np.array_equal(Pp, rPp)


def test_iwb_dif_benchmark_grid(gpu, O):
    from parallelfdtd_gb300 import materials
    room, src, rec = bench_room((512, 384, 256))
    steps = 200
    n_mat = room.admittance.shape[0]
    flags = np.ones(n_mat, np.int32)
    table = materials.dif_table(materials.positive_real_filters(n_mat, 3, seed=77), 3)
    params = default_params(scheme="iwb")
    samples = rooms.impulse(steps)[None]
    with Domain(room.dims, "f32") as d:
        d.set_voxels(room.bid, room.mat, centred=True)
        d.set_materials(room.admittance)
        d.set_dif_filters(flags, table)
        d.set_params(params)
        d.set_scheme("iwb")
        d.set_sources(src, [1], samples)
        d.set_receivers(rec)
        g, _, st = d.run(steps)
        assert st == 0
        assert d.dif_count() > 0
        P = d.download_field(L.FIELD_CURRENT)
    pos, mat = O.encode_nodes(room.bid, room.mat, True)
    r, rP, _ = O.run(pos, mat, room.dims, room.admittance, params, [room.flat(*src[0])], [1],
                     samples, [room.flat(*x) for x in rec], steps, scheme=3, dif=(flags, table))
    assert np.abs(r).max() > 1e-6
    assert np.array_equal(g, r)
    assert np.array_equal(P, rP)


def test_batched_sixteen_fields(gpu, O):
    K, steps = 16, 200
    room, src, rec = bench_room((384, 320, 256), fields=K)
    src_f = list(range(K))
    rec_f = [i // 4 for i in range(4 * K)]
    samples = np.repeat(rooms.impulse(steps)[None], K, axis=0)
    with Domain(room.dims, "f32", fields=K) as d:
        d.set_voxels(room.bid, room.mat, centred=False)
        d.set_materials(room.admittance)
        d.set_params(default_params())
        d.set_scheme("forward")
        d.set_sources(src, [1] * K, samples, fields=src_f)
        d.set_receivers(rec, fields=rec_f)
        g, _, st = d.run(steps)
        assert st == 0
    pos, mat = O.encode_nodes(room.bid, room.mat, False)
    for f in (3, 12):
        mine = [i for i, rf in enumerate(rec_f) if rf == f]
        r, _, _ = O.run(pos, mat, room.dims, room.admittance, default_params(),
                        [room.flat(*src[f])], [1], samples[f:f + 1],
                        [room.flat(*rec[i]) for i in mine], steps)
        assert np.abs(r).max() > 1e-6
        assert np.array_equal(g[mine], r), f"field {f}"
