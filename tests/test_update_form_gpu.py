"""The difference form of the forward update (PFDTD_FORM_DIFFERENCE).

The form is an addition with no counterpart in the reference: the same
forward update, equal in exact arithmetic, written so that a uniform field
gives an exactly zero Laplacian.  It is checked bit for bit against the
oracle's statement of the same form, on every kernel path that runs it (FP32
fields, the one storage it is built for), and its receiver error against an
FP64 run is checked against a 1e-4 relative L2 bound, which the reference
form misses in FP32.
"""
import numpy as np
import pytest

from parallelfdtd_gb300 import rooms
from parallelfdtd_gb300 import _lib as L
from parallelfdtd_gb300.domain import Domain, default_params

HERE_TOL = 1e-4


@pytest.fixture(scope="module")
def O(built):
    from oracle import oracle
    return oracle


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


def c1():
    room = rooms.shoebox((64, 64, 64), n_materials=6, seed=1)
    steps = 500
    return room, steps, rooms.gaussian_pulse(steps, 5.0)


def test_oracle_difference_form_meets_fp64_bound(O):
    """CPU: 64^3 shoebox, 500 steps.  Reference form in float: ~5e-4 against
    FP64; difference form: ~2e-6."""
    room, steps, pulse = c1()
    pos, mat = O.encode_nodes(room.bid, room.mat, False)
    args = (pos, mat, room.dims, room.admittance, default_params(), [room.flat(32, 32, 32)], [1],
            pulse[None], [room.flat(16, 40, 24)], steps)
    r64, _, _ = O.run(*args, double=True)
    ref, _, _ = O.run(*args)
    dif, _, _ = O.run(*args, form="difference")
    assert rel_l2(ref, r64) > HERE_TOL
    assert rel_l2(dif, r64) < HERE_TOL / 10


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["f32"])
@pytest.mark.parametrize("variant", ["auto", "zmarch"])
def test_difference_form_equals_oracle(gpu, O, prec, variant):
    room = rooms.boxes_room((96, 64, 48), n_boxes=6, edge=(5, 14), n_materials=6, seed=41)
    steps = 160
    srcs = room.random_air_nodes(2, seed=3)
    rec = room.random_air_nodes(4, seed=4)
    pulse = rooms.gaussian_pulse(steps, 4.0)
    samples = np.stack([pulse, -0.5 * pulse])
    with Domain(room.dims, prec) as d:
        d.set_voxels(room.bid, room.mat, centred=False)
        d.set_materials(room.admittance)
        d.set_params()
        d.set_scheme("forward")
        d.set_update_form("difference")
        d.set_kernel(variant)
        d.set_sources(srcs, [1, 1], samples)
        d.set_receivers(rec)
        g, _, st = d.run(steps)
        assert st == 0
        assert d.kernel() == ("tma" if variant == "auto" else "zmarch")
        P = d.download_field(L.FIELD_CURRENT)
    pos, mat = O.encode_nodes(room.bid, room.mat, False)
    r, rP, _ = O.run(pos, mat, room.dims, room.admittance, default_params(),
                     [room.flat(*s) for s in srcs], [1, 1], samples, [room.flat(*x) for x in rec],
                     steps, storage=(None if prec == "f32" else prec), form="difference")
    assert np.abs(r).max() > 1e-4
    assert np.array_equal(g, r)
    if prec == "f32":
        assert np.array_equal(P, rP)
    else:
        assert np.array_equal(P.view(np.uint16), rP.view(np.uint16))


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["f32"])
def test_difference_form_batched_fields(gpu, O, prec):
    """K = 8 fields sharing the room: each field equals an oracle run of it
    alone in the difference form."""
    K, steps = 8, 120
    room = rooms.boxes_room((64, 48, 40), n_boxes=4, edge=(5, 12), n_materials=5, seed=42)
    srcs = room.random_air_nodes(K, seed=5)
    rec = room.random_air_nodes(K, seed=6)
    pulse = rooms.gaussian_pulse(steps, 3.0)
    samples = np.stack([pulse * (1 + 0.1 * i) for i in range(K)])
    with Domain(room.dims, prec, fields=K) as d:
        d.set_voxels(room.bid, room.mat, centred=False)
        d.set_materials(room.admittance)
        d.set_params()
        d.set_update_form("difference")
        d.set_sources(srcs, [1] * K, samples, fields=list(range(K)))
        d.set_receivers(rec, fields=list(range(K)))
        g, _, st = d.run(steps)
        assert st == 0
    pos, mat = O.encode_nodes(room.bid, room.mat, False)
    for f in (0, 5):
        r, _, _ = O.run(pos, mat, room.dims, room.admittance, default_params(),
                        [room.flat(*srcs[f])], [1], samples[f:f + 1], [room.flat(*rec[f])], steps,
                        storage=(None if prec == "f32" else prec), form="difference")
        assert np.array_equal(g[f], r[0]), f"field {f}"


@pytest.mark.gpu
def test_difference_form_c1_error_against_fp64(gpu, O):
    """The 64^3 shoebox (500 steps, soft Gaussian, receiver
    (16, 40, 24)): the difference form in FP32 on the GPU stays within 1e-4
    relative L2 of the FP64 run; the reference form does not."""
    room, steps, pulse = c1()
    out = {}
    for prec, form in (("f32", "reference"), ("f32", "difference"), ("f64", "reference")):
        with Domain(room.dims, prec) as d:
            d.set_voxels(room.bid, room.mat, centred=False)
            d.set_materials(room.admittance)
            d.set_params()
            d.set_update_form(form)
            d.set_sources([(32, 32, 32)], [1], pulse[None])
            d.set_receivers([(16, 40, 24)])
            out[(prec, form)], _, _ = d.run(steps)
    r64 = out[("f64", "reference")]
    assert rel_l2(out[("f32", "reference")], r64) > HERE_TOL
    assert rel_l2(out[("f32", "difference")], r64) < HERE_TOL / 10


@pytest.mark.gpu
def test_difference_form_refusals(gpu):
    from parallelfdtd_gb300 import materials
    for prec in ("f64", "f16", "bf16"):  # built for FP32 fields only
        with Domain((32, 16, 16), prec) as d:
            with pytest.raises(Exception):
                d.set_update_form("difference")
    room = rooms.shoebox((32, 16, 16), n_materials=6, seed=1)
    with Domain(room.dims, "f32") as d:
        d.set_voxels(room.bid, room.mat, centred=False)
        d.set_materials(room.admittance)
        d.set_dif_filters(np.ones(6, np.int32),
                          materials.dif_table(materials.positive_real_filters(6, 3, seed=1), 3))
        d.set_params()
        d.set_update_form("difference")
        d.set_sources([(16, 8, 8)], [1], rooms.impulse(10)[None])
        with pytest.raises(Exception):
            d.run(10)
