"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

The kernels evaluate the reference's update rule with every product and sum
rounded separately and the per-class coefficients computed with the
reference's expressions, so receiver traces and fields are expected to be
bit-identical to the oracle (compiled with -ffp-contract=off).  The parity
tolerance of the path (relative L2 <= 1e-5 for FP32, <= 1e-12 for FP64) is
checked as well and reported on failure.
"""
import os

import numpy as np
import pytest

from parallelfdtd_gb300 import rooms
from parallelfdtd_gb300 import _lib as L
from parallelfdtd_gb300.domain import Domain, default_params

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
TOL = {"f32": 1e-5, "f64": 1e-12}


@pytest.fixture(scope="module")
def O(built):
    from oracle import oracle
    return oracle


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


def assert_parity(gpu, ref, prec):
    err = rel_l2(gpu, ref)
    assert err <= TOL[prec], f"relative L2 {err:.3e} > {TOL[prec]}"
    assert np.array_equal(gpu, ref), f"not bit-identical (relative L2 {err:.3e})"


def run_both(O, room, prec, centred, srcs, rec, samples, steps, quirks=0, params=None):
    params = default_params() if params is None else params
    dbl = prec == "f64"
    with Domain(room.dims, prec) as d:
        d.set_voxels(room.bid, room.mat, centred=centred)
        d.set_materials(room.admittance)
        d.set_params(params)
        d.set_scheme("centred" if centred else "forward")
        d.set_quirks(quirks)
        d.set_sources([s[0] for s in srcs], [s[1] for s in srcs], samples)
        d.set_receivers(rec)
        gpu, _, st = d.run(steps)
        assert st == 0
        P = d.download_field(L.FIELD_CURRENT)
        Pp = d.download_field(L.FIELD_PAST)
    pos, mat = O.encode_nodes(room.bid, room.mat, centred)
    ref, rP, rPp = O.run(pos, mat, room.dims, room.admittance, params,
                         [room.flat(*s[0]) for s in srcs], [s[1] for s in srcs], samples,
                         [room.flat(*r) for r in rec], steps, scheme=2 if centred else 0,
                         quirks=quirks, double=dbl)
    return gpu, ref, (P, Pp), (rP, rPp)


def c1_room():
    return rooms.shoebox((64, 64, 64), n_materials=6, admittance_range=(0.01, 0.5), seed=1)


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_c1_shoebox_forward(gpu, O, prec):
    """64^3 shoebox, 6 wall materials, soft Gaussian (sigma 5) at the centre,
    receiver (16, 40, 24), 500 steps, SRL forward."""
    room = c1_room()
    steps = 500
    pulse = rooms.gaussian_pulse(steps, 5.0)
    g, r, (P, Pp), (rP, rPp) = run_both(O, room, prec, False, [((32, 32, 32), 1)],
                                        [(16, 40, 24)], pulse[None], steps)
    assert np.abs(r).max() > 1e-4
    assert_parity(g, r, prec)
    assert np.array_equal(P, rP) and np.array_equal(Pp, rPp)


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_centred_boxes_room(gpu, O, prec):
    room = rooms.boxes_room((96, 64, 48), n_boxes=8, edge=(6, 20), n_materials=12, seed=4)
    steps = 300
    srcs = [(p, 1) for p in room.random_air_nodes(2, seed=1)]
    rec = room.random_air_nodes(4, seed=2)
    pulse = rooms.gaussian_pulse(steps, 4.0)
    g, r, (P, _), (rP, _) = run_both(O, room, prec, True, srcs, rec,
                                     np.stack([pulse, -0.5 * pulse]), steps)
    assert_parity(g, r, prec)
    assert np.array_equal(P, rP)


@pytest.mark.parametrize("quirks", [L.QUIRK_MATIDX, L.QUIRK_SOFTSRC,
                                    L.QUIRK_MATIDX | L.QUIRK_SOFTSRC])
def test_reference_quirks(gpu, O, quirks):
    room = rooms.shoebox((40, 36, 32), seed=5)
    steps = 200
    pulse = rooms.gaussian_pulse(steps, 4.0)
    g, r, _, _ = run_both(O, room, "f32", False, [((20, 18, 16), 1)], [(8, 9, 10)],
                          pulse[None], steps, quirks=quirks)
    assert_parity(g, r, "f32")


def test_octave_selects_coefficient(gpu, O):
    room = rooms.shoebox((40, 36, 32), seed=5)
    room.admittance[:, 3] *= 0.5
    steps = 150
    pulse = rooms.gaussian_pulse(steps, 4.0)
    params = default_params(octave=3)
    for centred in (False, True):
        g, r, _, _ = run_both(O, room, "f32", centred, [((20, 18, 16), 1)], [(8, 9, 10)],
                              pulse[None], steps, params=params)
        assert_parity(g, r, "f32")


def test_golden_fixture(gpu, O):
    g = np.load(os.path.join(HERE, "golden", "oracle_small.npz"))
    room = rooms.Room(tuple(int(v) for v in g["dims"]), g["bid"], g["mat"], g["admittance"])
    pulse = g["pulse"]
    srcs = [(tuple(int(v) for v in g["src"][0]), 1), (tuple(int(v) for v in g["src"][1]), 0)]
    rec = [tuple(int(v) for v in r) for r in g["rec"]]
    for centred in (False, True):
        for prec in ("f32", "f64"):
            with Domain(room.dims, prec) as d:
                d.set_voxels(room.bid, room.mat, centred)
                d.set_materials(room.admittance)
                d.set_params()
                d.set_scheme("centred" if centred else "forward")
                d.set_sources([s[0] for s in srcs], [s[1] for s in srcs],
                              np.stack([pulse, 0.5 * pulse]))
                d.set_receivers(rec)
                out, _, _ = d.run(pulse.size)
            key = f"rec_{'centred' if centred else 'forward'}_{prec}"
            assert np.array_equal(out, g[key]), key


def test_multiple_sources_same_node_in_order(gpu, O):
    """Hard then soft source at one node: applied in source order."""
    room = rooms.shoebox((32, 30, 28), seed=6)
    steps = 120
    pulse = rooms.gaussian_pulse(steps, 3.0)
    srcs = [((10, 10, 10), 0), ((10, 10, 10), 1), ((20, 15, 12), 2)]
    g, r, _, _ = run_both(O, room, "f32", False, srcs, [(10, 10, 10), (5, 5, 5)],
                          np.stack([pulse, 0.25 * pulse, -pulse]), steps)
    assert_parity(g, r, "f32")


def test_odd_sizes_and_edges(gpu, O):
    """X not a multiple of 32, Z = 3 (a single updated plane), receivers and
    sources outside the grid are skipped, step counts around the graph chunk."""
    for dims, steps in [((37, 13, 11), 51), ((33, 7, 3), 7), ((5, 5, 64), 101)]:
        room = rooms.shoebox(dims, seed=7)
        X, Y, Z = dims
        pulse = rooms.gaussian_pulse(steps, 2.0, t0=6.0)
        src = (X // 2, Y // 2, Z // 2)
        g, r, (P, Pp), (rP, rPp) = run_both(
            O, room, "f32", False, [(src, 1), ((1, 1, Z + 5), 1)],
            [src, (1, 1, Z), (X - 2, Y - 2, max(Z - 2, 1))], np.stack([pulse, pulse]), steps)
        assert np.array_equal(g, r)
        assert (g[1] == 0).all()
        assert np.array_equal(P, rP) and np.array_equal(Pp, rPp)


def test_full_size_grid_short_run(gpu, O):
    """The 512 x 384 x 256 room with 40 boxes, 20 materials: bit-identical
    receivers and fields after a short run (the full 2000-step run is in
    tests/test_full_size_gpu.py and tests/test_ref_parity_gpu.py)."""
    room = rooms.boxes_room((512, 384, 256), n_boxes=40, edge=(8, 64), n_materials=20, seed=2)
    steps = 12
    rec = room.random_air_nodes(8, seed=9)
    src = room.random_air_nodes(1, seed=8)[0]
    g, r, (P, _), (rP, _) = run_both(O, room, "f32", False, [(src, 1)], rec,
                                     rooms.impulse(steps)[None], steps)
    assert np.array_equal(g, r)
    assert np.array_equal(P, rP)


def test_step_mode_equals_run(gpu, O):
    room = rooms.shoebox((40, 36, 32), seed=3)
    steps = 60
    pulse = rooms.gaussian_pulse(steps, 3.0).astype(np.float32)
    rec = [(8, 9, 10), (30, 20, 25)]
    with Domain(room.dims, "f32") as d:
        d.set_voxels(room.bid, room.mat, False)
        d.set_materials(room.admittance)
        d.set_params()
        d.set_sources([(20, 18, 16)], [1], pulse[None])
        d.set_receivers(rec)
        run_out, _, _ = d.run(steps)
        P_run = d.download_field(L.FIELD_CURRENT)
        d.reset_fields()
        step_out = np.zeros((2, steps), np.float32)
        for s in range(steps):
            d.step(s, 1, step_out, steps)
        P_step = d.download_field(L.FIELD_CURRENT)
    assert np.array_equal(run_out, step_out)
    assert np.array_equal(P_run, P_step)


def test_time_reversal_step_direction(gpu, O):
    """A change of step direction skips the swap (kernels3d.cu:462-465)."""
    room = rooms.shoebox((24, 20, 18), seed=3)
    with Domain(room.dims, "f32") as d:
        d.set_voxels(room.bid, room.mat, False)
        d.set_materials(room.admittance)
        d.set_params()
        pulse = rooms.gaussian_pulse(30, 2.0, 5.0)
        pulse[10:] = 0.0  # nothing injected at the reversed step
        d.set_sources([(12, 10, 9)], [1], pulse[None])
        for s in range(10):
            d.step(s, 1)
        a = d.download_field(L.FIELD_CURRENT)
        d.step(10, -1)  # direction changed: no swap, current field unchanged
        b = d.download_field(L.FIELD_CURRENT)
    assert np.array_equal(a, b)


def test_samples_and_flip(gpu):
    room = rooms.shoebox((20, 20, 20), seed=1)
    with Domain(room.dims, "f32") as d:
        d.set_sample(0, 0, 0, 3.0)
        assert d.get_sample(0, 0, 0) == 3.0
        d.add_sample(0, 0, 0, 3.0)
        assert d.get_sample(0, 0, 0) == 6.0  # tests/CudaMeshTest.cpp:308-318
        d.set_sample(7, 7, 7, 1.0)
        assert d.get_sample(7, 7, 7) == 1.0
        d.flip()
        assert d.get_sample(7, 7, 7) == 0.0
        d.flip()
        assert d.get_sample(7, 7, 7) == 1.0
        d.reset_fields()
        assert d.get_sample(7, 7, 7) == 0.0
        with pytest.raises(L.PfdtdError):
            d.get_sample(0, 0, 25)


def test_device_setup_matches_oracle(gpu, O):
    room = rooms.boxes_room((64, 40, 36), n_boxes=6, edge=(4, 12), seed=12)
    for centred in (False, True):
        with Domain(room.dims, "f32") as d:
            d.set_voxels(room.bid, room.mat, centred)
            pos, mat = d.get_nodes()
            air_value = 0x80 if centred else 0x86
            counts = d.count_boundaries(air_value)
        rpos, rmat = O.encode_nodes(room.bid, room.mat, centred)
        assert np.array_equal(pos, rpos) and np.array_equal(mat, rmat)
        assert counts == O.count_boundaries(rpos, air_value)


def test_device_padding_matches_oracle(gpu, O, lib):
    import ctypes as C
    rng = np.random.default_rng(0)
    for dims, block in [((20, 20, 20), (32, 4, 2)), ((50, 37, 9), (32, 4, 1)), ((64, 64, 8), (32, 4, 1))]:
        n = dims[0] * dims[1] * dims[2]
        mesh = rng.integers(0, 28, n).astype(np.uint8)
        ref, rdims = O.pad(mesh, dims, block)
        # device round trip through a domain's node buffer as scratch input
        with Domain((n, 1, 3), "f32") as src_d, Domain((len(ref), 1, 3), "f32") as dst_d:
            src_d.set_nodes(np.concatenate([mesh, np.zeros(2 * n, np.uint8)]),
                            np.zeros(3 * n, np.uint8))
            sp, dp = C.c_void_p(), C.c_void_p()
            L.call("pfdtd_get_node_ptrs", src_d.handle, C.byref(sp), None)
            L.call("pfdtd_get_node_ptrs", dst_d.handle, C.byref(dp), None)
            d3 = (C.c_uint32 * 3)(*dims)
            od = (C.c_uint32 * 3)()
            L.call("pfdtd_pad_mesh", sp, n, d3, block[0], block[1], block[2], dp, od, 0)
            out, _ = dst_d.get_nodes()
        assert tuple(od) == rdims
        assert np.array_equal(out[:len(ref)], ref)


def test_slice_capture(gpu, O):
    room = rooms.shoebox((40, 36, 32), seed=3)
    steps = 40
    pulse = rooms.gaussian_pulse(steps, 3.0)
    with Domain(room.dims, "f32") as d:
        d.set_voxels(room.bid, room.mat, False)
        d.set_materials(room.admittance)
        d.set_params()
        d.set_sources([(20, 18, 16)], [1], pulse[None])
        d.run(steps)
        P = d.download_field(L.FIELD_CURRENT).reshape(32, 36, 40)
        pos, _ = d.get_nodes()
        pos = pos.reshape(32, 36, 40)
        xy, qxy = d.capture_slice(0, 16)
        xz, qxz = d.capture_slice(1, 18)
        yz, qyz = d.capture_slice(2, 20)
        with pytest.raises(L.PfdtdError):
            d.capture_slice(0, 32)
    assert np.array_equal(xy, P[16]) and np.array_equal(qxy, pos[16])
    # xz / yz leave the last z row uncaptured, as the reference's limit does
    assert np.array_equal(xz[:-1], P[:-1, 18, :]) and (xz[-1] == 0).all()
    assert np.array_equal(yz[:-1], P[:-1, :, 20]) and (qyz[-1] == 0).all()


def test_interrupt_and_progress(gpu):
    room = rooms.shoebox((48, 40, 32), seed=3)
    steps = 1000
    pulse = rooms.gaussian_pulse(steps, 3.0)
    seen = []
    calls = {"n": 0}

    def interrupt():
        calls["n"] += 1
        return calls["n"] > 3

    with Domain(room.dims, "f32") as d:
        d.set_voxels(room.bid, room.mat, False)
        d.set_materials(room.admittance)
        d.set_params()
        d.set_sources([(24, 20, 16)], [1], pulse[None])
        d.set_receivers([(10, 10, 10)])
        full, _, st = d.run(steps, progress=lambda s, m, t: seen.append((s, m)))
        assert st == 0 and [s for s, _ in seen] == list(range(0, steps, 100))
        d.reset_fields()  # a run starts from the fields as they are, as the reference
        part, _, st = d.run(steps, interrupt=interrupt)
    assert st == L.INTERRUPTED
    done = int(np.count_nonzero(part[0]))
    assert 0 < done < steps
    k = np.flatnonzero(part[0])[-1] + 1
    assert np.array_equal(part[0, :k], full[0, :k]) and (part[0, k:] == 0).all()


def test_errors_are_status_codes(gpu):
    room = rooms.shoebox((16, 16, 16), seed=1)
    with Domain(room.dims, "f32") as d:
        with pytest.raises(L.PfdtdError) as e:
            d.run(5)
        assert e.value.status == L.ERR_STATE
        d.set_voxels(room.bid, room.mat, False)
        d.set_materials(room.admittance[:2])  # shell uses materials 0..5
        d.set_params()
        with pytest.raises(L.PfdtdError) as e:
            d.run(5)
        assert e.value.status == L.ERR_MATERIAL
        with pytest.raises(L.PfdtdError):
            d.set_scheme(7)


@pytest.mark.parametrize("variant", ["zmarch", "tma"])
@pytest.mark.parametrize("prec,centred", [("f32", False), ("f32", True), ("f64", False), ("f64", True)])
def test_kernel_variants_bit_identical(gpu, O, variant, prec, centred):
    """Both update kernels (register z-marching and TMA-pipelined) against the
    oracle, on a room whose x extent is not a multiple of the TMA tile and
    whose y extent is not a multiple of the tile height."""
    room = rooms.boxes_room((208, 52, 40), n_boxes=6, edge=(5, 16), n_materials=9, seed=13)
    steps = 120
    srcs = [(p, 1) for p in room.random_air_nodes(2, seed=3)]
    rec = room.random_air_nodes(5, seed=4)
    pulse = rooms.gaussian_pulse(steps, 3.0)
    params = default_params()
    with Domain(room.dims, prec) as d:
        d.set_voxels(room.bid, room.mat, centred=centred)
        d.set_materials(room.admittance)
        d.set_params(params)
        d.set_scheme("centred" if centred else "forward")
        d.set_kernel(variant)
        d.set_sources([s[0] for s in srcs], [1, 1], np.stack([pulse, 0.3 * pulse]))
        d.set_receivers(rec)
        g, _, _ = d.run(steps)
        assert d.kernel() == variant
        P = d.download_field(L.FIELD_CURRENT)
    pos, mat = O.encode_nodes(room.bid, room.mat, centred)
    r, rP, _ = O.run(pos, mat, room.dims, room.admittance, params, [room.flat(*s[0]) for s in srcs],
                     [1, 1], np.stack([pulse, 0.3 * pulse]), [room.flat(*x) for x in rec], steps,
                     scheme=2 if centred else 0, double=(prec == "f64"))
    assert_parity(g, r, prec)
    assert np.array_equal(P, rP)


def test_tma_wrap_neighbours_on_outer_faces(gpu, O):
    """Inside nodes on the outer x/y faces read the flat-index wrapped
    neighbour, as the reference kernel does; both variants match the oracle."""
    X, Y, Z = 64, 20, 12
    rng = np.random.default_rng(5)
    pos = np.full(X * Y * Z, 0x86, np.uint8)      # every node inside, K = 6
    pos[rng.random(pos.size) < 0.1] = 0x84          # some K = 4 boundary nodes
    mat = rng.integers(0, 3, pos.size).astype(np.uint8)
    table = np.repeat(np.array([[0.1], [0.3], [0.6]]), 20, axis=1)
    steps = 30
    pulse = rooms.gaussian_pulse(steps, 2.0, t0=5.0)
    out = {}
    for variant in ("zmarch", "tma"):
        with Domain((X, Y, Z), "f32") as d:
            d.set_nodes(pos, mat)
            d.set_materials(table)
            d.set_params()
            d.set_kernel(variant)
            d.set_sources([(0, 0, 6), (X - 1, Y - 1, 5)], [1, 1], np.stack([pulse, -pulse]))
            d.set_receivers([(0, 5, 6), (X - 1, 7, 4), (31, 0, 3)])
            g, _, _ = d.run(steps)
            out[variant] = (g, d.download_field(L.FIELD_CURRENT))
    X_, Y_ = X, Y
    r, rP, _ = O.run(pos, mat, (X, Y, Z), table, default_params(),
                     [6 * X_ * Y_, 5 * X_ * Y_ + (Y - 1) * X + X - 1], [1, 1],
                     np.stack([pulse, -pulse]),
                     [6 * X * Y + 5 * X, 4 * X * Y + 7 * X + X - 1, 3 * X * Y + 31], steps)
    for variant, (g, P) in out.items():
        assert np.array_equal(g, r), variant
        assert np.array_equal(P, rP), variant


@pytest.mark.parametrize("tile", list(range(9)))
@pytest.mark.parametrize("centred", [False, True])
@pytest.mark.parametrize("wide", [False, True])
@pytest.mark.parametrize("X", [208, 200])
def test_tma_tile_shapes_bit_identical(gpu, O, tile, centred, wide, X):
    """FP32 tile shapes; wide: materials drawn per voxel, more than 256 node
    classes, so the class ids are 16-bit; X = 200: rows of class ids that are
    not 16-byte aligned (read from the padded copy)."""
    room = rooms.boxes_room((X, 52, 40), n_boxes=6, edge=(5, 16), n_materials=150 if wide else 9,
                            seed=14)
    if wide:
        room.mat[...] = np.random.default_rng(5).integers(0, 150, room.mat.shape, dtype=np.uint8)
    steps = 60
    src = room.random_air_nodes(1, seed=3)
    rec = room.random_air_nodes(4, seed=4)
    pulse = rooms.gaussian_pulse(steps, 3.0)
    with Domain(room.dims, "f32") as d:
        d.set_voxels(room.bid, room.mat, centred=centred)
        d.set_materials(room.admittance)
        d.set_params()
        d.set_scheme("centred" if centred else "forward")
        d.set_kernel("tma")
        L.call("pfdtd_set_tile", d.handle, tile)
        d.set_sources(src, [1], pulse[None])
        d.set_receivers(rec)
        g, _, _ = d.run(steps)
        assert d.kernel() == "tma"
        P = d.download_field(L.FIELD_CURRENT)
    pos, mat = O.encode_nodes(room.bid, room.mat, centred)
    r, rP, _ = O.run(pos, mat, room.dims, room.admittance, default_params(), [room.flat(*src[0])],
                     [1], pulse[None], [room.flat(*x) for x in rec], steps, scheme=2 if centred else 0)
    assert_parity(g, r, "f32")
    assert np.array_equal(P, rP)


@pytest.mark.parametrize("tile", list(range(11)))
@pytest.mark.parametrize("prec", ["f16", "bf16"])
@pytest.mark.parametrize("centred,wide", [(False, False), (True, False), (False, True),
                                          (True, True)])
@pytest.mark.parametrize("X", [208, 200])
def test_16bit_tile_shapes_bit_identical(gpu, O, tile, prec, centred, wide, X):
    """Every 16-bit tile shape (4 and 8 elements per thread, planes carried
    in registers or reloaded), forward and centred, with 8-bit class ids and
    (wide: materials drawn per voxel, more than 256 node classes) 16-bit
    class ids; X = 208 leaves partly filled tiles, X = 200 rows of class ids
    that are not 16-byte aligned, Z = 40 a z-chunk whose plane count is not a
    multiple of three.  Bit-identical to the oracle with the same storage
    rounding."""
    room = rooms.boxes_room((X, 52, 40), n_boxes=6, edge=(5, 16), n_materials=150 if wide else 9,
                            seed=16)
    if wide:
        room.mat[...] = np.random.default_rng(5).integers(0, 150, room.mat.shape, dtype=np.uint8)
    steps = 60
    src = room.random_air_nodes(1, seed=3)
    rec = [src[0]] + room.random_air_nodes(3, seed=4)  # the source node sees the pulse
    pulse = rooms.gaussian_pulse(steps, 3.0)
    pos, mat = O.encode_nodes(room.bid, room.mat, centred)
    Y, Z = room.dims[1], room.dims[2]
    keys = np.unique(pos.reshape(Z, -1)[1:Z - 1].astype(np.int32) * 256 + mat.reshape(Z, -1)[1:Z - 1])
    assert (len(keys) > 256) == wide
    with Domain(room.dims, prec) as d:
        d.set_voxels(room.bid, room.mat, centred=centred)
        d.set_materials(room.admittance)
        d.set_params()
        d.set_scheme("centred" if centred else "forward")
        d.set_kernel("tma")
        L.call("pfdtd_set_tile", d.handle, tile)
        d.set_sources(src, [1], pulse[None])
        d.set_receivers(rec)
        g, _, _ = d.run(steps)
        assert d.kernel() == "tma"
        P = d.download_field(L.FIELD_CURRENT)
    r, rP, _ = O.run(pos, mat, room.dims, room.admittance, default_params(), [room.flat(*src[0])],
                     [1], pulse[None], [room.flat(*x) for x in rec], steps,
                     scheme=2 if centred else 0, storage=prec)
    assert np.abs(r).max() > 1e-4
    assert np.array_equal(g, r)
    assert np.array_equal(P.view(np.uint16), rP.view(np.uint16))


@pytest.mark.parametrize("variant", ["zmarch", "tma"])
@pytest.mark.parametrize("prec", ["f16", "bf16"])
@pytest.mark.parametrize("centred", [False, True])
def test_16bit_storage_bit_identical(gpu, O, variant, prec, centred):
    """FP16 / BF16 field storage with FP32 arithmetic: bit-identical to the
    oracle that rounds its stored fields the same way; the error against the
    FP64 oracle is bounded (FP16 <= 1e-2, BF16 <= 1e-1 relative L2 here)."""
    room = rooms.boxes_room((256, 48, 40), n_boxes=6, edge=(5, 16), n_materials=9, seed=15)
    steps = 150
    src = room.random_air_nodes(1, seed=3)
    rec = room.random_air_nodes(4, seed=4)
    pulse = rooms.gaussian_pulse(steps, 4.0)
    with Domain(room.dims, prec) as d:
        d.set_voxels(room.bid, room.mat, centred=centred)
        d.set_materials(room.admittance)
        d.set_params()
        d.set_scheme("centred" if centred else "forward")
        d.set_kernel(variant)
        d.set_sources(src, [1], pulse[None])
        d.set_receivers(rec)
        g, _, _ = d.run(steps)
        assert d.kernel() == variant
        P = d.download_field(L.FIELD_CURRENT)
    pos, mat = O.encode_nodes(room.bid, room.mat, centred)
    args = (pos, mat, room.dims, room.admittance, default_params(), [room.flat(*src[0])], [1],
            pulse[None], [room.flat(*x) for x in rec], steps)
    r, rP, _ = O.run(*args, scheme=2 if centred else 0, storage=prec)
    assert np.array_equal(g, r)
    assert np.array_equal(P.view(np.uint16), rP.view(np.uint16))
    d64, _, _ = O.run(*args, scheme=2 if centred else 0, double=True)
    err = rel_l2(g, d64)
    assert err < (1e-2 if prec == "f16" else 1e-1), err


@pytest.mark.parametrize("prec", ["f32", "bf16"])
@pytest.mark.parametrize("variant", ["auto", "zmarch"])
def test_iwb_open_x_faces(gpu, O, prec, variant):
    """IWB with inside nodes on the x and y faces, where the flat-index
    neighbours x-1 / x+1 wrap to the neighbouring row (the TMA kernel reads
    them from global memory at the grid's x edges): equal to the oracle."""
    room = rooms.boxes_room((64, 48, 40), n_boxes=4, edge=(5, 12), n_materials=6, seed=14)
    bid = room.bid.copy().reshape(room.dims[2], room.dims[1], room.dims[0])
    bid[5:30, 6:40, 0] = 26   # open strips on both x faces and one y face
    bid[8:25, 3:30, -1] = 22
    bid[10:20, 0, 10:50] = 21
    steps = 120
    srcs = [(1, 20, 15), (62, 10, 12)]
    rec = [(0, 20, 15), (63, 12, 14), (30, 0, 15), (20, 20, 20)]
    pulse = rooms.gaussian_pulse(steps, 3.0)
    params = default_params(scheme="iwb")
    with Domain(room.dims, prec) as d:
        d.set_voxels(bid.reshape(-1), room.mat, centred=True)
        d.set_materials(room.admittance)
        d.set_params(params)
        d.set_scheme("iwb")
        d.set_kernel(variant)
        d.set_sources(srcs, [1, 1], np.stack([pulse, -0.5 * pulse]))
        d.set_receivers(rec)
        g, _, _ = d.run(steps)
        assert d.kernel() == ("tma" if variant == "auto" else "zmarch")
    pos, mat = O.encode_nodes(bid.reshape(-1), room.mat, True)
    r, _, _ = O.run(pos, mat, room.dims, room.admittance, params, [room.flat(*x) for x in srcs],
                    [1, 1], np.stack([pulse, -0.5 * pulse]), [room.flat(*x) for x in rec], steps,
                    scheme=3, storage=(prec if prec == "bf16" else None))
    assert np.abs(r).max() > 1e-3
    assert np.array_equal(g, r)


@pytest.mark.parametrize("prec", ["f32", "bf16"])
@pytest.mark.parametrize("shape", list(range(11)))
@pytest.mark.parametrize("X", [208, 200])
def test_iwb_tile_shapes(gpu, O, prec, shape, X):
    """Every IWB tile shape on the TMA path equals the oracle, with DIF walls:
    shapes 0..5 run the closure inside the streaming kernel, 6..10 leave the
    nodes with a closed neighbour to the closure pass, which also applies the
    DIF update of those nodes.  The room is not a multiple of the 64- or
    128-node tiles in x or of the tile rows in y; X = 200: rows of class ids
    that are not 16-byte aligned."""
    from parallelfdtd_gb300 import materials
    room = rooms.boxes_room((X, 44, 36), n_boxes=6, edge=(5, 12), n_materials=6, seed=16)
    steps = 90
    srcs = room.random_air_nodes(2, seed=1)
    rec = room.random_air_nodes(4, seed=2)
    pulse = rooms.gaussian_pulse(steps, 3.0)
    params = default_params(scheme="iwb")
    flags = np.array([m % 2 for m in range(6)], np.int32)
    table = materials.dif_table(materials.positive_real_filters(6, 3, seed=2), 3)
    with Domain(room.dims, prec) as d:
        d.set_voxels(room.bid, room.mat, centred=True)
        d.set_materials(room.admittance)
        d.set_params(params)
        d.set_scheme("iwb")
        d.set_dif_filters(flags, table)
        d.set_kernel("tma")
        L.call("pfdtd_set_tile", d.handle, shape)
        d.set_sources(srcs, [1, 1], np.stack([pulse, -0.5 * pulse]))
        d.set_receivers(rec)
        g, _, _ = d.run(steps)
        assert d.kernel() == "tma"
        P = d.download_field(L.FIELD_CURRENT)
    pos, mat = O.encode_nodes(room.bid, room.mat, True)
    r, rP, _ = O.run(pos, mat, room.dims, room.admittance, params, [room.flat(*s) for s in srcs],
                     [1, 1], np.stack([pulse, -0.5 * pulse]), [room.flat(*x) for x in rec], steps,
                     scheme=3, storage=(prec if prec == "bf16" else None), dif=(flags, table))
    assert np.abs(r).max() > 1e-4
    assert np.array_equal(g, r)
    if prec == "bf16":
        assert np.array_equal(P.view(np.uint16), rP.view(np.uint16))
    else:
        assert np.array_equal(P, rP)


@pytest.mark.parametrize("prec", ["f32", "bf16"])
def test_iwb_below_the_stability_limit(gpu, O, prec):
    """IWB at lambda = 0.95 (weights lambda^2 (1/4, 1/8, 1/16), centre
    2 - 7/2 lambda^2) with frequency-dependent walls: equal to the oracle."""
    from parallelfdtd_gb300 import materials
    room = rooms.boxes_room((64, 48, 40), n_boxes=5, edge=(5, 12), n_materials=6, seed=15)
    steps = 150
    srcs = room.random_air_nodes(2, seed=1)
    rec = room.random_air_nodes(4, seed=2)
    pulse = rooms.gaussian_pulse(steps, 3.0)
    params = default_params(scheme="iwb", lam=0.95)
    flags = np.array([m % 2 for m in range(6)], np.int32)
    table = materials.dif_table(materials.positive_real_filters(6, 3, seed=2), 3)
    with Domain(room.dims, prec) as d:
        d.set_voxels(room.bid, room.mat, centred=True)
        d.set_materials(room.admittance)
        d.set_params(params)
        d.set_scheme("iwb")
        d.set_dif_filters(flags, table)
        d.set_sources(srcs, [1, 1], np.stack([pulse, -0.5 * pulse]))
        d.set_receivers(rec)
        g, _, _ = d.run(steps)
    pos, mat = O.encode_nodes(room.bid, room.mat, True)
    r, _, _ = O.run(pos, mat, room.dims, room.admittance, params, [room.flat(*s) for s in srcs],
                    [1, 1], np.stack([pulse, -0.5 * pulse]), [room.flat(*x) for x in rec], steps,
                    scheme=3, storage=(prec if prec == "bf16" else None), dif=(flags, table))
    assert np.abs(r).max() > 1e-4
    assert np.array_equal(g, r)


@pytest.mark.parametrize("prec", ["f32", "f64", "f16", "bf16"])
def test_iwb_bit_identical(gpu, O, prec):
    """IWB 27-point scheme (specification in the oracle): the CUDA path equals
    the oracle bit for bit on a room with boxes (faces, edges, corners)."""
    room = rooms.boxes_room((96, 64, 48), n_boxes=8, edge=(6, 20), n_materials=12, seed=4)
    steps = 200
    srcs = room.random_air_nodes(2, seed=1)
    rec = room.random_air_nodes(4, seed=2)
    pulse = rooms.gaussian_pulse(steps, 3.0)
    params = default_params(scheme="iwb")
    with Domain(room.dims, prec) as d:
        d.set_voxels(room.bid, room.mat, centred=True)
        d.set_materials(room.admittance)
        d.set_params(params)
        d.set_scheme("iwb")
        d.set_sources(srcs, [1, 1], np.stack([pulse, -0.5 * pulse]))
        d.set_receivers(rec)
        g, _, _ = d.run(steps)
        P = d.download_field(L.FIELD_CURRENT)
    pos, mat = O.encode_nodes(room.bid, room.mat, True)
    r, rP, _ = O.run(pos, mat, room.dims, room.admittance, params, [room.flat(*s) for s in srcs],
                     [1, 1], np.stack([pulse, -0.5 * pulse]), [room.flat(*x) for x in rec], steps,
                     scheme=3, double=(prec == "f64"),
                     storage=(prec if prec in ("f16", "bf16") else None))
    assert np.abs(r).max() > 1e-4
    if prec in ("f16", "bf16"):
        assert np.array_equal(g, r) and np.array_equal(P.view(np.uint16), rP.view(np.uint16))
    else:
        assert_parity(g, r, prec)
        assert np.array_equal(P, rP)


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("scheme", ["forward", "centred", "iwb"])
def test_dif_boundaries_bit_identical(gpu, O, prec, scheme):
    """Frequency-dependent boundaries (3rd-order passive IIR admittances on
    half of the materials): the CUDA path equals the oracle bit for bit."""
    from parallelfdtd_gb300 import materials
    room = rooms.boxes_room((128, 64, 48), n_boxes=8, edge=(6, 20), n_materials=10, seed=6)
    steps = 300
    srcs = room.random_air_nodes(2, seed=1)
    rec = room.random_air_nodes(4, seed=2)
    pulse = rooms.gaussian_pulse(steps, 3.0)
    code = {"forward": 0, "centred": 2, "iwb": 3}[scheme]
    params = default_params(scheme=scheme)
    flags = np.array([m % 2 for m in range(10)], np.int32)
    table = materials.dif_table(materials.positive_real_filters(10, 3, seed=12), 3)
    with Domain(room.dims, prec) as d:
        d.set_voxels(room.bid, room.mat, centred=(scheme != "forward"))
        d.set_materials(room.admittance)
        d.set_params(params)
        d.set_scheme(scheme)
        d.set_dif_filters(flags, table)
        d.set_sources(srcs, [1, 1], np.stack([pulse, -0.5 * pulse]))
        d.set_receivers(rec)
        n_dif = d.dif_count()
        g, _, _ = d.run(steps)
        P = d.download_field(L.FIELD_CURRENT)
    pos, mat = O.encode_nodes(room.bid, room.mat, scheme != "forward")
    r, rP, _ = O.run(pos, mat, room.dims, room.admittance, params, [room.flat(*s) for s in srcs],
                     [1, 1], np.stack([pulse, -0.5 * pulse]), [room.flat(*x) for x in rec], steps,
                     scheme=code, double=(prec == "f64"), dif=(flags, table))
    X, Y, Z = room.dims
    inside = (pos.reshape(Z, Y, X)[1:-1] >> 7) == 1
    flagged = flags[mat.reshape(Z, Y, X)[1:-1]] == 1
    if scheme == "forward":
        boundary = (pos.reshape(Z, Y, X)[1:-1] & 0x7F) < 6
    else:
        boundary = (pos.reshape(Z, Y, X)[1:-1] & 0x07) != 0
    assert n_dif == int(np.count_nonzero(inside & flagged & boundary)) > 0
    assert_parity(g, r, prec)
    assert np.array_equal(P, rP)


@pytest.mark.parametrize("variant", ["zmarch", "auto"])
@pytest.mark.parametrize("fields,prec,scheme", [(4, "f32", "forward"), (16, "f32", "forward"),
                                                (16, "f16", "forward"), (4, "f64", "centred"),
                                                (8, "bf16", "centred"), (8, "f32", "iwb")])
def test_batched_fields_equal_independent_runs(gpu, O, fields, prec, scheme, variant):
    """K fields sharing one geometry: field f equals an independent oracle run
    of field f's source (bit-identical), with DIF boundaries on some materials."""
    from parallelfdtd_gb300 import materials
    room = rooms.boxes_room((64, 48, 40), n_boxes=5, edge=(5, 14), n_materials=6, seed=21)
    steps = 120
    pulse = rooms.gaussian_pulse(steps, 3.0)
    srcs = room.random_air_nodes(fields, seed=5)
    recs = room.random_air_nodes(2 * fields, seed=6)
    rec_fields = [i // 2 for i in range(2 * fields)]
    params = default_params(scheme=scheme)
    code = {"forward": 0, "centred": 2, "iwb": 3}[scheme]
    flags = np.array([m % 2 for m in range(6)], np.int32)
    table = materials.dif_table(materials.positive_real_filters(6, 2, seed=3), 2)
    with Domain(room.dims, prec, fields=fields) as d:
        d.set_voxels(room.bid, room.mat, centred=(scheme != "forward"))
        d.set_materials(room.admittance)
        d.set_params(params)
        d.set_scheme(scheme)
        d.set_dif_filters(flags, table)
        d.set_kernel(variant)
        d.set_sources(srcs, [1] * fields, np.repeat(pulse[None], fields, axis=0),
                      fields=list(range(fields)))
        d.set_receivers(recs, fields=rec_fields)
        g, _, _ = d.run(steps)
        if variant == "auto" and scheme != "iwb":
            assert d.kernel() == "tma"
    pos, mat = O.encode_nodes(room.bid, room.mat, scheme != "forward")
    for f in range(fields):
        r, _, _ = O.run(pos, mat, room.dims, room.admittance, params, [room.flat(*srcs[f])], [1],
                        pulse[None], [room.flat(*recs[2 * f]), room.flat(*recs[2 * f + 1])], steps,
                        scheme=code, double=(prec == "f64"),
                        storage=(prec if prec in ("f16", "bf16") else None), dif=(flags, table))
        assert np.array_equal(g[2 * f:2 * f + 2], r), f"field {f}"


@pytest.mark.parametrize("input_type,steps,n_ir", [(1, 600, 1000), (0, 900, 250), (3, 400, 0)])
def test_transparent_source_on_device(gpu, O, input_type, steps, n_ir):
    """The device transparent-source vector equals the oracle's per-step
    restatement of SimulationParameters::getTransparentSourceSample."""
    from parallelfdtd_gb300.domain import transparent_source
    rng = np.random.default_rng(3)
    h = (rng.standard_normal(n_ir) * 0.05).astype(np.float32) if n_ir else np.zeros(0, np.float32)
    data = rng.standard_normal(steps).astype(np.float32)
    regular = O.source_vector(1, input_type, steps, data=data if input_type == 3 else None)
    ref = O.source_vector(2, input_type, steps, data=data if input_type == 3 else None,
                          grid_ir=h if n_ir else None)
    got = transparent_source(regular, h)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("prec,depth", [("f32", 0), ("f16", 0), ("f32", 2)])
def test_run_with_slice_captures(gpu, prec, depth):
    """Slices captured asynchronously during one run equal run(s) followed by
    capture_slice, and the receivers equal a plain run."""
    room = rooms.boxes_room((64, 48, 40), n_boxes=4, edge=(5, 12), n_materials=6, seed=12)
    steps = 163
    pulse = rooms.gaussian_pulse(steps, 3.0)
    src = [tuple(p) for p in room.random_air_nodes(2, seed=1)]
    rec = [tuple(p) for p in room.random_air_nodes(3, seed=2)]
    caps = [(0, 0, 10), (37, 1, 20), (50, 2, 30), (100, 0, 25), (100, 2, 5), (163, 1, 47)]

    def make():
        d = Domain(room.dims, prec)
        d.set_voxels(room.bid, room.mat, centred=False)
        d.set_materials(room.admittance)
        d.set_params(default_params())
        d.set_sources(src, [1, 1], np.stack([pulse, -pulse]))
        d.set_receivers(rec)
        d.set_temporal_block(depth)
        return d

    with make() as d:
        g, got = d.run_captures(steps, caps)
    with make() as d:
        g0, _, _ = d.run(steps)
    assert np.array_equal(g, g0)
    for (s, o, sl), (p, q) in zip(caps, got):
        with make() as d:
            if s:
                d.run(s)
            rp, rq = d.capture_slice(o, sl)
        assert np.array_equal(p, rp), (s, o, sl)
        assert np.array_equal(q, rq)
    assert np.abs(got[3][0]).max() > 0


def test_post_filter_matches_scipy(gpu):
    """Receiver post-processing on the device (python/FDTDfilter.py,
    matlab/functions/FDTDpostFilter.m) against scipy's lfilter; double
    within 1e-12 of the largest output, float within 1e-5."""
    from scipy.signal import firwin, lfilter
    from parallelfdtd_gb300 import postfilter as pf
    rng = np.random.default_rng(4)
    x = rng.standard_normal((3000, 16))  # [samples, channels], as FDTDfilter.py
    y = pf.FDTDfilter(x, 8000.0, 48000.0, 0.2)
    taps = firwin(200, 8000 * 0.2 / 4000.0, window=("chebwin", 70.0))
    ref = lfilter(taps, 1.0, x, axis=0)
    assert y.shape == x.shape and np.max(np.abs(y - ref)) <= 1e-12 * np.max(np.abs(ref))
    a = pf.dcblock(5.0, 8000.0)
    ref2 = lfilter([1.0, -1.0], [1.0, -a], lfilter(firwin(201, 0.3, window="hamming"), 1.0,
                                                     x, axis=0), axis=0)
    for inp in (x, x.T):  # column or row traces: columns out
        z = pf.FDTDpostFilter(inp, 8000.0, 0.3)
        assert z.shape == x.shape and np.max(np.abs(z - ref2)) <= 1e-10 * np.max(np.abs(ref2))
    z1 = pf.FDTDpostFilter(x[:, 3], 8000.0, 0.3)
    assert np.max(np.abs(z1 - ref2[:, 3])) <= 1e-10 * np.max(np.abs(ref2))
    f = pf.FDTDfilter(x.astype(np.float32), 8000.0, 48000.0, 0.2)
    assert f.dtype == np.float32 and np.max(np.abs(f - ref)) <= 1e-5 * np.max(np.abs(ref))


@pytest.mark.parametrize("p,q,n", [(6, 1, 1000), (48000, 7350, 2001), (3, 4, 999), (1, 5, 400)])
def test_resample_matches_scipy(gpu, p, q, n):
    """Polyphase resampling on the device against scipy's resample_poly with
    the same taps (output alignment and length as MATLAB's resample)."""
    from scipy.signal import resample_poly
    from parallelfdtd_gb300 import postfilter as pf
    rng = np.random.default_rng(p + q)
    x = rng.standard_normal((n, 3))
    h = pf.resample_taps(p, q)
    y = pf.resample(x, p, q)
    ref = resample_poly(x, p, q, axis=0, window=h)
    assert y.shape == ref.shape == (-(-n * p // q), 3)
    assert np.max(np.abs(y - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_render_pipeline(gpu):
    """matlab/testBench.m:203-204 on a simulated response: post-filter, then
    resample to 48 kHz; equal to the scipy composition."""
    from scipy.signal import firwin, lfilter, resample_poly
    from parallelfdtd_gb300 import postfilter as pf
    fs = 7350
    rng = np.random.default_rng(9)
    p = rng.standard_normal((900, 2)) * np.exp(-np.arange(900) / 200.0)[:, None]
    y = pf.render(p, fs, 0.2, 48000)
    a = pf.dcblock(5.0, fs)
    f = lfilter([1.0, -1.0], [1.0, -a], lfilter(firwin(201, 0.2, window="hamming"), 1.0, p,
                                                  axis=0), axis=0)
    ref = resample_poly(f, 48000, fs, axis=0, window=pf.resample_taps(48000, fs))
    assert y.shape == ref.shape and np.max(np.abs(y - ref)) <= 1e-12 * np.max(np.abs(ref))


def _iwb_dif_room():
    from parallelfdtd_gb300 import materials
    room = rooms.boxes_room((208, 44, 36), n_boxes=6, edge=(5, 12), n_materials=6, seed=16)
    flags = np.array([m % 2 for m in range(6)], np.int32)
    table = materials.dif_table(materials.positive_real_filters(6, 3, seed=2), 3)
    return room, flags, table


@pytest.mark.parametrize("shape", [6, 7, 8, 9, 10])
def test_iwb_closure_pass_unfused_dif(gpu, O, monkeypatch, shape):
    """The closure pass with the DIF update left to its own pass
    (PFDTD_IWB_DIF_UNFUSED=1, the path a DIF node without a closure record
    takes) equals the fused closure pass and the oracle bit for bit."""
    room, flags, table = _iwb_dif_room()
    steps = 90
    srcs = room.random_air_nodes(2, seed=1)
    rec = room.random_air_nodes(4, seed=2)
    pulse = rooms.gaussian_pulse(steps, 3.0)
    params = default_params(scheme="iwb")
    out = {}
    for unfused in (False, True):
        if unfused:
            monkeypatch.setenv("PFDTD_IWB_DIF_UNFUSED", "1")
        else:
            monkeypatch.delenv("PFDTD_IWB_DIF_UNFUSED", raising=False)
        with Domain(room.dims, "f32") as d:
            d.set_voxels(room.bid, room.mat, centred=True)
            d.set_materials(room.admittance)
            d.set_params(params)
            d.set_scheme("iwb")
            d.set_dif_filters(flags, table)
            d.set_kernel("tma")
            L.call("pfdtd_set_tile", d.handle, shape)
            d.set_sources(srcs, [1, 1], np.stack([pulse, -0.5 * pulse]))
            d.set_receivers(rec)
            g, _, st = d.run(steps)
            assert st == 0
            out[unfused] = (g, d.download_field(L.FIELD_CURRENT))
    monkeypatch.delenv("PFDTD_IWB_DIF_UNFUSED", raising=False)
    assert np.array_equal(out[False][0], out[True][0])
    assert np.array_equal(out[False][1], out[True][1])
    pos, mat = O.encode_nodes(room.bid, room.mat, True)
    r, rP, _ = O.run(pos, mat, room.dims, room.admittance, params, [room.flat(*s) for s in srcs],
                     [1, 1], np.stack([pulse, -0.5 * pulse]), [room.flat(*x) for x in rec], steps,
                     scheme=3, dif=(flags, table))
    assert np.abs(r).max() > 1e-4
    assert np.array_equal(out[True][0], r) and np.array_equal(out[True][1], rP)


def test_autotune_mid_run_keeps_dif_state(gpu):
    """An IWB room with frequency-dependent walls: 40 steps, then the
    autotuner (whose timing launches advance the fields and the DIF filter
    states), then 50 more steps without a reset.  Receivers and fields equal
    a run that was never autotuned, bit for bit."""
    room, flags, table = _iwb_dif_room()
    steps, cut = 90, 40
    srcs = room.random_air_nodes(2, seed=1)
    rec = room.random_air_nodes(4, seed=2)
    pulse = rooms.gaussian_pulse(steps, 3.0)
    params = default_params(scheme="iwb")
    res = []
    for tune in (False, True):
        with Domain(room.dims, "f32") as d:
            d.set_voxels(room.bid, room.mat, centred=True)
            d.set_materials(room.admittance)
            d.set_params(params)
            d.set_scheme("iwb")
            d.set_dif_filters(flags, table)
            d.set_sources(srcs, [1, 1], np.stack([pulse, -0.5 * pulse]))
            d.set_receivers(rec)
            assert d.dif_count() > 0
            out = np.zeros((len(rec), steps), np.float32)
            for s in range(cut):
                d.step(s, 1, out, steps)
            if tune:
                d.autotune(max_depth=0, iters=3)
            for s in range(cut, steps):
                d.step(s, 1, out, steps)
            res.append((out, d.download_field(L.FIELD_CURRENT), d.download_field(L.FIELD_PAST)))
    assert np.abs(res[0][0]).max() > 1e-4
    for a, b in zip(res[0], res[1]):
        assert np.array_equal(a, b)


def test_pipeline_wait_timeout_reports_and_recovers(gpu, O):
    """The bounded waits of the TMA update kernel: with every pipeline wait
    limited to 1 ns, waits run out, the kernel raises the domain's error flag
    (after waiting, with its full bound, for the loads it already issued),
    later launches do nothing, and the run reports PFDTD_ERR_CUDA.  The same
    domain, back at the default bound, then runs and equals the oracle."""
    room = rooms.boxes_room((256, 96, 64), n_boxes=5, edge=(6, 16), n_materials=6, seed=43)
    steps = 60
    src = room.random_air_nodes(1, seed=1)
    rec = [src[0]] + room.random_air_nodes(2, seed=2)  # the source node sees the pulse
    pulse = rooms.gaussian_pulse(steps, 3.0)
    with Domain(room.dims, "f32") as d:
        d.set_voxels(room.bid, room.mat, centred=False)
        d.set_materials(room.admittance)
        d.set_params()
        d.set_kernel("tma")
        d.set_sources(src, [1], pulse[None])
        d.set_receivers(rec)
        L.call("pfdtd_set_wait_limit", d.handle, 1)
        with pytest.raises(L.PfdtdError) as ex:
            d.run(steps)
        assert ex.value.status == L.ERR_CUDA and "timed out" in str(ex.value)
        L.call("pfdtd_set_wait_limit", d.handle, 0)
        d.reset_fields()
        g, _, st = d.run(steps)
        assert st == 0 and d.kernel() == "tma"
    pos, mat = O.encode_nodes(room.bid, room.mat, False)
    r, _, _ = O.run(pos, mat, room.dims, room.admittance, default_params(),
                    [room.flat(*src[0])], [1], pulse[None], [room.flat(*x) for x in rec], steps)
    assert np.abs(r).max() > 1e-4
    assert np.array_equal(g, r)


@pytest.mark.parametrize("fields,prec", [(4, "f32"), (8, "f32"), (8, "f16"), (4, "f64")])
def test_batched_partly_filled_tiles(gpu, O, fields, prec):
    """Batched fields on the TMA path when a row of X*K elements ends inside
    a 256-element tile (X = 80: 320 or 640 elements), with inside nodes on
    both x faces so that the last node of a row reads the next row's first
    node through the flat index: every field equals an oracle run of it
    alone."""
    room = rooms.boxes_room((80, 40, 32), n_boxes=4, edge=(4, 10), n_materials=5, seed=44)
    X, Y, Z = room.dims
    bid = room.bid.copy().reshape(Z, Y, X)
    # air nodes on both x faces; their neighbours' node codes still describe
    # the closed room, so the field grows, and the run is kept short enough
    # for 16-bit storage
    bid[4:24, 5:30, 0] = 27
    bid[6:20, 3:28, -1] = 27
    steps = 40
    srcs = room.random_air_nodes(fields, seed=7)
    srcs[0] = (X - 1, 10, 10)
    srcs[1] = (0, 11, 12)
    recs = [(X - 1, 12, 12), (0, 12, 12)] + room.random_air_nodes(fields, seed=8)[2:]
    pulse = rooms.gaussian_pulse(steps, 3.0)
    samples = np.stack([pulse * (1.0 + 0.1 * f) for f in range(fields)])
    with Domain(room.dims, prec, fields=fields) as d:
        d.set_voxels(bid.reshape(-1), room.mat, centred=False)
        d.set_materials(room.admittance)
        d.set_params()
        d.set_sources(srcs, [1] * fields, samples, fields=list(range(fields)))
        d.set_receivers(recs, fields=list(range(fields)))
        g, _, st = d.run(steps)
        assert st == 0 and d.kernel() == "tma"
    pos, mat = O.encode_nodes(bid.reshape(-1), room.mat, False)
    for f in range(fields):
        r, _, _ = O.run(pos, mat, room.dims, room.admittance, default_params(),
                        [room.flat(*srcs[f])], [1], samples[f:f + 1], [room.flat(*recs[f])],
                        steps, double=(prec == "f64"),
                        storage=(prec if prec in ("f16", "bf16") else None))
        assert np.isfinite(r).all() and (f > 1 or np.abs(r).max() > 1e-6)
        assert np.array_equal(g[f], r[0]), f"field {f}"


@pytest.mark.parametrize("tile", [0, 1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("fields,prec", [(16, "f16"), (8, "bf16"), (4, "f16")])
@pytest.mark.parametrize("centred", [False, True])
@pytest.mark.parametrize("dims", [(64, 48, 40), (72, 40, 32)])
def test_batched_16bit_tile_shapes(gpu, O, monkeypatch, tile, fields, prec, centred, dims):
    """The batched 16-bit tile shapes (1: 256 x 4 elements, four CTAs per SM;
    2: 256 x 8, six stages; 3 and 4: 8 fields per thread, 5: the same with
    planes carried in registers, for K a multiple of 8, else the default
    shape) equal an oracle run of each field alone.  X = 72 leaves the last
    tile of a row partly filled."""
    monkeypatch.setenv("PFDTD_TMA_TILE", str(tile))
    room = rooms.boxes_room(dims, n_boxes=5, edge=(5, 14), n_materials=6, seed=45)
    steps = 90
    pulse = rooms.gaussian_pulse(steps, 3.0)
    srcs = room.random_air_nodes(fields, seed=5)
    recs = room.random_air_nodes(fields, seed=6)
    samples = np.stack([pulse * (1 + 0.1 * f) for f in range(fields)])
    with Domain(room.dims, prec, fields=fields) as d:
        d.set_voxels(room.bid, room.mat, centred=centred)
        d.set_materials(room.admittance)
        d.set_params()
        d.set_scheme("centred" if centred else "forward")
        d.set_sources(srcs, [1] * fields, samples, fields=list(range(fields)))
        d.set_receivers(recs, fields=list(range(fields)))
        g, _, st = d.run(steps)
        assert st == 0 and d.kernel() == "tma"
    monkeypatch.delenv("PFDTD_TMA_TILE", raising=False)
    pos, mat = O.encode_nodes(room.bid, room.mat, centred)
    for f in (0, fields - 1):
        r, _, _ = O.run(pos, mat, room.dims, room.admittance, default_params(),
                        [room.flat(*srcs[f])], [1], samples[f:f + 1], [room.flat(*recs[f])],
                        steps, storage=prec, scheme=2 if centred else 0)
        assert np.abs(r).max() > 1e-6
        assert np.array_equal(g[f], r[0]), f"field {f}"
