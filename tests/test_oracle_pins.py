"""The CPU oracle pinned against the known answers the reference's tests hold
and against properties of the update rule.  CPU only."""
import os

import numpy as np
import pytest

from parallelfdtd_gb300 import rooms
from parallelfdtd_gb300.domain import default_params

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def O(built):
    from oracle import oracle
    return oracle


def test_source_samples_kat(O):
    # IMPULSE fires at step 1 (tests/SimulationParametersTest.cpp:149-151)
    imp = O.source_vector(0, 0, 5)
    assert list(imp) == [0, 1, 0, 0, 0]
    # DATA indexing and zero past the end (:153-158)
    data = np.arange(200, dtype=np.float32)[:-1]
    v = O.source_vector(0, 3, 301, data=data)
    assert v[0] == 0 and v[1] == 1 and v[100] == 100 and v[300] == 0
    # GAUSSIAN centred at step 40 with width 4 (SimulationParameters.cpp:274-281)
    g = O.source_vector(0, 1, 81)
    assert g[40] == 1.0 and abs(g[44] - np.exp(-0.5)) < 1e-7 and g[36] == g[44]
    # double variant agrees
    gd = O.source_vector(0, 1, 81, double=True)
    assert np.max(np.abs(gd - g)) < 1e-7


def test_transparent_source_kat(O):
    # Transparent impulse gives 1/3 at step 3 with the grid IR
    # (tests/SimulationParametersTest.cpp:196-207)
    ir = np.loadtxt(os.path.join(HERE, "golden", "grid_ir_kat.txt")).astype(np.float32)
    assert ir[0] == 0.0 and ir[2] == np.float32(-0.333333343)
    t = O.source_vector(2, 0, 5, grid_ir=ir)
    assert t[0] == 0.0 and t[1] == 1.0 and t[3] == np.float32(1.0 / 3.0)


def test_encode_tables(O):
    ids = np.arange(28, dtype=np.uint8)
    pos_f, mat_f = O.encode_nodes(ids, np.full(28, 7, np.uint8), centred=False)
    assert pos_f[0] == 0 and mat_f[0] == 0 and (mat_f[1:] == 7).all()
    assert list(pos_f[1:9] & 0x7F) == [3] * 8
    assert list(pos_f[9:21] & 0x7F) == [4] * 12
    assert list(pos_f[21:27] & 0x7F) == [5] * 6
    assert pos_f[27] == 0x86 and (pos_f[1:] >> 7 == 1).all()
    pos_c, _ = O.encode_nodes(ids, np.zeros(28, np.uint8), centred=True)
    assert pos_c[27] == 0x80 and pos_c[0] == 0
    # number of boundary axes: corners 3, edges 2, faces 1
    ndir = [(p & 1) + ((p >> 1) & 1) + ((p >> 2) & 1) for p in pos_c]
    assert ndir[1:9] == [3] * 8 and ndir[9:21] == [2] * 12 and ndir[21:27] == [1] * 6


def test_room_ids_match_neighbour_counts(O):
    room = rooms.boxes_room((40, 36, 28), n_boxes=6, edge=(3, 12), n_materials=5, seed=3)
    X, Y, Z = room.dims
    pos, _ = O.encode_nodes(room.bid, room.mat, centred=False)
    solid = (room.bid == 0).reshape(Z, Y, X)
    k = pos.reshape(Z, Y, X) & 0x7F
    inner = (slice(1, -1),) * 3
    air_n = sum((~np.roll(solid, s, a))[inner].astype(int) for a in range(3) for s in (1, -1))
    assert np.array_equal(k[inner][~solid[inner]], air_n[~solid[inner]])


def test_count_boundaries(O):
    room = rooms.shoebox((20, 18, 16), seed=2)
    pos, _ = O.encode_nodes(room.bid, room.mat, centred=False)
    air, bnd = O.count_boundaries(pos, 0x86)
    assert air == 16 * 14 * 12 and bnd == 18 * 16 * 14 - air


def test_padding_element_index(O):
    # A 20^3 mesh padded to block (32, 4, 2) gives x = 32 and element
    # (10,10,10) at 10*20*32 + 10*32 + 10 (tests/CudaMeshTest.cpp:220-258)
    mesh = np.arange(20 * 20 * 20, dtype=np.uint32).astype(np.uint8)
    out, dims = O.pad(mesh, (20, 20, 20), (32, 4, 2))
    assert dims == (32, 20, 20)
    assert out[10 * 20 * 32 + 10 * 32 + 10] == mesh[10 * 400 + 10 * 20 + 10]
    assert out.reshape(20, 20, 32)[0].max() == 0  # plane z = 0 is cleared
    assert out.reshape(20, 20, 32)[:, 0].max() == 0
    assert out.reshape(20, 20, 32)[:, :, 0].max() == 0


def _c1(steps=120):
    room = rooms.shoebox((24, 22, 20), n_materials=6, seed=1)
    return room, steps, rooms.gaussian_pulse(steps, 3.0, t0=12.0)


def test_oracle_matches_golden(O):
    g = np.load(os.path.join(HERE, "golden", "oracle_small.npz"))
    dims = tuple(int(v) for v in g["dims"])
    X, Y, _ = dims
    src = [int(s[2]) * X * Y + int(s[1]) * X + int(s[0]) for s in g["src"]]
    rec = [int(r[2]) * X * Y + int(r[1]) * X + int(r[0]) for r in g["rec"]]
    pulse = g["pulse"]
    for centred in (False, True):
        pos, mat = O.encode_nodes(g["bid"], g["mat"], centred)
        for dbl in (False, True):
            out, _, _ = O.run(pos, mat, dims, g["admittance"], default_params(), src, [1, 0],
                              np.stack([pulse, 0.5 * pulse]), rec, pulse.size,
                              scheme=2 if centred else 0, double=dbl)
            key = f"rec_{'centred' if centred else 'forward'}_{'f64' if dbl else 'f32'}"
            assert np.array_equal(out, g[key]), key


def test_linearity_exact(O):
    room, steps, pulse = _c1()
    pos, mat = O.encode_nodes(room.bid, room.mat, False)
    args = (pos, mat, room.dims, room.admittance, default_params())
    src, rec = [room.flat(12, 11, 10)], [room.flat(5, 6, 7)]
    a, _, _ = O.run(*args, src, [1], pulse[None], rec, steps)
    b, _, _ = O.run(*args, src, [1], 2 * pulse[None], rec, steps)
    assert np.array_equal(2 * a, b)  # scaling by 2 is exact in binary floating point


def test_float_close_to_double(O):
    # The reference's single-precision arithmetic drifts from double at about
    # 5e-7 relative L2 per step in this reverberant room (1.1e-4 forward,
    # 1.6e-4 centred after 300 steps); bound it at 5e-4.
    room, steps, pulse = _c1(300)
    for centred in (False, True):
        pos, mat = O.encode_nodes(room.bid, room.mat, centred)
        args = (pos, mat, room.dims, room.admittance, default_params())
        src, rec = [room.flat(12, 11, 10)], [room.flat(5, 6, 7), room.flat(18, 15, 14)]
        f, _, _ = O.run(*args, src, [1], pulse[None], rec, steps, scheme=2 * centred)
        d, _, _ = O.run(*args, src, [1], pulse[None], rec, steps, scheme=2 * centred, double=True)
        err = np.linalg.norm(f - d) / np.linalg.norm(d)
        assert err < 5e-4, err


def test_hard_source_pins_node(O):
    room, steps, pulse = _c1(40)
    pos, mat = O.encode_nodes(room.bid, room.mat, False)
    s = room.flat(12, 11, 10)
    out, P, _ = O.run(pos, mat, room.dims, room.admittance, default_params(), [s], [0],
                      pulse[None], [s], steps)
    # A hard source overwrites the node each step before the update, so the
    # node is free only in the update itself.
    assert out.shape == (1, steps) and np.isfinite(out).all()


def test_quirk_soft_source_equals_hard(O):
    room, steps, pulse = _c1(60)
    pos, mat = O.encode_nodes(room.bid, room.mat, False)
    args = (pos, mat, room.dims, room.admittance, default_params())
    s, r = [room.flat(12, 11, 10)], [room.flat(5, 6, 7)]
    hard, _, _ = O.run(*args, s, [0], pulse[None], r, steps)
    soft_q, _, _ = O.run(*args, s, [1], pulse[None], r, steps, quirks=2)
    soft, _, _ = O.run(*args, s, [1], pulse[None], r, steps)
    assert np.array_equal(hard, soft_q) and not np.array_equal(soft, soft_q)


def test_quirk_material_index_octave0_reads_material0(O):
    room, steps, pulse = _c1(60)
    pos, mat = O.encode_nodes(room.bid, room.mat, False)
    tab = room.admittance.copy()
    one = tab.copy()
    one[:] = tab[0, 0]
    s, r = [room.flat(12, 11, 10)], [room.flat(5, 6, 7)]
    q, _, _ = O.run(pos, mat, room.dims, tab, default_params(), s, [1], pulse[None], r, steps, quirks=1)
    u, _, _ = O.run(pos, mat, room.dims, one, default_params(), s, [1], pulse[None], r, steps)
    assert np.array_equal(q, u)


def test_material_index_out_of_table_fails(O):
    room, steps, pulse = _c1(5)
    pos, mat = O.encode_nodes(room.bid, room.mat, False)
    with pytest.raises(RuntimeError):
        O.run(pos, mat, room.dims, room.admittance[:2], default_params(), [], [], np.zeros((0, 5)),
              [], steps)
