"""The IWB 27-point scheme (no reference implementation: parity unpinned by
the reference).  CPU checks of the oracle's specification."""
import numpy as np
import pytest

from parallelfdtd_gb300 import rooms
from parallelfdtd_gb300.domain import default_params


@pytest.fixture(scope="module")
def O(built):
    from oracle import oracle
    return oracle


def iwb_params():
    return default_params(scheme="iwb")


def test_constant_field_is_preserved(O):
    """Weights sum to 2 (6/4 + 12/8 + 8/16 - 3/2): a uniform field in an
    all-air periodic-free interior stays uniform."""
    X = Y = Z = 12
    pos = np.full(X * Y * Z, 0x80, np.uint8)       # inside, no boundary axes
    mat = np.zeros_like(pos)
    tab = np.zeros((1, 20))
    P0 = np.full(X * Y * Z, 0.5, np.float64)
    _, P, Pp = O.run(pos, mat, (X, Y, Z), tab, iwb_params(), [], [], np.zeros((0, 3)), [], 3,
                     scheme=3, double=True, P0=P0, Pp0=P0)
    inner = P.reshape(Z, Y, X)[3:-3, 3:-3, 3:-3]
    assert np.allclose(inner, 0.5, rtol=0, atol=1e-15)


def _box(admittance=0.3, dims=(28, 26, 24)):
    room = rooms.shoebox(dims, n_materials=1, seed=3)
    room.admittance[:] = admittance
    pos, mat = None, None
    return room


def test_stable_and_decaying(O):
    """Lossy walls: the sound decays.  Measured on the time-differenced trace:
    a soft source leaves a constant offset that no closed room removes, and at
    lambda = 1 the modes at omega*dt = pi (sign flip every step) are left
    undamped by the centred loss term, at a level far below the sound."""
    room = _box(0.4)
    pos, mat = O.encode_nodes(room.bid, room.mat, centred=True)
    steps = 1500
    pulse = rooms.gaussian_pulse(steps, 2.0, t0=8.0)
    out, _, _ = O.run(pos, mat, room.dims, room.admittance, iwb_params(), [room.flat(14, 13, 12)],
                      [1], pulse[None], [room.flat(6, 7, 8)], steps, scheme=3, double=True)
    ac = np.diff(out[0])
    e_early = np.sum(ac[0:300] ** 2)
    e_late = np.sum(ac[1200:1500] ** 2)
    assert np.isfinite(out).all() and e_late < 1e-2 * e_early


@pytest.mark.parametrize("admittance", [0.0, 0.5])
def test_obstacles_stay_bounded(O, admittance):
    """Rooms with solid boxes (obstacle edges and corners seen from the air):
    the finite-volume closure keeps an impulse response bounded, lossless or
    lossy, over 2000 steps."""
    room = rooms.boxes_room((40, 36, 32), n_boxes=4, edge=(3, 10), n_materials=4,
                            admittance_range=(0.01, 0.5), seed=5)
    pos, mat = O.encode_nodes(room.bid, room.mat, centred=True)
    steps = 2000
    src = room.random_air_nodes(1, seed=8)
    rec = room.random_air_nodes(3, seed=9)
    out, P, _ = O.run(pos, mat, room.dims, room.admittance * admittance, iwb_params(),
                      [room.flat(*s) for s in src], [1], rooms.impulse(steps)[None],
                      [room.flat(*r) for r in rec], steps, scheme=3, double=True)
    a = np.abs(out)
    assert np.isfinite(out).all()
    assert a[:, 1000:].max() < 3.0 * a[:, :1000].max() and np.abs(P).max() < 10.0


def test_rigid_walls_do_not_decay_blow_up(O):
    room = _box(0.0)
    pos, mat = O.encode_nodes(room.bid, room.mat, centred=True)
    steps = 1500
    pulse = rooms.gaussian_pulse(steps, 2.0, t0=8.0)
    out, _, _ = O.run(pos, mat, room.dims, room.admittance, iwb_params(), [room.flat(14, 13, 12)],
                      [1], pulse[None], [room.flat(6, 7, 8)], steps, scheme=3, double=True)
    assert np.isfinite(out).all() and np.abs(out).max() < 10.0


def test_mirror_symmetry(O):
    """A centred source in a box with one material: receivers mirrored in x
    see the same trace up to rounding."""
    dims = (27, 25, 23)
    room = _box(0.2, dims)
    pos, mat = O.encode_nodes(room.bid, room.mat, centred=True)
    steps = 300
    pulse = rooms.gaussian_pulse(steps, 2.0, t0=8.0)
    out, _, _ = O.run(pos, mat, dims, room.admittance, iwb_params(), [room.flat(13, 12, 11)], [1],
                      pulse[None], [room.flat(5, 9, 7), room.flat(21, 9, 7)], steps, scheme=3,
                      double=True)
    assert np.allclose(out[0], out[1], rtol=0, atol=1e-12 * np.abs(out).max())


def test_float_close_to_double(O):
    room = _box(0.3)
    pos, mat = O.encode_nodes(room.bid, room.mat, centred=True)
    steps = 300
    pulse = rooms.gaussian_pulse(steps, 3.0)
    args = (pos, mat, room.dims, room.admittance, iwb_params(), [room.flat(14, 13, 12)], [1],
            pulse[None], [room.flat(6, 7, 8)], steps)
    f, _, _ = O.run(*args, scheme=3)
    d, _, _ = O.run(*args, scheme=3, double=True)
    assert np.linalg.norm(f - d) / np.linalg.norm(d) < 1e-3


def test_nodes_outside_the_room_hold_plus_zero(O):
    """A node without the inside bit stores +0 every step (its update would be
    0 times a finite value, whose zero sign depends on neighbours no inside
    node reads); inside nodes are unaffected."""
    room = rooms.boxes_room((40, 32, 28), n_boxes=4, edge=(4, 10), n_materials=5, seed=9)
    pos, mat = O.encode_nodes(room.bid, room.mat, True)
    steps = 40
    pulse = rooms.gaussian_pulse(steps, 3.0)
    src = room.random_air_nodes(1, seed=1)
    for double in (False, True):
        _, P, Pp = O.run(pos, mat, room.dims, room.admittance, iwb_params(), [room.flat(*src[0])],
                         [1], pulse[None], [], steps, scheme=3, double=double)
        X, Y, Z = room.dims
        outside = (pos & 0x80) == 0
        planes = np.zeros((Z, Y, X), bool)
        planes[1:-1] = True  # planes 0 and Z-1 are never updated
        sel = (outside & planes.reshape(-1))
        for F in (P, Pp):
            v = np.asarray(F).reshape(-1)[sel]
            assert np.all(v == 0) and not np.any(np.signbit(v))
        inside = ~outside & planes.reshape(-1)
        assert np.abs(np.asarray(P).reshape(-1)[inside]).max() > 1e-6
