"""Procedural room generator invariants (CPU)."""
import numpy as np

from parallelfdtd_gb300 import rooms


def test_shoebox_counts():
    r = rooms.shoebox((16, 14, 12))
    counts = np.bincount(r.bid, minlength=28)
    assert counts[27] == 12 * 10 * 8           # pure air
    assert counts[0] == 16 * 14 * 12 - 14 * 12 * 10
    assert counts[1:9].sum() == 8               # one corner id per room corner
    assert counts[9:21].sum() == 4 * (12 + 10 + 8)


def test_no_unrepresentable_nodes():
    r = rooms.boxes_room((48, 40, 36), n_boxes=12, edge=(2, 9), seed=7)
    X, Y, Z = r.dims
    solid = (r.bid == 0).reshape(Z, Y, X)
    inner = (slice(1, -1),) * 3
    for axis in range(3):
        both = np.roll(solid, 1, axis) & np.roll(solid, -1, axis)
        assert not (both & ~solid)[inner].any()


def test_boundary_materials_from_first_solid_neighbour():
    r = rooms.shoebox((10, 9, 8), n_materials=6)
    X, Y, Z = r.dims
    mat = r.mat.reshape(Z, Y, X)
    assert mat[4, 4, 1] == 0 and mat[4, 4, X - 2] == 1
    assert mat[4, 1, 4] == 2 and mat[4, Y - 2, 4] == 3
    assert mat[1, 4, 4] == 4 and mat[Z - 2, 4, 4] == 5
    assert mat[4, 4, 4] == 0 and r.bid[r.flat(4, 4, 4)] == 27


def test_random_air_nodes_are_air():
    r = rooms.boxes_room((40, 36, 28), n_boxes=4, edge=(4, 10), seed=1)
    for p in r.random_air_nodes(10, seed=3):
        assert r.bid[r.flat(*p)] == 27
