"""GPU: the device voxelizer (triangle mesh -> boundary ids and materials).

The reference's voxelizer is an external library that is not vendored, so its
output is not pinned; the voxelizer here follows the conventions of the
procedural rooms (rooms.py), and a grid-aligned box mesh must voxelize to
exactly the procedural room, ids and materials.
"""
import numpy as np
import pytest

from parallelfdtd_gb300 import rooms
from parallelfdtd_gb300.geometry import box_mesh, merge, voxelize

pytestmark = pytest.mark.gpu


def test_box_room_equals_procedural_room(gpu):
    room = box_mesh((0, 0, 0), (20, 16, 12), materials=(0, 1, 2, 3, 4, 5))
    a = box_mesh((5, 4, 3), (9, 8, 6), materials=(6,) * 6)
    b = box_mesh((10, 4, 3), (13, 8, 6), materials=(6,) * 6)   # 1-voxel slot to box a
    c = box_mesh((14, 10, 2), (17, 13, 9), materials=(3,) * 6)
    v, t, m = merge(room, a, b, c)
    bid, mat, dims, origin = voxelize(v, t, m, 1.0)
    assert dims == (22, 18, 14)
    assert np.allclose(origin, (-1.0, -1.0, -1.0))
    ref = rooms.build_room(dims, rooms.admittance_table(7, 0.1, 0.5, 1),
                           boxes=[(6, 5, 4, 10, 9, 7, 6), (11, 5, 4, 14, 9, 7, 6),
                                  (15, 11, 3, 18, 14, 10, 3)])
    assert np.array_equal(bid, ref.bid)
    assert np.array_equal(mat, ref.mat)


def test_scaled_room_and_node_coordinates(gpu):
    """A room of 7.875 x 5.125 x 3.25 m at dx = 0.125 m: node i of an axis sits
    at (i - 1) dx from the mesh's minimum, as the reference's element
    coordinates ROUND(p/dx) + 1 assume, so the room holds 63 x 41 x 26 air
    nodes with one solid layer around them."""
    room = box_mesh((2.0, -1.0, 0.5), (9.875, 4.125, 3.75))
    bid, mat, dims, origin = voxelize(*room, 0.125)
    X, Y, Z = dims
    assert (X, Y, Z) == (65, 43, 28)
    assert np.allclose(origin, (1.875, -1.125, 0.375))
    b = bid.reshape(Z, Y, X)
    inside = b > 0
    assert inside[1:27, 1:42, 1:64].all() and inside.sum() == 63 * 41 * 26
    assert (b[1:27, 1:42, 1] != 27).all() and (b[2:26, 2:41, 2] == 27).all()


def test_sphere_volume_and_ids(gpu):
    """A closed UV sphere (radius 10, dx 0.5): the air volume is the sphere's
    within a few per cent, ids are valid and every boundary node touches
    solid."""
    n_lat, n_lon, r = 48, 96, 10.0
    verts = [(0, 0, r)]
    for i in range(1, n_lat):
        th = np.pi * i / n_lat
        for j in range(n_lon):
            ph = 2 * np.pi * j / n_lon
            verts.append((r * np.sin(th) * np.cos(ph), r * np.sin(th) * np.sin(ph), r * np.cos(th)))
    verts.append((0, 0, -r))
    tris = []
    for j in range(n_lon):
        tris.append((0, 1 + j, 1 + (j + 1) % n_lon))
    for i in range(n_lat - 2):
        a0, b0 = 1 + i * n_lon, 1 + (i + 1) * n_lon
        for j in range(n_lon):
            j1 = (j + 1) % n_lon
            tris += [(a0 + j, b0 + j, b0 + j1), (a0 + j, b0 + j1, a0 + j1)]
    last = len(verts) - 1
    base = 1 + (n_lat - 2) * n_lon
    for j in range(n_lon):
        tris.append((base + j, last, base + (j + 1) % n_lon))
    v = np.array(verts, np.float32)
    t = np.array(tris, np.uint32)
    bid, mat, dims, origin = voxelize(v, t, np.zeros(len(t), np.uint8), 0.5)
    air = np.count_nonzero(bid) * 0.5 ** 3
    assert abs(air / (4 / 3 * np.pi * r ** 3) - 1) < 0.03
    assert bid.max() <= 27
    X, Y, Z = dims
    b = bid.reshape(Z, Y, X)
    solid = b == 0
    boundary = (b > 0) & (b < 27)
    nb = np.zeros_like(solid)
    nb[:, :, 1:] |= solid[:, :, :-1]
    nb[:, :, :-1] |= solid[:, :, 1:]
    nb[:, 1:] |= solid[:, :-1]
    nb[:, :-1] |= solid[:, 1:]
    nb[1:] |= solid[:-1]
    nb[:-1] |= solid[1:]
    assert np.array_equal(boundary, (b > 0) & nb)


def test_app_voxelizes_its_mesh(gpu):
    """libPyFDTD flow with a triangle mesh (initializeGeometryPy, one material
    row per triangle) gives the same responses as the same room given as
    voxels (initializeVoxels)."""
    from parallelfdtd_gb300 import libPyFDTD as pf
    fs = 4000
    dx = 344.0 / (fs * np.sqrt(1.0 / 3.0))   # the reference's dx = c / (fs * lambda)
    L_ = (24 * dx, 18 * dx, 14 * dx)
    v, t, m = merge(box_mesh((0, 0, 0), L_, materials=(0, 1, 2, 3, 4, 5)),
                    box_mesh((6 * dx, 5 * dx, 4 * dx), (10 * dx, 9 * dx, 7 * dx), materials=(6,) * 6))
    adm = np.linspace(0.1, 0.7, 7)
    coefs = np.repeat(adm[m][:, None], 20, axis=1)          # one row per triangle
    steps = 120

    def run(app):
        app.setSpatialFs(fs)
        app.setNumSteps(steps)
        app.setUpdateType(0)
        app.addSurfaceMaterials(coefs.flatten().tolist(), len(t), 20)
        app.addSource(12 * dx, 9 * dx, 7 * dx, 1, 0, 0)
        app.addReceiver(16 * dx, 12 * dx, 5 * dx)
        app.runSimulation()
        r = app.getResponse(0)
        app.close()
        return r

    a = pf.App()
    a.initializeDevices()
    a.initializeGeometryPy(t.flatten().tolist(), v.flatten().tolist())
    r_mesh = run(a)
    bid, mat, dims, _ = voxelize(v, t, m, dx)
    b = pf.App()
    b.initializeDevices()
    b.initializeGeometryPy(t.flatten().tolist(), v.flatten().tolist())  # materials per triangle
    b.initializeVoxels(bid, mat, dims)
    r_vox = run(b)
    assert np.abs(r_mesh).max() > 0
    assert np.array_equal(r_mesh, r_vox)
