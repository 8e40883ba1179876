"""Triangle-mesh geometry and its voxelization on the GPU (pfdtd_voxelize).

The reference turns the room's boundary mesh into node bytes with an external
voxelizer (src/kernels/voxelizationUtils.cu:55-136); ``voxelize`` does that
on the device, with the conventions of ``rooms`` (one boundary id 0..27 and
one material byte per node).  ``box_mesh`` builds axis-aligned boxes as
triangle meshes, e.g. a shoebox room and obstacles inside it.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence, Tuple

import numpy as np

from . import _lib as L


def box_mesh(lo: Sequence[float], hi: Sequence[float], materials: Sequence[int] = (0,) * 6):
    """12 triangles of the box [lo, hi]; face materials in the order -x, +x,
    -y, +y, -z, +z.  Returns (vertices [8, 3], triangles [12, 3], tri_mat [12])."""
    x0, y0, z0 = (float(v) for v in lo)
    x1, y1, z1 = (float(v) for v in hi)
    v = np.array([[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0],
                  [x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1]], dtype=np.float32)
    faces = [(0, 3, 7, 4), (1, 2, 6, 5), (0, 1, 5, 4), (3, 2, 6, 7), (0, 1, 2, 3), (4, 5, 6, 7)]
    tris, mats = [], []
    for f, (a, b, c, d) in enumerate(faces):
        tris += [(a, b, c), (a, c, d)]
        mats += [materials[f], materials[f]]
    return v, np.array(tris, dtype=np.uint32), np.array(mats, dtype=np.uint8)


def merge(*meshes):
    """One mesh from several (vertices, triangles, tri_mat) tuples."""
    vs, ts, ms, off = [], [], [], 0
    for v, t, m in meshes:
        vs.append(np.asarray(v, np.float32))
        ts.append(np.asarray(t, np.uint32) + off)
        ms.append(np.asarray(m, np.uint8))
        off += len(v)
    return np.concatenate(vs), np.concatenate(ts), np.concatenate(ms)


def voxelize(vertices: np.ndarray, triangles: np.ndarray, tri_materials: np.ndarray,
             voxel_edge: float, device: int = 0) -> Tuple[np.ndarray, np.ndarray, tuple, tuple]:
    """(bid, mat, dims (X, Y, Z), origin) of the mesh; bid/mat flat x-fastest."""
    v = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 3)
    t = np.ascontiguousarray(triangles, dtype=np.uint32).reshape(-1, 3)
    m = np.ascontiguousarray(tri_materials, dtype=np.uint8).reshape(-1)
    dims = (C.c_uint32 * 3)()
    origin = (C.c_double * 3)()
    L.call("pfdtd_voxelize", v.ctypes.data, v.shape[0], t.ctypes.data, t.shape[0], m.ctypes.data,
           float(voxel_edge), int(device), dims, origin, None, None)
    n = int(dims[0]) * int(dims[1]) * int(dims[2])
    bid = np.empty(n, np.uint8)
    mat = np.empty(n, np.uint8)
    L.call("pfdtd_voxelize", v.ctypes.data, v.shape[0], t.ctypes.data, t.shape[0], m.ctypes.data,
           float(voxel_edge), int(device), dims, origin, bid.ctypes.data, mat.ctypes.data)
    return bid, mat, (int(dims[0]), int(dims[1]), int(dims[2])), tuple(origin)
