"""Procedural rooms in the voxelizer's output format.

The reference voxelizes a triangle mesh with an external GPU voxelizer whose
output is one byte per node: a boundary id 0..27 (0 = solid/outside,
1..8 corners, 9..20 edges, 21..26 faces, 27 = air) and one material byte
(src/kernels/voxelizationUtils.cu:55-136).  The scheme translation
(src/kernels/cudaMesh.cu:328-480) then turns the id into the forward K count
or the centred DIR/SIGN bits.  This module builds the same pair of byte arrays
for axis-aligned rooms, so that the kernels can be driven without a triangle
mesh: a shoebox with a 1-voxel solid shell and, optionally, seeded solid boxes
inside it.

Conventions (shared by the CUDA path and the CPU oracle, which both consume
these arrays):
  * arrays are flat, x fastest: index = z*X*Y + y*X + x (cudaMesh.h:247-249);
  * the six shell faces carry materials 0..5 in the order -x,+x,-y,+y,-z,+z;
  * an air node whose neighbours are solid on both sides of one axis has no
    boundary id in the voxelizer's table; such nodes are turned solid
    (repeated until none is left);
  * a boundary node takes the material of its first solid neighbour in the
    order -x,+x,-y,+y,-z,+z; air nodes keep material 0.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import numpy as np

# Missing-neighbour masks (bit set = that neighbour is solid).
_XM, _XP, _YM, _YP, _ZM, _ZP = 1, 2, 4, 8, 16, 32

# Boundary id for each missing-neighbour set.  The voxelizer's ids name the
# neighbours that are present ("Left, Right, In, Out, Down" ...), as spelled
# out next to the centred translation in src/kernels/cudaMesh.cu:372-478:
# Left/Right = -x/+x, In/Out = -y/+y, Down/Up = -z/+z.
_BID_OF_MISSING = {
    0: 27,
    _ZP: 21, _YM: 22, _YP: 23, _XM: 24, _XP: 25, _ZM: 26,
    _ZP | _YP: 9, _ZP | _YM: 10, _ZP | _XP: 11, _ZP | _XM: 12,
    _ZM | _YP: 13, _ZM | _YM: 14, _ZM | _XP: 15, _ZM | _XM: 16,
    _XP | _YP: 17, _XM | _YP: 18, _XP | _YM: 19, _XM | _YM: 20,
    _ZP | _XP | _YP: 1, _ZP | _XM | _YP: 2, _ZP | _XP | _YM: 3, _ZP | _XM | _YM: 4,
    _ZM | _XP | _YP: 5, _ZM | _XM | _YP: 6, _ZM | _XP | _YM: 7, _ZM | _XM | _YM: 8,
}

BID_LUT = np.zeros(64, dtype=np.uint8)
_VALID = np.zeros(64, dtype=bool)
for _m, _b in _BID_OF_MISSING.items():
    BID_LUT[_m] = _b
    _VALID[_m] = True


@dataclass
class Room:
    """A voxelized room: boundary ids and material bytes, x fastest."""

    dims: Tuple[int, int, int]          # (X, Y, Z)
    bid: np.ndarray                     # uint8 [N], 0..27
    mat: np.ndarray                     # uint8 [N]
    admittance: np.ndarray              # float64 [n_mat, 20]
    boxes: List[Tuple[int, int, int, int, int, int]] = field(default_factory=list)

    @property
    def n_nodes(self) -> int:
        X, Y, Z = self.dims
        return X * Y * Z

    @property
    def n_materials(self) -> int:
        return int(self.admittance.shape[0])

    def flat(self, x: int, y: int, z: int) -> int:
        X, Y, _ = self.dims
        return z * X * Y + y * X + x

    def coords(self, idx: int) -> Tuple[int, int, int]:
        X, Y, _ = self.dims
        return int(idx % X), int((idx // X) % Y), int(idx // (X * Y))

    def air_nodes(self) -> np.ndarray:
        """Flat indices of pure air nodes (id 27: all six neighbours air)."""
        return np.flatnonzero(self.bid == 27)

    def boundary_fraction(self) -> float:
        inside = np.count_nonzero(self.bid)
        return float(np.count_nonzero((self.bid > 0) & (self.bid < 27))) / max(inside, 1)

    def random_air_nodes(self, n: int, seed: int, margin: int = 2) -> List[Tuple[int, int, int]]:
        """n distinct seeded air nodes at least `margin` nodes from the shell."""
        rng = np.random.default_rng(seed)
        X, Y, Z = self.dims
        out: List[Tuple[int, int, int]] = []
        seen = set()
        tries = 0
        while len(out) < n:
            tries += 1
            if tries > 1000000:
                raise RuntimeError("room has too few air nodes")
            x = int(rng.integers(margin, X - margin))
            y = int(rng.integers(margin, Y - margin))
            z = int(rng.integers(margin, Z - margin))
            if (x, y, z) in seen or self.bid[self.flat(x, y, z)] != 27:
                continue
            seen.add((x, y, z))
            out.append((x, y, z))
        return out


def _neighbour_missing(solid: np.ndarray) -> np.ndarray:
    """6-bit missing-neighbour mask per node (array shape (Z, Y, X))."""
    m = np.zeros(solid.shape, dtype=np.uint8)
    s = solid
    m[:, :, 1:] |= np.where(s[:, :, :-1], _XM, 0).astype(np.uint8)
    m[:, :, :-1] |= np.where(s[:, :, 1:], _XP, 0).astype(np.uint8)
    m[:, 1:, :] |= np.where(s[:, :-1, :], _YM, 0).astype(np.uint8)
    m[:, :-1, :] |= np.where(s[:, 1:, :], _YP, 0).astype(np.uint8)
    m[1:, :, :] |= np.where(s[:-1, :, :], _ZM, 0).astype(np.uint8)
    m[:-1, :, :] |= np.where(s[1:, :, :], _ZP, 0).astype(np.uint8)
    # Nodes on the outer faces have no neighbour outside the grid; those
    # nodes are always solid (shell), so the value there is irrelevant.
    return m


def _first_solid_material(solid: np.ndarray, smat: np.ndarray) -> np.ndarray:
    """Material of the first solid neighbour in the order -x,+x,-y,+y,-z,+z."""
    out = np.zeros(solid.shape, dtype=np.uint8)
    done = np.zeros(solid.shape, dtype=bool)

    def take(dst_sl, src_sl):
        cand = solid[src_sl] & ~done[dst_sl]
        out[dst_sl] = np.where(cand, smat[src_sl], out[dst_sl])
        done[dst_sl] |= cand

    take((slice(None), slice(None), slice(1, None)), (slice(None), slice(None), slice(None, -1)))
    take((slice(None), slice(None), slice(None, -1)), (slice(None), slice(None), slice(1, None)))
    take((slice(None), slice(1, None), slice(None)), (slice(None), slice(None, -1), slice(None)))
    take((slice(None), slice(None, -1), slice(None)), (slice(None), slice(1, None), slice(None)))
    take((slice(1, None), slice(None), slice(None)), (slice(None, -1), slice(None), slice(None)))
    take((slice(None, -1), slice(None), slice(None)), (slice(1, None), slice(None), slice(None)))
    return out


def build_room(dims: Sequence[int], admittance: np.ndarray,
               boxes: Sequence[Tuple[int, int, int, int, int, int, int]] = ()) -> Room:
    """Room with a solid shell (face materials 0..5) and solid boxes.

    `boxes` holds (x0, y0, z0, x1, y1, z1, material) with half-open extents.
    """
    X, Y, Z = (int(d) for d in dims)
    if min(X, Y, Z) < 3:
        raise ValueError("room needs at least 3 nodes per axis")
    solid = np.zeros((Z, Y, X), dtype=bool)
    smat = np.zeros((Z, Y, X), dtype=np.uint8)
    faces = [
        ((slice(None), slice(None), 0), 0), ((slice(None), slice(None), X - 1), 1),
        ((slice(None), 0, slice(None)), 2), ((slice(None), Y - 1, slice(None)), 3),
        ((0, slice(None), slice(None)), 4), ((Z - 1, slice(None), slice(None)), 5),
    ]
    n_mat = admittance.shape[0]
    for sl, m in faces:
        solid[sl] = True
        smat[sl] = m % n_mat
    kept = []
    for (x0, y0, z0, x1, y1, z1, m) in boxes:
        x0, x1 = max(x0, 1), min(x1, X - 1)
        y0, y1 = max(y0, 1), min(y1, Y - 1)
        z0, z1 = max(z0, 1), min(z1, Z - 1)
        if x0 >= x1 or y0 >= y1 or z0 >= z1:
            continue
        solid[z0:z1, y0:y1, x0:x1] = True
        smat[z0:z1, y0:y1, x0:x1] = m % n_mat
        kept.append((x0, y0, z0, x1, y1, z1))
    # Close slots that leave an air node with solid on both sides of an axis.
    while True:
        miss = _neighbour_missing(solid)
        bad = (~solid) & ~_VALID[miss]
        if not bad.any():
            break
        fill = _first_solid_material(solid, smat)
        smat = np.where(bad, fill, smat)
        solid |= bad
    miss = _neighbour_missing(solid)
    bid = np.where(solid, 0, BID_LUT[miss]).astype(np.uint8)
    bmat = _first_solid_material(solid, smat)
    mat = np.where((bid > 0) & (bid < 27), bmat, 0).astype(np.uint8)
    return Room((X, Y, Z), bid.reshape(-1), mat.reshape(-1),
                np.asarray(admittance, dtype=np.float64), kept)


def admittance_table(n_mat: int, low: float, high: float, seed: int) -> np.ndarray:
    """Frequency-independent admittances: all 20 coefficients equal, U(low, high)."""
    rng = np.random.default_rng(seed)
    y = rng.uniform(low, high, size=n_mat)
    return np.repeat(y[:, None], 20, axis=1)


def shoebox(dims: Sequence[int] = (64, 64, 64), n_materials: int = 6,
            admittance_range=(0.01, 0.5), seed: int = 1) -> Room:
    """Air interior, 1-voxel solid shell, one material per wall face."""
    tab = admittance_table(n_materials, admittance_range[0], admittance_range[1], seed)
    return build_room(dims, tab)


def boxes_room(dims: Sequence[int] = (512, 384, 256), n_boxes: int = 40,
               edge=(8, 64), n_materials: int = 20, admittance_range=(0.01, 0.9),
               seed: int = 2) -> Room:
    """Shoebox with seeded axis-aligned solid boxes (edges U{edge}) inside."""
    rng = np.random.default_rng(seed)
    tab = admittance_table(n_materials, admittance_range[0], admittance_range[1], seed + 1)
    X, Y, Z = (int(d) for d in dims)
    boxes = []
    for _ in range(n_boxes):
        ex, ey, ez = (int(rng.integers(edge[0], edge[1] + 1)) for _ in range(3))
        x0 = int(rng.integers(1, max(2, X - 1 - ex)))
        y0 = int(rng.integers(1, max(2, Y - 1 - ey)))
        z0 = int(rng.integers(1, max(2, Z - 1 - ez)))
        m = int(rng.integers(0, n_materials))
        boxes.append((x0, y0, z0, x0 + ex, y0 + ey, z0 + ez, m))
    return build_room(dims, tab, boxes)


def gaussian_pulse(n_steps: int, sigma: float = 5.0, t0: Optional[float] = None) -> np.ndarray:
    """exp(-0.5((n - t0)/sigma)^2), t0 = 8 sigma by default."""
    if t0 is None:
        t0 = 8.0 * sigma
    n = np.arange(n_steps, dtype=np.float64)
    return np.exp(-0.5 * ((n - t0) / sigma) ** 2)


def impulse(n_steps: int) -> np.ndarray:
    """1 at step 1, as the reference's IMPULSE input (SimulationParameters.cpp:266-273)."""
    v = np.zeros(n_steps, dtype=np.float64)
    if n_steps > 1:
        v[1] = 1.0
    return v
