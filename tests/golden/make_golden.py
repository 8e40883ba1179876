"""Generate the committed golden fixtures of tests/golden/.

* grid_ir_kat.txt — the free-field impulse response of the SRL grid at
  lambda^2 = 1/3 seen at the excited node: h[0] = 0 and h[n] = p^n(0) for
  p^0 = delta, p^-1 = 0, p^{n+1} = lambda^2 * (sum of the six neighbours) -
  p^{n-1}.  It carries the values the reference's tests assert for its grid
  IR file (h[0] = 0, h[2] = -0.333333343 once read as float; ParallelFDTD
  tests/SimulationParametersTest.cpp:187-194), computed in float64 on a grid
  large enough that no wall is reached.
* oracle_small.npz — receiver traces of the CPU oracle on a small procedural
  room (forward and centred, float and double), pinning the oracle against
  later regressions.

Run: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def grid_ir(n_steps: int = 64) -> np.ndarray:
    R = n_steps // 2 + 3
    n = 2 * R + 1
    l2 = 1.0 / 3.0
    prev = np.zeros((n, n, n), np.float64)
    cur = np.zeros((n, n, n), np.float64)
    cur[R, R, R] = 1.0
    h = np.zeros(n_steps, np.float64)
    for k in range(1, n_steps):
        s = np.zeros_like(cur)
        s[1:-1, 1:-1, 1:-1] = (cur[2:, 1:-1, 1:-1] + cur[:-2, 1:-1, 1:-1] + cur[1:-1, 2:, 1:-1]
                               + cur[1:-1, :-2, 1:-1] + cur[1:-1, 1:-1, 2:] + cur[1:-1, 1:-1, :-2])
        nxt = l2 * s - prev
        prev, cur = cur, nxt
        h[k] = cur[R, R, R]
    return h


def oracle_small():
    from oracle import oracle as O
    from parallelfdtd_gb300 import rooms
    from parallelfdtd_gb300.domain import default_params
    room = rooms.boxes_room((40, 36, 28), n_boxes=4, edge=(4, 10), n_materials=5, seed=11)
    steps = 80
    srcs = room.random_air_nodes(2, seed=5)
    recs = room.random_air_nodes(3, seed=6)
    pulse = rooms.gaussian_pulse(steps, 3.0, t0=12.0)
    out = {"bid": room.bid, "mat": room.mat, "dims": np.array(room.dims),
           "admittance": room.admittance, "src": np.array(srcs), "rec": np.array(recs),
           "pulse": pulse}
    for centred in (False, True):
        pos, mat = O.encode_nodes(room.bid, room.mat, centred)
        for dbl in (False, True):
            r, _, _ = O.run(pos, mat, room.dims, room.admittance, default_params(),
                            [room.flat(*s) for s in srcs], [1, 0],
                            np.stack([pulse, 0.5 * pulse]), [room.flat(*r) for r in recs], steps,
                            scheme=2 if centred else 0, double=dbl, threads=1)
            out[f"rec_{'centred' if centred else 'forward'}_{'f64' if dbl else 'f32'}"] = r
    return out


if __name__ == "__main__":
    h = grid_ir(64)
    with open(os.path.join(HERE, "grid_ir_kat.txt"), "w") as f:
        f.write("\n".join(repr(float(v)) for v in h) + "\n")
    np.savez_compressed(os.path.join(HERE, "oracle_small.npz"), **oracle_small())
    print("h[:4] =", h[:4])
