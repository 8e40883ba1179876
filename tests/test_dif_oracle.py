"""Frequency-dependent (IIR admittance) boundaries: the filter design and
the oracle's specification (no reference implementation: parity unpinned by
the reference).  CPU only."""
import numpy as np
import pytest

from parallelfdtd_gb300 import materials, rooms
from parallelfdtd_gb300.domain import default_params


@pytest.fixture(scope="module")
def O(built):
    from oracle import oracle
    return oracle


def test_filters_passive_and_stable():
    for order in (1, 2, 3):
        f = materials.positive_real_filters(12, order=order, seed=order)
        for row in f:
            assert materials.is_passive(row, order)
        t = materials.dif_table(f, order)
        assert t.shape == (12, 7) and np.allclose(t[:, 0], f[:, 0])


@pytest.mark.parametrize("scheme", [0, 2, 3])
def test_order0_filter_equals_frequency_independent(O, scheme):
    room = rooms.shoebox((24, 22, 20), n_materials=6, admittance_range=(0.05, 0.6), seed=2)
    centred = scheme != 0
    pos, mat = O.encode_nodes(room.bid, room.mat, centred)
    steps = 200
    pulse = rooms.gaussian_pulse(steps, 3.0)
    params = default_params(scheme="iwb" if scheme == 3 else "forward")
    coefs = np.zeros((6, 7))
    coefs[:, 0] = room.admittance[:, 0]
    args = (pos, mat, room.dims, room.admittance, params, [room.flat(12, 11, 10)], [1],
            pulse[None], [room.flat(5, 6, 7)], steps)
    fi, _, _ = O.run(*args, scheme=scheme, double=True)
    dif, _, _ = O.run(*args, scheme=scheme, double=True, dif=(np.ones(6), coefs))
    assert np.allclose(dif, fi, rtol=0, atol=1e-12 * np.abs(fi).max())


@pytest.mark.parametrize("scheme", [0, 2, 3])
def test_passive_filters_decay(O, scheme):
    room = rooms.shoebox((26, 24, 22), n_materials=6, seed=4)
    centred = scheme != 0
    pos, mat = O.encode_nodes(room.bid, room.mat, centred)
    steps = 2000
    pulse = rooms.gaussian_pulse(steps, 3.0)
    params = default_params(scheme="iwb" if scheme == 3 else "forward")
    table = materials.dif_table(materials.positive_real_filters(6, 3, seed=9), 3)
    out, _, _ = O.run(pos, mat, room.dims, room.admittance, params, [room.flat(13, 12, 11)], [1],
                      pulse[None], [room.flat(6, 7, 8)], steps, scheme=scheme, double=True,
                      dif=(np.ones(6), table))
    assert np.isfinite(out).all()
    # A soft source leaves a constant pressure offset that an impedance
    # boundary does not absorb (its loss acts on dp/dt); the sound (the time
    # differences) decays.
    ac = np.diff(out[0])
    assert np.sum(ac[1600:] ** 2) < 1e-2 * np.sum(ac[100:500] ** 2)
    fi, _, _ = O.run(pos, mat, room.dims, room.admittance, params, [room.flat(13, 12, 11)], [1],
                     pulse[None], [room.flat(6, 7, 8)], 400, scheme=scheme, double=True)
    assert not np.allclose(out[0, :400], fi[0])
