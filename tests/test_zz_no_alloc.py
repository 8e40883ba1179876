"""The slice capture that allocates nothing (pfdtd_capture_slice_noalloc).

Callers that cannot allocate device memory while a simulation runs — a
serving loop whose HBM budget is already given to resident domains, or a
per-step capture loop that must not stall on cudaFree — use this variant; it
gathers into a fixed scratch array compiled into the library.  Its output
must equal the allocating capture's, bit for bit (the tolerance of every
parity test here), on consecutive calls that reuse the shared scratch.  This
file is collected last so that a failure here stops a run only after every
other test has run.
"""
import numpy as np
import pytest

from parallelfdtd_gb300 import _lib as L
from parallelfdtd_gb300 import rooms
from parallelfdtd_gb300.domain import Domain

pytestmark = pytest.mark.gpu


def _domain(dims, prec="f32"):
    room = rooms.boxes_room(dims, n_boxes=3, edge=(4, 9), n_materials=4, seed=21)
    d = Domain(room.dims, prec)
    d.set_voxels(room.bid, room.mat, centred=False)
    d.set_materials(room.admittance)
    d.set_params()
    d.set_sources([(dims[0] // 2, dims[1] // 2, dims[2] // 2)], [1],
                  rooms.gaussian_pulse(200, 3.0)[None])
    return d


def test_noalloc_capture_matches_allocating_capture(gpu):
    with _domain((48, 40, 36)) as d:
        d.run(30)
        for call in range(2):  # two calls in a row per slice, with steps between
            for orientation, slc in [(0, 17), (1, 20), (2, 23), (0, 3), (2, 46)]:
                ref_p, ref_q = d.capture_slice(orientation, slc)
                p, q = d.capture_slice_noalloc(orientation, slc)
                assert np.array_equal(p, ref_p), (call, orientation, slc)
                assert np.array_equal(q, ref_q), (call, orientation, slc)
            d.run(25)
        assert np.abs(d.capture_slice_noalloc(0, 18)[0]).max() > 0


def test_noalloc_capture_other_precision_and_order(gpu):
    # A smaller slice after a larger one: stale scratch contents must not leak.
    with _domain((64, 60, 20), "f64") as d:
        d.run(20)
        big = d.capture_slice_noalloc(0, 10)
        small_p, small_q = d.capture_slice_noalloc(2, 30)
        ref_p, ref_q = d.capture_slice(2, 30)
        assert big[0].shape == (60, 64)
        assert np.array_equal(small_p, ref_p) and np.array_equal(small_q, ref_q)


def test_noalloc_capture_rejects_oversized_slices(gpu):
    with Domain((1100, 1000, 3), "f32") as d:
        with pytest.raises(L.PfdtdError) as e:
            d.capture_slice_noalloc(0, 1)
        assert e.value.status == L.ERR_ARG and "exceeds" in str(e.value)
        p, q = d.capture_slice_noalloc(1, 10)  # 1100 x 3 nodes fits
        ref_p, ref_q = d.capture_slice(1, 10)
        assert np.array_equal(p, ref_p) and np.array_equal(q, ref_q)
