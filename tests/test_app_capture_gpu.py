"""GPU: App::runCapture through the libPyFDTD mirror.  The asynchronous
captured run (slice captures only) writes the same bitmaps and responses as
the reference's stepping loop (taken here because a mesh capture is
scheduled, at a step the run never reaches)."""
import os

import numpy as np
import pytest

from parallelfdtd_gb300 import libPyFDTD as pf
from parallelfdtd_gb300 import rooms

pytestmark = pytest.mark.gpu


def _run(tmp, with_mesh_capture):
    room = rooms.boxes_room((48, 40, 36), n_boxes=3, edge=(4, 10), n_materials=4, seed=5)
    cwd = os.getcwd()
    os.makedirs(tmp, exist_ok=True)
    os.chdir(tmp)
    try:
        app = pf.App()
        app.initializeDevices()
        app.initializeVoxels(room.bid, room.mat, room.dims)
        app.addSurfaceMaterials(room.admittance.flatten().tolist(), room.admittance.shape[0], 20)
        fs = 5000
        dx = 344.0 / (fs * np.sqrt(1.0 / 3.0))
        app.setSpatialFs(fs)
        app.setNumSteps(90)
        app.setUpdateType(0)
        app.addSource(24 * dx, 20 * dx, 18 * dx, 1, 1, 0)
        app.addReceiver(30 * dx, 14 * dx, 12 * dx)
        for slc, step, o in [(18, 20, 0), (20, 45, 1), (24, 45, 2), (18, 90, 0), (99, 30, 0)]:
            app.addSliceToCapture(slc, step, o)
        if with_mesh_capture:
            app.addMeshToCapture(10_000)
        app.runCapture()
        r = app.getResponse(0)
        app.close()
        files = sorted(f for f in os.listdir(".") if f.startswith("capture_"))
        return r, {f: open(f, "rb").read() for f in files}
    finally:
        os.chdir(cwd)


def test_async_capture_equals_stepping(gpu, tmp_path):
    r1, f1 = _run(str(tmp_path / "async"), False)
    r2, f2 = _run(str(tmp_path / "step"), True)
    assert sorted(f1) == sorted(f2) and len(f1) == 4
    assert f1 == f2
    assert np.array_equal(r1, r2) and np.abs(r1).max() > 0
