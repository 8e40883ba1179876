"""App: the reference's Python class libPyFDTD.App (ParallelFDTD
src/AppPy.cpp:96-133) over the C ABI of FDTD::App (include/pfdtd_app.h).

Method names, argument order and meaning follow the boost::python module, so
a script written for ``import libPyFDTD as pf`` runs with
``from parallelfdtd_gb300 import libPyFDTD as pf``.  Lists may be Python
lists or numpy arrays.  initializeGeometry voxelizes the triangle mesh on the
device (csrc/voxelize.cu).  Two additions: initializeVoxels (geometry that is
already voxelized, as boundary ids and materials) and setReferenceQuirks.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import _lib as L


class App:
    def __init__(self):
        self._lib = L.load()
        h = C.c_void_p()
        L.call("pfdtd_app_create", C.byref(h))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None:
            try:
                self._lib.pfdtd_app_destroy(h)
            except Exception:
                pass
            self._h = None

    def _c(self, name, *args):
        return L.call(name, self._h, *args)

    # --- methods of libPyFDTD.App ---------------------------------------
    def initializeDevices(self):
        self._c("pfdtd_app_initialize_devices")

    def initializeGeometryPy(self, indices: Sequence[int], vertices: Sequence[float]):
        idx = np.ascontiguousarray(indices, dtype=np.uint32).reshape(-1)
        ver = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1)
        self._c("pfdtd_app_initialize_geometry", idx.ctypes.data_as(C.POINTER(C.c_uint32)),
                idx.size, ver.ctypes.data_as(C.POINTER(C.c_float)), ver.size)

    def setLayerIndices(self, indices: Sequence[int], name: str):
        """Layer bookkeeping of the geometry handler; not used by the solver."""
        self._layers = getattr(self, "_layers", {})
        self._layers[name] = list(indices)

    def addSource(self, x, y, z, type_, signal, input_signal_idx):
        self._c("pfdtd_app_add_source", float(x), float(y), float(z), int(type_), int(signal),
                int(input_signal_idx))

    def addSourceDataFloat(self, src_data, num_steps, num_sources):
        d = np.ascontiguousarray(src_data, dtype=np.float32).reshape(-1)
        self._c("pfdtd_app_add_source_data_float", d.ctypes.data_as(C.POINTER(C.c_float)),
                int(num_steps), int(num_sources))

    def addSourceDataDouble(self, src_data, num_steps, num_sources):
        d = np.ascontiguousarray(src_data, dtype=np.float64).reshape(-1)
        self._c("pfdtd_app_add_source_data_double", d.ctypes.data_as(C.POINTER(C.c_double)),
                int(num_steps), int(num_sources))

    def addReceiver(self, x, y, z):
        self._c("pfdtd_app_add_receiver", float(x), float(y), float(z))

    def addSurfaceMaterials(self, material_coefficients, number_of_surfaces, number_of_coefficients):
        m = np.ascontiguousarray(material_coefficients, dtype=np.float32).reshape(-1)
        self._c("pfdtd_app_add_surface_materials", m.ctypes.data_as(C.POINTER(C.c_float)),
                int(number_of_surfaces), int(number_of_coefficients))

    def setSpatialFs(self, fs):
        self._c("pfdtd_app_set_spatial_fs", int(fs))

    def setNumSteps(self, n):
        self._c("pfdtd_app_set_num_steps", int(n))

    def setUpdateType(self, i):
        self._c("pfdtd_app_set_update_type", int(i))

    def setUniformMaterial(self, R):
        self._c("pfdtd_app_set_uniform_material", float(R))

    setUniform = setUniformMaterial

    def runVisualization(self):
        self._c("pfdtd_app_run_visualization")

    def runSimulation(self):
        self._c("pfdtd_app_run_simulation")

    def runCapture(self):
        self._c("pfdtd_app_run_capture")

    def _num_steps(self) -> int:
        n = C.c_uint()
        self._c("pfdtd_app_get_num_steps", C.byref(n))
        return int(n.value)

    def getResponse(self, rec) -> np.ndarray:
        out = np.zeros(self._num_steps(), dtype=np.float32)
        self._c("pfdtd_app_get_response", int(rec), out.ctypes.data_as(C.POINTER(C.c_float)), out.size)
        return out

    def getResponseDouble(self, rec) -> np.ndarray:
        out = np.zeros(self._num_steps(), dtype=np.float64)
        self._c("pfdtd_app_get_response_double", int(rec),
                out.ctypes.data_as(C.POINTER(C.c_double)), out.size)
        return out

    def forcePartitionTo(self, n):
        self._c("pfdtd_app_force_partition_to", int(n))

    def addSliceToCapture(self, slice_, step, orientation):
        self._c("pfdtd_app_add_slice_to_capture", int(slice_), int(step), int(orientation))

    def addMeshToCapture(self, step):
        self._c("pfdtd_app_add_mesh_to_capture", int(step))

    def setDouble(self, set_to):
        self._c("pfdtd_app_set_double", 1 if set_to else 0)

    def setCapturedB(self, db):
        self._c("pfdtd_app_set_captured_b", float(db))

    def close(self):
        self._c("pfdtd_app_close")

    def getMvox(self) -> float:
        v = C.c_float()
        self._c("pfdtd_app_get_mvox", C.byref(v))
        return float(v.value)

    def getNumElems(self) -> int:
        v = C.c_uint()
        self._c("pfdtd_app_get_num_elems", C.byref(v))
        return int(v.value)

    # --- additions --------------------------------------------------------
    def initializeVoxels(self, boundary_ids, materials, dims):
        ids = np.ascontiguousarray(boundary_ids, dtype=np.uint8).reshape(-1)
        mats = np.ascontiguousarray(materials, dtype=np.uint8).reshape(-1)
        d = (C.c_uint32 * 3)(*[int(v) for v in dims])
        if ids.size != d[0] * d[1] * d[2] or mats.size != ids.size:
            raise ValueError("voxel arrays must hold dims[0]*dims[1]*dims[2] bytes")
        self._c("pfdtd_app_initialize_voxels", C.c_void_p(ids.ctypes.data),
                C.c_void_p(mats.ctypes.data), d)

    def setReferenceQuirks(self, quirks: int):
        self._c("pfdtd_app_set_reference_quirks", int(quirks))

    def setOctave(self, octave: int):
        self._c("pfdtd_app_set_octave", int(octave))

    def getTimePerStep(self) -> float:
        v = C.c_float()
        self._c("pfdtd_app_get_time_per_step", C.byref(v))
        return float(v.value)

    def getMeshDims(self):
        d = (C.c_uint32 * 3)()
        self._c("pfdtd_app_get_mesh_dims", d)
        return tuple(int(v) for v in d)

    def getDx(self) -> float:
        v = C.c_float()
        self._c("pfdtd_app_get_dx", C.byref(v))
        return float(v.value)
