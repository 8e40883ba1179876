"""ctypes binding of libpfdtd.so (the C ABI declared in include/pfdtd.h and
include/pfdtd_app.h).

The library is the product: there is no fallback.  If libpfdtd.so is missing
or cannot be loaded, importing anything that needs it raises, naming the build
step (``python -c "import __graft_entry__ as g; g.build()"`` or
``python -m parallelfdtd_gb300.build``).
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libpfdtd.so")

# Status codes (pfdtd.h)
OK = 0
INTERRUPTED = 1
ERR_ARG = -1
ERR_CUDA = -2
ERR_MATERIAL = -3
ERR_NOMEM = -4
ERR_STATE = -5
ERR_UNSUPPORTED = -6

F32, F64, F16, BF16 = 0, 1, 2, 3
SRL_FORWARD, SHARED, SRL, IWB = 0, 1, 2, 3
SRC_HARD, SRC_SOFT, SRC_TRANSPARENT = 0, 1, 2
QUIRK_MATIDX, QUIRK_SOFTSRC = 1, 2
FIELD_CURRENT, FIELD_PAST = 0, 1
KERNEL_AUTO, KERNEL_ZMARCH, KERNEL_TMA, KERNEL_TB = 0, 1, 2, 3

INTERRUPT_FN = C.CFUNCTYPE(C.c_int)
PROGRESS_FN = C.CFUNCTYPE(None, C.c_int, C.c_int, C.c_float)

_vp = C.c_void_p
_i64 = C.c_int64
_i32 = C.c_int
_u32 = C.c_uint32
_pu8 = C.POINTER(C.c_uint8)

# name: (restype, argtypes)
_SIGNATURES = {
    "pfdtd_last_error": (C.c_char_p, []),
    "pfdtd_version": (C.c_char_p, []),
    "pfdtd_device_count": (_i32, [C.POINTER(_i32)]),
    "pfdtd_create": (_i32, [_i64, _i64, _i64, _i32, _i32, C.POINTER(_vp)]),
    "pfdtd_destroy": (_i32, [_vp]),
    "pfdtd_create_batched": (_i32, [_i64, _i64, _i64, _i32, _i32, _i32, C.POINTER(_vp)]),
    "pfdtd_get_fields": (_i32, [_vp, C.POINTER(_i32)]),
    "pfdtd_set_sources_batched": (_i32, [_vp, _i32, C.POINTER(_i64), C.POINTER(C.c_int32),
                                         C.POINTER(C.c_int32), _vp, _i64]),
    "pfdtd_set_receivers_batched": (_i32, [_vp, _i32, C.POINTER(_i64), C.POINTER(C.c_int32)]),
    "pfdtd_get_dims": (_i32, [_vp, C.POINTER(_i64)]),
    "pfdtd_get_precision": (_i32, [_vp, C.POINTER(_i32)]),
    "pfdtd_get_serial": (_i32, [_vp, C.POINTER(_i64)]),
    "pfdtd_set_quirks": (_i32, [_vp, _i32]),
    "pfdtd_set_nodes": (_i32, [_vp, _vp, _vp, _i32]),
    "pfdtd_get_node_ptrs": (_i32, [_vp, C.POINTER(_vp), C.POINTER(_vp)]),
    "pfdtd_nodes_changed": (_i32, [_vp]),
    "pfdtd_get_nodes": (_i32, [_vp, _vp, _vp]),
    "pfdtd_set_materials": (_i32, [_vp, C.POINTER(C.c_double), _i32, _i32]),
    "pfdtd_set_params": (_i32, [_vp, C.POINTER(C.c_double)]),
    "pfdtd_set_dif_filters": (_i32, [_vp, _i32, C.POINTER(C.c_int32), C.POINTER(C.c_double)]),
    "pfdtd_get_dif_count": (_i32, [_vp, C.POINTER(_i64)]),
    "pfdtd_set_sources": (_i32, [_vp, _i32, C.POINTER(_i64), C.POINTER(C.c_int32), _vp, _i64]),
    "pfdtd_set_receivers": (_i32, [_vp, _i32, C.POINTER(_i64)]),
    "pfdtd_set_scheme": (_i32, [_vp, _i32]),
    "pfdtd_set_update_form": (_i32, [_vp, _i32]),
    "pfdtd_set_wait_limit": (_i32, [_vp, C.c_uint64]),
    "pfdtd_run": (_i32, [_vp, _i64, _vp, INTERRUPT_FN, PROGRESS_FN, C.POINTER(C.c_double)]),
    "pfdtd_run_device": (_i32, [_vp, _i64, _vp]),
    "pfdtd_profile_update": (_i32, [_vp, _i32]),
    "pfdtd_step": (_i32, [_vp, _i64, _i32, _vp, _i64]),
    "pfdtd_set_sample": (_i32, [_vp, _i64, _i64, _i64, C.c_double]),
    "pfdtd_add_sample": (_i32, [_vp, _i64, _i64, _i64, C.c_double]),
    "pfdtd_get_sample": (_i32, [_vp, _i64, _i64, _i64, C.POINTER(C.c_double)]),
    "pfdtd_flip": (_i32, [_vp]),
    "pfdtd_reset_fields": (_i32, [_vp]),
    "pfdtd_get_field_ptr": (_i32, [_vp, _i32, C.POINTER(_vp)]),
    "pfdtd_download_field": (_i32, [_vp, _i32, _vp]),
    "pfdtd_upload_field": (_i32, [_vp, _i32, _vp]),
    "pfdtd_capture_slice": (_i32, [_vp, _i32, _i64, _vp, _vp]),
    "pfdtd_capture_slice_noalloc": (_i32, [_vp, _i32, _i64, _vp, _vp]),
    "pfdtd_get_stream": (_i32, [_vp, C.POINTER(_vp)]),
    "pfdtd_set_kernel": (_i32, [_vp, _i32]),
    "pfdtd_set_tile": (_i32, [_vp, _i32]),
    "pfdtd_get_kernel": (_i32, [_vp, C.POINTER(_i32)]),
    "pfdtd_set_temporal_block": (_i32, [_vp, _i32]),
    "pfdtd_run_async": (_i32, [_vp, _i64]),
    "pfdtd_run_captures": (_i32, [_vp, _i64, _vp, _i32, C.POINTER(_i64), C.POINTER(C.c_int32),
                                  C.POINTER(_i64), C.POINTER(_vp), C.POINTER(_vp)]),
    "pfdtd_host_alloc": (_i32, [C.c_size_t, C.POINTER(_vp)]),
    "pfdtd_host_free": (_i32, [_vp]),
    "pfdtd_query": (_i32, [_vp, C.POINTER(_i32)]),
    "pfdtd_fetch_receivers": (_i32, [_vp, _vp]),
    "pfdtd_encode_nodes_host": (_i32, [_i32, _vp, _vp, _i64]),
    "pfdtd_transparent_source": (_i32, [_vp, _i64, _vp, _i64, _vp, _i32]),
    "pfdtd_resample": (_i32, [_vp, _i64, _i64, _i32, C.POINTER(C.c_double), _i32, _i32, _i32,
                              _i64, _i64, _vp, _i32]),
    "pfdtd_post_filter": (_i32, [_vp, _i64, _i64, _i32, C.POINTER(C.c_double), _i32, _i32,
                                 C.c_double, _vp, _i32]),
    "pfdtd_voxelize": (_i32, [_vp, _i64, _vp, _i64, _vp, C.c_double, _i32,
                              C.POINTER(C.c_uint32), C.POINTER(C.c_double), _vp, _vp]),
    # request loop (pfdtd_server.h)
    "pfdtd_request_create": (_i32, [_i64, _i64, _i64, _i32, _i32, _i32, _i64, C.POINTER(_vp)]),
    "pfdtd_request_set_voxels": (_i32, [_vp, _vp, _vp]),
    "pfdtd_request_set_nodes": (_i32, [_vp, _vp, _vp]),
    "pfdtd_request_set_materials": (_i32, [_vp, C.POINTER(C.c_double), _i32, _i32]),
    "pfdtd_request_set_dif_filters": (_i32, [_vp, _i32, C.POINTER(C.c_int32),
                                             C.POINTER(C.c_double)]),
    "pfdtd_request_set_params": (_i32, [_vp, C.POINTER(C.c_double)]),
    "pfdtd_request_set_sources": (_i32, [_vp, _i32, C.POINTER(_i64), C.POINTER(C.c_int32),
                                         C.POINTER(C.c_int32), C.POINTER(C.c_double), _i64]),
    "pfdtd_request_set_receivers": (_i32, [_vp, _i32, C.POINTER(_i64), C.POINTER(C.c_int32)]),
    "pfdtd_request_set_temporal_block": (_i32, [_vp, _i32]),
    "pfdtd_request_bytes": (_i32, [_vp, C.POINTER(C.c_uint64)]),
    "pfdtd_request_destroy": (_i32, [_vp]),
    "pfdtd_server_create": (_i32, [_i32, C.c_uint64, _i32, C.POINTER(_vp)]),
    "pfdtd_server_submit": (_i32, [_vp, _vp, C.POINTER(_i64)]),
    "pfdtd_server_wait": (_i32, [_vp, _i64, C.c_double, C.POINTER(_i32)]),
    "pfdtd_server_result": (_i32, [_vp, _i64, _vp, C.POINTER(C.c_double)]),
    "pfdtd_server_request_error": (C.c_char_p, [_vp, _i64]),
    "pfdtd_server_release": (_i32, [_vp, _i64]),
    "pfdtd_server_stats_get": (_i32, [_vp, _vp]),
    "pfdtd_server_drain": (_i32, [_vp, C.c_double]),
    "pfdtd_server_destroy": (_i32, [_vp]),
    "pfdtd_set_tb_shape": (_i32, [_vp, _i32]),
    "pfdtd_autotune": (_i32, [_vp, _i32, _i32, C.POINTER(_i32), C.POINTER(_i32),
                              C.POINTER(C.c_double)]),
    "pfdtd_get_temporal_block": (_i32, [_vp, C.POINTER(_i32), C.POINTER(_i32), C.c_char_p,
                                        C.c_size_t]),
    "pfdtd_synchronize": (_i32, [_vp]),
    "pfdtd_kernel_launches": (_i64, []),
    "pfdtd_encode_nodes": (_i32, [_i32, _vp, _vp, _i64, _i32]),
    "pfdtd_count_boundaries": (_i32, [_vp, _i64, C.c_uint8, C.c_uint8, _i32,
                                      C.POINTER(_u32), C.POINTER(_u32)]),
    "pfdtd_pad_mesh": (_i32, [_vp, _i64, C.POINTER(_u32), _u32, _u32, _u32, _vp,
                              C.POINTER(_u32), _i32]),
    # App C ABI (pfdtd_app.h)
    "pfdtd_app_create": (_i32, [C.POINTER(_vp)]),
    "pfdtd_app_destroy": (_i32, [_vp]),
    "pfdtd_app_initialize_devices": (_i32, [_vp]),
    "pfdtd_app_initialize_geometry": (_i32, [_vp, C.POINTER(_u32), _i64, C.POINTER(C.c_float), _i64]),
    "pfdtd_app_initialize_voxels": (_i32, [_vp, _vp, _vp, C.POINTER(_u32)]),
    "pfdtd_app_add_source": (_i32, [_vp, C.c_float, C.c_float, C.c_float, _i32, _i32, _i32]),
    "pfdtd_app_add_source_data_float": (_i32, [_vp, C.POINTER(C.c_float), _i32, _i32]),
    "pfdtd_app_add_source_data_double": (_i32, [_vp, C.POINTER(C.c_double), _i32, _i32]),
    "pfdtd_app_add_receiver": (_i32, [_vp, C.c_float, C.c_float, C.c_float]),
    "pfdtd_app_add_surface_materials": (_i32, [_vp, C.POINTER(C.c_float), C.c_uint, C.c_uint]),
    "pfdtd_app_set_spatial_fs": (_i32, [_vp, C.c_uint]),
    "pfdtd_app_set_num_steps": (_i32, [_vp, C.c_uint]),
    "pfdtd_app_set_update_type": (_i32, [_vp, _i32]),
    "pfdtd_app_set_uniform_material": (_i32, [_vp, C.c_float]),
    "pfdtd_app_run_simulation": (_i32, [_vp]),
    "pfdtd_app_run_capture": (_i32, [_vp]),
    "pfdtd_app_run_visualization": (_i32, [_vp]),
    "pfdtd_app_get_response": (_i32, [_vp, C.c_uint, C.POINTER(C.c_float), _i64]),
    "pfdtd_app_get_response_double": (_i32, [_vp, C.c_uint, C.POINTER(C.c_double), _i64]),
    "pfdtd_app_force_partition_to": (_i32, [_vp, _i32]),
    "pfdtd_app_add_slice_to_capture": (_i32, [_vp, C.c_uint, C.c_uint, C.c_uint]),
    "pfdtd_app_add_mesh_to_capture": (_i32, [_vp, C.c_uint]),
    "pfdtd_app_set_double": (_i32, [_vp, _i32]),
    "pfdtd_app_set_captured_b": (_i32, [_vp, C.c_float]),
    "pfdtd_app_close": (_i32, [_vp]),
    "pfdtd_app_get_mvox": (_i32, [_vp, C.POINTER(C.c_float)]),
    "pfdtd_app_get_num_elems": (_i32, [_vp, C.POINTER(C.c_uint)]),
    "pfdtd_app_get_num_steps": (_i32, [_vp, C.POINTER(C.c_uint)]),
    "pfdtd_app_get_time_per_step": (_i32, [_vp, C.POINTER(C.c_float)]),
    "pfdtd_app_set_octave": (_i32, [_vp, C.c_uint]),
    "pfdtd_app_set_reference_quirks": (_i32, [_vp, _i32]),
    "pfdtd_app_get_mesh_dims": (_i32, [_vp, C.POINTER(_u32)]),
    "pfdtd_app_get_dx": (_i32, [_vp, C.POINTER(C.c_float)]),
}


class PfdtdError(RuntimeError):
    """A C ABI call returned a negative status."""

    def __init__(self, status: int, func: str, message: str):
        super().__init__(f"{func} -> {status}: {message}")
        self.status = status


_lib: Optional[C.CDLL] = None


def load(path: str = LIB_PATH) -> C.CDLL:
    """Load libpfdtd.so and declare every exported signature."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(
            f"{path} is missing: build it with `python -m parallelfdtd_gb300.build` "
            "(or __graft_entry__.build()); there is no CPU fallback")
    lib = C.CDLL(path)
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_names():
    return list(_SIGNATURES.keys())


def check(status: int, func: str) -> int:
    if status < 0:
        msg = load().pfdtd_last_error()
        raise PfdtdError(status, func, msg.decode() if msg else "")
    return status


def call(name: str, *args) -> int:
    lib = load()
    return check(getattr(lib, name)(*args), name)
