"""GB300-native implementation of ParallelFDTD's time-stepping hot path.

libpfdtd.so (built by parallelfdtd_gb300.build) holds the sm_103a CUDA
kernels, the C ABI (include/pfdtd.h, include/pfdtd_app.h) and the C++ host
API with the reference's class names (include/pfdtd/).  This package is the
Python side: Domain (one grid on one GPU), App / libPyFDTD (the reference's
Python class) and procedural rooms.
"""

__all__ = ["Domain", "App", "rooms"]


def __getattr__(name):
    if name == "Domain":
        from .domain import Domain
        return Domain
    if name == "App":
        from .app import App
        return App
    raise AttributeError(name)
