"""Drop-in module name of the reference's boost::python extension
(ParallelFDTD src/AppPy.cpp:96): ``from parallelfdtd_gb300 import libPyFDTD as pf``."""
from .app import App  # noqa: F401
