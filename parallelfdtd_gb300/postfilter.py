"""Post-processing of receiver traces, the reference's two recipes with the
filtering on the GPU (pfdtd_post_filter):

* ``fdtd_filter(x, sfs, normalized_cutoff)`` — python/FDTDfilter.py:13-19: a
  200-tap FIR low-pass designed with a Chebyshev window (70 dB), applied
  causally;
* ``fdtd_post_filter(ir, fs, frac)`` — matlab/functions/FDTDpostFilter.m:
  an order-200 FIR low-pass (Hamming window, as MATLAB's fir1), then a DC
  blocker with its cut-on at 5 Hz (dcblock.m, J. de Freitas 2007:
  a = (sqrt(3) - 2 sin(pi Fc)) / (sin(pi Fc) + sqrt(3) cos(pi Fc)),
  Fc = 2 fc / fs).

Taps are designed on the host with scipy.signal, as the reference does; the
traces (one per row) are filtered on the device in double arithmetic.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib as L


def apply(x: np.ndarray, taps: np.ndarray, dc_coef: float | None = None, device: int = 0):
    """Filter each row of x with the FIR taps, then the DC blocker if given."""
    a = np.asarray(x)
    dt = np.float64 if a.dtype == np.float64 else np.float32
    xs = np.ascontiguousarray(a, dtype=dt)
    shape = xs.shape
    xs2 = xs.reshape(-1, shape[-1]) if xs.ndim > 1 else xs.reshape(1, -1)
    out = np.empty_like(xs2)
    b = np.ascontiguousarray(taps, dtype=np.float64).reshape(-1)
    L.call("pfdtd_post_filter", xs2.ctypes.data, xs2.shape[0], xs2.shape[1],
           1 if dt == np.float64 else 0, b.ctypes.data_as(C.POINTER(C.c_double)), b.size,
           0 if dc_coef is None else 1, float(dc_coef or 0.0), out.ctypes.data, int(device))
    return out.reshape(shape)


def dc_block_coef(fc: float, fs: float) -> float:
    fn = 2.0 * fc / fs
    return (math.sqrt(3) - 2 * math.sin(math.pi * fn)) / (
        math.sin(math.pi * fn) + math.sqrt(3) * math.cos(math.pi * fn))


def fdtd_filter(x: np.ndarray, sfs: float, normalized_cutoff: float, device: int = 0):
    """FIR low-pass of python/FDTDfilter.py (200 taps, Chebyshev window 70 dB)."""
    from scipy.signal import firwin
    nyq = sfs / 2.0
    taps = firwin(200, sfs * normalized_cutoff / nyq, window=("chebwin", 70.0))
    return apply(x, taps, None, device)


def fdtd_post_filter(ir: np.ndarray, fs: float, frac: float, device: int = 0):
    """FDTDpostFilter.m: fir1(200, frac) low-pass, then the 5 Hz DC blocker."""
    from scipy.signal import firwin
    taps = firwin(201, frac, window="hamming")
    return apply(ir, taps, dc_block_coef(5.0, fs), device)
