"""Post-processing of receiver traces: the reference's recipes, with the
filtering on the GPU (pfdtd_post_filter, pfdtd_resample).

* ``FDTDfilter(x, sfs, fs, normalized_cutoff)`` — python/FDTDfilter.py:13-19:
  a 200-tap FIR low-pass designed with a Chebyshev window (70 dB ripple),
  applied causally along axis 0 (``fs`` is unused, as in the reference);
* ``FDTDpostFilter(ir, fs, frac)`` — matlab/functions/FDTDpostFilter.m: an
  order-200 FIR low-pass (Hamming window and unit DC gain, as MATLAB's
  ``fir1``), then a DC blocker with its cut-on at 5 Hz (``dcblock``); like
  the MATLAB function it takes row or column traces and returns columns
  (``[samples, channels]``);
* ``resample(x, p, q)`` — the rational resampler of matlab/testBench.m:204
  (MATLAB's ``resample``: an anti-aliasing low-pass of length
  2·10·max(p, q) + 1, least-squares ideal low-pass at 1/(2·max(p, q)) times a
  Kaiser window with beta 5, gain p, applied polyphase with the filter delay
  removed; ``ceil(n·p/q)`` output samples), along axis 0.

Filter taps are designed on the host with scipy.signal, as the reference
does; the traces are filtered on the device in double arithmetic.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib as L


def _rows(x):
    """(contiguous float32/float64 2-D array, original dtype kind)."""
    a = np.asarray(x)
    dt = np.float64 if a.dtype == np.float64 else np.float32
    return np.ascontiguousarray(a, dtype=dt), dt


def fir(x: np.ndarray, taps: np.ndarray, dc_coef: float | None = None, device: int = 0):
    """Filter each row of x (the last axis is time) with the causal FIR taps
    (lfilter(taps, 1, x)), then, if dc_coef is given, the DC blocker
    y[n] = x[n] - x[n-1] + dc_coef y[n-1]."""
    xs, dt = _rows(x)
    shape = xs.shape
    xs2 = xs.reshape(-1, shape[-1]) if xs.ndim > 1 else xs.reshape(1, -1)
    out = np.empty_like(xs2)
    b = np.ascontiguousarray(taps, dtype=np.float64).reshape(-1)
    L.call("pfdtd_post_filter", xs2.ctypes.data, xs2.shape[0], xs2.shape[1],
           1 if dt == np.float64 else 0, b.ctypes.data_as(C.POINTER(C.c_double)), b.size,
           0 if dc_coef is None else 1, float(dc_coef or 0.0), out.ctypes.data, int(device))
    return out.reshape(shape)


def polyphase(x: np.ndarray, h: np.ndarray, up: int, down: int, device: int = 0):
    """Resample each row of x by up/down with the linear-phase FIR h (unit DC
    gain before the factor `up` is applied), the filter's delay removed and
    ceil(n·up/down) samples kept (the output alignment of MATLAB's resample
    and scipy's resample_poly)."""
    g = math.gcd(int(up), int(down))
    up, down = int(up) // g, int(down) // g
    xs, dt = _rows(x)
    shape = xs.shape
    xs2 = xs.reshape(-1, shape[-1]) if xs.ndim > 1 else xs.reshape(1, -1)
    n_in = xs2.shape[1]
    if up == down == 1:
        return xs.copy()
    n_out = -(-n_in * up // down)
    h = np.asarray(h, dtype=np.float64).reshape(-1) * up
    half = (h.size - 1) // 2
    pre_pad = down - half % down
    offset = (half + pre_pad) // down
    taps = np.ascontiguousarray(np.concatenate([np.zeros(pre_pad), h]))
    out = np.empty((xs2.shape[0], n_out), dtype=dt)
    L.call("pfdtd_resample", xs2.ctypes.data, xs2.shape[0], n_in, 1 if dt == np.float64 else 0,
           taps.ctypes.data_as(C.POINTER(C.c_double)), taps.size, up, down, offset, n_out,
           out.ctypes.data, int(device))
    return out.reshape(shape[:-1] + (n_out,))


def dcblock(fc: float, fs: float) -> float:
    """Pole of the DC blocker y[n] = x[n] - x[n-1] + a y[n-1] whose gain at
    fc Hz is half its gain at Nyquist (J. de Freitas, "The DC Blocking
    Filter", 2007; matlab/functions/FileExchange/dcblock.m): Fc = 2 fc / fs,
    a = (sqrt(3) - 2 sin(pi Fc)) / (sin(pi Fc) + sqrt(3) cos(pi Fc))."""
    fn = 2.0 * fc / fs
    return (math.sqrt(3) - 2 * math.sin(math.pi * fn)) / (
        math.sin(math.pi * fn) + math.sqrt(3) * math.cos(math.pi * fn))


def fir1_taps(order: int, frac: float) -> np.ndarray:
    """MATLAB fir1(order, frac): Hamming-windowed low-pass, unit DC gain."""
    from scipy.signal import firwin
    return firwin(order + 1, frac, window="hamming")


def FDTDfilter(x: np.ndarray, sfs: float, fs: float, normalized_cutoff: float, device: int = 0):
    """python/FDTDfilter.py:13-19 with the filtering on the device; time
    along axis 0."""
    from scipy.signal import firwin
    nyq_rate = sfs / 2.0
    taps = firwin(200, sfs * normalized_cutoff / nyq_rate, window=("chebwin", 70.0))
    a = np.asarray(x)
    return np.moveaxis(fir(np.moveaxis(a, 0, -1), taps, None, device), -1, 0)


def FDTDpostFilter(ir: np.ndarray, fs: float, frac: float, device: int = 0):
    """matlab/functions/FDTDpostFilter.m with the filtering on the device:
    returns [samples, channels] (a 1-D trace stays 1-D)."""
    a = np.asarray(ir)
    if a.ndim == 1:
        return fir(a, fir1_taps(200, frac), dcblock(5.0, fs), device)
    if a.shape[0] > a.shape[1]:  # column traces
        a = a.T
    return fir(a, fir1_taps(200, frac), dcblock(5.0, fs), device).T


def resample_taps(p: int, q: int, n: int = 10, beta: float = 5.0) -> np.ndarray:
    """Anti-aliasing filter of MATLAB's resample(x, p, q) with unit DC gain:
    the least-squares ideal low-pass at 1/(2·max(p, q)) of length
    2·n·max(p, q) + 1 times a Kaiser window (beta)."""
    from scipy.signal import firls
    from scipy.signal.windows import kaiser
    g = math.gcd(int(p), int(q))
    pq = max(int(p) // g, int(q) // g)
    fc = 1.0 / (2.0 * pq)
    length = 2 * n * pq + 1
    h = firls(length, [0.0, 2 * fc, 2 * fc, 1.0], [1.0, 1.0, 0.0, 0.0]) * kaiser(length, beta)
    return h / h.sum()


def resample(x: np.ndarray, p: int, q: int, n: int = 10, beta: float = 5.0, device: int = 0):
    """MATLAB resample(x, p, q) along axis 0 (a 1-D trace stays 1-D)."""
    a = np.asarray(x)
    if int(p) == int(q):
        return _rows(a)[0].copy()
    h = resample_taps(p, q, n, beta)
    if a.ndim == 1:
        return polyphase(a, h, p, q, device)
    return np.moveaxis(polyphase(np.moveaxis(a, 0, -1), h, p, q, device), -1, 0)


def render(p: np.ndarray, fs: float, frac: float = 0.2, fs_out: int = 48000, device: int = 0):
    """matlab/testBench.m:203-204: resample(FDTDpostFilter(p, fs, frac), fs_out, fs)."""
    return resample(FDTDpostFilter(np.asarray(p, dtype=np.float64), fs, frac, device),
                    int(fs_out), int(round(fs)), device=device)
