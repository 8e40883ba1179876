"""Frequency-dependent boundary admittance filters (digital impedance filters).

The reference has placeholders only ("Digital impedance filters not
implemented", ParallelFDTD src/kernels/cudaMesh.h:88, :122-123).  Here a
material may carry a rational admittance

    Y(z) = (b0 + b1 z^-1 + ... + bN z^-N) / (1 + a1 z^-1 + ... + aN z^-N),  N <= 3,

applied at boundary nodes in place of the frequency-independent value.
Filters built by `positive_real_filters` are passive by construction: a sum
of a constant and first-order sections c (1 + p z^-1) / (1 - p z^-1) with
c > 0 and real |p| < 1, each of which has a positive real part on the unit
circle, so Re Y(e^jw) > 0 at every frequency and every pole lies inside the
unit circle.
"""
from __future__ import annotations

from typing import Tuple

import numpy as np

MAX_ORDER = 3


def _section_sum(c0: float, c: np.ndarray, p: np.ndarray) -> Tuple[np.ndarray, np.ndarray]:
    """Numerator/denominator of c0 + sum_k c_k (1 + p_k z^-1) / (1 - p_k z^-1)."""
    den = np.array([1.0])
    for pk in p:
        den = np.convolve(den, [1.0, -pk])
    num = c0 * den
    for k, (ck, pk) in enumerate(zip(c, p)):
        part = np.array([ck, ck * pk])
        for j, pj in enumerate(p):
            if j != k:
                part = np.convolve(part, [1.0, -pj])
        num = num + np.pad(part, (0, len(den) - len(part)))
    return num, den


def positive_real_filters(n_mat: int, order: int = 3, seed: int = 5, max_pole: float = 0.95,
                          level=(0.01, 0.5)) -> np.ndarray:
    """n_mat seeded passive admittance filters of the given order.

    Returns [n_mat, 2*order + 1]: b0..b_order, a1..a_order.  The admittance
    at DC and at Nyquist lies in `level`-scaled ranges.
    """
    if not 0 <= order <= MAX_ORDER:
        raise ValueError(f"filter order must be 0..{MAX_ORDER}")
    rng = np.random.default_rng(seed)
    out = np.zeros((n_mat, 2 * order + 1))
    for m in range(n_mat):
        p = rng.uniform(-max_pole, max_pole, size=order)
        c0 = rng.uniform(level[0], level[1]) * 0.5
        # keep each section's gain (1+|p|)/(1-|p|) c within the level range
        c = rng.uniform(level[0], level[1], size=order) * (1 - np.abs(p)) / (1 + np.abs(p)) / max(order, 1)
        num, den = _section_sum(c0, c, p)
        out[m, :order + 1] = num
        out[m, order + 1:] = den[1:]
    return out


def frequency_response(coefs: np.ndarray, order: int, n: int = 1024) -> np.ndarray:
    """Y(e^jw) on n frequencies in [0, pi] for one filter row."""
    w = np.linspace(0, np.pi, n)
    zi = np.exp(-1j * w)
    b = coefs[:order + 1]
    a = np.concatenate([[1.0], coefs[order + 1:]])
    num = sum(bk * zi ** k for k, bk in enumerate(b))
    den = sum(ak * zi ** k for k, ak in enumerate(a))
    return num / den


def is_passive(coefs: np.ndarray, order: int) -> bool:
    """Stable denominator and positive real part on the unit circle."""
    a = np.concatenate([[1.0], coefs[order + 1:]])
    if order and np.max(np.abs(np.roots(a))) >= 1.0:
        return False
    return bool(np.min(frequency_response(coefs, order).real) > 0)


def dif_table(coefs: np.ndarray, order: int) -> np.ndarray:
    """[n, 2*order+1] filter rows -> [n, 7] rows b0..b3, a1..a3 (zero padded)."""
    coefs = np.asarray(coefs, dtype=np.float64).reshape(-1, 2 * order + 1)
    out = np.zeros((coefs.shape[0], 7))
    out[:, :order + 1] = coefs[:, :order + 1]
    out[:, 4:4 + order] = coefs[:, order + 1:]
    return out
