"""CPU: the host-side filter designs of the receiver post-processing
(python/FDTDfilter.py:13-19, matlab/functions/FDTDpostFilter.m,
matlab/testBench.m:204).  The device filtering is checked in the GPU
parity tests."""
import numpy as np
import pytest

from parallelfdtd_gb300 import postfilter as pf


@pytest.mark.parametrize("fs", [7350.0, 8000.0, 44100.0, 96000.0])
def test_dcblock_half_gain_at_cut_on(fs):
    a = pf.dcblock(5.0, fs)
    assert 0.9 < a < 1.0
    z = np.exp(1j * 2 * np.pi * 5.0 / fs)
    h = abs((1 - 1 / z) / (1 - a / z))
    assert abs(h / (2 / (1 + a)) - 0.5) < 1e-12  # relative to the gain at Nyquist


def test_fir1_design():
    h = pf.fir1_taps(200, 0.2)
    assert h.size == 201 and abs(h.sum() - 1.0) < 1e-12 and np.allclose(h, h[::-1])


@pytest.mark.parametrize("p,q", [(6, 1), (48000, 7350), (3, 4), (1, 5)])
def test_resample_design(p, q):
    import math
    g = math.gcd(p, q)
    pq = max(p // g, q // g)
    h = pf.resample_taps(p, q)
    assert h.size == 2 * 10 * pq + 1 and abs(h.sum() - 1.0) < 1e-12
    assert np.allclose(h, h[::-1], atol=1e-15)
    # pass band flat, stop band attenuated above the new Nyquist
    w = np.linspace(0, np.pi, 4097)
    resp = np.abs(np.exp(-1j * np.outer(w, np.arange(h.size))) @ h)
    assert np.all(np.abs(resp[w < 0.5 * np.pi / pq] - 1) < 0.02)
    assert np.all(resp[w > 1.5 * np.pi / pq] < 0.01)
