"""Restatement of the reference's filter-design study.  TEST INFRASTRUCTURE ONLY.

writing_and_wiki/notebooks/Filter design.ipynb compares anti-aliasing filters by the share of
their image-plane response that falls outside the imaged field.  This module restates its sample
grid (cell 4), its two energy integrals (cells 5 and 6), its three filters (cells 8, 10 and 12)
and the figure of cell 13, so that any tabulated kernel (the PSWF of bullseye_gb300.filters in
particular) can be scored the way the reference scores its own.  Pinned against
tests/golden/filter_design.npz, which running the notebook's cells produced.
"""
from __future__ import annotations

import numpy as np
from scipy import special as sp

HALF_SUPPORT = 20
OVERSAMPLE = 63


def grid(half_support: int = HALF_SUPPORT, oversample: int = OVERSAMPLE):
    """Cell 4: full support and the sample positions x (cells), W * os samples about 0."""
    full = 2 * half_support + 1
    x = (np.arange(0, full * oversample) - (full * oversample) // 2) / float(oversample)
    return full, x


def response(filt: np.ndarray) -> np.ndarray:
    """Cells 8, 10, 12: the real part of the shifted FFT of the (unit-sum) filter."""
    return np.real(np.fft.ifftshift(np.fft.fft(np.fft.fftshift(filt))))


def aliasing_percent(resp: np.ndarray, full: int, oversample: int, step: float = 1e-6) -> float:
    """Cells 5, 6 and 13: 100 x (|response| integrated from index (W//2 + 1) os on) / (all of it)."""
    lb = (full // 2 + 1) * oversample
    outside = np.trapezoid(np.abs(resp[lb:]), dx=step) * 2
    total = np.trapezoid(np.abs(resp), dx=step) * 2
    return float(outside / total * 100.0)


def notebook_filters(half_support: int = HALF_SUPPORT, oversample: int = OVERSAMPLE) -> dict:
    """Cells 8, 10 and 12: sinc, sinc x Hamming and sinc x Kaiser-Bessel, each of unit sum."""
    full, x = grid(half_support, oversample)
    sinc = np.sinc(x)
    box = sinc / np.sum(sinc)
    ham = np.sinc(x) * np.hamming(full * oversample)
    ham /= np.sum(ham)
    beta = (7.43 - 2.39) / (5.0 - 2.0) * full - 0.366833
    inner = 1 - (2 * x / float(full)) ** 2
    kb = 1.0 / full * sp.i0(beta * np.sqrt(inner)) * np.sinc(x)
    kb /= np.sum(kb)
    return {"sinc": box, "sinc_hamming": ham, "kb": kb}
