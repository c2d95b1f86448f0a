"""Convolution kernels: the PSWF, the windowed sincs, the w-projection stack and the detaper.

The reference offers no PSWF (bullseye/mo/convolution_filter.py:93 lists sinc, kb and hamming).
Its filter-design study (writing_and_wiki/notebooks/Filter design.ipynb) scores filters by the
share of their image-plane response outside the imaged field; tests/golden/filter_design.npz holds
that study's own filters and figures (made by running its cells, tests/golden/make_filter_design.py).
The restatement in oracle/filter_design.py is pinned to them, and the PSWF is then scored the same
way: it must beat every filter of the study.
"""
import os

import numpy as np
import pytest

from bullseye_gb300 import filters
from oracle import filter_design as fd

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def study():
    return np.load(os.path.join(HERE, "golden", "filter_design.npz"))


def test_restatement_matches_study(study):
    full, x = fd.grid()
    assert full == int(study["full_support"])
    assert np.array_equal(x, study["x"])
    got = fd.notebook_filters()
    # cell 12 rebinds `sinc` to the raw np.sinc(x); cell 8's unit-sum box survives in fft_sinc
    assert np.allclose(study["sinc"], np.sinc(x), rtol=1e-15, atol=0)
    for name in ("sinc_hamming", "kb"):
        assert np.allclose(got[name], study[name], rtol=1e-13, atol=0), name
    for name in ("sinc", "sinc_hamming", "kb"):
        assert np.allclose(fd.response(got[name]), study["fft_" + name], rtol=0, atol=1e-15), name
    figs = [fd.aliasing_percent(fd.response(got[n]), full, fd.OVERSAMPLE) for n in ("sinc", "sinc_hamming", "kb")]
    assert np.allclose(figs, study["aliasing"], rtol=1e-9)


def test_pswf_beats_every_study_filter(study):
    full, x = fd.grid()
    k = filters.pswf(np.pi * full / 2.0, 2.0 * x / full)
    k /= np.sum(k)
    fig = fd.aliasing_percent(fd.response(k), full, fd.OVERSAMPLE)
    assert fig < float(np.min(study["aliasing"])) * 1e-3, (fig, study["aliasing"])


def test_pswf_is_the_prolate_eigenfunction():
    """psi_0(c, .) solves  int_{-1}^{1} e^{i c x t} psi(t) dt = lambda psi(x)  (Slepian & Pollak 1961)."""
    c = 9.0
    t, w = np.polynomial.legendre.leggauss(200)
    psi = filters.pswf(c, t)
    xs = np.linspace(-1, 1, 41)
    lhs = np.array([np.sum(w * np.cos(c * xv * t) * psi) for xv in xs])
    lam = lhs[20] / 1.0  # psi(0) = 1
    rhs = lam * filters.pswf(c, xs)
    assert abs(filters.pswf(c, np.array([0.0]))[0] - 1.0) < 1e-14
    assert np.max(np.abs(lhs - rhs)) <= 1e-10 * abs(lam)
    assert np.allclose(psi, psi[::-1], atol=1e-13)  # even


@pytest.mark.parametrize("s,os_", [(3, 63), (7, 15), (31, 15)])
def test_kernel_layouts(s, os_):
    K = filters.kernel_length(s, os_)
    assert K == (2 * s + 3) + (2 * s + 2) * (os_ - 1)
    for k in (filters.pswf_kernel(s, os_), filters.aa_kernel(s, os_, "sinc"), filters.aa_kernel(s, os_, "kb"),
              filters.aa_kernel(s, os_, "hamming")):
        assert k.shape == (K,)
        assert abs(np.sum(k) - 1.0) < 1e-12
        assert np.allclose(k, k[::-1], atol=1e-15)
    # the PSWF is exactly zero beyond W/2 cells, so the padding taps vanish
    k = filters.pswf_kernel(s, os_)
    off = (np.arange(K) - K // 2) / os_
    assert np.all(k[np.abs(off) > (2 * s + 1) / 2.0] == 0)


def test_pswf_aliasing_below_windowed_sincs():
    s, os_ = 3, 63
    a = filters.aliasing_fraction(filters.pswf_kernel(s, os_), s, os_)
    for win in ("sinc", "kb", "hamming"):
        assert a < filters.aliasing_fraction(filters.aa_kernel(s, os_, win), s, os_), win


def test_wproj_stack_supports_and_symmetry():
    s, os_, P = 7, 9, 6
    stack, sup = filters.wproj_kernels(s, os_, P, wmax=2000.0, fov_rad=np.deg2rad(1.0), min_support=5)
    K = filters.kernel_length(s, os_)
    assert stack.shape == (P, K)
    assert sup[0] == 5 and sup[-1] == 2 * s + 1 and np.all(np.diff(sup) >= 0)
    off = (np.arange(K) - K // 2) / os_
    for p in range(P):
        assert np.all(stack[p][np.abs(off) > sup[p] / 2.0] == 0), p
        assert abs(np.sum(stack[p].real) - 1.0) < 1e-12
        assert np.allclose(stack[p], stack[p][::-1], atol=1e-14)  # even in u: l^2 chirp
    # plane 0 (w = 0) is real up to the transform's rounding
    assert np.max(np.abs(stack[0].imag)) < 1e-12


def test_gridding_correction_is_the_kernel_dft():
    s, os_, n = 3, 15, 40
    k = filters.pswf_kernel(s, os_)
    c = filters.gridding_correction(k, s, os_, n)
    x = (np.arange(k.size) - k.size // 2) / os_
    for i in (0, 7, n // 2, n - 1):
        l = (i - n // 2) / n
        direct = np.sum(k * np.exp(2j * np.pi * x * l)).real / np.sum(k)
        assert abs(c[i] - direct) < 1e-13
    assert c[n // 2] == pytest.approx(1.0, abs=1e-15)
