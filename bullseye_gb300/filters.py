"""Convolution-kernel tables in the layouts the imaging ABI expects, and the gridding correction.

Layouts (bullseye/mo/convolution_filter.py:95-149; consumed by
bullseye/mo/cpu_algorithm/convolution_policies.h:70-118 and
bullseye/mo/gpu_algorithm/convolution_policies.h:78-206):

* full support ``W = 2 s + 1`` cells, padded to ``W + 2``;
* ``K = (W + 2) + (W + 1)(os - 1)`` oversampled samples, centre sample ``K // 2``;
* ``1D_AA``: real ``[K]``; separable taps are ``k[fu + j os] * k[fv + i os]``;
* ``1D_WPROJ``: complex ``[P, K]``, one separable kernel per w plane (GPU ABI);
* ``2D_WPROJ``: complex ``[P, K, K]`` (CPU ABI).  :func:`outer_stack` builds it from a
  ``1D_WPROJ`` stack so the CPU oracle and the GPU drop-in grid the same mathematics.

Kernels offered here:

* :func:`aa_kernel` -- windowed sinc exactly as the reference's ``1D_AA`` generator
  (sinc(x/os) x window, normalised to unit sum; convolution_filter.py:104-107);
* :func:`pswf_kernel` -- prolate spheroidal wave function psi_0(c, eta), c = pi W / 2
  (Slepian & Pollak 1961; the spheroidal gridding function of Schwab 1984 with alpha = 0),
  computed from the Legendre-series eigenproblem of Bouwkamp (1947) / Xiao, Rokhlin &
  Yarvin (2001).  The reference offers no PSWF (convolution_filter.py:93);
* :func:`wproj_kernels` -- separable small-angle w-projection stack with a per-plane support;
* :func:`gridding_correction` -- the detaper: the DFT of the tabulated kernel at the image
  pixel positions, normalised at the centre.  Absent in the reference (only a dead index
  variable at bullseye/mo/cpu_gpu_common/fft_and_repacking_routines.cpp:113).
"""
from __future__ import annotations

import numpy as np
from numpy.polynomial import legendre as npleg


def kernel_length(half_support: int, oversample: int) -> int:
    W = 2 * half_support + 1
    return (W + 2) + (W + 1) * (oversample - 1)


def _offsets(half_support: int, oversample: int) -> np.ndarray:
    """Sample offsets from the kernel centre, in oversampled units (integers)."""
    K = kernel_length(half_support, oversample)
    c = K // 2
    return np.arange(-c, c + 1, dtype=np.float64)


def aa_kernel(half_support: int, oversample: int, window: str = "sinc") -> np.ndarray:
    """Windowed-sinc anti-aliasing kernel, ``1D_AA`` layout (float64 [K]).

    ``window`` is one of 'sinc' (no window), 'kb' or 'hamming', following
    bullseye/mo/convolution_filter.py:62-75 and :104-107.
    """
    x = _offsets(half_support, oversample)
    K = x.size
    Wp = 2 * half_support + 3
    aa = np.sinc(x / float(oversample))
    if window == "kb":
        xs = x / float(oversample)
        inner = 1.0 - (xs / float(Wp)) ** 2
        from scipy import special as sp
        aa = aa * sp.i0(Wp * np.sqrt(np.clip(inner, 0.0, None))) * oversample * sp.i0(Wp)
    elif window == "hamming":
        aa = aa * np.hamming(Wp + (Wp - 1) * (oversample - 1))[:K]
    elif window != "sinc":
        raise ValueError(f"unknown window {window!r}")
    return aa / np.sum(aa)


def pswf(c: float, eta: np.ndarray, terms: int | None = None) -> np.ndarray:
    """Zeroth-order prolate spheroidal wave function psi_0(c, eta) on |eta| <= 1 (0 outside).

    Expands psi_0 in normalised even Legendre polynomials; the coefficient vector is the
    eigenvector of the smallest eigenvalue of the symmetric tridiagonal matrix of the
    prolate differential operator  -d/deta (1 - eta^2) d/deta + c^2 eta^2  in that basis.
    Normalised to psi_0(c, 0) = 1.
    """
    eta = np.asarray(eta, dtype=np.float64)
    n = terms or int(2 * c + 40)
    k = 2 * np.arange(n, dtype=np.float64)  # even degrees
    diag = k * (k + 1) + c * c * (2 * k * (k + 1) - 1) / ((2 * k + 3) * (2 * k - 1))
    off = c * c * (k[:-1] + 2) * (k[:-1] + 1) / ((2 * k[:-1] + 3) * np.sqrt((2 * k[:-1] + 1) * (2 * k[:-1] + 5)))
    mat = np.diag(diag) + np.diag(off, 1) + np.diag(off, -1)
    vals, vecs = np.linalg.eigh(mat)
    beta = vecs[:, np.argmin(vals)]
    coef = np.zeros(2 * n)
    coef[0::2] = beta * np.sqrt(k + 0.5)  # normalised -> standard Legendre
    inside = np.abs(eta) <= 1.0
    out = np.zeros_like(eta)
    out[inside] = npleg.legval(eta[inside], coef)
    centre = npleg.legval(0.0, coef)
    return out / centre


def pswf_kernel(half_support: int, oversample: int) -> np.ndarray:
    """PSWF anti-aliasing kernel in ``1D_AA`` layout (float64 [K]), unit sum.

    C(x) = psi_0(c, 2x / W) for |x| <= W/2 cells (W = 2s+1, c = pi W / 2), zero beyond.
    """
    W = 2 * half_support + 1
    x = _offsets(half_support, oversample) / float(oversample)
    k = pswf(np.pi * W / 2.0, 2.0 * x / W)
    return k / np.sum(k)


def aliasing_fraction(kernel: np.ndarray, half_support: int, oversample: int) -> float:
    """Fraction of the kernel's image-plane response lying outside the imaged field.

    Same figure as the reference's filter-design study (writing_and_wiki/notebooks/Filter
    design.ipynb, cells 5-6 and 13): |FFT(kernel)| integrated beyond the image edge over
    |FFT(kernel)| integrated everywhere.  The imaged field spans 1/os of the transform.
    """
    K = kernel.size
    resp = np.abs(np.fft.fftshift(np.fft.fft(np.fft.ifftshift(kernel))))
    c = K // 2
    half_field = K / (2.0 * oversample)
    idx = np.arange(K) - c
    outside = np.abs(idx) > half_field
    return float(resp[outside].sum() / resp.sum())


def plane_supports(wplanes: int, w_min_support: int, w_max_support: int) -> np.ndarray:
    """Odd full supports growing linearly from ``w_min_support`` (plane 0) to ``w_max_support``."""
    if wplanes <= 1:
        return np.array([w_max_support])
    s = np.linspace(w_min_support, w_max_support, wplanes)
    s = 2 * np.floor(s / 2.0).astype(int) + 1
    return np.clip(s, w_min_support | 1, w_max_support | 1)


def wproj_kernels(half_support: int, oversample: int, wplanes: int, wmax: float, fov_rad: float,
                  aa: np.ndarray | None = None, min_support: int | None = None,
                  sign: float = -1.0) -> tuple[np.ndarray, np.ndarray]:
    """Separable small-angle w-projection stack, ``1D_WPROJ`` layout (complex128 [P, K]).

    For plane p (w_p = p * wmax / (P - 1)) the image-plane kernel is the AA taper times the
    small-angle w phase exp(sign * i pi w_p l^2) (l = direction cosine, the field is
    ``fov_rad`` wide); its transform sampled at the oversampled uv offsets is truncated to a
    per-plane full support W_p (odd, from ``min_support`` at w = 0 to 2s+1 at wmax) and
    normalised to unit real sum.  Returns (stack, supports).
    """
    x = _offsets(half_support, oversample)
    K = x.size
    W = 2 * half_support + 1
    if aa is None:
        aa = pswf_kernel(half_support, oversample)
    supports = plane_supports(wplanes, min_support or W, W)
    # image-plane taper of the AA kernel on the oversampled transform grid
    taper = np.fft.fftshift(np.fft.ifft(np.fft.ifftshift(aa))) * K
    phi = x / K * oversample          # fraction of the field, spans +-os/2 fields
    lm = phi * fov_rad
    step = wmax / float(max(1, wplanes - 1))
    stack = np.zeros((wplanes, K), dtype=np.complex128)
    for p in range(wplanes):
        chirp = np.exp(sign * 1j * np.pi * (p * step) * lm ** 2)
        k = np.fft.fftshift(np.fft.fft(np.fft.ifftshift(taper * chirp))) / K
        half = supports[p] / 2.0
        k[np.abs(x / oversample) > half] = 0.0
        k /= np.sum(k.real)
        stack[p] = k
    return stack, supports


def outer_stack(stack_1d: np.ndarray) -> np.ndarray:
    """2-D w-projection stack [P, K, K] with entry [p, v, u] = k[p, u] * k[p, v].

    This is the ``2D_WPROJ`` layout of the CPU library (convolution_policies.h:262-281,
    row index v, column index u); it reproduces the GPU library's separable product
    (gpu_algorithm/convolution_policies.h:200) so both grid the same mathematics.
    """
    s = np.asarray(stack_1d)
    return s[:, None, :] * s[:, :, None]


def gridding_correction(kernel_1d: np.ndarray, half_support: int, oversample: int, n: int) -> np.ndarray:
    """Detaper factor c(l) per image pixel (float64 [n]), normalised to c(centre) = 1.

    c is the DFT of the tabulated 1-D kernel at the pixel positions: for pixel i (after the
    reference's fftshift, pixel n//2 is the field centre), l_i = (i - n//2) / n cycles per
    cell and c(l) = sum_j k_j cos(2 pi x_j l) with x_j the tap offsets in cells.  Complex
    kernels (w-projection plane 0) use their real part.  Dividing the image by
    c(l_x) c(m_y) undoes the kernel's taper.
    """
    x = _offsets(half_support, oversample) / float(oversample)
    k = np.real(np.asarray(kernel_1d, dtype=np.complex128))
    l = (np.arange(n) - n // 2) / float(n)
    c = np.cos(2.0 * np.pi * np.outer(l, x)) @ k
    centre = np.sum(k)
    return c / centre
