"""Precision of a tensor-core form of the footprint update, emulated on the CPU (numpy).

Within a run of visibilities that share a footprint corner, gridding one support class is a complex
GEMM over the run: G[y][x] += sum_v A[y][v] B[v][x], with A[y][v] = vis_v k_v(y) (the visibility
premultiplied by its row taps) and B[v][x] = k_v(x) (its column taps).  tcgen05's FP32-class
operand type is TF32 (10 explicit mantissa bits), accumulated in FP32.  The library's bar is 1e-5
relative to the FP64 oracle, so the design question is which operand split holds it:

* one TF32 pass: A and B rounded to TF32;
* three TF32 passes: x = big + small with big = tf32(x), small = tf32(x - big), and
  A B ~ big_A big_B + big_A small_B + small_A big_B (the small x small term dropped);
* the CUDA-core form the library uses: FP32 operands, one FMA per product.

Over 1,024 products a plain FP32 accumulator already drifts to about 1e-6 of the tile's largest
value (3e-6 for the three-pass split), so a tile form would still flush its FP32 (TMEM)
accumulators into compensated grid words at intervals, as the CUDA-core form flushes its registers.

Taps are the benchmark's w-projection stack (half support 31, oversampling 15, 64 planes), at
random sub-pixel offsets, for one plane of each of three supports; visibilities are complex
Gaussian.  Errors are the tile's largest deviation from the FP64 product over the tile's largest
value, as the library's parity tests measure grids.
"""
import numpy as np
import pytest

from bullseye_gb300.filters import wproj_kernels

HALF, OS, PLANES = 31, 15, 64


def tf32(x: np.ndarray) -> np.ndarray:
    """Round float32 values to TF32 (10 explicit mantissa bits), to nearest with ties away from
    zero, as the float-to-TF32 conversion does."""
    b = np.asarray(x, np.float32).view(np.uint32)
    return ((b + np.uint32(0x1000)) & np.uint32(0xFFFFE000)).view(np.float32)


def fma32(a, b, c):
    """float32 fused multiply-add: the product is exact in float64, one rounding to float32."""
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(np.float32)


def real_gemm(a, b, form):
    """a [M][K] @ b [K][N] in float32 arithmetic, accumulated over K in order, in one of the forms."""
    acc = np.zeros((a.shape[0], b.shape[1]), np.float32)
    if form == "tf32x1":
        a1, b1 = tf32(a), tf32(b)
        for k in range(a.shape[1]):
            acc = fma32(a1[:, k:k + 1], b1[k:k + 1, :], acc)
    elif form == "tf32x3":
        ab, bb = tf32(a), tf32(b)
        asml, bsml = tf32(a - ab), tf32(b - bb)
        for k in range(a.shape[1]):
            # the small products first, then the large one, each accumulated in float32
            acc = fma32(asml[:, k:k + 1], bb[k:k + 1, :], acc)
            acc = fma32(ab[:, k:k + 1], bsml[k:k + 1, :], acc)
            acc = fma32(ab[:, k:k + 1], bb[k:k + 1, :], acc)
    else:  # fp32: CUDA-core FMAs
        a32, b32 = a.astype(np.float32), b.astype(np.float32)
        for k in range(a.shape[1]):
            acc = fma32(a32[:, k:k + 1], b32[k:k + 1, :], acc)
    return acc


def complex_gemm(A, B, form):
    """Four real GEMMs, as a tensor-core complex product would run."""
    re = real_gemm(A.real, B.real, form) - real_gemm(A.imag, B.imag, form)
    im = real_gemm(A.real, B.imag, form) + real_gemm(A.imag, B.real, form)
    return re.astype(np.float64) + 1j * im.astype(np.float64)


@pytest.fixture(scope="module")
def taps():
    fov = 1024 * 5.0 * np.pi / (180 * 3600)
    stack, supports = wproj_kernels(HALF, OS, PLANES, 8000.0, fov, min_support=15)
    return stack.astype(np.complex64), supports


def run_operands(stack, supports, plane, nvis, seed):
    """A [W][V] and B [V][W] of one run: nvis visibilities at random sub-pixel offsets on `plane`."""
    rng = np.random.default_rng(seed)
    W = int(supports[plane])
    lo = (2 * HALF + 1 - W) // 2  # the plane's nonzero window among the full support's cells
    fu = rng.integers(OS // 2, 3 * OS // 2 + 1, nvis)
    fv = rng.integers(OS // 2, 3 * OS // 2 + 1, nvis)
    cells = lo + np.arange(W)
    ku = stack[plane][fu[:, None] + cells[None, :] * OS]  # [V][W]
    kv = stack[plane][fv[:, None] + cells[None, :] * OS]  # [V][W]
    vis = (rng.standard_normal(nvis) + 1j * rng.standard_normal(nvis)).astype(np.complex64)
    A = (vis[:, None] * kv).T.astype(np.complex64)  # premultiplied in float32, as on the device
    return A, ku.astype(np.complex64)


def rel_err(G, ref):
    return float(np.max(np.abs(G - ref)) / np.max(np.abs(ref)))


@pytest.mark.parametrize("plane", [0, 32, 63])
@pytest.mark.parametrize("nvis", [64, 1024])
def test_three_pass_tf32_holds_the_bar_and_one_pass_does_not(plane, nvis, taps):
    stack, supports = taps
    A, B = run_operands(stack, supports, plane, nvis, seed=plane * 7919 + nvis)
    ref = A.astype(np.complex128) @ B.astype(np.complex128)
    errs = {form: rel_err(complex_gemm(A, B, form), ref) for form in ("tf32x1", "tf32x3", "fp32")}
    assert errs["tf32x1"] > 1e-5, errs      # one TF32 pass misses the library's bar (2.7e-4 .. 9e-4)
    assert errs["tf32x3"] <= 1e-5, errs     # three passes hold it (3e-7 .. 3e-6)
    assert errs["fp32"] <= 1e-5, errs       # as the CUDA-core form does (1.5e-7 .. 1.1e-6)
    assert errs["tf32x3"] <= 5 * errs["fp32"] + 1e-7, errs  # within a few FP32 roundings of it
