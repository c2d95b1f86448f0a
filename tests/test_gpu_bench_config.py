"""GPU parity at the benchmarked shapes, against the oracle.

* The plain single-facet workload at full size: 64 antennas on a 2 km disc, 120 timesteps, 1
  channel at 1.4 GHz, a 1024^2 grid of 2 arcsec cells, the PSWF kernel with W = 7 and os = 63, no
  w-projection, natural weighting; grid_4_cor and grid_single_pol.  The 64-bit library must match
  the FP64 oracle to 1e-12 (grids, normalisation) and the 32-bit library must be within 1e-5 of it.
* The multi-facet workload's kernel and facet shape with fewer rows: the reference benchmark's
  EVLA-27 layout, 16 facets of 1024^2 (5 arcsec cells) within 3 deg, Jones terms, w-projection with
  64 planes of supports 15..63 (padded to 63) at os = 15, uniform weighting; the reference exports
  (facet_4_cor_corrections + facet_sampling_function) run the batched, support-aware gridder with
  its class windows, tuned layouts and compensated FP32 (bullseye_grid_batched).  The oracle grids
  the same inputs over the full 63 x 63 support of the 2-D kernel stack.

The reference semantics are those of bullseye/mo/cpu_algorithm/templated_gridder.h:17-103 and
convolution_policies.h:231-289, which the oracle restates.
"""
import numpy as np
import pytest

from bullseye_gb300 import synth
from bullseye_gb300.imaging import run_imaging
from tests.golden.cases import cpu_conv
from tests.test_gpu_parity import FP32_TOL, FP64_TOL, gpu_libs, oracle_libs, rel, run_gpu  # noqa: F401

pytestmark = pytest.mark.gpu


def dirty(grid):
    g = np.asarray(grid, np.complex128)
    return np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(g, axes=(-2, -1))), axes=(-2, -1)).real


@pytest.fixture(scope="module")
def config1_full():
    return synth.config1("double")  # 64 antennas, 120 timesteps, 1024^2, W = 7, os = 63


def exact_aa_normalisation(p):
    """The normalisation sum of a single-channel, unfaceted AA problem with unit weights, summed
    exactly (math.fsum) from per-visibility terms sum_j k[fu + j os] x sum_k k[fv + k os] at the
    gridder's own FP64 cell and tap choice (floor; corner >= 0 and corner + W + 2 < n)."""
    import math
    arcsec = float(np.float32(np.pi / (180.0 * 3600.0)))
    W, os_, K, s = 2 * p.conv_support + 1, p.conv_oversample, p.conv.shape[-1], p.conv_support
    inv = 1.0 / float(p.wavelengths[0, 0])
    u = (p.uvw[:, 0].astype(np.float64) * inv) * (p.nx * float(p.cell_x) * arcsec)
    v = (p.uvw[:, 1].astype(np.float64) * inv) * -(p.ny * float(p.cell_y) * arcsec)
    fu_r, fv_r = np.floor(u), np.floor(v)
    du, dv = fu_r + (p.nx // 2 - s), fv_r + (p.ny // 2 - s)
    keep = (du >= 0) & (dv >= 0) & (du + W + 2 < p.nx) & (dv + W + 2 < p.ny)
    fu = ((1.0 - u + fu_r) * os_).astype(np.int64)[keep]
    fv = ((1.0 - v + fv_r) * os_).astype(np.int64)[keep]
    conv = p.conv.astype(np.float64)
    rows = np.zeros(2 * os_ + 1)
    for f in range(2 * os_ + 1):
        idx = f + np.arange(W) * os_
        rows[f] = conv[idx[idx < K]].sum()
    return math.fsum((rows[fu] * rows[fv]).tolist())


@pytest.mark.parametrize("call", ["grid_4_cor", "grid_single_pol"])
def test_plain_workload_full_size(call, config1_full, gpu_libs, oracle_libs):
    """Grids to 1e-12 of the reference.  The normalisation sum (241,920 terms) is held to 1e-12 of
    its exactly rounded value: the reference accumulates it sequentially with every FP64 operation
    rounded down (its AA path sets FE_DOWNWARD, convolution_policies.h:73-75), which leaves its own
    sum low by up to N ulp / 2, about 1e-11 here, so against the reference it is held to N x eps."""
    p64 = config1_full
    assert (p64.nx, p64.rows, 2 * p64.conv_support + 1, p64.conv_oversample) == (1024, 2016 * 120, 7, 63)
    ref = run_imaging(oracle_libs["double"], p64, call, keep_raw=True)
    assert np.max(np.abs(ref.raw_grid)) > 0
    r64 = run_gpu(gpu_libs["double"], p64, call, keep_raw=True)
    assert rel(r64.raw_grid, ref.raw_grid) <= FP64_TOL
    exact = exact_aa_normalisation(p64)
    n_eps = p64.rows * np.finfo(np.float64).eps
    assert rel(r64.normalization, np.full_like(r64.normalization, exact)) <= FP64_TOL
    assert rel(ref.normalization, np.full_like(ref.normalization, exact)) <= n_eps
    assert rel(r64.normalization, ref.normalization) <= n_eps
    # dirty images: equal to 1e-12 once both are normalised by the same sum
    scale = (ref.normalization / r64.normalization).reshape(1, 1, -1, 1, 1)
    assert rel(dirty(r64.grid), dirty(ref.grid * scale)) <= FP64_TOL
    assert rel(dirty(r64.grid), dirty(ref.grid)) <= n_eps
    p32 = p64.astype("single")
    ref32in = run_imaging(oracle_libs["double"], p32.astype("double"), call, keep_raw=True)
    r32 = run_gpu(gpu_libs["single"], p32, call, keep_raw=True)
    assert rel(r32.raw_grid, ref32in.raw_grid) <= FP32_TOL
    assert rel(dirty(r32.grid), dirty(ref32in.grid)) <= FP32_TOL


@pytest.fixture(scope="module")
def multifacet_shape():
    # the benchmark's kernel stack and facets; 16 timesteps x 8 channels of the 2000 x 64
    return synth.config2("single", n_times=16, n_chan=8, n_facets=16, nx=1024, cell=5.0, wplanes=64, s=31,
                         min_support=15, os=15, n_src=50)


def test_multifacet_shape_batched_fp32(multifacet_shape, gpu_libs, oracle_libs):
    p32 = multifacet_shape
    assert (p32.n_facets, p32.nx, p32.wplanes, p32.conv_oversample, p32.n_antennas) == (16, 1024, 64, 15, 27)
    lib = gpu_libs["single"]
    lib.bullseye_set_batched_calls(1)
    r32 = run_gpu(lib, p32, "facet_4_cor_corrections", keep_raw=True, uniform=True)
    p64 = p32.astype("double")
    ref = run_imaging(oracle_libs["double"], p64.with_conv(cpu_conv(p64)), "facet_4_cor_corrections", keep_raw=True,
                      uniform=True)
    assert rel(r32.normalization, ref.normalization) <= 1e-6
    for f in range(16):
        assert rel(r32.raw_grid[f], ref.raw_grid[f]) <= FP32_TOL, f"facet {f} raw grid"
        assert rel(dirty(r32.grid[f]), dirty(ref.grid[f])) <= FP32_TOL, f"facet {f} dirty image"


def test_multifacet_shape_batched_fp64(multifacet_shape, gpu_libs, oracle_libs):
    p64 = multifacet_shape.astype("double")
    lib = gpu_libs["double"]
    lib.bullseye_set_batched_calls(1)
    r64 = run_gpu(lib, p64, "facet_4_cor_corrections", keep_raw=True, uniform=True)
    ref = run_imaging(oracle_libs["double"], p64.with_conv(cpu_conv(p64)), "facet_4_cor_corrections", keep_raw=True,
                      uniform=True)
    assert rel(r64.raw_grid, ref.raw_grid) <= FP64_TOL
    assert rel(r64.normalization, ref.normalization) <= FP64_TOL
    assert rel(dirty(r64.grid), dirty(ref.grid)) <= FP64_TOL
