"""GPU parity: the drop-in CUDA library against the reference's outputs and the oracle.

* double precision: the GPU library must reproduce the reference CPU library's grids,
  normalisation and images to 1e-12 relative (max |difference| / max |reference|);
* single precision: the GPU library (FP32 data and accumulation, FP64 phase/uvw, compensated
  grid flushes) must be within 1e-5 relative of the FP64 oracle run on the same float inputs.

All calls go through the C-ABI with the pipeliner's sequence (bullseye_gb300.imaging.run_imaging),
including repack_input_data and chunked gridding.
"""
import numpy as np
import pytest

from bullseye_gb300 import synth
from bullseye_gb300.imaging import run_imaging
from tests.golden.cases import CASES, PRECISIONS, cpu_conv, load_case

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32_TOL = 1e-5


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    s = np.max(np.abs(b))
    d = np.max(np.abs(a - b))
    return float(d / s) if s else float(d)


@pytest.fixture(scope="module")
def gpu_libs(gpu_required, built_libraries):
    from bullseye_gb300.library import load_library
    return {p: load_library("GPU", p) for p in PRECISIONS}


@pytest.fixture(scope="module")
def oracle_libs(oracle_built):
    from oracle.harness import load_oracle
    return {p: load_oracle(p) for p in PRECISIONS}


@pytest.fixture(params=["batched", "plain"])
def form(request, gpu_libs):
    """The 4-correlation and sampling-function exports through the batched, support-aware gridder
    (the default) or the plain per-track kernels."""
    for lib in gpu_libs.values():
        lib.bullseye_set_batched_calls(1 if request.param == "batched" else 0)
    yield request.param
    for lib in gpu_libs.values():
        lib.bullseye_set_batched_calls(1)


def run_gpu(lib, p, call, **kw):
    from bullseye_gb300.library import check
    res = run_imaging(lib, p, call, repack=True, norm_bins=(2 * p.conv_support + 1) ** 2, **kw)
    check(lib)
    return res


@pytest.mark.parametrize("name", sorted(CASES))
def test_fp64_matches_reference_fixture(name, gpu_libs, form):
    """GPU FP64 vs the reference CPU library's own outputs (golden fixtures)."""
    call, _, rkw = CASES[name]
    p, out = load_case(name, "double")
    res = run_gpu(gpu_libs["double"], p, call, keep_raw=True, **rkw)
    assert rel(res.raw_grid, out["raw_grid"]) <= FP64_TOL
    assert rel(res.normalization, out["normalization"]) <= FP64_TOL
    # uniform weighting divides by 1e-7 + the sampling function, which amplifies rounding in
    # almost-empty cells; the contract is on the dirty image (checked below), the weighted grid
    # itself is held to 1e-10
    assert rel(res.grid, out["grid"]) <= (1e-10 if rkw.get("uniform") else FP64_TOL)
    img_gpu = np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(res.grid, axes=(-2, -1))), axes=(-2, -1))
    img_ref = np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(out["grid"], axes=(-2, -1))), axes=(-2, -1))
    assert rel(img_gpu.real, img_ref.real) <= FP64_TOL
    if "sampling" in out:
        assert rel(res.sampling, out["sampling"]) <= FP64_TOL
    if "image" in out:
        # float32 packing of an FP64 transform: agreement to float32 rounding
        assert rel(res.image, out["image"]) <= 1e-6
    if "psf" in out:
        assert rel(res.psf, out["psf"]) <= 1e-6


@pytest.mark.parametrize("name", sorted(CASES))
def test_fp32_within_1e5_of_fp64(name, gpu_libs, oracle_libs, form):
    """GPU FP32 vs the FP64 oracle run on the same (float) inputs."""
    call, _, rkw = CASES[name]
    p32, _ = load_case(name, "single")
    p64 = p32.astype("double")
    res = run_gpu(gpu_libs["single"], p32, call, keep_raw=True, **rkw)
    ref = run_imaging(oracle_libs["double"], p64.with_conv(cpu_conv(p64)), call, keep_raw=True, **rkw)
    assert rel(res.raw_grid, ref.raw_grid) <= FP32_TOL
    assert rel(res.normalization, ref.normalization) <= 1e-6
    img = np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(res.grid.astype(np.complex128), axes=(-2, -1))), axes=(-2, -1))
    img_ref = np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(ref.grid, axes=(-2, -1))), axes=(-2, -1))
    assert rel(img.real, img_ref.real) <= FP32_TOL
    if not rkw.get("uniform"):
        assert rel(res.grid, ref.grid) <= FP32_TOL
    if ref.image is not None:
        assert rel(res.image, ref.image) <= FP32_TOL


def _cfg1_like(precision, nx=256, n_ant=24, n_times=40, seed=3):
    return synth.config1(precision, n_ant=n_ant, n_times=n_times, nx=nx, cell=8.0, seed=seed)


@pytest.mark.parametrize("call", ["grid_4_cor", "grid_single_pol", "grid_duel_pol"])
def test_cfg1_shape_fp64_and_fp32(call, gpu_libs, oracle_libs):
    """Config-1 kernel shape (W = 7, os = 63, PSWF) at a reduced size, both precisions."""
    p64 = _cfg1_like("double")
    r_gpu = run_gpu(gpu_libs["double"], p64, call, keep_raw=True, uniform=False, psf=True, do_finalize=True)
    r_orc = run_imaging(oracle_libs["double"], p64, call, keep_raw=True, psf=True, do_finalize=True)
    assert rel(r_gpu.raw_grid, r_orc.raw_grid) <= FP64_TOL
    assert rel(r_gpu.normalization, r_orc.normalization) <= FP64_TOL
    assert rel(r_gpu.image, r_orc.image) <= 1e-6
    p32 = _cfg1_like("single")
    r32 = run_gpu(gpu_libs["single"], p32, call, keep_raw=True)
    r64 = run_imaging(oracle_libs["double"], p32.astype("double"), call, keep_raw=True)
    assert rel(r32.raw_grid, r64.raw_grid) <= FP32_TOL
    assert rel(r32.grid, r64.grid) <= FP32_TOL


def test_chunked_equals_single_chunk(gpu_libs):
    p = synth.small_problem("double", nx=64, n_ant=7, n_times=10, n_chan=3, n_facets=2, jones=True)
    one = run_gpu(gpu_libs["double"], p, "facet_4_cor_corrections", keep_raw=True)
    three = run_gpu(gpu_libs["double"], p, "facet_4_cor_corrections", chunks=3, keep_raw=True)
    assert rel(three.raw_grid, one.raw_grid) <= FP64_TOL
    assert rel(three.normalization, one.normalization) <= FP64_TOL


def test_no_repack_fixed_segments(gpu_libs, oracle_libs):
    """Without repack_input_data the library grids fixed row segments; results are unchanged."""
    from bullseye_gb300.library import check
    p = synth.small_problem("double", nx=64, n_ant=6, n_times=9, n_chan=2, n_facets=2)
    res = run_imaging(gpu_libs["double"], p, "facet_4_cor", keep_raw=True, norm_bins=(2 * p.conv_support + 1) ** 2)
    check(gpu_libs["double"])
    ref = run_imaging(oracle_libs["double"], p, "facet_4_cor", keep_raw=True)
    assert rel(res.raw_grid, ref.raw_grid) <= FP64_TOL


def test_wproj_large_support_fp64(gpu_libs, oracle_libs):
    """w-projection with W = 31 (the J = 2 ownership layout) against the oracle."""
    p = synth.small_problem("double", nx=128, n_ant=6, n_times=8, n_chan=2, s=15, os=5, wplanes=5,
                            min_support=9, n_facets=2, jones=True)
    res = run_gpu(gpu_libs["double"], p, "facet_4_cor_corrections", keep_raw=True)
    ref = run_imaging(oracle_libs["double"], p.with_conv(cpu_conv(p)), "facet_4_cor_corrections", keep_raw=True)
    assert rel(res.raw_grid, ref.raw_grid) <= FP64_TOL
    assert rel(res.normalization, ref.normalization) <= FP64_TOL


@pytest.mark.parametrize("s", [11, 31])
def test_wproj_large_support_fp32(s, gpu_libs, oracle_libs):
    """W = 23 and W = 63 (J = 1 / J = 8 layouts) in single precision against the FP64 oracle."""
    p32 = synth.small_problem("single", nx=192, n_ant=5, n_times=6, n_chan=2, s=s, os=3, wplanes=4,
                              min_support=7, n_facets=1, jones=True)
    res = run_gpu(gpu_libs["single"], p32, "facet_4_cor_corrections", keep_raw=True)
    p64 = p32.astype("double")
    ref = run_imaging(oracle_libs["double"], p64.with_conv(cpu_conv(p64)), "facet_4_cor_corrections", keep_raw=True)
    assert rel(res.raw_grid, ref.raw_grid) <= FP32_TOL


def test_gridding_correction_divides_image(gpu_libs):
    """finalize with a registered detaper equals the plain image divided by c(l) c(m)."""
    import ctypes
    from bullseye_gb300.filters import gridding_correction
    from bullseye_gb300.library import check
    p = synth.small_problem("double", nx=64, ny=48, n_ant=6, n_times=8, n_chan=1)
    plain = run_gpu(gpu_libs["double"], p, "grid_4_cor", do_finalize=True)
    lib = gpu_libs["double"]
    cx = gridding_correction(p.conv, p.conv_support, p.conv_oversample, p.nx)
    cy = gridding_correction(p.conv, p.conv_support, p.conv_oversample, p.ny)
    orig_init = lib.initLibrary

    class Hooked:
        def __getattr__(self, k):
            return getattr(lib, k)

        def initLibrary(self, st):
            orig_init(st)
            lib.bullseye_set_gridding_correction(cx.ctypes.data_as(ctypes.c_void_p), p.nx,
                                                 cy.ctypes.data_as(ctypes.c_void_p), p.ny)

    corr = run_imaging(Hooked(), p, "grid_4_cor", repack=True, do_finalize=True,
                       norm_bins=(2 * p.conv_support + 1) ** 2)
    check(lib)
    expect = plain.image / (cy[None, None, :, None] * cx[None, None, None, :])
    assert rel(corr.image, expect) <= 1e-6


def test_singular_jones_reports_error(gpu_libs):
    from bullseye_gb300.library import ImagingError, check
    p = synth.small_problem("double", nx=48, n_ant=5, n_times=4, n_chan=1, n_facets=1, jones=True)
    p.jones[0, 0, 0, 0, 0, :] = 0
    lib = gpu_libs["double"]
    run_imaging(lib, p, "facet_4_cor_corrections", repack=True, norm_bins=49)
    with pytest.raises(ImagingError, match="singular"):
        check(lib)
    # the library stays usable after the error
    q = synth.small_problem("double", nx=48, n_ant=5, n_times=4, n_chan=1)
    run_gpu(lib, q, "grid_4_cor")


def test_calls_before_init_report_error(gpu_libs):
    import ctypes
    from bullseye_gb300.abi import gridding_parameters_type
    from bullseye_gb300.library import ImagingError, check
    lib = gpu_libs["single"]
    st = gridding_parameters_type("single")()
    lib.grid_4_cor(ctypes.byref(st))
    with pytest.raises(ImagingError, match="before initLibrary"):
        check(lib)
