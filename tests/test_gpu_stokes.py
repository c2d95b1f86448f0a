"""bullseye_finalize_stokes: the Stokes combination and facet compaction done on the device before
the transform must equal the host combination (the pairs bullseye/data/stokes.py:90-172 forms,
each cube slice's term moved to slice c of its facet block) followed by finalize."""
import ctypes

import numpy as np
import pytest

from bullseye_gb300 import synth
from bullseye_gb300.abi import gridding_parameters_type

pytestmark = pytest.mark.gpu

CUBE = 2


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def _init(lib, precision, keep):
    """A library initialised for 4 correlations, CUBE cube slices and 2 facets (nothing gridded)."""
    p = synth.small_problem(precision, nx=64, n_ant=4, n_times=4, n_chan=4, n_facets=2, s=3, os=15)
    rd = np.float32 if precision == "single" else np.float64
    st = gridding_parameters_type(precision)()
    conv = np.ascontiguousarray(p.conv)
    lam = np.ascontiguousarray(p.wavelengths.reshape(-1), rd)
    enabled = np.ones(p.channels, np.bool_)
    cgi = np.ascontiguousarray(np.arange(p.channels) % CUBE, np.uintp)
    fc = np.ascontiguousarray(p.facet_centres, rd)
    keep += [conv, lam, enabled, cgi, fc]
    st.chunk_max_row_count = 1
    st.nx = st.ny = p.nx
    st.cell_size_x, st.cell_size_y = p.cell_x, p.cell_y
    st.conv = _ptr(conv)
    st.conv_support, st.conv_oversample = p.conv_support, p.conv_oversample
    st.phase_centre_ra, st.phase_centre_dec = p.phase_centre
    st.channel_grid_indicies = _ptr(cgi)
    st.cube_channel_dim_size = CUBE
    st.number_of_polarization_terms = st.number_of_polarization_terms_being_gridded = 4
    st.spw_count, st.channel_count = 1, p.channels
    st.antenna_count = p.n_antennas
    st.enabled_channels = _ptr(enabled)
    st.reference_wavelengths = _ptr(lam)
    st.num_facet_centres = 2
    st.facet_centres = _ptr(fc)
    st.wplanes, st.wmax_est = 1, p.wmax
    grid0 = np.zeros((2, CUBE, 4, p.ny, p.nx), np.complex64 if precision == "single" else np.complex128)
    keep.append(grid0)
    st.output_buffer = _ptr(grid0)
    lib.initLibrary(ctypes.byref(st))
    return st, p.nx


def _images(grid, nx):
    """The float32 images finalize packs into the host buffer, read as float32: facet f's cube
    images start at float index f * (cube * 4) * nx * ny (fft_and_repacking_routines.cpp:85-117)."""
    F = grid.shape[0]
    nxy = nx * nx
    per = CUBE * 4
    floats = grid.reshape(-1).view(np.uint8).view(np.float32)
    return np.stack([floats[f * per * nxy:f * per * nxy + CUBE * nxy] for f in range(F)]).reshape(F, CUBE, nx, nx)


@pytest.mark.parametrize("precision", ["single", "double"])
@pytest.mark.parametrize("a,b,sign", [(0, 3, 1), (0, 3, -1), (1, 2, 1), (1, 2, -1), (2, 2, 1)])
def test_device_stokes_matches_host_combination(precision, a, b, sign, gpu_required, built_libraries):
    from bullseye_gb300.library import check, load_library
    lib = load_library("GPU", precision)
    keep = []
    st, nx = _init(lib, precision, keep)
    try:
        check(lib)
        cd = np.complex64 if precision == "single" else np.complex128
        rng = np.random.default_rng(11 + 5 * a + b)
        G = (rng.standard_normal((2, CUBE, 4, nx, nx)) + 1j * rng.standard_normal((2, CUBE, 4, nx, nx))).astype(cd)
        # host: the Stokes term of every (facet, cube slice), compacted to slice c of the facet block
        host = G.copy()
        terms = (G[:, :, a] + cd(sign) * G[:, :, b]) / cd(2)
        flat = host.reshape(2, CUBE * 4, nx, nx)
        for c in range(CUBE):
            flat[:, c] = terms[:, c]
        st.output_buffer = _ptr(host)
        lib.finalize(ctypes.byref(st))
        check(lib)
        dev = G.copy()
        st.output_buffer = _ptr(dev)
        lib.bullseye_finalize_stokes(ctypes.byref(st), a, b, sign)
        check(lib)
        want, got = _images(host, nx), _images(dev, nx)
        assert np.max(np.abs(want)) > 0
        assert np.max(np.abs(got - want)) <= 1e-6 * np.max(np.abs(want))
    finally:
        lib.releaseLibrary()


def test_device_stokes_rejects_bad_correlations(gpu_required, built_libraries):
    from bullseye_gb300.library import ImagingError, check, load_library
    lib = load_library("GPU", "single")
    keep = []
    st, _ = _init(lib, "single", keep)
    try:
        check(lib)
        lib.bullseye_finalize_stokes(ctypes.byref(st), 0, 4, 1)
        with pytest.raises(ImagingError, match="bullseye_finalize_stokes"):
            check(lib)
        lib.bullseye_finalize_stokes(ctypes.byref(st), 0, 3, 2)
        with pytest.raises(ImagingError, match="bullseye_finalize_stokes"):
            check(lib)
    finally:
        lib.bullseye_clear_error()
        lib.releaseLibrary()
