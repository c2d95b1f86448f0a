"""The allocation-free gridding entry point against the library's regular entry point.

bullseye_facet_4_cor_corrections_noalloc serves callers that cannot allocate device memory while
they grid (an application that owns a fixed device arena and forbids further cudaMalloc/cudaFree,
or code where an allocation would synchronise the device or is not permitted).  It must produce
what facet_4_cor_corrections produces: the grids and normalisation sums are compared, within the
single-precision tolerance of the other parity tests, on two calls in a row (the second call must
not see anything the first left in the shared scratch array).  This file is collected last so a
failure here never hides the other tests.
"""
import ctypes

import numpy as np
import pytest

from bullseye_gb300 import synth
from bullseye_gb300.imaging import baseline_index, run_imaging

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _rel(a, b):
    s = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / s) if s else float(np.max(np.abs(a - b)))


def _problem():
    return synth.small_problem("single", nx=96, n_ant=7, n_times=10, n_chan=3, n_facets=3, jones=True, s=4, os=9,
                               wplanes=4, min_support=5)


def _device_struct(p, torch, lib_keep):
    """gridding_parameters whose array fields are device pointers (rows in baseline-major order)."""
    from bullseye_gb300.abi import gridding_parameters_type
    dev = torch.device("cuda")
    b = baseline_index(p.antenna1, p.antenna2, p.n_antennas)
    order = np.argsort(b, kind="stable")
    counts = np.bincount(b, minlength=p.baseline_count)
    starts = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    F = max(1, p.n_facets)
    t = lambda a, dt=None: torch.as_tensor(np.ascontiguousarray(a if dt is None else a.astype(dt)), device=dev)
    arrs = dict(
        vis=t(p.vis[order]), uvw=t(p.uvw[order]), wt=t(p.weights[order]), fl=t(p.flags[order], np.uint8),
        fr=t(p.flagged_rows[order], np.uint8), field=t(p.field_ids[order], np.int32), spw=t(p.spw_ids[order], np.int32),
        a1=t(p.antenna1[order], np.int32), a2=t(p.antenna2[order], np.int32), tid=t(p.timestamp_ids[order], np.int64),
        jones=t(p.jones), starts=t(starts), conv=t(p.conv), lam=t(p.wavelengths.reshape(-1)),
        en=t(np.ones(p.spws * p.channels, np.uint8)), cgi=t(np.zeros(p.spws * p.channels, np.int64)),
        fc=t(p.facet_centres),
        grid=torch.zeros((F, p.cube, 4, p.ny, p.nx), dtype=torch.complex64, device=dev),
        norm=torch.zeros(F * p.cube * 4, dtype=torch.float64, device=dev),
    )
    lib_keep.append(arrs)
    st = gridding_parameters_type("single")()
    P = lambda x: ctypes.c_void_p(x.data_ptr())
    st.visibilities, st.uvw_coords, st.visibility_weights = P(arrs["vis"]), P(arrs["uvw"]), P(arrs["wt"])
    st.flags, st.flagged_rows, st.field_array = P(arrs["fl"]), P(arrs["fr"]), P(arrs["field"])
    st.spw_index_array, st.antenna_1_ids, st.antenna_2_ids = P(arrs["spw"]), P(arrs["a1"]), P(arrs["a2"])
    st.timestamp_ids, st.jones_terms, st.baseline_starting_indexes = P(arrs["tid"]), P(arrs["jones"]), P(arrs["starts"])
    st.conv, st.reference_wavelengths = P(arrs["conv"]), P(arrs["lam"])
    st.enabled_channels, st.channel_grid_indicies, st.facet_centres = P(arrs["en"]), P(arrs["cgi"]), P(arrs["fc"])
    st.output_buffer, st.normalization_terms = P(arrs["grid"]), P(arrs["norm"])
    st.row_count = p.rows
    st.baseline_count = p.baseline_count
    st.channel_count, st.spw_count = p.channels, p.spws
    st.number_of_polarization_terms = st.number_of_polarization_terms_being_gridded = 4
    st.no_timestamps_read, st.antenna_count = p.n_timestamps, p.n_antennas
    st.nx, st.ny = p.nx, p.ny
    st.cell_size_x, st.cell_size_y = p.cell_x, p.cell_y
    st.conv_support, st.conv_oversample = p.conv_support, p.conv_oversample
    st.phase_centre_ra, st.phase_centre_dec = p.phase_centre
    st.num_facet_centres = F
    st.cube_channel_dim_size = p.cube
    st.wplanes, st.wmax_est = p.wplanes, p.wmax
    st.imaging_field = p.imaging_field
    return st, arrs


def test_noalloc_matches_regular_entry_point_on_two_calls(gpu_required, built_libraries):
    import torch
    from bullseye_gb300.library import check, load_library
    torch.cuda.set_device(0)
    lib = load_library("GPU", "single")
    p = _problem()
    ref = run_imaging(lib, p, "facet_4_cor_corrections", repack=True, keep_raw=True,
                      norm_bins=(2 * p.conv_support + 1) ** 2)
    check(lib)
    keep = []
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        st, arrs = _device_struct(p, torch, keep)
        rc = lib.bullseye_facet_4_cor_corrections_noalloc(ctypes.byref(st), stream)
        assert rc == 0, f"call {call}: status {rc}"
        torch.cuda.synchronize()
        check(lib)
        grid = arrs["grid"].cpu().numpy()
        norm = arrs["norm"].cpu().numpy().reshape(ref.normalization.shape)
        assert _rel(grid, ref.raw_grid) <= TOL, f"call {call}: grid rel err {_rel(grid, ref.raw_grid):.2e}"
        assert _rel(norm, ref.normalization) <= TOL, f"call {call}: norm rel err {_rel(norm, ref.normalization):.2e}"


def test_workspace_entry_is_support_aware_and_matches_full_support(gpu_required, built_libraries):
    """bullseye_facet_4_cor_corrections_ws grids each w plane's nonzero window only, with the support
    windows, the window table and the run schedule built in the caller's workspace.  Its grids and
    normalisation must match the plain kernels over the full padded support (31 taps, planes of 11 to
    31), on two calls in a row."""
    import torch
    from bullseye_gb300.library import check, load_library
    torch.cuda.set_device(0)
    lib = load_library("GPU", "single")
    p = synth.small_problem("single", nx=128, n_ant=7, n_times=10, n_chan=3, n_facets=2, jones=True, s=15, os=5,
                            wplanes=8, min_support=5)
    lib.bullseye_set_batched_calls(0)
    try:
        ref = run_imaging(lib, p, "facet_4_cor_corrections", repack=True, keep_raw=True,
                          norm_bins=(2 * p.conv_support + 1) ** 2)
    finally:
        lib.bullseye_set_batched_calls(1)
    check(lib)
    keep = []
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        st, arrs = _device_struct(p, torch, keep)  # fresh Jones each call: the entry inverts them in place
        nbytes = int(lib.bullseye_facet_4_cor_corrections_ws_bytes(ctypes.byref(st)))
        ws = torch.empty(nbytes + 256, dtype=torch.uint8, device="cuda")
        base = (ws.data_ptr() + 255) // 256 * 256
        rc = lib.bullseye_facet_4_cor_corrections_ws(ctypes.byref(st), ctypes.c_void_p(base), nbytes, stream)
        assert rc == 0, f"call {call}: status {rc}"
        torch.cuda.synchronize()
        check(lib)
        grid = arrs["grid"].cpu().numpy()
        norm = arrs["norm"].cpu().numpy().reshape(ref.normalization.shape)
        assert np.max(np.abs(ref.raw_grid)) > 0
        assert _rel(grid, ref.raw_grid) <= TOL, f"call {call}: grid rel err {_rel(grid, ref.raw_grid):.2e}"
        assert _rel(norm, ref.normalization) <= TOL, f"call {call}: norm rel err {_rel(norm, ref.normalization):.2e}"


def test_noalloc_rejects_grids_beyond_the_scratch(gpu_required, built_libraries):
    import torch
    from bullseye_gb300.library import ImagingError, check, load_library
    torch.cuda.set_device(0)
    lib = load_library("GPU", "single")
    keep = []
    st, _ = _device_struct(_problem(), torch, keep)
    st.nx = st.ny = 2048  # 3 facets x 4 x 2048^2 cells > 5,242,880
    rc = lib.bullseye_facet_4_cor_corrections_noalloc(ctypes.byref(st), ctypes.c_void_p(0))
    assert rc == 5
    with pytest.raises(ImagingError, match="scratch"):
        check(lib)
