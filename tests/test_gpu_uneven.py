"""Batched gridding of an uneven facet layout (bullseye_grid_batched_facets).

Three facets with different grid sizes, cell sizes and per-facet row masks are gridded in one
batched call into caller-owned device buffers.  Each facet must equal what the regular per-call
entry point (facet_4_cor / grid_4_cor) gives for that facet alone on a problem of its own size and
cell, with the masked rows flagged: 1e-12 relative in the 64-bit library, 1e-5 in the 32-bit one.
A second call accumulates (graph replay) and must give twice the first.
"""
import ctypes
from dataclasses import replace

import numpy as np
import pytest

from bullseye_gb300 import synth
from bullseye_gb300.imaging import baseline_index, run_imaging

pytestmark = pytest.mark.gpu

SIZES = [(64, 1.5), (96, 1.0), (128, 0.75)]  # (grid size, cell relative to the base cell)
TOL = {"double": 1e-12, "single": 1e-5}


def _rel(a, b):
    s = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / s)


def _problem(precision, wplanes):
    return synth.small_problem(precision, nx=96, n_ant=7, n_times=10, n_chan=3, n_facets=3, jones=False, s=4, os=9,
                               wplanes=wplanes, min_support=5 if wplanes > 1 else None, seed=31)


def _masks(p):
    rng = np.random.default_rng(4)
    return np.stack([rng.uniform(0, 1, p.rows) >= frac for frac in (0.0, 0.3, 0.6)])  # [F][R], True = kept


def _init_struct(p, torch, keep):
    """initLibrary struct: host tables, device rows in baseline-major order (device-input mode)."""
    from bullseye_gb300.abi import gridding_parameters_type
    dev = torch.device("cuda")
    b = baseline_index(p.antenna1, p.antenna2, p.n_antennas)
    order = np.argsort(b, kind="stable")
    counts = np.bincount(b, minlength=p.baseline_count)
    starts = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    t = lambda a, dt=None: torch.as_tensor(np.ascontiguousarray(a if dt is None else a.astype(dt)), device=dev)  # noqa: E731
    h = lambda a, dt: np.ascontiguousarray(np.asarray(a).astype(dt))  # noqa: E731
    F = max(1, p.n_facets)
    cd = np.complex64 if p.precision == "single" else np.complex128
    arrs = dict(
        vis=t(p.vis[order]), uvw=t(p.uvw[order]), wt=t(p.weights[order]), fl=t(p.flags[order], np.uint8),
        fr=t(p.flagged_rows[order], np.uint8), field=t(p.field_ids[order], np.int32), spw=t(p.spw_ids[order], np.int32),
        a1=t(p.antenna1[order], np.int32), a2=t(p.antenna2[order], np.int32), tid=t(p.timestamp_ids[order], np.int64),
        starts=t(starts),
        conv=np.ascontiguousarray(p.conv), lam=h(p.wavelengths.reshape(-1), p.wavelengths.dtype),
        en=np.ones(p.spws * p.channels, np.uint8), cgi=np.zeros(p.spws * p.channels, np.uintp),
        fc=h(p.facet_centres, p.uvw.dtype), grid=np.zeros((F, p.cube, 4, p.ny, p.nx), cd))
    keep.append(arrs)
    st = gridding_parameters_type(p.precision)()
    D = lambda x: ctypes.c_void_p(x.data_ptr())  # noqa: E731
    H = lambda x: ctypes.c_void_p(x.ctypes.data)  # noqa: E731
    st.visibilities, st.uvw_coords, st.visibility_weights = D(arrs["vis"]), D(arrs["uvw"]), D(arrs["wt"])
    st.flags, st.flagged_rows, st.field_array = D(arrs["fl"]), D(arrs["fr"]), D(arrs["field"])
    st.spw_index_array, st.antenna_1_ids, st.antenna_2_ids = D(arrs["spw"]), D(arrs["a1"]), D(arrs["a2"])
    st.timestamp_ids, st.baseline_starting_indexes = D(arrs["tid"]), D(arrs["starts"])
    st.conv, st.reference_wavelengths = H(arrs["conv"]), H(arrs["lam"])
    st.enabled_channels, st.channel_grid_indicies, st.facet_centres = H(arrs["en"]), H(arrs["cgi"]), H(arrs["fc"])
    st.output_buffer = H(arrs["grid"])
    st.row_count = st.chunk_max_row_count = p.rows
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
    return st, order


@pytest.mark.parametrize("precision", ["double", "single"])
@pytest.mark.parametrize("call,wplanes", [("facet_4_cor", 4), ("facet_4_cor", 1), ("grid_4_cor", 4)])
def test_uneven_facets_match_per_facet_calls(precision, call, wplanes, gpu_required, built_libraries):
    import torch
    from bullseye_gb300.abi import BullseyeFacet
    from bullseye_gb300.library import check, load_library
    torch.cuda.set_device(0)
    lib = load_library("GPU", precision)
    p = _problem(precision, wplanes)
    masks = _masks(p)
    F = len(SIZES)
    # references: each facet alone on a problem of its own size and cell, masked rows flagged
    refs = []
    for f, (n, cf) in enumerate(SIZES):
        pf = replace(p, nx=n, ny=n, cell_x=p.cell_x * cf, cell_y=p.cell_y * cf,
                     facet_centres=p.facet_centres[f:f + 1], flagged_rows=p.flagged_rows | ~masks[f])
        refs.append(run_imaging(lib, pf, call, keep_raw=True, norm_bins=(2 * p.conv_support + 1) ** 2))
        check(lib)
    # one batched call over the uneven layout
    keep = []
    facets = (BullseyeFacet * F)()
    offs, off = [], 0
    for f, (n, cf) in enumerate(SIZES):
        ra, dec = (p.facet_centres[f] if call.startswith("facet") else p.phase_centre)
        facets[f] = BullseyeFacet(float(ra), float(dec), p.cell_x * cf, p.cell_y * cf, n, n, off)
        offs.append(off)
        off += p.cube * 4 * n * n
    ct = torch.complex64 if precision == "single" else torch.complex128
    grids = torch.zeros(off, dtype=ct, device="cuda")
    lo = torch.zeros(off, dtype=ct, device="cuda")
    norms = torch.zeros(F * p.cube * 4, dtype=torch.float64, device="cuda")
    lib.bullseye_set_device_inputs(1)
    try:
        st, order = _init_struct(p, torch, keep)
        lib.initLibrary(ctypes.byref(st))
        check(lib)
        mask_dev = torch.as_tensor(np.ascontiguousarray(masks[:, order].astype(np.uint8)), device="cuda")
        torch.cuda.synchronize()  # torch's zero fills and copies run on its own stream
        code = {"facet_4_cor": 1, "grid_4_cor": 2}[call]
        results = []
        for rep in range(2):
            rc = lib.bullseye_grid_batched_facets(ctypes.byref(st), ctypes.cast(facets, ctypes.c_void_p), F,
                                                  ctypes.c_void_p(mask_dev.data_ptr()), ctypes.c_void_p(grids.data_ptr()),
                                                  ctypes.c_void_p(lo.data_ptr()), ctypes.c_void_p(norms.data_ptr()), code)
            assert rc == 0
            lib.gridding_barrier()
            check(lib)
            results.append(((grids + lo).cpu().numpy(), norms.cpu().numpy().reshape(F, p.cube, 4)))
        lib.releaseLibrary()
    finally:
        lib.bullseye_set_device_inputs(0)
    for rep, (g, nrm) in enumerate(results):
        for f, (n, _) in enumerate(SIZES):
            got = g[offs[f]:offs[f] + p.cube * 4 * n * n].reshape(p.cube, 4, n, n)
            want = refs[f].raw_grid[0] * (rep + 1)
            assert _rel(got, want) <= TOL[precision], (rep, f, _rel(got, want))
            wn = refs[f].normalization[0] * (rep + 1)
            assert np.max(np.abs(nrm[f] - wn)) <= TOL[precision] * np.max(np.abs(wn)), (rep, f)


def test_uneven_rejects_bad_layouts(gpu_required, built_libraries):
    from bullseye_gb300.abi import BullseyeFacet, gridding_parameters_type
    from bullseye_gb300.library import load_library
    lib = load_library("GPU", "single")
    st = gridding_parameters_type("single")()
    f = (BullseyeFacet * 1)(BullseyeFacet(0.0, 0.0, 1.0, 1.0, 64, 64, 0))
    # before initLibrary: refused without touching the GPU
    assert lib.bullseye_grid_batched_facets(ctypes.byref(st), ctypes.cast(f, ctypes.c_void_p), 1, None,
                                            ctypes.c_void_p(1), None, ctypes.c_void_p(1), 1) != 0
    lib.bullseye_clear_error()
