"""Inputs for the nearest-neighbour sampling-count fixtures (tests/golden/nn_counts_<precision>.npz).

Rows are drawn so that the cell decision is delicate: a third of the pixel coordinates lie within
1e-5 pixels of a half-integer, where the nearest-even rounding of the reference's own float or
double operation sequence decides the cell; others fall off the grid on every side.  Flagged rows,
rows of another field, a disabled channel and two sampling-function channels are included.
"""
from __future__ import annotations

import ctypes

import numpy as np

from bullseye_gb300.abi import gridding_parameters_type, real_dtype

NX, NY = 64, 48
SPWS, CHANS = 2, 3
SF_CH = 2
FACETS = 3
CELL = 7.0
ARCSEC = float(np.float32(np.pi / (180.0 * 3600.0)))


def make_inputs(precision: str, seed: int = 11, rows: int = 900) -> dict:
    rd = real_dtype(precision)
    rng = np.random.default_rng(seed)
    lam = rng.uniform(0.2, 0.25, (SPWS, CHANS)).astype(rd)
    spw = rng.integers(0, SPWS, rows).astype(np.uint32)
    px = rng.uniform(-6, NX + 6, rows)
    py = rng.uniform(-6, NY + 6, rows)
    near = rng.uniform(0, 1, rows) < 1 / 3
    px[near] = np.floor(px[near]) + 0.5 + rng.uniform(-1e-5, 1e-5, near.sum())
    py[near] = np.floor(py[near]) + 0.5 + rng.uniform(-1e-5, 1e-5, near.sum())
    u_scale = NX * CELL * ARCSEC
    v_scale = -(NY * CELL * ARCSEC)
    # metres for channel 0 of the row's spw; other channels scale with their wavelength
    lam0 = lam[spw, 0].astype(np.float64)
    uvw = np.zeros((rows, 3))
    uvw[:, 0] = (px - NX // 2) / u_scale * lam0
    uvw[:, 1] = (py - NY // 2) / v_scale * lam0
    uvw[:, 2] = rng.uniform(-500, 500, rows)
    enabled = np.ones(SPWS * CHANS, np.bool_)
    enabled[4] = False
    return dict(
        uvw=uvw.astype(rd), lam=lam.reshape(-1), spw=spw,
        field=np.where(rng.uniform(0, 1, rows) < 0.05, 1, 0).astype(np.uint32),
        flagged_rows=rng.uniform(0, 1, rows) < 0.05, enabled=enabled,
        sfcgi=np.array([0, 1, 0, 1, 1, 0], np.uintp), facet_centres=rng.uniform(-3000, 3000, (FACETS, 2)).astype(rd),
        phase_centre=np.array([0.0, -108000.0]))


def make_struct(precision: str, d: dict, faceting: bool, ptr, buffer_ptr):
    """gridding_parameters for the sampling-count call; ``ptr`` turns an array into a pointer."""
    st = gridding_parameters_type(precision)()
    st.uvw_coords = ptr(d["uvw"])
    st.reference_wavelengths = ptr(d["lam"])
    st.spw_index_array = ptr(d["spw"])
    st.field_array = ptr(d["field"])
    st.flagged_rows = ptr(d["flagged_rows"])
    st.enabled_channels = ptr(d["enabled"])
    st.sampling_function_channel_grid_indicies = ptr(d["sfcgi"])
    st.facet_centres = ptr(d["facet_centres"])
    st.sampling_function_buffer = buffer_ptr
    st.sampling_function_channel_count = SF_CH
    st.row_count = d["uvw"].shape[0]
    st.channel_count, st.spw_count = CHANS, SPWS
    st.nx, st.ny = NX, NY
    st.cell_size_x = st.cell_size_y = CELL
    st.num_facet_centres = FACETS if faceting else 1
    st.phase_centre_ra, st.phase_centre_dec = d["phase_centre"]
    st.imaging_field = 0
    st.conv_support = 0
    st.conv_oversample = 1
    return st


def host_ptr(a):
    return ctypes.c_void_p(np.ascontiguousarray(a).ctypes.data)
