"""Host-side driver for the imaging C-ABI: problem description and the pipeliner's call sequence.

A :class:`GriddingProblem` holds every array the pipeliner hands to the imaging library, in the
ABI's layouts (bullseye/mo/cpu_gpu_common/gridding_parameters.h:44-109).  :func:`run_imaging`
replays the pipeliner's sequence against any library exporting that ABI
(bullseye/bin/bullseye_pipeliner.py:260-424):

    initLibrary -> per chunk { [repack_input_data] -> grid/facet call -> [sampling-function
    call] -> gridding_barrier } -> [weight_uniformly] -> normalize -> [finalize] ->
    [finalize_psf] -> releaseLibrary

It works unchanged with the GPU drop-in (``bullseye_gb300.library``) and with any CPU library
of the same ABI, which is how the tests compare them on identical inputs.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field, replace
from typing import Optional

import numpy as np

from .abi import complex_dtype, gridding_parameters_type, real_dtype

#: ABI entry point per gridding mode (bullseye/bin/bullseye_pipeliner.py:359-378)
GRID_CALLS = {
    "grid_single_pol": (1, False),
    "facet_single_pol": (1, True),
    "grid_duel_pol": (2, False),
    "facet_duel_pol": (2, True),
    "grid_4_cor": (4, False),
    "facet_4_cor": (4, True),
    "facet_4_cor_corrections": (4, True),
}


def baseline_index(a1, a2, n_antennas):
    """Baseline slot of an antenna pair, autocorrelations included.

    Same quadratic-series enumeration as bullseye/mo/gpu_algorithm/wrapper.cu:358-366:
    S = min(a1, a2);  b = S * (2N + 1 - S) / 2 + |a1 - a2|.
    """
    a1 = np.asarray(a1, dtype=np.int64)
    a2 = np.asarray(a2, dtype=np.int64)
    s = np.minimum(a1, a2)
    return (s * (2 * n_antennas + 1 - s)) // 2 + np.abs(a1 - a2)


@dataclass
class GriddingProblem:
    """All inputs of one imaging run in ABI layout.

    Shapes: R rows, Ch channels per spw, S spws, P polarisation terms per (row, channel),
    F facets (F = 0 means no faceting: one grid at the phase centre).
    """
    precision: str
    vis: np.ndarray            # complex [R, Ch, P]
    uvw: np.ndarray            # real [R, 3] metres
    wavelengths: np.ndarray    # real [S, Ch] metres
    weights: np.ndarray        # real [R, Ch, P]
    flags: np.ndarray          # bool [R, Ch, P]
    flagged_rows: np.ndarray   # bool [R]
    field_ids: np.ndarray      # uint32 [R]
    spw_ids: np.ndarray        # uint32 [R]
    antenna1: np.ndarray       # uint32 [R]
    antenna2: np.ndarray       # uint32 [R]
    timestamp_ids: np.ndarray  # uintp [R]
    n_antennas: int
    n_timestamps: int
    nx: int
    ny: int
    cell_x: float              # arcsec
    cell_y: float              # arcsec
    conv: np.ndarray           # real [K] (no w) | complex [Pw, K] (separable w) | complex [Pw, K, K]
    conv_support: int          # half support s; full support W = 2s + 1
    conv_oversample: int
    wplanes: int = 1
    wmax: float = 1.0
    phase_centre: tuple = (0.0, 0.0)   # (ra, dec) arcsec
    facet_centres: Optional[np.ndarray] = None  # real [F, 2] arcsec
    jones: Optional[np.ndarray] = None  # complex [T, A, F, S, Ch, 4]
    pol_index: int = 0
    second_pol_index: int = 3
    enabled_channels: Optional[np.ndarray] = None       # bool [S*Ch]
    channel_grid_index: Optional[np.ndarray] = None     # uintp [S*Ch]
    cube: int = 1
    sampling_channel_grid_index: Optional[np.ndarray] = None  # uintp [S*Ch]
    sampling_channel_count: int = 1
    imaging_field: int = 0

    @property
    def rows(self) -> int:
        return int(self.uvw.shape[0])

    @property
    def channels(self) -> int:
        return int(self.wavelengths.shape[1])

    @property
    def spws(self) -> int:
        return int(self.wavelengths.shape[0])

    @property
    def n_pol(self) -> int:
        return int(self.vis.shape[2])

    @property
    def n_facets(self) -> int:
        return 0 if self.facet_centres is None else int(self.facet_centres.shape[0])

    @property
    def baseline_count(self) -> int:
        n = self.n_antennas
        return n * (n - 1) // 2 + n

    def astype(self, precision: str) -> "GriddingProblem":
        """Same problem with real/complex arrays converted to ``precision``."""
        rd, cd = real_dtype(precision), complex_dtype(precision)
        conv = self.conv.astype(cd if np.iscomplexobj(self.conv) else rd)
        fc = None if self.facet_centres is None else self.facet_centres.astype(rd)
        jn = None if self.jones is None else self.jones.astype(cd)
        return replace(self, precision=precision, vis=self.vis.astype(cd), uvw=self.uvw.astype(rd),
                       wavelengths=self.wavelengths.astype(rd), weights=self.weights.astype(rd),
                       conv=conv, facet_centres=fc, jones=jn)

    def with_conv(self, conv: np.ndarray) -> "GriddingProblem":
        return replace(self, conv=conv)


@dataclass
class ImagingResult:
    grid: np.ndarray                 # complex [F', cube, C, ny, nx] after normalize (and weighting)
    normalization: np.ndarray        # float64 as published by the library
    sampling: Optional[np.ndarray] = None   # complex [F', sf, 1, ny, nx]
    image: Optional[np.ndarray] = None      # float32 [F', cube, ny, nx] after finalize
    psf: Optional[np.ndarray] = None        # float32 [F', sf, ny, nx] after finalize_psf
    raw_grid: Optional[np.ndarray] = None   # grid before weighting/normalisation
    gridding_walltime: float = 0.0
    inversion_walltime: float = 0.0
    extras: dict = field(default_factory=dict)


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _contig(a, dtype=None):
    return np.ascontiguousarray(a if dtype is None else a.astype(dtype, copy=False))


def pinned_host(offset: int = 0):
    """A ``host_alloc`` for run_imaging: every array in its own page-locked (pinned torch) buffer,
    starting ``offset`` bytes into it (an offset that is not a multiple of the element size gives
    unaligned arrays)."""
    import torch

    def new(shape, dtype):
        dtype = np.dtype(dtype)
        n = int(np.prod(shape)) * dtype.itemsize
        buf = torch.empty(n + offset, dtype=torch.uint8, pin_memory=True)
        return buf.numpy()[offset:offset + n].view(dtype).reshape(shape)

    return new


def run_imaging(lib, problem: GriddingProblem, call: str, *, chunks: int = 1, repack: bool = False,
                uniform: bool = False, psf: bool = False, do_finalize: bool = False,
                norm_bins: int = 1, keep_raw: bool = False, host_alloc=None) -> ImagingResult:
    """Run the pipeliner's ABI sequence for ``call`` on ``lib`` and return the host outputs.

    ``norm_bins`` is the number of float64 normalisation bins per (facet, cube, correlation)
    that the library publishes: 1 for the CPU libraries (wrapper.cpp:102-105), W*W for the
    GPU library layout (wrapper.cu:222-230).  The returned ``normalization`` is summed over
    bins.  Caller arrays are copied before every call that may modify them.  ``host_alloc(shape,
    dtype)`` makes the caller's grids, rows and Jones terms (numpy memory by default; see
    pinned_host).
    """
    alloc = host_alloc or (lambda shape, dtype: np.empty(shape, dtype))

    def place(a):
        out = alloc(a.shape, a.dtype)
        out[...] = a
        return out

    if call not in GRID_CALLS:
        raise ValueError(f"unknown gridding call {call!r}")
    n_corr, faceting = GRID_CALLS[call]
    p = problem
    prec = p.precision
    rd, cd = real_dtype(prec), complex_dtype(prec)
    F = max(1, p.n_facets)
    nxy = p.nx * p.ny
    S, Ch = p.spws, p.channels

    grid = place(np.zeros((F, p.cube, n_corr, p.ny, p.nx), dtype=cd))
    want_sf = uniform or psf
    sf = place(np.zeros((F, p.sampling_channel_count, 1, p.ny, p.nx), dtype=cd)) if want_sf else None

    enabled = _contig(p.enabled_channels if p.enabled_channels is not None else np.ones(S * Ch, bool), np.bool_)
    cgi = _contig(p.channel_grid_index if p.channel_grid_index is not None else np.zeros(S * Ch, np.uintp), np.uintp)
    sfcgi = _contig(p.sampling_channel_grid_index if p.sampling_channel_grid_index is not None
                    else np.zeros(S * Ch, np.uintp), np.uintp)
    lam = _contig(p.wavelengths, rd)
    conv = _contig(p.conv)
    fc = _contig(p.facet_centres, rd) if p.facet_centres is not None else np.zeros((1, 2), rd)

    st = gridding_parameters_type(prec)()
    st.chunk_max_row_count = int(np.ceil(p.rows / chunks)) if p.rows else 0
    st.nx, st.ny = p.nx, p.ny
    st.cell_size_x, st.cell_size_y = p.cell_x, p.cell_y
    st.conv = _ptr(conv)
    st.conv_support = p.conv_support
    st.conv_oversample = p.conv_oversample
    st.phase_centre_ra, st.phase_centre_dec = p.phase_centre
    st.should_invert_jones_terms = call == "facet_4_cor_corrections"
    st.imaging_field = p.imaging_field
    st.channel_grid_indicies = _ptr(cgi)
    st.cube_channel_dim_size = p.cube
    st.output_buffer = _ptr(grid)
    st.baseline_count = p.baseline_count
    st.number_of_polarization_terms = p.n_pol
    st.number_of_polarization_terms_being_gridded = n_corr
    st.spw_count = S
    st.channel_count = Ch
    st.antenna_count = p.n_antennas
    st.enabled_channels = _ptr(enabled)
    st.reference_wavelengths = _ptr(lam)
    st.should_grid_sampling_function = want_sf
    if want_sf:
        st.sampling_function_buffer = _ptr(sf)
        st.sampling_function_channel_grid_indicies = _ptr(sfcgi)
        st.sampling_function_channel_count = p.sampling_channel_count
    st.num_facet_centres = F
    st.facet_centres = _ptr(fc)
    st.polarization_index = p.pol_index
    st.second_polarization_index = p.second_pol_index
    st.wplanes = p.wplanes
    st.wmax_est = p.wmax
    keep = [grid, sf, enabled, cgi, sfcgi, lam, conv, fc]

    lib.initLibrary(ctypes.byref(st))
    norm_ptr = st.normalization_terms
    bounds = np.linspace(0, p.rows, chunks + 1).astype(np.int64) if p.rows else np.zeros(chunks + 1, np.int64)
    for ci in range(chunks):
        lo, hi = int(bounds[ci]), int(bounds[ci + 1])
        lib.gridding_barrier()
        arrs = dict(
            vis=place(_contig(p.vis[lo:hi], cd)), uvw=place(_contig(p.uvw[lo:hi], rd)),
            wt=place(_contig(p.weights[lo:hi], rd)), fl=place(_contig(p.flags[lo:hi], np.bool_)),
            fr=place(_contig(p.flagged_rows[lo:hi], np.bool_)), field=place(_contig(p.field_ids[lo:hi], np.uint32)),
            spw=place(_contig(p.spw_ids[lo:hi], np.uint32)), a1=place(_contig(p.antenna1[lo:hi], np.uint32)),
            a2=place(_contig(p.antenna2[lo:hi], np.uint32)),
            t=place(_contig(p.timestamp_ids[lo:hi], np.uintp)),
        )
        keep.append(arrs)
        st.visibilities = _ptr(arrs["vis"])
        st.uvw_coords = _ptr(arrs["uvw"])
        st.visibility_weights = _ptr(arrs["wt"])
        st.flags = _ptr(arrs["fl"])
        st.flagged_rows = _ptr(arrs["fr"])
        st.field_array = _ptr(arrs["field"])
        st.spw_index_array = _ptr(arrs["spw"])
        st.row_count = hi - lo
        st.no_timestamps_read = p.n_timestamps
        st.is_final_data_chunk = ci == chunks - 1
        st.antenna_1_ids = _ptr(arrs["a1"])
        st.antenna_2_ids = _ptr(arrs["a2"])
        st.timestamp_ids = _ptr(arrs["t"])
        if repack:
            starts = np.zeros(p.baseline_count + 1, dtype=np.uintp)
            arrs["starts"] = starts
            st.baseline_starting_indexes = _ptr(starts)
            lib.repack_input_data(ctypes.byref(st))
        if call == "facet_4_cor_corrections":
            jn = place(_contig(p.jones, cd))
            arrs["jones"] = jn
            st.jones_terms = _ptr(jn)
        getattr(lib, call)(ctypes.byref(st))
        if want_sf:
            (lib.facet_sampling_function if faceting else lib.grid_sampling_function)(ctypes.byref(st))
    lib.gridding_barrier()
    raw = grid.copy() if keep_raw else None
    if uniform:
        lib.weight_uniformly(ctypes.byref(st))
    nbins = F * p.cube * n_corr * norm_bins
    norm = np.ctypeslib.as_array(ctypes.cast(norm_ptr, ctypes.POINTER(ctypes.c_double)), shape=(nbins,)).copy()
    lib.normalize(ctypes.byref(st))
    res = ImagingResult(grid=grid.copy(), normalization=norm.reshape(F, p.cube, n_corr, norm_bins).sum(-1),
                        sampling=None if sf is None else sf.copy(), raw_grid=raw)
    if do_finalize:
        lib.finalize(ctypes.byref(st))
        fl = grid.view(np.float32).reshape(-1)
        off = p.cube * n_corr * nxy
        res.image = np.stack([fl[off * f: off * f + p.cube * nxy].reshape(p.cube, p.ny, p.nx) for f in range(F)]).copy()
        if psf:
            lib.finalize_psf(ctypes.byref(st))
            fl = sf.view(np.float32).reshape(-1)
            off = p.sampling_channel_count * nxy
            res.psf = np.stack([fl[off * f: off * f + off].reshape(p.sampling_channel_count, p.ny, p.nx)
                                for f in range(F)]).copy()
    res.gridding_walltime = float(lib.get_gridding_walltime())
    res.inversion_walltime = float(lib.get_inversion_walltime())
    lib.releaseLibrary()
    del keep
    return res
