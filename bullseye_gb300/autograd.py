"""Differentiable faceted gridding: grids as a torch function of the visibilities and Jones terms.

:func:`facet_grid` grids four-correlation visibilities into per-facet grids exactly as
``facet_4_cor_corrections`` does (Jones correction J_p^-1 V J_q^-H, per-facet phase rotation and
planar uv transform, Romein gridding with the AA or w-projection kernel:
bullseye/mo/gpu_algorithm/wrapper.cu:988-1150 and the CPU policies it mirrors,
correlation_gridding_policies.h:503-542, phase_transform_policies.h:110-134,
baseline_transform_policies.h:117-149).  The forward pass runs the library's workspace entry point
(bullseye_facet_4_cor_corrections_ws, with a torch-allocated workspace) on torch's current stream; the backward pass runs the library's adjoint (degridding) kernel
and returns dL/dV and dL/dJ in PyTorch's complex-gradient convention (dL = Re sum conj(g) dz).

Both passes are the CUDA library: there is no PyTorch or CPU implementation here, and a missing
library raises.  ``complex64`` inputs run the 32-bit library (compensated FP32 gridding),
``complex128`` the 64-bit one.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from .abi import gridding_parameters_type
from .imaging import GriddingProblem, baseline_index
from .library import ImagingError, check, load_library


def _precision(dtype: torch.dtype) -> str:
    if dtype == torch.complex64:
        return "single"
    if dtype == torch.complex128:
        return "double"
    raise TypeError(f"visibilities must be complex64 or complex128, not {dtype}")


@dataclass
class FacetGeometry:
    """Device-resident, gradient-free inputs of a faceted gridding problem.

    Rows are stored baseline-major (stable within a baseline); ``order`` maps the stored rows to the
    problem's rows, so visibilities for :func:`facet_grid` are ``problem.vis[order]`` and gradients
    come back in the same order.
    """
    precision: str
    order: np.ndarray
    arrays: dict
    scalars: dict

    @classmethod
    def from_problem(cls, p: GriddingProblem, device=None) -> "FacetGeometry":
        if p.n_pol != 4:
            raise ValueError("four-correlation data required")
        device = torch.device(device or "cuda")
        b = baseline_index(p.antenna1, p.antenna2, p.n_antennas)
        order = np.argsort(b, kind="stable")
        counts = np.bincount(b, minlength=p.baseline_count)
        starts = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
        S, C = p.spws, p.channels
        en = np.ones(S * C, np.uint8) if p.enabled_channels is None else np.asarray(p.enabled_channels, np.uint8)
        cgi = np.zeros(S * C, np.int64) if p.channel_grid_index is None else np.asarray(p.channel_grid_index, np.int64)
        fc = np.zeros((1, 2), p.uvw.dtype) + np.asarray(p.phase_centre, p.uvw.dtype) if p.facet_centres is None \
            else p.facet_centres

        def t(a, dt=None):
            return torch.as_tensor(np.ascontiguousarray(a if dt is None else np.asarray(a).astype(dt)), device=device)

        arrays = dict(
            uvw=t(p.uvw[order]), wt=t(p.weights[order]), fl=t(p.flags[order], np.uint8),
            fr=t(p.flagged_rows[order], np.uint8), field=t(p.field_ids[order], np.uint32),
            spw=t(p.spw_ids[order], np.uint32), a1=t(p.antenna1[order], np.uint32), a2=t(p.antenna2[order], np.uint32),
            tid=t(p.timestamp_ids[order], np.int64), starts=t(starts), conv=t(p.conv),
            lam=t(p.wavelengths.reshape(-1)), en=t(en), cgi=t(cgi), fc=t(fc))
        scalars = dict(
            rows=p.rows, baselines=p.baseline_count, channels=C, spws=S, times=p.n_timestamps, antennas=p.n_antennas,
            nx=p.nx, ny=p.ny, cell=(p.cell_x, p.cell_y), support=p.conv_support, oversample=p.conv_oversample,
            phase_centre=tuple(p.phase_centre), facets=int(fc.shape[0]), cube=p.cube, wplanes=p.wplanes,
            wmax=p.wmax, field=p.imaging_field)
        return cls(p.precision, order, arrays, scalars)

    @property
    def grid_shape(self):
        s = self.scalars
        return (s["facets"], s["cube"], 4, s["ny"], s["nx"])

    @property
    def jones_shape(self):
        s = self.scalars
        return (s["times"], s["antennas"], s["facets"], s["spws"], s["channels"], 4)

    def struct(self, vis: torch.Tensor, jones: torch.Tensor | None, grid=None, norm=None):
        """gridding_parameters with device pointers into this geometry and the given tensors."""
        s = self.scalars
        st = gridding_parameters_type(self.precision)()
        A = self.arrays
        P = lambda x: ctypes.c_void_p(x.data_ptr()) if x is not None else None  # noqa: E731
        st.visibilities, st.uvw_coords, st.visibility_weights = P(vis), P(A["uvw"]), P(A["wt"])
        st.flags, st.flagged_rows, st.field_array = P(A["fl"]), P(A["fr"]), P(A["field"])
        st.spw_index_array, st.antenna_1_ids, st.antenna_2_ids = P(A["spw"]), P(A["a1"]), P(A["a2"])
        st.timestamp_ids, st.jones_terms, st.baseline_starting_indexes = P(A["tid"]), P(jones), P(A["starts"])
        st.conv, st.reference_wavelengths = P(A["conv"]), P(A["lam"])
        st.enabled_channels, st.channel_grid_indicies, st.facet_centres = P(A["en"]), P(A["cgi"]), P(A["fc"])
        st.output_buffer, st.normalization_terms = P(grid), P(norm)
        st.row_count, st.baseline_count = s["rows"], s["baselines"]
        st.channel_count, st.spw_count = s["channels"], s["spws"]
        st.number_of_polarization_terms = st.number_of_polarization_terms_being_gridded = 4
        st.no_timestamps_read, st.antenna_count = s["times"], s["antennas"]
        st.nx, st.ny = s["nx"], s["ny"]
        st.cell_size_x, st.cell_size_y = s["cell"]
        st.conv_support, st.conv_oversample = s["support"], s["oversample"]
        st.phase_centre_ra, st.phase_centre_dec = s["phase_centre"]
        st.num_facet_centres = s["facets"]
        st.cube_channel_dim_size = s["cube"]
        st.wplanes, st.wmax_est = s["wplanes"], s["wmax"]
        st.imaging_field = s["field"]
        return st

    def _check(self, vis, jones):
        s = self.scalars
        if vis.shape != (s["rows"], s["channels"], 4) or not vis.is_contiguous():
            raise ValueError(f"visibilities must be contiguous [{s['rows']}, {s['channels']}, 4], got {tuple(vis.shape)}")
        if _precision(vis.dtype) != self.precision:
            raise TypeError(f"{self.precision} geometry needs {'complex64' if self.precision == 'single' else 'complex128'}")
        if jones is not None and (tuple(jones.shape) != self.jones_shape or jones.dtype != vis.dtype
                                  or not jones.is_contiguous()):
            raise ValueError(f"jones must be contiguous {self.jones_shape} of {vis.dtype}")
        if vis.device != self.arrays["uvw"].device or (jones is not None and jones.device != vis.device):
            raise ValueError("all tensors must be on the geometry's device")


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def grid_adjoint(geom: FacetGeometry, vis: torch.Tensor, jones: torch.Tensor | None, grad_grid: torch.Tensor,
                 faceting: bool = True):
    """(dL/dV, dL/dJ or None) for the grids produced from ``vis`` and ``jones`` given dL/dG."""
    geom._check(vis, jones)
    if tuple(grad_grid.shape) != geom.grid_shape or grad_grid.dtype != vis.dtype:
        raise ValueError(f"grad_grid must be {geom.grid_shape} of {vis.dtype}")
    lib = load_library("GPU", geom.precision)
    grad_grid = grad_grid.contiguous()
    grad_vis = torch.empty_like(vis)
    grad_jones = torch.zeros_like(jones) if jones is not None else None
    st = geom.struct(vis, jones)
    rc = lib.bullseye_grid_adjoint(ctypes.byref(st), ctypes.c_void_p(grad_grid.data_ptr()),
                                   ctypes.c_void_p(grad_vis.data_ptr()),
                                   ctypes.c_void_p(grad_jones.data_ptr()) if grad_jones is not None else None,
                                   1 if faceting else 0, _stream())
    if rc != 0:
        check(lib)
        raise ImagingError(f"bullseye_grid_adjoint failed with status {rc}")
    return grad_vis, grad_jones


class _FacetGrid(torch.autograd.Function):
    @staticmethod
    def forward(ctx, vis, jones, geom):
        lib = load_library("GPU", geom.precision)
        grid = torch.zeros(geom.grid_shape, dtype=vis.dtype, device=vis.device)
        norm = torch.zeros(geom.grid_shape[:3], dtype=torch.float64, device=vis.device)
        work = jones.detach().clone()  # the entry point inverts the terms in place
        st = geom.struct(vis.detach(), work, grid, norm)
        nbytes = int(lib.bullseye_facet_4_cor_corrections_ws_bytes(ctypes.byref(st)))
        ws = torch.empty(nbytes + 256, dtype=torch.uint8, device=vis.device)
        aligned = (ws.data_ptr() + 255) // 256 * 256
        rc = lib.bullseye_facet_4_cor_corrections_ws(ctypes.byref(st), ctypes.c_void_p(aligned), nbytes, _stream())
        if rc != 0:
            check(lib)
            raise ImagingError(f"bullseye_facet_4_cor_corrections_ws failed with status {rc}")
        # device-side errors (singular Jones terms, ids out of range): waits for the forward kernels
        rc = lib.bullseye_facet_4_cor_corrections_status(ctypes.byref(st), ctypes.c_void_p(aligned), _stream())
        if rc != 0:
            check(lib)
            raise ImagingError(f"bullseye_facet_4_cor_corrections_ws reported device status {rc}")
        ctx.geom = geom
        ctx.save_for_backward(vis, jones)
        ctx.mark_non_differentiable(norm)
        return grid, norm

    @staticmethod
    def backward(ctx, grad_grid, grad_norm):
        vis, jones = ctx.saved_tensors
        if grad_grid is None:
            return None, None, None
        gv, gj = grid_adjoint(ctx.geom, vis.detach(), jones.detach(), grad_grid, faceting=True)
        return (gv if ctx.needs_input_grad[0] else None), (gj if ctx.needs_input_grad[1] else None), None


def facet_grid(geom: FacetGeometry, vis: torch.Tensor, jones: torch.Tensor):
    """Per-facet grids [F, cube, 4, ny, nx] and normalisation sums [F, cube, 4] (float64, no gradient).

    ``vis`` is [rows, channels, 4] in the geometry's row order, ``jones`` the raw (not inverted)
    terms [T, A, F, S, Ch, 4]; both complex64 (32-bit library) or both complex128 (64-bit).
    Differentiable with respect to both.  The forward waits for its kernels and raises
    :class:`ImagingError` on a device-side error (a singular Jones matrix, ids out of range).
    """
    geom._check(vis, jones)
    if jones is None:
        raise ValueError("jones terms are required (use identity matrices for none)")
    return _FacetGrid.apply(vis, jones, geom)


def predict(geom: FacetGeometry, model: torch.Tensor, jones: torch.Tensor | None = None, *, faceting: bool = True,
            normalise: bool = False, from_grid: bool = False, taper=None) -> torch.Tensor:
    """Model visibilities [rows, channels, 4] (the geometry's row order) predicted by the library's
    bullseye_predict from per-facet models [F, cube, 4, ny, nx]: images (divided by the gridding
    correction ``taper`` = (taper_x [nx], taper_y [ny]) float64 tensors when given, then transformed
    to uv grids) or, with ``from_grid``, uv grids.  ``jones`` (raw terms [T, A, F, S, Ch, 4]) are
    applied forward; ``normalise`` divides each facet's degridded value by its tap sum (the
    reference's prototype degridder).  Not differentiable."""
    lib = load_library("GPU", geom.precision)
    s = geom.scalars
    dt = torch.complex64 if geom.precision == "single" else torch.complex128
    if tuple(model.shape) != geom.grid_shape or model.dtype != dt or not model.is_contiguous():
        raise ValueError(f"model must be contiguous {geom.grid_shape} of {dt}")
    out = torch.empty((s["rows"], s["channels"], 4), dtype=dt, device=model.device)
    st = geom.struct(None, jones)
    ws, ws_ptr, nbytes = None, None, 0
    if not from_grid:
        nbytes = int(lib.bullseye_predict_ws_bytes(ctypes.byref(st)))
        ws = torch.empty(nbytes + 256, dtype=torch.uint8, device=model.device)
        ws_ptr = ctypes.c_void_p((ws.data_ptr() + 255) // 256 * 256)
    tx = ty = None
    if taper is not None:
        tx = ctypes.c_void_p(taper[0].data_ptr())
        ty = ctypes.c_void_p(taper[1].data_ptr())
    flags = (1 if normalise else 0) | (2 if from_grid else 0)
    rc = lib.bullseye_predict(ctypes.byref(st), ctypes.c_void_p(model.data_ptr()), tx, ty, 1 if faceting else 0, flags,
                              ctypes.c_void_p(out.data_ptr()), ws_ptr, nbytes, _stream())
    if rc != 0:
        check(lib)
        raise ImagingError(f"bullseye_predict failed with status {rc}")
    if ws is not None:
        torch.cuda.current_stream().synchronize()  # the workspace is released on return
    return out
