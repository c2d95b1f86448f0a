"""Footprint geometry of the gridder in numpy FP64, for reporting (which visibilities land off a
facet's grid).

The library computes the same geometry on the device for every (row, channel, facet): the facet's
planar uv transform (u -= w l0/n0, v -= w m0/n0 with l0, m0, n0 of the facet centre,
bullseye/mo/cpu_gpu_common/baseline_transform_policies.h:117-149, phase_transform_policies.h:110-134),
the scale to pixels (nx x cell and -(ny x cell) in radians, templated_gridder.h:23-24), the footprint
corner floor(u) + nx/2 - s (AA, convolution_policies.h:70-118) or rint(u) + nx/2 - s (w-projection,
:231-289), and the acceptance test corner >= 0 and corner + W + 2 < n.  The reference drops the
visibilities that fail it without a count; `offgrid_pairs` counts them.
"""
from __future__ import annotations

import numpy as np

ARCSEC_F32 = float(np.float32(np.pi / (180.0 * 3600.0)))  # the library's float ARCSEC_TO_RAD


def facet_uv_terms(ra0: float, dec0: float, ra: float, dec: float) -> tuple[float, float]:
    """(l0 / n0, m0 / n0) of a facet centred at (ra, dec) arcsec for phase centre (ra0, dec0)."""
    d_ra = (ra - ra0) * ARCSEC_F32
    n_dec, o_dec = dec * ARCSEC_F32, dec0 * ARCSEC_F32
    li0 = np.cos(n_dec) * np.sin(d_ra)
    mi0 = np.sin(n_dec) * np.cos(o_dec) - np.cos(n_dec) * np.sin(o_dec) * np.cos(d_ra)
    ni0 = np.sin(n_dec) * np.sin(o_dec) + np.cos(n_dec) * np.cos(o_dec) * np.cos(d_ra)
    return float(li0 / ni0), float(mi0 / ni0)


def offgrid_pairs(p, faceting: bool = True) -> np.ndarray:
    """Per facet, the (row, channel) samples of problem ``p`` whose footprint leaves the facet's grid
    (counted whether flagged or not: the gridder visits flagged samples with zero weight)."""
    F = max(1, p.n_facets)
    W = 2 * p.conv_support + 1
    wproj = p.wplanes > 1
    u_scale = p.nx * float(p.cell_x) * ARCSEC_F32
    v_scale = -(p.ny * float(p.cell_y) * ARCSEC_F32)
    gcx, gcy = p.nx // 2 - p.conv_support, p.ny // 2 - p.conv_support
    uvw = np.asarray(p.uvw, np.float64)
    lam = np.asarray(p.wavelengths, np.float64).reshape(-1)
    spw = np.asarray(p.spw_ids, np.int64)
    ra0, dec0 = (float(x) for x in p.phase_centre)
    out = np.zeros(F, np.int64)
    for f in range(F):
        ut = vt = 0.0
        if faceting and p.facet_centres is not None:
            ut, vt = facet_uv_terms(ra0, dec0, float(p.facet_centres[f, 0]), float(p.facet_centres[f, 1]))
        for c in range(p.channels):
            inv = 1.0 / lam[spw * p.channels + c]
            u, v, w = uvw[:, 0] * inv, uvw[:, 1] * inv, uvw[:, 2] * inv
            if faceting:
                u, v = u - w * ut, v - w * vt
            u, v = u * u_scale, v * v_scale
            if wproj:
                flip = w < 0
                u, v = np.where(flip, -u, u), np.where(flip, -v, v)
            rnd = np.rint if wproj else np.floor
            du, dv = rnd(u) + gcx, rnd(v) + gcy
            ok = (du >= 0) & (dv >= 0) & (du + W + 2 < p.nx) & (dv + W + 2 < p.ny)
            if wproj:  # the w plane rint(|w| (P - 1) / wmax) must exist
                plane = np.rint(np.abs(w) * ((p.wplanes - 1) / float(np.float32(p.wmax))))
                ok &= plane < p.wplanes
            out[f] += int(np.count_nonzero(~ok))
    return out
