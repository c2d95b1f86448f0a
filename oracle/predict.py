"""Restatement of prediction (degridding as a forward operator) in FP64 numpy.  TEST INFRASTRUCTURE ONLY.

Only tests import this module: it is the checker of the library's bullseye_predict.  The reference
has no prediction in its imaging library; what it does have is pinned here piece by piece:

* the cell, tap, w-plane, phase and uv-transform choice of the reference's CPU gridder, which a
  degridder must read back from the same footprint: the AA policy rounds the footprint corner and
  the tap offset down (bullseye/mo/cpu_algorithm/convolution_policies.h:70-118, under FE_DOWNWARD),
  the w-projection policy rounds half to even, takes plane rint(|w| (P - 1) / (float) wmax) and
  grids the conjugate at (-u, -v) for w < 0 (convolution_policies.h:231-289); a footprint is
  accepted when corner >= 0 and corner + W + 2 < n; the phase offsets and the planar uv transform
  follow bullseye/mo/cpu_gpu_common/phase_transform_policies.h:110-134 and
  baseline_transform_policies.h:117-149 (uvw in wavelengths, u -= w l0/n0, v -= w m0/n0, then
  scaled by nx cell and -(ny cell) in radians);
* the degridded value of the reference's prototype degridder
  (writing_and_wiki/notebooks/Resampling.ipynb cell 17): the sum of grid x tap over the footprint,
  divided by the sum of the taps in the normalised form.  tests/test_predict_oracle.py pins this
  restatement to the notebook's own output (tests/golden/notebook_degrid.npz);
* the model image to model grid step as the inverse of the reference's finalize
  (bullseye/mo/cpu_gpu_common/fft_and_repacking_routines.cpp:83-118: ifftshift, backward transform,
  fftshift): grid = fftshift(fft2(ifftshift(image / taper))), unnormalised.

The forward model per (row, channel): V = sum over facets of J_p (e^{-i phi_f} D_f') J_q^H with
D_f = sum grid_f conj(tap) [/ Re sum tap] and D_f' = D_f, or conj(D_f) for w < 0.
"""
from __future__ import annotations

import numpy as np

ARCSEC_F32 = float(np.float32(np.pi / (180.0 * 3600.0)))  # the reference's float ARCSEC_TO_RAD


def model_grids(images: np.ndarray, taper_x=None, taper_y=None) -> np.ndarray:
    """[..., ny, nx] model images -> uv grids (divided by the taper, unnormalised forward transform
    with numpy's shifts)."""
    img = np.asarray(images, np.complex128)
    if taper_x is not None:
        img = img / (np.asarray(taper_y, np.float64)[:, None] * np.asarray(taper_x, np.float64)[None, :])
    return np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(img, axes=(-2, -1))), axes=(-2, -1))


def facet_constants(ra0, dec0, ra, dec):
    """(u_term, v_term, dl, dm, dn) of a facet centred at (ra, dec) arcsec for phase centre
    (ra0, dec0) (phase_transform_policies.h:110-134, baseline_transform_policies.h:117-149)."""
    d_ra = (ra - ra0) * ARCSEC_F32
    n_dec, o_dec = dec * ARCSEC_F32, dec0 * ARCSEC_F32
    c_d_ra, s_d_ra = np.cos(d_ra), np.sin(d_ra)
    c_n, s_n, c_o, s_o = np.cos(n_dec), np.sin(n_dec), np.cos(o_dec), np.sin(o_dec)
    li0, mi0, ni0 = c_n * s_d_ra, s_n * c_o - c_n * s_o * c_d_ra, s_n * s_o + c_n * c_o * c_d_ra
    dl, dm = -c_n * s_d_ra, -(s_n * c_o - c_n * s_o * c_d_ra)
    return li0 / ni0, mi0 / ni0, dl, dm, 1.0 - np.sqrt(1.0 - dl * dl - dm * dm)


def predict(p, grids: np.ndarray, *, faceting: bool, normalise: bool) -> np.ndarray:
    """Visibilities [R][Ch][4] (complex128) predicted from model grids [F][cube][4][ny][nx] of
    GriddingProblem ``p`` (its conv is the 1-D AA table or the separable [P][K] w stack)."""
    R, Ch, S = p.rows, p.channels, p.spws
    F = max(1, p.n_facets)
    W, os_ = 2 * p.conv_support + 1, p.conv_oversample
    wproj = p.wplanes > 1
    conv = np.asarray(p.conv, np.complex128).reshape(-1 if wproj else 1, np.asarray(p.conv).shape[-1])
    K = conv.shape[1]
    u_scale = p.nx * float(p.cell_x) * ARCSEC_F32
    v_scale = -(p.ny * float(p.cell_y) * ARCSEC_F32)
    gcx, gcy = float(p.nx // 2 - p.conv_support), float(p.ny // 2 - p.conv_support)
    wmax = float(np.float32(p.wmax))
    plane_scale = (p.wplanes - 1) / wmax if wproj else 0.0
    enabled = np.ones(S * Ch, bool) if p.enabled_channels is None else np.asarray(p.enabled_channels, bool)
    cgi = np.zeros(S * Ch, np.int64) if p.channel_grid_index is None else np.asarray(p.channel_grid_index, np.int64)
    uvw = np.asarray(p.uvw, np.float64)
    spw = np.asarray(p.spw_ids, np.int64)
    out = np.zeros((R, Ch, 4), np.complex128)
    ra0, dec0 = (float(x) for x in p.phase_centre)
    jones = None if p.jones is None else np.asarray(p.jones, np.complex128)
    jw = np.arange(W)
    for f in range(F):
        if faceting and p.facet_centres is not None:
            ut, vt, dl, dm, dn = facet_constants(ra0, dec0, float(p.facet_centres[f, 0]), float(p.facet_centres[f, 1]))
        else:
            ut = vt = dl = dm = dn = 0.0
        for c in range(Ch):
            sc = spw * Ch + c
            g = cgi[sc]
            live = enabled[sc] & (g < p.cube)
            inv = 1.0 / np.asarray(p.wavelengths, np.float64).reshape(-1)[sc]
            u, v, w = uvw[:, 0] * inv, uvw[:, 1] * inv, uvw[:, 2] * inv
            ph = np.exp(1j * (2 * np.pi * (u * dl + v * dm + w * dn))) if faceting else np.ones(R, np.complex128)
            if faceting:
                u, v = u - w * ut, v - w * vt
            u, v = u * u_scale, v * v_scale
            flip = wproj & (w < 0)
            u, v, w = np.where(flip, -u, u), np.where(flip, -v, v), np.where(flip, -w, w)
            rnd = np.rint if wproj else np.floor
            ru, rv = rnd(u), rnd(v)
            du, dv = rnd(u + gcx), rnd(v + gcy)
            plane = np.rint(np.abs(w) * plane_scale) if wproj else np.zeros(R)
            ok = live & (du >= 0) & (dv >= 0) & (du + W + 2 < p.nx) & (dv + W + 2 < p.ny) & (plane >= 0) & \
                (plane < max(1, p.wplanes))
            idx = np.nonzero(ok)[0]
            if idx.size == 0:
                continue
            fu = ((1.0 - u[idx] + ru[idx]) * os_).astype(np.int64)
            fv = ((1.0 - v[idx] + rv[idx]) * os_).astype(np.int64)
            pl = plane[idx].astype(np.int64)
            iu = fu[:, None] + jw[None, :] * os_
            iv = fv[:, None] + jw[None, :] * os_
            tu = np.where(iu < K, conv[pl[:, None], np.minimum(iu, K - 1)], 0)
            tv = np.where(iv < K, conv[pl[:, None], np.minimum(iv, K - 1)], 0)
            tap = tv[:, :, None] * tu[:, None, :]  # [n][y][x]
            ys = dv[idx].astype(np.int64)[:, None] + jw[None, :]
            xs = du[idx].astype(np.int64)[:, None] + jw[None, :]
            X = np.zeros((idx.size, 4), np.complex128)
            for k in range(4):
                G = np.asarray(grids[f], np.complex128)[g[idx], k]  # [n][ny][nx]
                patch = G[np.arange(idx.size)[:, None, None], ys[:, :, None], xs[:, None, :]]
                X[:, k] = np.sum(patch * np.conj(tap), axis=(1, 2))
            if normalise:
                ts = np.sum(tap.real, axis=(1, 2))
                X = X / np.where(ts != 0, ts, 1.0)[:, None]
            X = np.where(flip[idx][:, None], np.conj(X), X) * np.conj(ph[idx])[:, None]
            if jones is not None:
                t = np.asarray(p.timestamp_ids, np.int64)[idx]
                a1 = np.asarray(p.antenna1, np.int64)[idx]
                a2 = np.asarray(p.antenna2, np.int64)[idx]
                Jp = jones[t, a1, f, spw[idx], c].reshape(-1, 2, 2)
                Jq = jones[t, a2, f, spw[idx], c].reshape(-1, 2, 2)
                M = X.reshape(-1, 2, 2)
                X = (Jp @ M @ np.conj(np.transpose(Jq, (0, 2, 1)))).reshape(-1, 4)
            out[idx, c] += X
    return out
