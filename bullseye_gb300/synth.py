"""Seeded synthetic interferometer data for the imaging workloads.

The reference images Measurement Sets read through casacore (bullseye/data/data_set_loader.py),
which is not available here; the benchmark workloads are therefore generated: antenna layouts,
Earth-rotation uvw tracks, point-source visibilities with noise, per-antenna 2x2 gains and facet
centres, all from numpy ``default_rng`` seeds.  Rows are in Measurement-Set order (time-major,
then baseline), antenna pairs cross-correlations only, so the ABI's baseline slots include empty
autocorrelations (bullseye/data/data_set_loader.py:89).

uvw follow the Earth-rotation relation used by the reference's benchmark generator
(bullseye/mo/benchmarks/benchmark.cpp:192-202): for baseline vector (Lx, Ly, Lz) in the local
equatorial frame, hour angle H and declination d,
    u = -sin H Lx + cos H Ly
    v = -sin d cos H Lx - sin d sin H Ly + cos d Lz
    w =  cos d cos H Lx + cos d sin H Ly + sin d Lz
"""
from __future__ import annotations

import numpy as np

from .filters import aa_kernel, pswf_kernel, wproj_kernels
from .imaging import GriddingProblem

C_LIGHT = 299792458.0
ARCSEC = np.pi / (180.0 * 3600.0)


def disc_layout(n: int, diameter_m: float, seed: int) -> np.ndarray:
    """``n`` antennas uniform in a disc, local (east, north, up) metres."""
    rng = np.random.default_rng(seed)
    r = 0.5 * diameter_m * np.sqrt(rng.uniform(0, 1, n))
    th = rng.uniform(0, 2 * np.pi, n)
    return np.stack([r * np.cos(th), r * np.sin(th), np.zeros(n)], axis=1)


def y_layout(n: int, arm_m: float, seed: int) -> np.ndarray:
    """``n`` antennas on a three-armed (Y) array with power-law spacing along each arm."""
    rng = np.random.default_rng(seed)
    per_arm = int(np.ceil(n / 3))
    pos = []
    for a in range(3):
        ang = np.deg2rad(5.0 + 120.0 * a)
        d = arm_m * (np.arange(1, per_arm + 1) / per_arm) ** 1.716
        d = d * (1 + rng.normal(0, 0.02, per_arm))
        for di in d:
            pos.append((di * np.sin(ang), di * np.cos(ang), 0.0))
    return np.asarray(pos[:n])


# Geocentric (ITRF) positions in metres of the 27 EVLA antennas that the reference's benchmark
# simulates (bullseye/mo/benchmarks/benchmark.cpp:68-95, taken there from a measurement set of an
# observation of G55.7+3.4).  The same numbers, so that the multi-facet workload grids the
# reference benchmark's uv coverage.
EVLA27_ITRF = np.array([
    [-1601710.017000, -5042006.925200, 3554602.355600], [-1601150.060300, -5042000.619800, 3554860.729400],
    [-1600715.950800, -5042273.187000, 3554668.184500], [-1601189.030140, -5042000.493300, 3554843.425700],
    [-1601614.091000, -5042001.652900, 3554652.509300], [-1601162.591000, -5041828.999000, 3555095.896400],
    [-1601014.462000, -5042086.252000, 3554800.799800], [-1601185.634945, -5041978.156586, 3554876.424700],
    [-1600951.588000, -5042125.911000, 3554773.012300], [-1601177.376760, -5041925.073200, 3554954.584100],
    [-1601068.790300, -5042051.910200, 3554824.835300], [-1600801.926000, -5042219.366500, 3554706.448200],
    [-1601155.635800, -5041783.843800, 3555162.374100], [-1601447.198000, -5041992.502500, 3554739.687600],
    [-1601225.255200, -5041980.383590, 3554855.675000], [-1601526.387300, -5041996.840100, 3554698.327400],
    [-1601139.485100, -5041679.036800, 3555316.533200], [-1601315.893000, -5041985.320170, 3554808.304600],
    [-1601168.786100, -5041869.054000, 3555036.936000], [-1601192.467800, -5042022.856800, 3554810.438800],
    [-1601173.979400, -5041902.657700, 3554987.517500], [-1600880.571400, -5042170.388000, 3554741.457400],
    [-1601377.009500, -5041988.665500, 3554776.393400], [-1601180.861480, -5041947.453400, 3554921.628700],
    [-1601265.153600, -5041982.533050, 3554834.858400], [-1601114.365500, -5042023.151800, 3554844.944000],
    [-1601147.940400, -5041733.837000, 3555235.956000],
])


def evla27_equatorial() -> np.ndarray:
    """The EVLA-27 positions in the local equatorial frame of the array (X towards the local meridian
    at H = 0, Y east, Z pole): the geocentric positions rotated about the pole by the array's
    longitude, centred on the array."""
    xyz = EVLA27_ITRF - EVLA27_ITRF.mean(axis=0)
    lon = np.arctan2(EVLA27_ITRF[:, 1].mean(), EVLA27_ITRF[:, 0].mean())
    c, s_ = np.cos(lon), np.sin(lon)
    return np.stack([c * xyz[:, 0] + s_ * xyz[:, 1], -s_ * xyz[:, 0] + c * xyz[:, 1], xyz[:, 2]], axis=1)


def enu_to_equatorial(enu: np.ndarray, lat_rad: float) -> np.ndarray:
    """Local (east, north, up) to the local equatorial frame (X towards H = 0, Y east, Z pole)."""
    e, nn, u = enu[:, 0], enu[:, 1], enu[:, 2]
    X = -np.sin(lat_rad) * nn + np.cos(lat_rad) * u
    Y = e
    Z = np.cos(lat_rad) * nn + np.sin(lat_rad) * u
    return np.stack([X, Y, Z], axis=1)


def earth_rotation_rows(xyz: np.ndarray, n_times: int, dec_rad: float, ha_span_rad: float):
    """uvw [R, 3] metres plus antenna1/antenna2/time ids for time-major rows of cross baselines."""
    n = xyz.shape[0]
    a1, a2 = np.triu_indices(n, k=1)
    nb = a1.size
    H = (np.arange(n_times) - (n_times - 1) / 2.0) * (ha_span_rad / max(1, n_times - 1))
    L = xyz[a1] - xyz[a2]  # [nb, 3]
    sH, cH = np.sin(H)[:, None], np.cos(H)[:, None]
    sd, cd = np.sin(dec_rad), np.cos(dec_rad)
    Lx, Ly, Lz = L[None, :, 0], L[None, :, 1], L[None, :, 2]
    u = -sH * Lx + cH * Ly
    v = -sd * cH * Lx - sd * sH * Ly + cd * Lz
    w = cd * cH * Lx + cd * sH * Ly + sd * Lz
    uvw = np.stack([u, v, w], axis=-1).reshape(n_times * nb, 3)
    ant1 = np.tile(a1, n_times).astype(np.uint32)
    ant2 = np.tile(a2, n_times).astype(np.uint32)
    tid = np.repeat(np.arange(n_times), nb).astype(np.uintp)
    return uvw, ant1, ant2, tid


def point_source_vis(uvw_m: np.ndarray, wavelengths: np.ndarray, l: np.ndarray, m: np.ndarray,
                     flux: np.ndarray, chunk: int = 1 << 16) -> np.ndarray:
    """Sum of point sources, V = sum_s S_s exp(-2 pi i (u l + v m + w (n - 1))), complex128 [R, Ch]."""
    R = uvw_m.shape[0]
    lam = np.asarray(wavelengths).reshape(-1)
    n = np.sqrt(1.0 - l ** 2 - m ** 2)
    out = np.zeros((R, lam.size), dtype=np.complex128)
    for lo in range(0, R, chunk):
        hi = min(R, lo + chunk)
        ph = (uvw_m[lo:hi, 0:1] * l[None, :] + uvw_m[lo:hi, 1:2] * m[None, :] +
              uvw_m[lo:hi, 2:3] * (n[None, :] - 1.0))  # [r, s] metres
        for ci, lm_ in enumerate(lam):
            out[lo:hi, ci] = np.exp(-2j * np.pi * ph / lm_) @ flux
    return out


def _problem(precision, uvw, a1, a2, tid, n_ant, n_times, freqs, vis_c, seed, *, nx, ny, cell,
             conv, s, os, wplanes=1, wmax=1.0, phase_centre=(0.0, 0.0), facet_centres=None,
             jones=None, noise=0.01, flag_fraction=0.0):
    rng = np.random.default_rng(seed + 101)
    R, Ch = vis_c.shape
    vis = np.zeros((R, Ch, 4), dtype=np.complex128)
    nz = lambda: (rng.normal(0, noise, (R, Ch)) + 1j * rng.normal(0, noise, (R, Ch)))
    vis[:, :, 0] = vis_c + nz()
    vis[:, :, 1] = nz()
    vis[:, :, 2] = nz()
    vis[:, :, 3] = vis_c + nz()
    weights = np.ones((R, Ch, 4))
    flags = np.zeros((R, Ch, 4), dtype=bool)
    if flag_fraction > 0:
        flags |= rng.uniform(0, 1, (R, Ch, 1)) < flag_fraction
    lam = (C_LIGHT / np.asarray(freqs)).reshape(1, -1)
    return GriddingProblem(
        precision="double", vis=vis, uvw=uvw, wavelengths=lam, weights=weights, flags=flags,
        flagged_rows=np.zeros(R, bool), field_ids=np.zeros(R, np.uint32), spw_ids=np.zeros(R, np.uint32),
        antenna1=a1, antenna2=a2, timestamp_ids=tid, n_antennas=n_ant, n_timestamps=n_times,
        nx=nx, ny=ny, cell_x=cell, cell_y=cell, conv=conv, conv_support=s, conv_oversample=os,
        wplanes=wplanes, wmax=wmax, phase_centre=phase_centre, facet_centres=facet_centres, jones=jones,
        channel_grid_index=np.zeros(Ch, np.uintp), sampling_channel_grid_index=np.zeros(Ch, np.uintp),
    ).astype(precision)


def random_gains(n_times: int, n_ant: int, n_dir: int, n_chan: int, seed: int,
                 amp_sigma: float = 0.1, leak: float = 0.05) -> np.ndarray:
    """Per (time, antenna, direction, spw=1, channel) 2x2 complex gains, complex128 [T, A, F, 1, Ch, 4].

    Diagonal: amplitude 1 +- amp_sigma (uniform) with a uniformly random phase; off-diagonal:
    small complex leakage of scale ``leak``.
    """
    rng = np.random.default_rng(seed)
    shape = (n_times, n_ant, n_dir, 1, n_chan)
    g = np.zeros(shape + (4,), dtype=np.complex128)
    for k in (0, 3):
        amp = 1.0 + rng.uniform(-amp_sigma, amp_sigma, shape)
        g[..., k] = amp * np.exp(1j * rng.uniform(-np.pi, np.pi, shape))
    for k in (1, 2):
        g[..., k] = leak * (rng.normal(0, 1, shape) + 1j * rng.normal(0, 1, shape)) / np.sqrt(2)
    return g


def config1(precision="single", *, n_ant=64, n_times=120, nx=1024, cell=2.0, s=3, os=63,
            kernel="pswf", seed=1, noise=0.01) -> GriddingProblem:
    """Plain single-facet gridding: 64 antennas on a seeded 2 km disc, 120 timesteps at dec
    -30 deg, 1 channel at 1.4 GHz, 3 point sources (0.1-2 Jy) + N(0, 0.01) noise, 1024^2 grid,
    2 arcsec cells, AA kernel W = 7, os = 63, no w-projection, natural weighting."""
    dec = np.deg2rad(-30.0)
    enu = disc_layout(n_ant, 2000.0, seed)
    xyz = enu_to_equatorial(enu, np.deg2rad(-30.0))
    uvw, a1, a2, tid = earth_rotation_rows(xyz, n_times, dec, np.deg2rad(90.0))
    freqs = np.array([1.4e9])
    rng = np.random.default_rng(seed + 7)
    fov = nx * cell * ARCSEC
    ls = rng.uniform(-0.3, 0.3, 3) * fov
    ms = rng.uniform(-0.3, 0.3, 3) * fov
    flux = rng.uniform(0.1, 2.0, 3)
    vis_c = point_source_vis(uvw, C_LIGHT / freqs, ls, ms, flux)
    conv = pswf_kernel(s, os) if kernel == "pswf" else aa_kernel(s, os, kernel)
    return _problem(precision, uvw, a1, a2, tid, n_ant, n_times, freqs, vis_c, seed, nx=nx, ny=nx,
                    cell=cell, conv=conv, s=s, os=os, phase_centre=(0.0, dec / ARCSEC), noise=noise)


def config2(precision="single", *, n_ant=27, n_times=2000, n_chan=64, n_facets=16, nx=1024,
            cell=10.0, wplanes=64, s=31, min_support=15, os=63, n_src=50, seed=2,
            jones=True, vis_chunk=1 << 14) -> GriddingProblem:
    """Multi-facet with phase rotation and Jones: 27 antennas (the reference benchmark's EVLA
    positions, or a Y layout for other counts), 2000 timesteps, 64 channels 1.0-1.5 GHz, 50
    sources, per-antenna/time gains, 16 facets of 1024^2 within 3 deg, w-projection with 64 planes
    and supports 15..63 (padded to 63 in the ABI table)."""
    dec = np.deg2rad(-30.0)
    xyz = evla27_equatorial() if n_ant == 27 else enu_to_equatorial(y_layout(n_ant, 600.0, seed), np.deg2rad(34.0))
    uvw, a1, a2, tid = earth_rotation_rows(xyz, n_times, dec, np.deg2rad(120.0))
    freqs = np.linspace(1.0e9, 1.5e9, n_chan)
    rng = np.random.default_rng(seed + 7)
    lim = np.deg2rad(3.0)
    ls = rng.uniform(-lim, lim, n_src)
    ms = rng.uniform(-lim, lim, n_src)
    flux = rng.uniform(0.1, 2.0, n_src)
    vis_c = point_source_vis(uvw, C_LIGHT / freqs, ls, ms, flux, chunk=vis_chunk)
    fl = rng.uniform(-lim, lim, n_facets)
    fm = rng.uniform(-lim, lim, n_facets)
    dec0 = dec / ARCSEC
    facet_centres = np.stack([fl / np.cos(dec) / ARCSEC, dec0 + fm / ARCSEC], axis=1)
    maxb = np.max(np.linalg.norm(uvw, axis=1))
    wmax = maxb / (C_LIGHT / freqs.max())
    fov = nx * cell * ARCSEC
    stack, _ = wproj_kernels(s, os, wplanes, wmax, fov, min_support=min_support)
    g = random_gains(n_times, n_ant, n_facets, n_chan, seed + 11) if jones else None
    return _problem(precision, uvw, a1, a2, tid, n_ant, n_times, freqs, vis_c, seed, nx=nx, ny=nx,
                    cell=cell, conv=stack, s=s, os=os, wplanes=wplanes, wmax=wmax,
                    phase_centre=(0.0, dec0), facet_centres=facet_centres, jones=g)


def config3(precision="single", *, n_ant=64, n_times=120, nx=4096, cell=0.25, s=3, os=63,
            diameter_m=80000.0, facet_offsets_deg=(0.0, 0.5, 1.0, 2.0), seed=1, noise=0.01) -> GriddingProblem:
    """Precision form: the config-1 observation (64 antennas, 120 timesteps at dec -30 deg, 1 channel
    at 1.4 GHz, 3 point sources + noise, PSWF W = 7, os = 63) on an 80 km disc, imaged on 4096^2
    facets of 0.25 arcsec cells (3.7e5 lambda baselines, all on the grid).  Facets sit at the phase
    centre and at the given offsets in l (the phase-rotation argument grows with the offset)."""
    dec = np.deg2rad(-30.0)
    enu = disc_layout(n_ant, diameter_m, seed)
    xyz = enu_to_equatorial(enu, np.deg2rad(-30.0))
    uvw, a1, a2, tid = earth_rotation_rows(xyz, n_times, dec, np.deg2rad(90.0))
    freqs = np.array([1.4e9])
    rng = np.random.default_rng(seed + 7)
    fov = nx * cell * ARCSEC
    ls = rng.uniform(-0.3, 0.3, 3) * fov
    ms = rng.uniform(-0.3, 0.3, 3) * fov
    flux = rng.uniform(0.1, 2.0, 3)
    vis_c = point_source_vis(uvw, C_LIGHT / freqs, ls, ms, flux)
    conv = pswf_kernel(s, os)
    dec0 = dec / ARCSEC
    off = np.deg2rad(np.asarray(facet_offsets_deg, dtype=np.float64))
    facet_centres = np.stack([off / np.cos(dec) / ARCSEC, np.full(off.shape, dec0)], axis=1)
    return _problem(precision, uvw, a1, a2, tid, n_ant, n_times, freqs, vis_c, seed, nx=nx, ny=nx, cell=cell,
                    conv=conv, s=s, os=os, phase_centre=(0.0, dec0), facet_centres=facet_centres, noise=noise)


def small_problem(precision="double", *, n_ant=8, n_times=12, n_chan=3, nx=96, ny=None, cell=60.0,
                  s=3, os=15, wplanes=1, n_facets=0, jones=False, seed=5, flag_fraction=0.1,
                  kernel="pswf", min_support=None, n_spw=1) -> GriddingProblem:
    """A seconds-sized problem exercising every code path (parity tests)."""
    ny = ny or nx
    dec = np.deg2rad(-40.0)
    enu = disc_layout(n_ant, 1500.0, seed)
    xyz = enu_to_equatorial(enu, np.deg2rad(-30.0))
    uvw, a1, a2, tid = earth_rotation_rows(xyz, n_times, dec, np.deg2rad(60.0))
    freqs = np.linspace(1.2e9, 1.5e9, n_chan)
    rng = np.random.default_rng(seed + 7)
    fov = nx * cell * ARCSEC
    ls = rng.uniform(-0.3, 0.3, 4) * fov
    ms = rng.uniform(-0.3, 0.3, 4) * fov
    vis_c = point_source_vis(uvw, C_LIGHT / freqs, ls, ms, rng.uniform(0.1, 2.0, 4))
    fc = None
    dec0 = dec / ARCSEC
    if n_facets:
        fl = rng.uniform(-0.4, 0.4, n_facets) * fov
        fm = rng.uniform(-0.4, 0.4, n_facets) * fov
        fc = np.stack([fl / np.cos(dec) / ARCSEC, dec0 + fm / ARCSEC], axis=1)
    if wplanes > 1:
        maxb = np.max(np.linalg.norm(uvw, axis=1))
        wmax = maxb / (C_LIGHT / freqs.max()) * 1.01
        conv, _ = wproj_kernels(s, os, wplanes, wmax, fov, min_support=min_support)
    else:
        wmax = 1.0
        conv = pswf_kernel(s, os) if kernel == "pswf" else aa_kernel(s, os, kernel)
    g = random_gains(n_times, n_ant, max(1, n_facets), n_chan, seed + 11) if jones else None
    p = _problem("double", uvw, a1, a2, tid, n_ant, n_times, freqs, vis_c, seed, nx=nx, ny=ny, cell=cell,
                 conv=conv, s=s, os=os, wplanes=wplanes, wmax=wmax, phase_centre=(0.0, dec0),
                 facet_centres=fc, jones=g, flag_fraction=flag_fraction)
    rng2 = np.random.default_rng(seed + 13)
    p.weights = rng2.uniform(0.5, 1.5, p.weights.shape)
    p.flagged_rows = rng2.uniform(0, 1, p.rows) < 0.05
    return p.astype(precision)
