#!/usr/bin/env python3
"""Benchmark: gridded Mvis/s on one GB300 for the multi-facet Jones + w-projection workload.

Workload (one "step" = one pass of the facet-imaging hot path over the whole visibility set):
  27 antennas (351 baselines) at the EVLA positions of the reference's benchmark
  (bullseye/mo/benchmarks/benchmark.cpp:68-95), 2000 timesteps of Earth rotation, 64 channels
  1.0-1.5 GHz -> 702,000 rows x 64 channels = 44.93 M visibilities (4 correlations, complex64);
  50 seeded point sources + noise; seeded per-antenna, per-time, per-facet 2x2 gains; 16 facets
  of 1024^2 within 3 deg; w-projection with 64 planes, supports 15..63 (ABI table padded to 63,
  oversampling 15); uniform weighting, so each step grids the visibilities (facet_4_cor_corrections)
  and the sampling function (facet_sampling_function).  Throughput counts (visibility x facet)
  pairs that pass flags: 44.93 M x 16 = 718.8 M per step.

Lines printed (rank 0, one JSON line):
  value     Mvis/s with inputs resident in HBM (device pointers through the C-ABI), CUDA events
            on the library stream around each step;
  e2e       the same metric through the reference-facing C-ABI with host buffers: initLibrary,
            facet_4_cor_corrections + facet_sampling_function (pinned host inputs, final-chunk
            copy-back), weight_uniformly, normalize, finalize, releaseLibrary every step;
  roofline  the gridder kernel against the measured FP32 FMA rate of this GPU (the gridder is
            FP32-issue bound; HBM traffic is reported alongside);
  cpu_baseline  the oracle port of the reference CPU library (OpenMP over facets) on a bounded
            sample of rows, on this machine's host cores;
  precision the precision form: per-facet max / RMS relative dirty-image error of the FP32
            library (compensated and plain flushes) against the FP64 library, config 3 (80 km,
            4 facets of 4096^2).

With N ranks (torchrun) each rank grids its own 16 facets of a 16 N-facet field (facet sharding,
no collective on the data path); the step time is the max over ranks.

--impl reference prints the reference arm: the oracle port of the reference's CPU path, timed on
bounded row samples of the same workload, all host threads.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

N_ANT, N_TIMES, N_CHAN, N_FACETS, NX = 27, 2000, 64, 16, 1024
WPLANES, S_HALF, MIN_SUPPORT, OS = 64, 31, 15, 15
CELL = 5.0
N_SRC = 50
WORKLOAD = ("facet_4_cor_corrections+facet_sampling_function, 27 ant x 2000 t x 64 ch (44.93M vis, 4 corr), "
            "16 facets 1024^2, w-proj 64 planes support 15-63 (padded 63), os 15, Jones, uniform")


# DRAM traffic of one batched step (dram__bytes_read.sum + dram__bytes_write.sum, every launch of
# the step), captured with ncu on the 16-channel, 4-facet cut of this workload (11.20 GB for
# 44.93 M vis-facet pairs, visibility records included) and scaled by vis-facet pairs: an upper
# estimate for the full step, where 16 facets rather than 4 share each row's loads.
TRAFFIC_BYTES_PER_PAIR = 11.20e9 / 44928000
TRAFFIC_SOURCE = ("ncu dram bytes of one eager step of the 16-channel 4-facet case (11.20 GB / 44.93 M pairs, "
                  "visibility records written and read once), scaled by vis-facet pairs (upper estimate: more "
                  "facets share each row's loads)")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--time-frac", type=float, default=1.0, help="fraction of timesteps (quick runs)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-comp", action="store_true", help="plain (uncompensated) FP32 grid flushes")
    ap.add_argument("--chans", type=int, default=0, help="override the channel count (profiling cases)")
    ap.add_argument("--form", default="batched", choices=["batched", "plain"],
                    help="batched: bullseye_grid_batched; plain: the per-call drop-in ABI path")
    ap.add_argument("--no-other", action="store_true", help="skip timing the other form")
    ap.add_argument("--facets", type=int, default=0, help="override the facet count (profiling cases)")
    ap.add_argument("--no-precision", action="store_true", help="skip the per-facet FP32 error report")
    ap.add_argument("--adj-times", type=int, default=0, help="differentiation workload: override the timestep count")
    ap.add_argument("--workload", default="facets16", choices=["facets16", "uneven", "adjoint", "predict"],
                    help="facets16: the 16-facet Jones workload (default); uneven: 96 facets of uneven sizes and masks; "
                         "adjoint: the differentiation form at scale with a finite-difference check; "
                         "predict: degridding 16 facet model images back to the visibilities")
    ap.add_argument("--no-class-profile", action="store_true",
                    help="skip the eager, per-support-class timed step after the timed region")
    ap.add_argument("--eager", action="store_true",
                    help="batched form without graph replay (per-class launches with events; for profilers)")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the parity check of the batched FP32 path against the FP64 oracle on the row sample")
    ap.add_argument("--sample-baselines", type=int, default=0,
                    help="baselines (all their timesteps) in the CPU-baseline / parity row sample (0: sized by time)")
    ap.add_argument("--clocks-dir", default=None, help="also write the raw nvidia-smi clock samples into this folder")
    ap.add_argument("--grid-groups", type=int, default=1,
                    help="e2e: groups of row chunks gridded while later chunks upload (bullseye_set_grid_groups)")
    ap.add_argument("--no-records", action="store_true",
                    help="batched form: prepare every staged visibility in the class launches instead of by the "
                         "visibility-record kernel (bullseye_set_visibility_records(0))")
    ap.add_argument("--host-copy", type=int, default=1, choices=[0, 1],
                    help="e2e: 1 copies mapped page-locked host buffers with SM kernels, 0 with the copy engines "
                         "(bullseye_set_host_copy)")
    ap.add_argument("--reference-vs-port", action="store_true",
                    help="time the reference's own CPU build (oracle/_ref, where it is built) against the oracle "
                         "port on the same row sample, and exit (CPU only)")
    return ap.parse_args()


# ----------------------------------------------------------------------------- workload
def geometry(n_times, world=1, rank=0):
    """Rows, baseline order and facet centres.  With N ranks the field holds 16 N facets and each
    rank grids its own 16 (facet sharding, no collective on the data path)."""
    from bullseye_gb300 import synth
    from bullseye_gb300.sharding import facet_shard
    dec = np.deg2rad(-30.0)
    xyz = synth.evla27_equatorial()  # the reference benchmark's EVLA-27 positions
    uvw, a1, a2, tid = synth.earth_rotation_rows(xyz, n_times, dec, np.deg2rad(120.0))
    freqs = np.linspace(1.0e9, 1.5e9, N_CHAN)
    lam = synth.C_LIGHT / freqs
    rng = np.random.default_rng(9)
    lim = np.deg2rad(3.0)
    fl, fm = rng.uniform(-lim, lim, N_FACETS * world), rng.uniform(-lim, lim, N_FACETS * world)
    dec0 = dec / synth.ARCSEC
    facets = np.stack([fl / np.cos(dec) / synth.ARCSEC, dec0 + fm / synth.ARCSEC], axis=1)
    shard = facet_shard(N_FACETS * world, world, rank)
    facets = facets[shard.start:shard.stop]
    # baseline-major order (what repack_input_data produces), stable in time
    from bullseye_gb300.imaging import baseline_index
    b = baseline_index(a1, a2, N_ANT)
    order = np.argsort(b, kind="stable")
    nb = N_ANT * (N_ANT - 1) // 2 + N_ANT
    starts = np.zeros(nb + 1, dtype=np.uintp)
    np.add.at(starts, b + 1, 1)
    starts = np.cumsum(starts).astype(np.uintp)
    maxb = np.max(np.linalg.norm(uvw, axis=1))
    wmax = maxb / lam.min()
    return dict(uvw=uvw[order], a1=a1[order], a2=a2[order], tid=tid[order], lam=lam, facets=facets,
                starts=starts, dec0=dec0, wmax=wmax, n_times=n_times, nb=nb)


def kernel_stack(wmax):
    from bullseye_gb300.filters import wproj_kernels
    fov = NX * CELL * np.pi / (180 * 3600)
    stack, supports = wproj_kernels(S_HALF, OS, WPLANES, wmax, fov, min_support=MIN_SUPPORT)
    return stack.astype(np.complex64), supports


def plane_vis_counts(geo):
    """Visibilities per w plane over all channels (the gridder's plane rule)."""
    w = np.abs(geo["uvw"][:, 2])
    cnt = np.zeros(WPLANES, np.int64)
    for lam in geo["lam"]:
        pl = np.rint(w / lam * ((WPLANES - 1) / geo["wmax"])).astype(np.int64)
        cnt += np.bincount(np.clip(pl, 0, WPLANES - 1), minlength=WPLANES)
    return cnt


def class_taps(counts, plane_width):
    """Per support-class width: (visibilities, sum of W_class^2) over (row, channel), per facet."""
    out = {}
    for p, cw in enumerate(plane_width):
        vis, taps = out.get(int(cw), (0, 0.0))
        out[int(cw)] = (vis + int(counts[p]), taps + float(counts[p]) * float(cw) ** 2)
    return out


def batched_plane_widths(lib):
    arr = np.zeros(WPLANES, np.int32)
    n = lib.bullseye_batched_plane_classes(arr.ctypes.data_as(ctypes.c_void_p), WPLANES)
    return arr[:n] if n else None


def class_profile(lib, step, counts, plane_width):
    """One eager batched step with a CUDA event pair around each support-class launch."""
    lib.bullseye_set_batched_profiling(1)
    try:
        step()
    finally:
        lib.bullseye_set_batched_profiling(0)
    n = 128
    arrs = [np.zeros(n, np.int32) for _ in range(5)] + [np.zeros(n, np.float32)]
    cnt = lib.bullseye_batched_profile(*[a.ctypes.data_as(ctypes.c_void_p) for a in arrs], n)
    width, nc, J, wide, items, ms = arrs
    taps = class_taps(counts, plane_width)
    rows = []
    for i in range(min(cnt, n)):
        vis, t = taps.get(int(width[i]), (0, 0.0))
        flops = t * (N_FACETS * 8 * 4 if nc[i] == 4 else 8)
        if int(width[i]) == 0:  # the visibility-record kernel that precedes the build's class launches
            rows.append({"kernel": "record_kernel", "corr": int(nc[i]), "ms": float(ms[i])})
            continue
        rows.append({"width": int(width[i]), "corr": int(nc[i]), "J": int(J[i]), "wide": bool(wide[i] & 1),
                     "registers": int(wide[i]) >> 1,
                     "work_items": int(items[i]), "vis": vis, "ms": float(ms[i]),
                     "executed_tflops": flops / (float(ms[i]) * 1e-3) / 1e12 if ms[i] > 0 else None})
    return rows


def device_inputs(geo, torch):
    """Visibilities, weights, flags and gains generated on the GPU (float32 phases)."""
    dev = torch.device("cuda")
    R = geo["uvw"].shape[0]
    rng = np.random.default_rng(7)
    lim = np.deg2rad(3.0)
    l = torch.tensor(rng.uniform(-lim, lim, N_SRC), dtype=torch.float32, device=dev)
    m = torch.tensor(rng.uniform(-lim, lim, N_SRC), dtype=torch.float32, device=dev)
    flux = torch.tensor(rng.uniform(0.1, 2.0, N_SRC), dtype=torch.complex64, device=dev)
    nm1 = torch.sqrt(1 - l * l - m * m) - 1
    uvw = torch.tensor(geo["uvw"], dtype=torch.float32, device=dev)
    vis = torch.empty((R, N_CHAN, 4), dtype=torch.complex64, device=dev)
    gen = torch.Generator(device=dev)
    gen.manual_seed(11)
    step = 1 << 15
    for ci, lam in enumerate(geo["lam"]):
        for lo in range(0, R, step):
            hi = min(R, lo + step)
            u, v, w = uvw[lo:hi, 0:1], uvw[lo:hi, 1:2], uvw[lo:hi, 2:3]
            ph = (u * l + v * m + w * nm1) * (-2 * np.pi / lam)
            s = torch.polar(torch.ones_like(ph), ph) @ flux
            vis[lo:hi, ci, 0] = s
            vis[lo:hi, ci, 3] = s
            vis[lo:hi, ci, 1] = 0
            vis[lo:hi, ci, 2] = 0
    vis += (torch.randn(vis.shape, dtype=torch.complex64, device=dev, generator=gen) * 0.01)
    weights = torch.ones((R, N_CHAN, 4), dtype=torch.float32, device=dev)
    flags = torch.zeros((R, N_CHAN, 4), dtype=torch.uint8, device=dev)
    T = geo["n_times"]
    shape = (T, N_ANT, N_FACETS, 1, N_CHAN)
    jones = torch.zeros(shape + (4,), dtype=torch.complex64, device=dev)
    for k in (0, 3):
        amp = 1 + (torch.rand(shape, device=dev, generator=gen) * 0.2 - 0.1)
        phase = (torch.rand(shape, device=dev, generator=gen) * 2 - 1) * np.pi
        jones[..., k] = torch.polar(amp, phase)
    for k in (1, 2):
        jones[..., k] = 0.05 * torch.randn(shape, dtype=torch.complex64, device=dev, generator=gen)
    return dict(
        vis=vis, weights=weights, flags=flags, uvw=uvw, jones=jones,
        flagged_rows=torch.zeros(R, dtype=torch.uint8, device=dev),
        field=torch.zeros(R, dtype=torch.int32, device=dev),
        spw=torch.zeros(R, dtype=torch.int32, device=dev),
        a1=torch.tensor(geo["a1"].astype(np.int32), device=dev),
        a2=torch.tensor(geo["a2"].astype(np.int32), device=dev),
        tid=torch.tensor(geo["tid"].astype(np.int64), device=dev),
        starts=torch.tensor(geo["starts"].astype(np.int64), device=dev),
    )


class Tables:
    """Host-side tables and output buffers handed to initLibrary (kept alive by this object)."""

    def __init__(self, geo, conv):
        self.conv = np.ascontiguousarray(conv)
        self.lam = geo["lam"].astype(np.float32).reshape(1, -1)
        self.enabled = np.ones(N_CHAN, dtype=np.bool_)
        self.cgi = np.zeros(N_CHAN, dtype=np.uintp)
        self.sfcgi = np.zeros(N_CHAN, dtype=np.uintp)
        self.facets = geo["facets"].astype(np.float32)
        self.grid = np.zeros((N_FACETS, 1, 4, NX, NX), dtype=np.complex64)
        self.sf = np.zeros((N_FACETS, 1, 1, NX, NX), dtype=np.complex64)

    def fill(self, st, geo, rows):
        P = ctypes.c_void_p
        st.chunk_max_row_count = rows
        st.nx = st.ny = NX
        st.cell_size_x = st.cell_size_y = CELL
        st.conv = self.conv.ctypes.data_as(P)
        st.conv_support = S_HALF
        st.conv_oversample = OS
        st.phase_centre_ra = 0.0
        st.phase_centre_dec = geo["dec0"]
        st.should_invert_jones_terms = True
        st.imaging_field = 0
        st.channel_grid_indicies = self.cgi.ctypes.data_as(P)
        st.cube_channel_dim_size = 1
        st.output_buffer = self.grid.ctypes.data_as(P)
        st.baseline_count = geo["nb"]
        st.number_of_polarization_terms = 4
        st.number_of_polarization_terms_being_gridded = 4
        st.spw_count = 1
        st.channel_count = N_CHAN
        st.antenna_count = N_ANT
        st.enabled_channels = self.enabled.ctypes.data_as(P)
        st.reference_wavelengths = self.lam.ctypes.data_as(P)
        st.should_grid_sampling_function = True
        st.sampling_function_buffer = self.sf.ctypes.data_as(P)
        st.sampling_function_channel_grid_indicies = self.sfcgi.ctypes.data_as(P)
        st.sampling_function_channel_count = 1
        st.num_facet_centres = N_FACETS
        st.facet_centres = self.facets.ctypes.data_as(P)
        st.wplanes = WPLANES
        st.wmax_est = geo["wmax"]
        st.no_timestamps_read = geo["n_times"]
        st.row_count = rows


def set_rows(st, d, ptr):
    st.visibilities = ptr(d["vis"])
    st.uvw_coords = ptr(d["uvw"])
    st.visibility_weights = ptr(d["weights"])
    st.flags = ptr(d["flags"])
    st.flagged_rows = ptr(d["flagged_rows"])
    st.field_array = ptr(d["field"])
    st.spw_index_array = ptr(d["spw"])
    st.antenna_1_ids = ptr(d["a1"])
    st.antenna_2_ids = ptr(d["a2"])
    st.timestamp_ids = ptr(d["tid"])
    st.jones_terms = ptr(d["jones"])
    st.baseline_starting_indexes = ptr(d["starts"])


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clock and throttle-reason samples every 200 ms between start() and stop(); the raw
    samples are also written to `path` when one is given."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, path=None):
        self.path = path
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            out = self.proc.communicate(timeout=5)[0] or ""
        except Exception:
            self.proc.kill()
            out = ""
        if self.path:
            with open(self.path, "w") as fh:
                fh.write(out)
        sm, mx, reasons = [], [], set()
        for line in out.splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"),
                                 parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


CLOCKS_DIR = None  # --clocks-dir


def clocks_path(name):
    """Where the raw clock samples go: the --clocks-dir folder when one was given, else nowhere."""
    return os.path.join(CLOCKS_DIR, name) if CLOCKS_DIR else None


# ----------------------------------------------------------------------------- CPU (oracle port) and parity
def sample_baselines(geo, n):
    """``n`` cross baselines spread over the baseline slots, each with all its timesteps: the row
    sample of the CPU baseline and of the parity check (whole tracks, as the gridder sees them)."""
    starts = geo["starts"].astype(np.int64)
    full = np.nonzero(starts[1:] > starts[:-1])[0]
    pick = np.unique(full[np.linspace(0, full.size - 1, max(1, n)).astype(np.int64)])
    rows = np.concatenate([np.arange(starts[b], starts[b + 1]) for b in pick])
    return pick, rows


def host_sample(geo, pick, vis=None, jones=None, seed=3):
    """Host arrays of the rows of baselines ``pick`` (baseline-major, as the workload), with their
    track starts.  ``vis`` [R, Ch, 4] and ``jones`` [T, A', F, 1, Ch, 4] (A' = the antennas the sample
    uses, ascending) are the workload's own arrays when given (complex64), else seeded stand-ins of
    the same distributions.  Antenna ids are renumbered to the antennas the sample uses."""
    starts_all = geo["starts"].astype(np.int64)
    counts = starts_all[pick + 1] - starts_all[pick]
    rows = np.concatenate([np.arange(starts_all[b], starts_all[b + 1]) for b in pick])
    a1, a2 = geo["a1"][rows], geo["a2"][rows]
    ants = np.unique(np.concatenate([a1, a2]))
    remap = np.full(N_ANT, -1, np.int64)
    remap[ants] = np.arange(ants.size)
    R, T = rows.size, geo["n_times"]
    rng = np.random.default_rng(seed)
    if vis is None:
        vis = (rng.normal(0, 1, (R, N_CHAN, 4)) + 1j * rng.normal(0, 1, (R, N_CHAN, 4))).astype(np.complex64)
    if jones is None:
        shape = (T, ants.size, N_FACETS, 1, N_CHAN)
        jones = np.zeros(shape + (4,), np.complex64)
        for k in (0, 3):
            jones[..., k] = (1 + rng.uniform(-0.1, 0.1, shape)) * np.exp(1j * rng.uniform(-np.pi, np.pi, shape))
        for k in (1, 2):
            jones[..., k] = 0.05 * (rng.normal(0, 1, shape) + 1j * rng.normal(0, 1, shape)) / np.sqrt(2)
    return dict(vis=np.ascontiguousarray(vis, np.complex64), uvw=geo["uvw"][rows].astype(np.float32),
                weights=np.ones((R, N_CHAN, 4), np.float32), flags=np.zeros((R, N_CHAN, 4), np.bool_),
                flagged_rows=np.zeros(R, np.bool_), field=np.zeros(R, np.uint32), spw=np.zeros(R, np.uint32),
                a1=remap[a1].astype(np.uint32), a2=remap[a2].astype(np.uint32),
                tid=geo["tid"][rows].astype(np.uintp), jones=np.ascontiguousarray(jones, np.complex64),
                starts=np.concatenate([[0], np.cumsum(counts)]).astype(np.uintp), n_ant=int(ants.size),
                rows=rows, ants=ants)


def run_sample(lib, precision, geo, conv, smp, post=True):
    """The pipeliner's call sequence on the row sample: initLibrary, facet_4_cor_corrections +
    facet_sampling_function (timed), then weight_uniformly and normalize when ``post``.  Returns the
    seconds of the gridding calls and the normalised grids [F, 1, 4, NX, NX]."""
    from bullseye_gb300.abi import complex_dtype, gridding_parameters_type, real_dtype
    cd, rd = complex_dtype(precision), real_dtype(precision)
    arr = {k: (v.astype(cd) if v.dtype == np.complex64 else v.astype(rd) if v.dtype == np.float32 else v)
           for k, v in smp.items() if isinstance(v, np.ndarray) and k not in ("rows", "ants")}
    arr = {k: np.ascontiguousarray(v) for k, v in arr.items()}
    tab = Tables(geo, np.ascontiguousarray(conv.astype(cd)))
    tab.lam = tab.lam.astype(rd)
    tab.facets = tab.facets.astype(rd)
    tab.grid = np.zeros((N_FACETS, 1, 4, NX, NX), dtype=cd)
    tab.sf = np.zeros((N_FACETS, 1, 1, NX, NX), dtype=cd)
    st = gridding_parameters_type(precision)()
    R = arr["uvw"].shape[0]
    tab.fill(st, geo, R)
    st.antenna_count = smp["n_ant"]
    st.baseline_count = smp["n_ant"] * (smp["n_ant"] - 1) // 2 + smp["n_ant"]  # slots of the renumbered antennas
    P = ctypes.c_void_p
    lib.initLibrary(ctypes.byref(st))
    set_rows(st, arr, lambda a: a.ctypes.data_as(P))
    st.baseline_starting_indexes = None  # the GPU library sorts by baseline itself; the oracle reads no starts
    st.is_final_data_chunk = True
    t0 = time.perf_counter()
    lib.facet_4_cor_corrections(ctypes.byref(st))
    lib.facet_sampling_function(ctypes.byref(st))
    lib.gridding_barrier()
    dt = time.perf_counter() - t0
    if post:
        lib.weight_uniformly(ctypes.byref(st))
        lib.normalize(ctypes.byref(st))
    lib.releaseLibrary()
    return dt, tab.grid


def cpu_baseline(geo, conv1d, target_s, smp=None, nbl=0):
    """The oracle port of the reference CPU library (single precision, OpenMP over facets) timed on
    a sample of whole baselines of the workload."""
    from bullseye_gb300.filters import outer_stack
    from oracle.harness import load_oracle
    lib = load_oracle("single")
    conv2d = outer_stack(conv1d.astype(np.complex128)).astype(np.complex64)
    if smp is None:
        if not nbl:
            # one baseline first, to size the sample to about target_s seconds
            pick, _ = sample_baselines(geo, 1)
            dt1, _ = run_sample(lib, "single", geo, conv2d, host_sample(geo, pick), post=False)
            nbl = int(max(1, min(64, round(target_s / max(dt1, 1e-3)))))
        pick, _ = sample_baselines(geo, nbl)
        smp = host_sample(geo, pick)
    dt, _ = run_sample(lib, "single", geo, conv2d, smp, post=False)
    R = smp["uvw"].shape[0]
    pairs = R * N_CHAN * N_FACETS
    return {"value": pairs / dt / 1e6, "unit": "Mvis/s", "cores": min(os.cpu_count() or 1, N_FACETS), "kind": "port",
            "sample": f"{smp['starts'].size - 1} whole baselines ({R} rows, all {geo['n_times']} timesteps) x "
                      f"{N_CHAN} ch x {N_FACETS} facets = {pairs} vis-facet pairs of the same workload with its "
                      f"per-time Jones terms, oracle port of the reference CPU library (FP32, OpenMP over facets, "
                      f"{os.cpu_count()} cores available, one thread per facet), {dt:.1f} s"}


def dirty(grid):
    """Dirty images of grids [..., ny, nx] with the reference's shifts (FP64)."""
    g = np.asarray(grid, np.complex128)
    return np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(g, axes=(-2, -1))), axes=(-2, -1)).real


def parity_check(lib32, geo, conv1d, smp):
    """The batched FP32 path against the FP64 oracle on the row sample: the same reference exports
    through the C-ABI (host inputs; the exports run the support-aware batched gridder with the
    tuned class layouts and compensated FP32) and the oracle port in double precision on the same
    values, both followed by weight_uniformly and normalize.  Per facet: max and RMS relative error
    of the weighted, normalised grids and of the dirty images."""
    from bullseye_gb300.filters import outer_stack
    from bullseye_gb300.library import check
    from oracle.harness import load_oracle
    t0 = time.perf_counter()
    _, g32 = run_sample(lib32, "single", geo, conv1d, smp)
    check(lib32)
    conv2d = outer_stack(conv1d.astype(np.complex128))
    _, g64 = run_sample(load_oracle("double"), "double", geo, conv2d, smp)
    facets = []
    for f in range(N_FACETS):
        a, b = g64[f, 0], g32[f, 0].astype(np.complex128)
        ia, ib = dirty(a), dirty(b)
        d, di = b - a, ib - ia
        facets.append({"grid_max_rel": float(np.max(np.abs(d)) / np.max(np.abs(a))),
                       "grid_rms_rel": float(np.sqrt(np.mean(np.abs(d) ** 2) / np.mean(np.abs(a) ** 2))),
                       "image_max_rel": float(np.max(np.abs(di)) / np.max(np.abs(ia))),
                       "image_rms_rel": float(np.sqrt(np.mean(di * di) / np.mean(ia * ia)))})
    worst = max(x["image_max_rel"] for x in facets)
    return {"against": "oracle port of the reference CPU library in FP64 (same input values, 2-D w-kernel stack "
                       "of the FP32 1-D stack), weight_uniformly + normalize on both",
            "form": "reference exports facet_4_cor_corrections + facet_sampling_function on the batched "
                    "support-aware gridder (tuned class layouts, compensated FP32)",
            "sample": f"{smp['starts'].size - 1} whole baselines, {smp['uvw'].shape[0]} rows x {N_CHAN} ch x "
                      f"{N_FACETS} facets",
            "max_rel": worst, "rms_rel": max(x["image_rms_rel"] for x in facets),
            "grid_max_rel": max(x["grid_max_rel"] for x in facets), "tolerance": 1e-5, "pass": worst <= 1e-5,
            "per_facet": facets, "seconds": time.perf_counter() - t0}


# ----------------------------------------------------------------------------- precision form
def precision_report():
    """Dirty-image error of the FP32 library against the FP64 library, per facet (config 3).

    The config-1 observation on an 80 km disc, 4 facets of 4096^2 (0.25 arcsec) at l offsets of
    0, 0.5, 1 and 2 deg, facet_4_cor + normalize + finalize through the C-ABI.  Both libraries get
    the same input values (the single-precision arrays, widened for the FP64 run), so the figures
    are the arithmetic error of the FP32 path: compensated (the precision form) and plain FP32
    flushes.  max_rel = max|I32 - I64| / max|I64|, rms_rel = rms(I32 - I64) / rms(I64), on the XX
    image of each facet.
    """
    from bullseye_gb300 import synth
    from bullseye_gb300.imaging import run_imaging
    from bullseye_gb300.library import check, load_library
    p32 = synth.config3("single")
    p64 = p32.astype("double")
    lib64 = load_library("GPU", "double")
    ref = run_imaging(lib64, p64, "facet_4_cor", repack=True, do_finalize=True)
    check(lib64)
    lib32 = load_library("GPU", "single")
    from bullseye_gb300.geometry import offgrid_pairs
    out = {"workload": "config-1 observation, 80 km disc, 4 facets 4096^2 at 0/0.5/1/2 deg, PSWF W=7 os=63, "
                       "facet_4_cor, XX dirty image", "reference": "64-bit library on the same input values",
           "rows": p32.rows,
           # samples whose footprint leaves each facet's grid (the reference drops them uncounted)
           "offgrid_samples_per_facet": [int(x) for x in offgrid_pairs(p64)]}
    for comp in (1, 0):
        lib32.bullseye_set_compensated(comp)
        res = run_imaging(lib32, p32, "facet_4_cor", repack=True, do_finalize=True)
        check(lib32)
        rows = []
        for f in range(ref.image.shape[0]):
            a = ref.image[f, 0].astype(np.float64)
            b = res.image[f, 0].astype(np.float64)
            d = b - a
            rows.append({"max_rel": float(np.max(np.abs(d)) / np.max(np.abs(a))),
                         "rms_rel": float(np.sqrt(np.mean(d * d)) / np.sqrt(np.mean(a * a)))})
        out["fp32_compensated" if comp else "fp32_plain"] = rows
    lib32.bullseye_set_compensated(1)
    return out


# ----------------------------------------------------------------------------- uneven facets
UNEVEN_FACETS, UNEVEN_TIMES, UNEVEN_PLANES = 96, 2226, 128


UNEVEN_MIN_VIS, UNEVEN_MAX_VIS = 1e5, 5e7


def uneven_layout(seed=21):
    """96 facets with sizes log-uniform in [256, 4096] (multiples of 64), 5 arcsec cells, centres
    within 3 deg, and per-facet visibility counts log-uniform in [1e5, 5e7] (the facet's kept
    fraction of the 5e7 shared visibilities)."""
    rng = np.random.default_rng(seed)
    sizes = (np.exp(rng.uniform(np.log(256), np.log(4096), UNEVEN_FACETS)) // 64 * 64).astype(np.int64)
    sizes = np.clip(sizes, 256, 4096)
    lim = np.deg2rad(3.0)
    counts = np.exp(rng.uniform(np.log(UNEVEN_MIN_VIS), np.log(UNEVEN_MAX_VIS), UNEVEN_FACETS))
    return sizes, rng.uniform(-lim, lim, UNEVEN_FACETS), rng.uniform(-lim, lim, UNEVEN_FACETS), counts


def uneven_masks(geo, counts, seed=22):
    """[F][R] uint8 masks from baseline and time flagging: facet f keeps a random subset of the
    baselines and one contiguous time range, each about sqrt(kept fraction) of the whole, so that it
    keeps about counts[f] visibilities (rows x channels)."""
    from bullseye_gb300.imaging import baseline_index
    rng = np.random.default_rng(seed)
    b = baseline_index(geo["a1"], geo["a2"], N_ANT)
    t = np.asarray(geo["tid"], np.int64)
    T = int(t.max()) + 1
    ub = np.unique(b)
    total = b.size * N_CHAN
    out = np.zeros((len(counts), b.size), np.uint8)
    for f, n in enumerate(counts):
        frac = min(1.0, float(n) / total)
        keep_b = np.zeros(int(b.max()) + 1, bool)
        nbk = max(1, int(round(ub.size * np.sqrt(frac))))
        keep_b[rng.choice(ub, nbk, replace=False)] = True
        span = max(1, min(T, int(round(frac * b.size / max(1, np.count_nonzero(keep_b[b])) * T))))
        t0 = int(rng.integers(0, T))
        keep_t = ((t - t0) % T) < span
        out[f] = keep_b[b] & keep_t
    return out


def uneven_main(args):
    """The batching form on an uneven layout: one bullseye_grid_batched_facets call per step over 96
    facets of different sizes with different row masks, w-projection with 128 planes."""
    global N_FACETS, WPLANES, NX
    import torch
    from bullseye_gb300.abi import BullseyeFacet, gridding_parameters_type
    from bullseye_gb300.library import check, load_library
    N_FACETS, WPLANES = 1, UNEVEN_PLANES
    torch.cuda.set_device(0)
    geo = geometry(UNEVEN_TIMES)
    conv, supports = kernel_stack(geo["wmax"])  # w kernels for a 1024-pixel field
    NX = 256  # the library's own grid only hosts the tuner
    R = geo["uvw"].shape[0]
    sizes, fl, fm, targets = uneven_layout()
    masks = uneven_masks(geo, targets)
    kept_rows = masks.sum(axis=1).astype(np.int64)
    pairs_per_step = int(kept_rows.sum()) * N_CHAN
    dec = geo["dec0"] * np.pi / (180 * 3600)
    facets = (BullseyeFacet * UNEVEN_FACETS)()
    off = 0
    for f in range(UNEVEN_FACETS):
        ra_as = fl[f] / np.cos(dec) * 180 * 3600 / np.pi
        dec_as = geo["dec0"] + fm[f] * 180 * 3600 / np.pi
        n = int(sizes[f])
        facets[f] = BullseyeFacet(float(ra_as), float(dec_as), CELL, CELL, n, n, off)
        off += 4 * n * n
    lib = load_library("GPU", "single")
    lib.bullseye_set_visibility_records(0 if args.no_records else 1)
    d = device_inputs(geo, torch)
    grids = torch.zeros(off, dtype=torch.complex64, device="cuda")
    lo = torch.zeros(off, dtype=torch.complex64, device="cuda")
    norms = torch.zeros(UNEVEN_FACETS * 4, dtype=torch.float64, device="cuda")
    mask_dev = torch.as_tensor(masks, device="cuda")
    torch.cuda.synchronize()
    tab = Tables(geo, conv)
    st = gridding_parameters_type("single")()
    tab.fill(st, geo, R)
    st.should_grid_sampling_function = False
    lib.bullseye_set_device_inputs(1)
    lib.bullseye_set_compensated(0 if args.no_comp else 1)
    lib.initLibrary(ctypes.byref(st))
    check(lib)
    set_rows(st, d, lambda t: ctypes.c_void_p(t.data_ptr()))
    st.is_final_data_chunk = False
    stream = torch.cuda.ExternalStream(lib.bullseye_get_stream())
    lo_ptr = None if args.no_comp else ctypes.c_void_p(lo.data_ptr())

    def step():
        rc = lib.bullseye_grid_batched_facets(ctypes.byref(st), ctypes.cast(facets, ctypes.c_void_p), UNEVEN_FACETS,
                                              ctypes.c_void_p(mask_dev.data_ptr()), ctypes.c_void_p(grids.data_ptr()),
                                              lo_ptr, ctypes.c_void_p(norms.data_ptr()), 1)
        if rc:
            check(lib)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    check(lib)
    lib.bullseye_reset_counters()
    clocks = ClockSampler(clocks_path("clocks.csv"))
    clocks.start()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    clk = clocks.stop()
    launches = int(lib.bullseye_kernel_launches())
    check(lib)
    fp32_peak = lib.bullseye_fp32_fma_tflops(4096)
    # algorithmic flops on each visibility's true w-plane support, over the rows each facet keeps
    w = np.abs(geo["uvw"][:, 2])
    true_taps = 0.0
    sup2 = np.asarray(supports, np.float64) ** 2
    for lam in geo["lam"]:
        pl = np.clip(np.rint(w / lam * ((WPLANES - 1) / geo["wmax"])).astype(np.int64), 0, WPLANES - 1)
        true_taps += float((masks.astype(np.float64) @ sup2[pl]).sum())
    step_flops = true_taps * 8 * 4 + pairs_per_step * (6 * 4)
    achieved = step_flops / (ms * 1e-3) / 1e12
    # load balance: one eager step with an event pair around every support-class launch
    lib.bullseye_set_batched_profiling(1)
    try:
        step()
        torch.cuda.synchronize()
    finally:
        lib.bullseye_set_batched_profiling(0)
    nrec = 128
    arrs = [np.zeros(nrec, np.int32) for _ in range(5)] + [np.zeros(nrec, np.float32)]
    cnt = lib.bullseye_batched_profile(*[a.ctypes.data_as(ctypes.c_void_p) for a in arrs], nrec)
    width, _, Jl, _, items, cms = arrs
    classes = [{"width": int(width[i]), "J": int(Jl[i]), "work_items": int(items[i]), "ms": float(cms[i])}
               for i in range(min(cnt, nrec))]
    busy = float(sum(c["ms"] for c in classes))
    lib.releaseLibrary()
    check(lib)
    parity, cpu = None, None
    if not args.no_parity:
        parity, cpu = uneven_parity(lib, geo, conv, sizes, fl, fm, masks, d, torch, args.no_comp)
    lib.bullseye_set_device_inputs(0)
    value = pairs_per_step / (ms * 1e-3) / 1e6
    line = {"metric": "gridded Mvis/s (vis x facet pairs)", "value": value, "unit": "Mvis/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"uneven facets: {UNEVEN_FACETS} facets of {int(sizes.min())}^2..{int(sizes.max())}^2 "
                                   f"(log-uniform), 5 arcsec cells, per-facet baseline/time flagging masks keeping "
                                   f"1e5..5e7 visibilities per facet (log-uniform), "
                                   f"27 ant x {UNEVEN_TIMES} t x {N_CHAN} ch ({R * N_CHAN / 1e6:.1f}M vis), w-proj "
                                   f"{WPLANES} planes support {MIN_SUPPORT}-{2 * S_HALF + 1}, facet_4_cor, compensated FP32",
                       "facet_vis_min": int(kept_rows.min()) * N_CHAN, "facet_vis_max": int(kept_rows.max()) * N_CHAN,
                       "grid_cells": off, "vis_facet_pairs_per_step": pairs_per_step,
                       "form": "bullseye_grid_batched_facets (persistent per-class launches, CUDA graph replay)"},
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                         "frac": achieved / fp32_peak if fp32_peak else None, "traffic": None,
                         "peak_source": "measured FP32 FMA probe on this GPU"},
            "clocks": clk, "gpu_launches": launches, "e2e": None, "cpu_baseline": cpu, "parity": parity,
            "load_balance": {"class_launches": classes, "class_ms_sum": busy,
                             "class_share_of_eager_step": busy / (ms if ms else 1.0),
                             "what": "per-class persistent launches of one eager step (event pair each) against the "
                                     "graph step time; the launches of a step run back to back on one stream"}}
    print(json.dumps(line))


def uneven_parity(lib, geo, conv1d, sizes, fl, fm, masks, d, torch, no_comp, nbl=3):
    """The uneven layout's batched form against the FP64 oracle on a sample: the rows of `nbl` whole
    baselines, the facets of smallest and largest kept count and the median one among facets of at
    most 2048^2, each facet's row mask applied.  The GPU grids the sample's facets in one
    bullseye_grid_batched_facets call; the oracle grids each facet on its own grid (masked rows
    flagged) with the 2-D stack of the same w kernels.  Also times the oracle port in FP32 on the
    same facet runs as the CPU baseline."""
    from bullseye_gb300.abi import BullseyeFacet, gridding_parameters_type
    from bullseye_gb300.filters import outer_stack
    from bullseye_gb300.imaging import GriddingProblem, run_imaging
    from bullseye_gb300.library import check
    from oracle.harness import load_oracle
    t0 = time.perf_counter()
    pick, rows = sample_baselines(geo, nbl)
    ms_rows = masks[:, rows]
    kept = ms_rows.sum(axis=1)
    small = np.nonzero((sizes <= 2048) & (kept > 0))[0]
    sel = sorted({int(small[np.argmin(kept[small])]), int(small[np.argmax(kept[small])]),
                  int(small[np.argsort(kept[small])[small.size // 2]])})
    R = rows.size
    dec = geo["dec0"] * np.pi / (180 * 3600)
    ras = [float(fl[f] / np.cos(dec) * 180 * 3600 / np.pi) for f in sel]
    decs = [float(geo["dec0"] + fm[f] * 180 * 3600 / np.pi) for f in sel]
    facets = (BullseyeFacet * len(sel))()
    off, offs = 0, []
    for i, f in enumerate(sel):
        n = int(sizes[f])
        facets[i] = BullseyeFacet(ras[i], decs[i], CELL, CELL, n, n, off)
        offs.append(off)
        off += 4 * n * n
    idx = torch.as_tensor(rows.astype(np.int64), device="cuda")
    ds = {k: (v if k in ("jones", "starts") else v[idx].contiguous()) for k, v in d.items()}
    ds["starts"] = torch.as_tensor(np.concatenate([[0], np.cumsum(geo["starts"][pick + 1] - geo["starts"][pick])])
                                   .astype(np.int64), device="cuda")
    grids = torch.zeros(off, dtype=torch.complex64, device="cuda")
    lo = torch.zeros(off, dtype=torch.complex64, device="cuda")
    norms = torch.zeros(len(sel) * 4, dtype=torch.float64, device="cuda")
    mask_dev = torch.as_tensor(np.ascontiguousarray(ms_rows[sel]), device="cuda")
    tab = Tables(geo, conv1d)
    st = gridding_parameters_type("single")()
    tab.fill(st, geo, R)
    st.should_grid_sampling_function = False
    st.num_facet_centres = 1
    lib.bullseye_set_device_inputs(1)
    lib.initLibrary(ctypes.byref(st))
    set_rows(st, ds, lambda t: ctypes.c_void_p(t.data_ptr()))
    st.baseline_count = pick.size
    st.is_final_data_chunk = False
    rc = lib.bullseye_grid_batched_facets(ctypes.byref(st), ctypes.cast(facets, ctypes.c_void_p), len(sel),
                                          ctypes.c_void_p(mask_dev.data_ptr()), ctypes.c_void_p(grids.data_ptr()),
                                          None if no_comp else ctypes.c_void_p(lo.data_ptr()),
                                          ctypes.c_void_p(norms.data_ptr()), 1)
    torch.cuda.synchronize()
    lib.releaseLibrary()
    check(lib)
    assert rc == 0
    G = (grids + lo).cpu().numpy()
    N = norms.cpu().numpy().reshape(len(sel), 4)
    host = {k: v.cpu().numpy() for k, v in ds.items() if k not in ("jones", "starts")}
    conv2d = outer_stack(conv1d.astype(np.complex128))
    per_facet, cpu_pairs, cpu_s = [], 0, 0.0
    for i, f in enumerate(sel):
        n = int(sizes[f])
        prob = GriddingProblem(
            precision="double", vis=host["vis"].astype(np.complex128), uvw=host["uvw"].astype(np.float64),
            wavelengths=geo["lam"].astype(np.float32).astype(np.float64).reshape(1, -1),
            weights=host["weights"].astype(np.float64), flags=host["flags"].astype(bool),
            flagged_rows=~ms_rows[f].astype(bool), field_ids=np.zeros(R, np.uint32), spw_ids=np.zeros(R, np.uint32),
            antenna1=host["a1"].astype(np.uint32), antenna2=host["a2"].astype(np.uint32),
            timestamp_ids=host["tid"].astype(np.uintp), n_antennas=N_ANT, n_timestamps=geo["n_times"], nx=n, ny=n,
            cell_x=CELL, cell_y=CELL, conv=conv2d, conv_support=S_HALF, conv_oversample=OS, wplanes=WPLANES,
            wmax=float(np.float32(geo["wmax"])), phase_centre=(0.0, float(np.float32(geo["dec0"]))),
            facet_centres=np.array([[ras[i], decs[i]]], np.float64))  # the GPU's facet centres are FP64
        ref = run_imaging(load_oracle("double"), prob, "facet_4_cor", keep_raw=True)
        g = G[offs[i]:offs[i] + 4 * n * n].reshape(4, n, n).astype(np.complex128)
        a = ref.raw_grid[0, 0]
        ia = dirty(a / ref.normalization[0, 0][:, None, None])
        ib = dirty(g / N[i][:, None, None])
        d_ = g - a
        per_facet.append({"facet": f, "grid": n, "vis_in_sample": int(kept[f]) * N_CHAN,
                          "grid_max_rel": float(np.max(np.abs(d_)) / np.max(np.abs(a))),
                          "image_max_rel": float(np.max(np.abs(ib - ia)) / np.max(np.abs(ia))),
                          "image_rms_rel": float(np.sqrt(np.mean((ib - ia) ** 2) / np.mean(ia * ia)))})
        p32 = prob.astype("single").with_conv(conv2d.astype(np.complex64))
        c0 = time.perf_counter()
        run_imaging(load_oracle("single"), p32, "facet_4_cor")
        cpu_s += time.perf_counter() - c0
        cpu_pairs += int(kept[f]) * N_CHAN
    worst = max(x["image_max_rel"] for x in per_facet)
    parity = {"against": "oracle port of the reference CPU library in FP64 on each facet's own grid (masked rows "
                         "flagged), 2-D stack of the FP32 1-D w kernels",
              "form": "bullseye_grid_batched_facets over the sampled facets (device inputs, compensated FP32)",
              "sample": f"{pick.size} whole baselines ({R} rows x {N_CHAN} ch), facets {sel}",
              "max_rel": worst, "tolerance": 1e-5, "pass": worst <= 1e-5, "per_facet": per_facet,
              "seconds": time.perf_counter() - t0}
    cpu = {"value": cpu_pairs / cpu_s / 1e6, "unit": "Mvis/s", "cores": 1, "kind": "port",
           "sample": f"the parity sample's {len(sel)} facet runs (one facet per call, so one OpenMP thread), "
                     f"{cpu_pairs} vis-facet pairs, oracle port in FP32 with initLibrary/releaseLibrary, {cpu_s:.1f} s"}
    return parity, cpu


# ----------------------------------------------------------------------------- prediction
def predict_main(args):
    """Prediction (degridding as a forward operator) on the multi-facet workload: 16 model images of
    1024^2 (point sources, 4 correlations) are divided by the gridding correction, transformed with
    the inverse of finalize's shifts and degridded to the 44.93 M visibilities with the Jones terms
    and the facet phases applied forward, summed over facets (bullseye_predict, device inputs,
    normalised form).  One step = one bullseye_predict call over every (visibility, facet) pair."""
    import torch
    from bullseye_gb300.abi import gridding_parameters_type
    from bullseye_gb300.filters import gridding_correction
    from bullseye_gb300.library import check, load_library
    torch.cuda.set_device(0)
    n_times = max(8, int(N_TIMES * args.time_frac))  # fewer timesteps only for profiling captures
    geo = geometry(n_times)
    conv, supports = kernel_stack(geo["wmax"])
    R = geo["uvw"].shape[0]
    pairs = R * N_CHAN * N_FACETS
    lib = load_library("GPU", "single")
    lib.bullseye_set_visibility_records(0 if args.no_records else 1)
    d = device_inputs(geo, torch)
    dev = torch.device("cuda")
    # model images: 20 point sources per facet with random fluxes, the same on the 4 correlations
    rng = np.random.default_rng(31)
    model = torch.zeros((N_FACETS, 1, 4, NX, NX), dtype=torch.complex64, device=dev)
    for f in range(N_FACETS):
        ys, xs = rng.integers(NX // 4, 3 * NX // 4, 20), rng.integers(NX // 4, 3 * NX // 4, 20)
        flux = torch.as_tensor(rng.uniform(0.1, 2.0, 20), dtype=torch.complex64, device=dev)
        for k in range(4):
            model[f, 0, k, torch.as_tensor(ys, device=dev), torch.as_tensor(xs, device=dev)] = flux
    k0 = np.real(conv[0]).astype(np.float64)
    taper = torch.as_tensor(gridding_correction(k0, S_HALF, OS, NX), device=dev)
    arrays = dict(conv=torch.as_tensor(conv, device=dev), lam=torch.as_tensor(geo["lam"].astype(np.float32), device=dev),
                  en=torch.ones(N_CHAN, dtype=torch.uint8, device=dev), cgi=torch.zeros(N_CHAN, dtype=torch.int64, device=dev),
                  fc=torch.as_tensor(geo["facets"].astype(np.float32), device=dev))
    st = gridding_parameters_type("single")()
    Tables(geo, conv).fill(st, geo, R)
    set_rows(st, d, lambda t: ctypes.c_void_p(t.data_ptr()))
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    st.conv, st.reference_wavelengths = P(arrays["conv"]), P(arrays["lam"])
    st.enabled_channels, st.channel_grid_indicies, st.facet_centres = P(arrays["en"]), P(arrays["cgi"]), P(arrays["fc"])
    st.baseline_starting_indexes = None
    out = torch.empty((R, N_CHAN, 4), dtype=torch.complex64, device=dev)
    nbytes = int(lib.bullseye_predict_ws_bytes(ctypes.byref(st)))
    ws = torch.empty(nbytes + 256, dtype=torch.uint8, device=dev)
    ws_ptr = ctypes.c_void_p((ws.data_ptr() + 255) // 256 * 256)
    stream = torch.cuda.current_stream()

    def step():
        rc = lib.bullseye_predict(ctypes.byref(st), P(model), P(taper), P(taper), 1, 1, P(out), ws_ptr, nbytes,
                                  ctypes.c_void_p(stream.cuda_stream))
        if rc:
            check(lib)

    for _ in range(max(1, args.warmup)):
        step()
    torch.cuda.synchronize()
    check(lib)
    clocks = ClockSampler(clocks_path("clocks.csv"))
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    clk = clocks.stop()
    check(lib)
    fp32_peak = lib.bullseye_fp32_fma_tflops(4096)
    counts = plane_vis_counts(geo)
    true_taps = float(np.sum(counts.astype(np.float64) * np.asarray(supports, np.float64) ** 2))
    # per (vis, facet): the W_p^2 complex grid x conj(tap) products of 4 correlations (8 flops each),
    # the tap product per cell (6) and the tap sum (1), then the phase and the two 2x2 Jones products
    step_flops = true_taps * N_FACETS * (8 * 4 + 7) + pairs * (6 * 4 + 128)
    achieved = step_flops / (ms * 1e-3) / 1e12
    gather_bytes = true_taps * N_FACETS * 4 * 8  # grid values read per step (mostly from L1 / L2)
    line = {"metric": "predicted Mvis/s (vis x facet pairs)", "value": pairs / (ms * 1e-3) / 1e6, "unit": "Mvis/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD.replace("facet_4_cor_corrections+facet_sampling_function",
                                                    "bullseye_predict (normalised, Jones forward)"),
                       "model": "16 facets x 20 point sources, 4 correlations, detapered, forward FFT every call",
                       **({} if n_times == N_TIMES else {"timesteps": n_times})},
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                         "frac": achieved / fp32_peak if fp32_peak else None,
                         "flops_rule": "(8 x 4 corr + 7) x W_p^2 per (vis, facet) + 152 for phase and Jones",
                         "gather_gbs": gather_bytes / (ms * 1e-3) / 1e9,
                         "gather_rule": "4 corr x 8 B x W_p^2 grid values read per (vis, facet), from L1/L2",
                         "peak_source": "measured FP32 FMA probe on this GPU"},
            "clocks": clk, "e2e": None, "cpu_baseline": None}
    print(json.dumps(line))


# ----------------------------------------------------------------------------- differentiation
ADJ_ANT, ADJ_TIMES, ADJ_CHAN, ADJ_NX, ADJ_PLANES, ADJ_S, ADJ_MINSUP, ADJ_OS, ADJ_CELL = 64, 1000, 32, 4096, 32, 15, 7, 15, 2.0


def adjoint_main(args):
    """The differentiation form at scale: 64 antennas (2016 baselines) x 1000 timesteps x 32
    channels (64.5 M visibilities), one 4096^2 facet with Jones, w-projection with 32 planes.
    Loss = sum over the central 512^2 pixels of the (XX + YY) dirty image squared.  Times the
    forward (gridding) and the backward (adjoint + FFT) through torch.autograd, then checks the
    gradients by central finite differences (eps 1e-3) on 200 random coordinates (100 visibility,
    100 Jones).  Each difference is evaluated exactly on the full loss: gridding is linear in the
    visibilities and a Jones term touches only the rows of its antenna and time, so the grid change
    is gridded from those rows alone (64-bit library) and added to the full grid."""
    import torch
    from bullseye_gb300 import synth
    from bullseye_gb300.autograd import FacetGeometry, facet_grid
    from bullseye_gb300.filters import wproj_kernels
    from bullseye_gb300.imaging import GriddingProblem
    from bullseye_gb300.library import load_library
    torch.cuda.set_device(0)
    dev = torch.device("cuda")
    dec = np.deg2rad(-30.0)
    xyz = synth.enu_to_equatorial(synth.disc_layout(ADJ_ANT, 2000.0, 1), np.deg2rad(-30.0))
    global ADJ_TIMES
    if args.adj_times:
        ADJ_TIMES = args.adj_times
    uvw, a1, a2, tid = synth.earth_rotation_rows(xyz, ADJ_TIMES, dec, np.deg2rad(90.0))
    R = uvw.shape[0]
    freqs = np.linspace(1.0e9, 1.5e9, ADJ_CHAN)
    lam = synth.C_LIGHT / freqs
    wmax = np.max(np.linalg.norm(uvw, axis=1)) / lam.min()
    fov = ADJ_NX * ADJ_CELL * synth.ARCSEC
    conv, adj_supports = wproj_kernels(ADJ_S, ADJ_OS, ADJ_PLANES, wmax, fov, min_support=ADJ_MINSUP)
    dec0 = dec / synth.ARCSEC

    def problem(rows, prec, weights=None):
        n = len(rows)
        rd = np.float64 if prec == "double" else np.float32
        if weights is None:
            weights = np.broadcast_to(np.ones((1, 1, 1), rd), (n, ADJ_CHAN, 4))
        return GriddingProblem(
            precision=prec, vis=np.broadcast_to(np.zeros((1, 1, 1), np.complex64), (n, ADJ_CHAN, 4)),
            uvw=uvw[rows].astype(np.float32).astype(np.float64 if prec == "double" else np.float32),
            wavelengths=lam.reshape(1, -1).astype(np.float32).astype(np.float64 if prec == "double" else np.float32),
            weights=weights.astype(rd),
            flags=np.broadcast_to(np.zeros((1, 1, 1), bool), (n, ADJ_CHAN, 4)), flagged_rows=np.zeros(n, bool),
            field_ids=np.zeros(n, np.uint32), spw_ids=np.zeros(n, np.uint32), antenna1=a1[rows], antenna2=a2[rows],
            timestamp_ids=tid[rows], n_antennas=ADJ_ANT, n_timestamps=ADJ_TIMES, nx=ADJ_NX, ny=ADJ_NX, cell_x=ADJ_CELL,
            cell_y=ADJ_CELL, conv=conv.astype(np.complex64 if prec == "single" else np.complex128), conv_support=ADJ_S,
            conv_oversample=ADJ_OS, wplanes=ADJ_PLANES, wmax=float(wmax), phase_centre=(0.0, dec0),
            facet_centres=np.array([[0.0, dec0]], dtype=rd), jones=None)

    geom = FacetGeometry.from_problem(problem(np.arange(R), "single"), device=dev)
    order = geom.order
    # visibilities of 20 point sources (row order of the geometry) and near-identity gains
    rng = np.random.default_rng(5)
    lim = 0.4 * fov / 2
    ls, ms = rng.uniform(-lim, lim, 20), rng.uniform(-lim, lim, 20)
    flux = torch.tensor(rng.uniform(0.1, 2.0, 20), dtype=torch.complex64, device=dev)
    l_t = torch.tensor(ls, dtype=torch.float32, device=dev)
    m_t = torch.tensor(ms, dtype=torch.float32, device=dev)
    nm1 = torch.sqrt(1 - l_t * l_t - m_t * m_t) - 1
    uvw_o = torch.tensor(uvw[order], dtype=torch.float32, device=dev)
    V = torch.empty((R, ADJ_CHAN, 4), dtype=torch.complex64, device=dev)
    for ci, lm in enumerate(lam):
        for lo in range(0, R, 1 << 16):
            hi = min(R, lo + (1 << 16))
            u, v, w = uvw_o[lo:hi, 0:1], uvw_o[lo:hi, 1:2], uvw_o[lo:hi, 2:3]
            sv = torch.polar(torch.ones_like(u * l_t), (u * l_t + v * m_t + w * nm1) * (-2 * np.pi / lm)) @ flux
            V[lo:hi, ci, 0] = sv
            V[lo:hi, ci, 3] = sv
            V[lo:hi, ci, 1] = 0
            V[lo:hi, ci, 2] = 0
    gen = torch.Generator(device=dev)
    gen.manual_seed(3)
    shape = (ADJ_TIMES, ADJ_ANT, 1, 1, ADJ_CHAN)
    J = torch.zeros(shape + (4,), dtype=torch.complex64, device=dev)
    for k in (0, 3):
        J[..., k] = torch.polar(1 + 0.2 * (torch.rand(shape, device=dev, generator=gen) - 0.5),
                                (2 * torch.rand(shape, device=dev, generator=gen) - 1) * np.pi)
    for k in (1, 2):
        J[..., k] = 0.05 * torch.randn(shape, dtype=torch.complex64, device=dev, generator=gen)
    c0, c1 = ADJ_NX // 2 - 256, ADJ_NX // 2 + 256

    def loss_of(G):
        s_ = G[0, 0, 0] + G[0, 0, 3]
        img = torch.fft.fftshift(torch.fft.ifft2(torch.fft.ifftshift(s_))).real
        cut = img[c0:c1, c0:c1]
        return (cut * cut).sum()

    def run(timed):
        Vg = V.clone().requires_grad_(True)
        Jg = J.clone().requires_grad_(True)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        ev[0].record()
        G, _ = facet_grid(geom, Vg, Jg)
        ev[1].record()
        L = loss_of(G)
        L.backward()
        ev[2].record()
        torch.cuda.synchronize()
        return ev[0].elapsed_time(ev[1]), ev[1].elapsed_time(ev[2]), G.detach(), L.item(), Vg.grad, Jg.grad

    for _ in range(args.warmup):
        run(False)
    fwd, bwd = [], []
    for _ in range(args.steps):
        f_ms, b_ms, G, Lval, gV, gJ = run(True)
        fwd.append(f_ms)
        bwd.append(b_ms)
    f_ms, b_ms = float(np.median(fwd)), float(np.median(bwd))
    # finite differences on 200 coordinates, the loss evaluated in FP64
    G0 = G[0, 0][[0, 3]].to(torch.complex128)
    del G

    def loss64(dG):  # dG: [2][ny][nx] change of the XX and YY grids
        s_ = (G0[0] + dG[0]) + (G0[1] + dG[1])
        img = torch.fft.fftshift(torch.fft.ifft2(torch.fft.ifftshift(s_))).real
        cut = img[c0:c1, c0:c1]
        return float((cut * cut).sum())

    J64 = J.to(torch.complex128)
    eps = 1e-3
    rng = np.random.default_rng(17)
    errs = {"vis": [], "jones": []}
    scale = {"vis": float(gV.abs().max()), "jones": float(gJ.abs().max())}
    for i in range(100):
        r = int(rng.integers(R))
        ch, k, part = int(rng.integers(ADJ_CHAN)), int(rng.choice([0, 3])), int(rng.integers(2))
        g1 = FacetGeometry.from_problem(problem(np.array([order[r]]), "double"), device=dev)
        e = torch.zeros((1, ADJ_CHAN, 4), dtype=torch.complex128, device=dev)
        e[0, ch, k] = 1.0 if part == 0 else 1j
        Ge, _ = facet_grid(g1, e, J64)
        dG = Ge[0, 0][[0, 3]]
        fd = (loss64(eps * dG) - loss64(-eps * dG)) / (2 * eps)
        an = float(gV[r, ch, k].real if part == 0 else gV[r, ch, k].imag)
        errs["vis"].append(abs(fd - an) / scale["vis"])
    inv = np.empty(R, np.int64)
    inv[order] = np.arange(R)
    for i in range(100):
        t, a = int(rng.integers(ADJ_TIMES)), int(rng.integers(ADJ_ANT))
        ch, k, part = int(rng.integers(ADJ_CHAN)), int(rng.integers(4)), int(rng.integers(2))
        rows = np.nonzero((tid == t) & ((a1 == a) | (a2 == a)))[0]
        wts = np.zeros((rows.size, ADJ_CHAN, 4), np.float64)
        wts[:, ch, :] = 1.0
        gs = FacetGeometry.from_problem(problem(rows, "double", weights=wts), device=dev)
        Vs = V[torch.as_tensor(inv[rows][gs.order], device=dev)].to(torch.complex128).contiguous()
        grids = []
        for sign in (1, -1, 0):
            Jp = J64.clone()
            Jp[t, a, 0, 0, ch, k] += sign * eps * (1.0 if part == 0 else 1j)
            Gs, _ = facet_grid(gs, Vs, Jp)
            grids.append(Gs[0, 0][[0, 3]])
        fd = (loss64(grids[0] - grids[2]) - loss64(grids[1] - grids[2])) / (2 * eps)
        g = gJ[t, a, 0, 0, ch, k]
        an = float(g.real if part == 0 else g.imag)
        errs["jones"].append(abs(fd - an) / scale["jones"])
    vis_pairs = R * ADJ_CHAN
    # algorithmic flops on each visibility's true w-plane support (one facet): the forward grids
    # 8 x 4 corr x W_p^2 (+ 152 for phase and Jones); the backward gathers the same footprint
    # (8 x 4 corr x W_p^2) and applies the chain rule through Jones (about 400 flops per item)
    true_taps = 0.0
    sup2 = np.asarray(adj_supports, np.float64) ** 2
    for lm in lam:
        pl = np.clip(np.rint(np.abs(uvw[:, 2]) / lm * ((ADJ_PLANES - 1) / wmax)).astype(np.int64), 0, ADJ_PLANES - 1)
        true_taps += float(sup2[pl].sum())
    fp32_peak = float(load_library("GPU", "single").bullseye_fp32_fma_tflops(4096))
    fwd_tf = (true_taps * 32 + vis_pairs * 152) / (f_ms * 1e-3) / 1e12
    bwd_tf = (true_taps * 32 + vis_pairs * 400) / (b_ms * 1e-3) / 1e12
    line = {"metric": "gridded Mvis/s (vis x facet pairs)", "value": vis_pairs / (f_ms * 1e-3) / 1e6, "unit": "Mvis/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": f_ms + b_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"differentiation: {ADJ_ANT} ant ({ADJ_ANT * (ADJ_ANT - 1) // 2} baselines) x "
                                   f"{ADJ_TIMES} t x {ADJ_CHAN} ch ({vis_pairs / 1e6:.1f}M vis), one {ADJ_NX}^2 facet with "
                                   f"Jones, w-proj {ADJ_PLANES} planes; loss = sum over the central 512^2 pixels of the "
                                   f"(XX+YY) dirty image squared"},
            "roofline": {"bound": "fp32", "achieved": fwd_tf, "peak": fp32_peak, "unit": "TFLOP/s",
                         "frac": fwd_tf / fp32_peak if fp32_peak else None, "kernel": "forward (workspace gridding)",
                         "backward_achieved": bwd_tf, "backward_frac": bwd_tf / fp32_peak if fp32_peak else None,
                         "backward_gather_gbs": true_taps * 32 / (b_ms * 1e-3) / 1e9,
                         "flops_rule": "8 x 4 corr x W_p^2 per visibility (true w-plane support) + 152 forward / "
                                       "about 400 backward for phase, Jones and the chain rule",
                         "peak_source": "measured FP32 FMA probe on this GPU"},
            "forward_ms": f_ms, "backward_ms": b_ms,
            "backward_mvis_s": vis_pairs / (b_ms * 1e-3) / 1e6, "loss": Lval,
            "finite_differences": {"eps": eps, "coordinates": 200,
                                   "max_err_vis": max(errs["vis"]), "max_err_jones": max(errs["jones"]),
                                   "tolerance": 1e-4, "relative_to": "largest gradient magnitude of each kind",
                                   "pass": max(errs["vis"]) <= 1e-4 and max(errs["jones"]) <= 1e-4}}
    print(json.dumps(line))


# ----------------------------------------------------------------------------- main
def reference_vs_port(geo, conv1d, nbl, reps=3):
    """The reference's own CPU library (oracle/_ref, compiled from its sources) against the oracle
    port on the same sample of whole baselines: best of `reps` seconds of the gridding calls and a
    checksum of the normalised grids; prints one JSON line."""
    from bullseye_gb300.filters import outer_stack
    from oracle.harness import load_oracle, load_reference, reference_available
    if not reference_available():
        print(json.dumps({"reference_vs_port": None, "why": "oracle/_ref is not built here"}))
        return
    conv2d = outer_stack(conv1d.astype(np.complex128)).astype(np.complex64)
    pick, rows = sample_baselines(geo, nbl)
    smp = host_sample(geo, pick)
    out = {"sample": f"{pick.size} whole baselines x {geo['n_times']} timesteps x {N_CHAN} ch x {N_FACETS} facets "
                     f"({rows.size * N_CHAN * N_FACETS} vis-facet pairs)", "threads": os.cpu_count()}
    for name, lib in (("port", load_oracle("single")), ("reference", load_reference("single"))):
        ts, g = [], None
        for _ in range(reps):
            dt, g = run_sample(lib, "single", geo, conv2d, smp, post=True)
            ts.append(dt)
        out[name] = {"seconds": min(ts), "mvis_s": rows.size * N_CHAN * N_FACETS / min(ts) / 1e6,
                     "checksum": float(np.abs(g).astype(np.float64).sum())}
    out["port_over_reference_speed"] = out["reference"]["seconds"] / out["port"]["seconds"]
    print(json.dumps(out))


def relaunch(n):
    """`bench.py --gpus N` started without torchrun: run N local ranks under torch.distributed.run
    (one per GPU, rendezvous on 127.0.0.1) with the same arguments and return its exit status."""
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr", "127.0.0.1", f"--master-port={port}", os.path.abspath(__file__)] + sys.argv[1:]
    return subprocess.call(cmd)


def main():
    args = parse()
    global CLOCKS_DIR
    CLOCKS_DIR = args.clocks_dir
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(relaunch(args.gpus))
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world != args.gpus:
        print(f"bench.py: --gpus {args.gpus} but WORLD_SIZE {world}", file=sys.stderr)
        sys.exit(2)
    if args.workload == "uneven":
        return uneven_main(args)
    if args.workload == "adjoint":
        return adjoint_main(args)
    if args.workload == "predict":
        return predict_main(args)
    global N_CHAN, N_FACETS
    if args.chans:
        N_CHAN = args.chans
    if args.facets:
        N_FACETS = args.facets
    n_times = max(8, int(N_TIMES * args.time_frac))
    geo = geometry(n_times, world, rank)
    conv, supports = kernel_stack(geo["wmax"])
    R = geo["uvw"].shape[0]
    pairs_per_step = R * N_CHAN * N_FACETS
    if args.reference_vs_port:
        return reference_vs_port(geo, conv, args.sample_baselines or 2)

    if args.impl == "reference":
        if rank != 0:
            return
        # the warm-up sizes the sample (whole baselines) to a bounded time per step
        per = max(2.0, min(20.0, 150.0 / max(1, args.steps + args.warmup)))
        from oracle.harness import load_oracle
        from bullseye_gb300.filters import outer_stack
        conv2d = outer_stack(conv.astype(np.complex128)).astype(np.complex64)
        pick, _ = sample_baselines(geo, 1)
        dt1, _ = run_sample(load_oracle("single"), "single", geo, conv2d, host_sample(geo, pick), post=False)
        nbl = args.sample_baselines or int(max(1, min(64, round(per / max(dt1, 1e-3)))))
        pick, _ = sample_baselines(geo, nbl)
        smp = host_sample(geo, pick)
        steps, base = [], None
        for _ in range(max(1, args.steps)):
            base = cpu_baseline(geo, conv, per, smp=smp)
            steps.append(base["value"])
        v = float(np.median(steps))
        line = {"impl": "reference", "metric": "gridded Mvis/s (vis x facet pairs)", "value": v, "unit": "Mvis/s",
                "n_gpus": 0, "steps": args.steps, "warmup": args.warmup, "ms_per_step": pairs_per_step / v / 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": WORKLOAD, "l2": "inputs 4.2 GB > L2"},
                "cpu_baseline": {"value": v, "unit": "Mvis/s", "cores": base["cores"], "kind": "port",
                                 "sample": base["sample"] + "; each step times this sample, ms_per_step extrapolates "
                                                            "to the whole workload"},
                "e2e": {"value": v, "unit": "Mvis/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from bullseye_gb300.abi import gridding_parameters_type
    from bullseye_gb300.library import check, load_library
    lib = load_library("GPU", "single")
    lib.bullseye_set_visibility_records(0 if args.no_records else 1)
    d = device_inputs(geo, torch)
    torch.cuda.synchronize()

    # ------------------------------------------------------------- device-resident value
    tab = Tables(geo, conv)
    st = gridding_parameters_type("single")()
    tab.fill(st, geo, R)
    lib.bullseye_set_device_inputs(1)
    lib.bullseye_set_compensated(0 if args.no_comp else 1)
    lib.initLibrary(ctypes.byref(st))
    check(lib)
    set_rows(st, d, lambda t: ctypes.c_void_p(t.data_ptr()))
    st.is_final_data_chunk = False
    stream = torch.cuda.ExternalStream(lib.bullseye_get_stream())

    def step_plain():
        # the reference's exports on the plain per-track kernels (full padded support)
        lib.bullseye_set_batched_calls(0)
        lib.facet_4_cor_corrections(ctypes.byref(st))
        lib.facet_sampling_function(ctypes.byref(st))
        lib.bullseye_set_batched_calls(1)

    if args.eager:
        lib.bullseye_set_batched_profiling(1)

    def step_batched():
        rc = lib.bullseye_grid_batched(ctypes.byref(st), 0, 1)
        if rc:
            check(lib)

    step = step_plain if args.form == "plain" else step_batched

    # the other form, timed the same way, reported beside the headline form
    other = step_batched if args.form == "plain" else step_plain
    other_ms = None
    if not args.no_other:
        other()
        torch.cuda.synchronize()
        check(lib)
        o0 = torch.cuda.Event(enable_timing=True)
        o1 = torch.cuda.Event(enable_timing=True)
        o0.record(stream)
        other()
        o1.record(stream)
        torch.cuda.synchronize()
        other_ms = o0.elapsed_time(o1)
        lib.bullseye_zero_grids()

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    check(lib)
    lib.bullseye_reset_counters()
    clocks = ClockSampler(clocks_path("clocks.csv"))
    clocks.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    if world > 1:
        from bullseye_gb300.sharding import max_over_ranks
        torch.distributed.barrier()
        ms = max_over_ranks(ms, device="cuda")
    clk = clocks.stop()
    launches = int(lib.bullseye_kernel_launches())
    counts = plane_vis_counts(geo)
    plane_width = batched_plane_widths(lib)
    classes = None
    if args.form == "batched" and rank == 0 and not args.no_class_profile and plane_width is not None:
        classes = class_profile(lib, step, counts, plane_width)
        check(lib)
    cnt = ctypes.c_longlong(0)
    vis_kernel_ms = lib.bullseye_gridder_kernel_ms(0, ctypes.byref(cnt))
    n_vis_launch = max(1, cnt.value)
    sf_kernel_ms = lib.bullseye_gridder_kernel_ms(1, ctypes.byref(cnt))
    check(lib)
    ms_per_step = ms / args.steps
    value = pairs_per_step * world / (ms_per_step * 1e-3) / 1e6
    fp32_peak = lib.bullseye_fp32_fma_tflops(4096)
    W = 2 * S_HALF + 1
    bytes_per_pair = 8 * 4 + 4 * 4 + 4 + 12 + 64
    # algorithmic flops: every visibility convolved with its own w plane's true support W_p
    # (complex tap x complex visibility x 4 correlations per facet, the sampling function once),
    # plus phase and Jones per pair -- whatever padding an implementation executes
    true_taps = float(np.sum(counts.astype(np.float64) * np.asarray(supports, np.float64) ** 2))
    step_flops = true_taps * N_FACETS * 8 * 4 + true_taps * 8 + pairs_per_step * (6 * 4 + 128)
    flops_per_pair = step_flops / pairs_per_step
    if args.form == "plain":
        # the visibility gridder launch (CUDA events around it in the library), padded W = 63
        launch_ms = vis_kernel_ms / n_vis_launch
        step_flops = true_taps * N_FACETS * 8 * 4 + pairs_per_step * (6 * 4 + 128)  # visibility launch only
        executed_taps = float(counts.sum()) * W * W
        kernel_name = "romein_grid_kernel<4,wproj,J=8,wide> (visibilities, padded W=63)"
    else:
        # batched: the per-class persistent launches make up the step (timed whole)
        launch_ms = ms_per_step
        executed_taps = sum(t for _, t in class_taps(counts, plane_width).values()) if plane_width is not None else None
        kernel_name = "romein_segment_kernel per support class (whole batched step)"
    achieved = step_flops / (launch_ms * 1e-3) / 1e12
    hbm_gbs = pairs_per_step * bytes_per_pair / (launch_ms * 1e-3) / 1e9
    peaks = json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(REPO, "MEASURED_PEAKS.json")) else {}
    lib.releaseLibrary()
    lib.bullseye_set_device_inputs(0)

    # the row sample of the CPU baseline and the parity check: whole baselines of this workload with
    # its own visibilities and Jones terms
    smp = None
    if rank == 0 and world == 1 and not (args.no_cpu and args.no_parity):
        pick, rows = sample_baselines(geo, args.sample_baselines or 3)
        ants = np.unique(np.concatenate([geo["a1"][rows], geo["a2"][rows]]))
        vis_s = d["vis"][torch.as_tensor(rows.astype(np.int64), device="cuda")].cpu().numpy()
        jones_s = d["jones"][:, torch.as_tensor(ants.astype(np.int64), device="cuda")].cpu().numpy()
        smp = host_sample(geo, pick, vis=vis_s, jones=jones_s)
        del vis_s, jones_s

    # ------------------------------------------------------------- end to end through the C-ABI
    e2e = None
    if not args.no_e2e:
        # the caller's arrays in Measurement Set order (time-major, as a reader delivers them), pinned;
        # each step runs the pipeliner's sequence including repack_input_data
        ms_order = torch.as_tensor(np.lexsort((np.arange(R), geo["tid"].astype(np.int64))), device="cuda")
        host = {k: (v if k in ("jones", "starts") else v[ms_order]).cpu().pin_memory() for k, v in d.items()}
        hnp = {k: v.numpy() for k, v in host.items()}
        hnp["flagged_rows"] = hnp["flagged_rows"].view(np.bool_)
        hnp["flags"] = hnp["flags"].view(np.bool_)
        hnp["starts"] = np.zeros(geo["nb"] + 1, np.uintp)  # filled by repack_input_data
        hnp["tid"] = hnp["tid"].view(np.uintp)
        del d
        torch.cuda.empty_cache()
        P = ctypes.c_void_p
        # the caller's output buffers, allocated once (pinned) and zeroed every step
        out_grid = torch.zeros((N_FACETS, 1, 4, NX, NX), dtype=torch.complex64).pin_memory()
        out_sf = torch.zeros((N_FACETS, 1, 1, NX, NX), dtype=torch.complex64).pin_memory()
        tab2 = Tables(geo, conv)
        tab2.grid, tab2.sf = out_grid.numpy(), out_sf.numpy()
        lib.bullseye_set_host_repack(0)
        lib.bullseye_set_grid_groups(args.grid_groups)
        lib.bullseye_set_host_copy(args.host_copy)

        def copy_gbs(src, dst):  # one large copy between pinned host and device memory
            torch.cuda.synchronize()
            c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            c0.record()
            dst.copy_(src, non_blocking=True)
            c1.record()
            torch.cuda.synchronize()
            return src.numel() * src.element_size() / (c0.elapsed_time(c1) * 1e-3) / 1e9

        probe_dev = torch.empty(host["jones"].numel(), dtype=host["jones"].dtype, device="cuda")
        copy_gbs(host["jones"].view(-1), probe_dev)
        bw = {"pinned_h2d_gbs": copy_gbs(host["jones"].view(-1), probe_dev),
              "pinned_d2h_gbs": copy_gbs(probe_dev, host["jones"].view(-1)), "bytes": int(host["jones"].nbytes)}
        del probe_dev
        probe_dev = torch.empty(host["vis"].numel(), dtype=host["vis"].dtype, device="cuda")
        bw["vis_h2d_gbs"] = copy_gbs(host["vis"].view(-1), probe_dev)
        del probe_dev
        torch.cuda.empty_cache()

        parts = {}

        def e2e_step():
            marks = [time.perf_counter()]
            out_grid.zero_()
            out_sf.zero_()
            s2 = gridding_parameters_type("single")()
            tab2.fill(s2, geo, R)
            lib.initLibrary(ctypes.byref(s2))
            set_rows(s2, hnp, lambda a: a.ctypes.data_as(P))
            s2.is_final_data_chunk = True
            marks.append(time.perf_counter())
            lib.repack_input_data(ctypes.byref(s2))
            # the reference's own call sequence; the exports run the batched gridder unless the
            # plain form is the headline
            lib.bullseye_set_batched_calls(0 if args.form == "plain" else 1)
            lib.facet_4_cor_corrections(ctypes.byref(s2))
            lib.facet_sampling_function(ctypes.byref(s2))
            lib.gridding_barrier()
            marks.append(time.perf_counter())
            lib.weight_uniformly(ctypes.byref(s2))
            marks.append(time.perf_counter())
            lib.normalize(ctypes.byref(s2))
            marks.append(time.perf_counter())
            lib.finalize(ctypes.byref(s2))
            img = float(tab2.grid.view(np.float32).reshape(-1)[0])
            marks.append(time.perf_counter())
            lib.releaseLibrary()
            check(lib)
            marks.append(time.perf_counter())
            for name, t0_, t1_ in zip(("init", "grid", "weight_uniformly", "normalize", "finalize", "release"),
                                      marks[:-1], marks[1:]):
                parts[name] = parts.get(name, 0.0) + (t1_ - t0_) * 1e3
            return img

        e2e_step()
        parts.clear()
        e2e_clocks = ClockSampler(clocks_path("clocks_e2e.csv"))
        e2e_clocks.start()
        if world > 1:
            torch.distributed.barrier()
        t0 = time.perf_counter()
        n_e2e = max(1, min(args.steps, 3))
        for _ in range(n_e2e):
            e2e_step()
        dt = (time.perf_counter() - t0) / n_e2e
        if world > 1:  # every rank runs its own facets concurrently: the slowest one sets the time
            from bullseye_gb300.sharding import max_over_ranks
            dt = max_over_ranks(dt, device="cuda")
        e2e_clk = e2e_clocks.stop()
        ms_by_call = {k: round(v / n_e2e, 1) for k, v in parts.items()}
        # one more step with phase tracing (it synchronises at phase boundaries, so it is not timed)
        lib.bullseye_set_tracing(1)
        e2e_step()
        buf = ctypes.create_string_buffer(1 << 16)
        lib.bullseye_trace_report(buf, len(buf))
        lib.bullseye_set_tracing(0)
        trace = buf.value.decode(errors="replace")
        lib.bullseye_set_host_repack(1)
        lib.bullseye_set_grid_groups(1)
        lib.bullseye_set_host_copy(1)
        h2d = sum(hnp[k].nbytes for k in ("vis", "weights", "flags", "uvw", "flagged_rows", "field", "spw", "a1",
                                          "a2", "tid", "jones"))
        h2d += tab.conv.nbytes + tab.grid.nbytes + tab.sf.nbytes  # tables and initial grids (initLibrary)
        h2d += N_FACETS * NX * NX * 8  # finalize uploads the first cube slice of each facet
        d2h = tab.grid.nbytes + tab.sf.nbytes + N_FACETS * NX * NX * (8 + 4)
        e2e = {"value": pairs_per_step * world / dt / 1e6, "unit": "Mvis/s", "h2d_bytes_per_step": int(h2d * world),
               "d2h_bytes_per_step": int(d2h * world), "s_per_step": dt,
               "ms_by_call": ms_by_call, "clocks": e2e_clk,
               "trace_of_one_step_ms": trace, "grid_groups": args.grid_groups, "copy_bandwidth": bw,
               "host_copy": "SM kernels" if args.host_copy else "copy engines",
               "calls": ("initLibrary, repack_input_data (baseline starts; rows sorted on the device), "
                         "facet_4_cor_corrections, facet_sampling_function (" +
                         ("plain kernels" if args.form == "plain" else "batched support-aware gridder") +
                         "), gridding_barrier, weight_uniformly, normalize, finalize, releaseLibrary; rows handed "
                         "over in Measurement Set (time-major) order from pinned host arrays, output buffers pinned "
                         "and zeroed every step")}

    cpu = None
    if not args.no_cpu and smp is not None:
        cpu = cpu_baseline(geo, conv, args.cpu_seconds, smp=smp)
    parity = None
    if not args.no_parity and smp is not None:
        lib.bullseye_set_batched_calls(0 if args.form == "plain" else 1)
        parity = parity_check(lib, geo, conv, smp)
        lib.bullseye_set_batched_calls(1)
    precision = None
    if not args.no_precision and rank == 0 and world == 1:
        precision = precision_report()

    if rank == 0:
        line = {
            "metric": "gridded Mvis/s (vis x facet pairs)", "value": value, "unit": "Mvis/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "rows": R, "channels": N_CHAN, "facets": N_FACETS,
                       "vis_facet_pairs_per_step": pairs_per_step, "l2": "inputs 4.2 GB per step > 129 MB L2",
                       "form": ("batched: bullseye_grid_batched (support-aware, persistent per-class launches, "
                                "CUDA graph, compensated FP32)" if args.form == "batched" else
                                "plain: per-call drop-in ABI path (padded support, compensated FP32)")},
            "other_form": None if other_ms is None else {
                "form": "plain" if args.form == "batched" else "batched", "ms_per_step": other_ms,
                "value": pairs_per_step * world / (other_ms * 1e-3) / 1e6, "unit": "Mvis/s"},
            "batched_over_plain": None if other_ms is None else (
                other_ms / ms_per_step if args.form == "batched" else ms_per_step / other_ms),
            "parity": parity,
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                         "frac": achieved / fp32_peak if fp32_peak else None,
                         "traffic": (TRAFFIC_BYTES_PER_PAIR * pairs_per_step
                                     if args.form == "batched" and not args.chans and not args.facets else None),
                         "traffic_source": TRAFFIC_SOURCE if args.form == "batched" else None,
                         "algorithmic_bytes": pairs_per_step * bytes_per_pair,
                         "peak_source": "measured FP32 FMA probe on this GPU (MEASURED_PEAKS.json has no FP32 rate)",
                         "kernel": kernel_name, "launch_ms": launch_ms,
                         "flops_per_pair": flops_per_pair,
                         "flops_rule": "8 x 4 corr x W_p^2 per (vis, facet) with W_p the visibility's w-plane "
                                       "support (+ sampling function once, + 152 for phase and Jones)",
                         "executed_taps_per_vis": executed_taps / float(counts.sum()) if executed_taps else None,
                         "true_taps_per_vis": true_taps / float(counts.sum()),
                         "hbm_gbs": hbm_gbs,
                         "hbm_frac_of_measured": hbm_gbs / peaks["hbm_gbs"] if peaks.get("hbm_gbs") else None,
                         "sampling_kernel_ms": sf_kernel_ms / max(1, cnt.value)},
            "clocks": clk, "gpu_launches": launches, "e2e": e2e, "cpu_baseline": cpu, "precision": precision,
            "class_profile": classes,
        }
        print(json.dumps(line))


if __name__ == "__main__":
    main()
