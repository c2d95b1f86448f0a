"""The batched, support-aware form against the per-call drop-in path and the oracle.

bullseye_grid_batched grids each visibility over its w plane's nonzero support window and builds
its schedule on the device (replayed as a CUDA graph); the grids must be the ones the per-call
ABI path produces: 1e-12 relative in double precision (against the oracle), 1e-5 in single
precision (against the FP64 oracle on the same float inputs).
"""
import numpy as np
import pytest

from bullseye_gb300 import synth
from bullseye_gb300.imaging import run_imaging
from tests.golden.cases import cpu_conv

pytestmark = pytest.mark.gpu

CALLS = {"facet_4_cor_corrections": 0, "facet_4_cor": 1, "grid_4_cor": 2}


class Batched:
    """Presents bullseye_grid_batched under the names run_imaging calls."""

    def __init__(self, lib, call):
        self._lib = lib
        self._call = call

    def __getattr__(self, name):
        import ctypes
        if name == self._call:
            def grid(st):
                rc = self._lib.bullseye_grid_batched(st, CALLS[self._call], 1)
                assert rc == 0, rc
            return grid
        if name in ("facet_sampling_function", "grid_sampling_function"):
            return lambda st: None  # gridded by the batched call
        return getattr(self._lib, name)


def rel(a, b):
    s = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / s) if s else float(np.max(np.abs(a - b)))


@pytest.fixture(scope="module")
def libs(gpu_required, built_libraries):
    from bullseye_gb300.library import load_library
    return {p: load_library("GPU", p) for p in ("single", "double")}


@pytest.fixture(scope="module")
def oracles(oracle_built):
    from oracle.harness import load_oracle
    return {p: load_oracle(p) for p in ("single", "double")}


def _run(lib, p, call, **kw):
    from bullseye_gb300.library import check
    res = run_imaging(Batched(lib, call), p, call, repack=True, keep_raw=True, psf=True,
                      norm_bins=(2 * p.conv_support + 1) ** 2, **kw)
    check(lib)
    return res


@pytest.mark.parametrize("call", sorted(CALLS))
def test_batched_wproj_fp64_matches_oracle(call, libs, oracles):
    nf = 3 if call.startswith("facet") else 0
    p = synth.small_problem("double", nx=128, n_ant=7, n_times=12, n_chan=3, s=15, os=5, wplanes=8, min_support=5,
                            n_facets=nf, jones=call.endswith("corrections"))
    res = _run(libs["double"], p, call)
    ref = run_imaging(oracles["double"], p.with_conv(cpu_conv(p)), call, keep_raw=True, psf=True)
    assert rel(res.raw_grid, ref.raw_grid) <= 1e-12
    assert rel(res.normalization, ref.normalization) <= 1e-12
    assert rel(res.sampling, ref.sampling) <= 1e-12


@pytest.mark.parametrize("chunks", [1, 3])
def test_batched_wproj_fp32_within_1e5(chunks, libs, oracles):
    p32 = synth.small_problem("single", nx=192, n_ant=7, n_times=14, n_chan=4, s=31, os=5, wplanes=16, min_support=7,
                              n_facets=4, jones=True)
    res = _run(libs["single"], p32, "facet_4_cor_corrections", chunks=chunks, uniform=True)
    p64 = p32.astype("double")
    ref = run_imaging(oracles["double"], p64.with_conv(cpu_conv(p64)), "facet_4_cor_corrections", keep_raw=True,
                      psf=True, uniform=True)
    assert rel(res.raw_grid, ref.raw_grid) <= 1e-5
    assert rel(res.normalization, ref.normalization) <= 1e-6
    assert rel(res.sampling, ref.sampling) <= 1e-5


def test_batched_aa_matches_per_call(libs):
    from bullseye_gb300.library import check
    p = synth.small_problem("single", nx=96, n_ant=8, n_times=10, n_chan=2, s=3, os=63)
    libs["single"].bullseye_set_batched_calls(0)  # the plain per-track kernels as the reference
    try:
        per_call = run_imaging(libs["single"], p, "grid_4_cor", repack=True, keep_raw=True, psf=True, norm_bins=49)
    finally:
        libs["single"].bullseye_set_batched_calls(1)
    check(libs["single"])
    res = _run(libs["single"], p, "grid_4_cor")
    assert rel(res.raw_grid, per_call.raw_grid) <= 1e-6
    assert rel(res.normalization, per_call.normalization) <= 1e-9
    assert rel(res.sampling, per_call.sampling) <= 1e-6


def test_batched_graph_replay_is_stable(libs):
    """Replaying the captured graph (same chunk twice) doubles the grids exactly as two calls would."""
    import ctypes
    from bullseye_gb300.library import check
    lib = libs["double"]
    p = synth.small_problem("double", nx=96, n_ant=6, n_times=8, n_chan=2, s=7, os=5, wplanes=4, min_support=5,
                            n_facets=2)
    one = _run(lib, p, "facet_4_cor")
    # two identical chunks: the second batched call replays the captured graph
    p2 = synth.small_problem("double", nx=96, n_ant=6, n_times=8, n_chan=2, s=7, os=5, wplanes=4, min_support=5,
                             n_facets=2)
    for name in ("vis", "uvw", "weights", "flags", "flagged_rows", "field_ids", "spw_ids", "antenna1", "antenna2",
                 "timestamp_ids"):
        setattr(p2, name, np.concatenate([getattr(p, name)] * 2))
    two = _run(lib, p2, "facet_4_cor", chunks=2)
    assert rel(two.raw_grid, 2 * one.raw_grid) <= 1e-12
    assert rel(two.normalization, 2 * one.normalization) <= 1e-12


@pytest.mark.parametrize("precision", ["single", "double"])
def test_bounded_wait_runs_out_and_reports(precision, gpu_required, built_libraries):
    """The tap-copy barrier's wait is bounded: a barrier that never completes (one arrival of two)
    makes the wait run out and record the timeout bit, and the context stays usable."""
    import torch
    from bullseye_gb300.library import load_library
    lib = load_library("GPU", precision)
    assert lib.bullseye_selftest_bounded_wait() == 16
    x = torch.ones(1024, device="cuda")
    assert float(x.sum()) == 1024.0  # the device still runs work afterwards


def test_tracing_reports_the_phases_of_a_call(libs):
    """bullseye_set_tracing records the phases of the batched gridding calls: upload and prepare,
    schedule/tune/capture, the class kernels and copy-back; the report empties the log."""
    import ctypes
    lib = libs["single"]
    p = synth.small_problem("single", nx=96, n_ant=6, n_times=8, n_chan=2, s=7, os=5, wplanes=4, min_support=5,
                            n_facets=2, jones=True)
    lib.bullseye_set_tracing(1)
    try:
        run_imaging(lib, p, "facet_4_cor_corrections", repack=True, keep_raw=True, psf=True)
        buf = ctypes.create_string_buffer(1 << 16)
        n = lib.bullseye_trace_report(buf, len(buf))
        log = buf.value.decode()
        assert n > 0 and n == len(log)
        for phase in ("vis.upload_prepare", "schedule_tune_capture", "vis.grid", "vis.copy_back", "sf.grid"):
            assert phase in log, (phase, log)
        assert lib.bullseye_trace_report(buf, len(buf)) == 0  # emptied by the report
    finally:
        lib.bullseye_set_tracing(0)
