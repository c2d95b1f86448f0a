"""Visibility records of the batched gridder (batched.cu record_kernel, gridder.cuh grid_track_pre).

A batched call first writes one record per (row, facet, channel) of its work and the
normalisation sums; the class launches then stage records and taps by bulk copies.  Work past the
record budget is prepared in place by the class launches, as with records off.  All three forms
must match the FP64 oracle (1e-12 for the 64-bit library, 1e-5 for the 32-bit one), with Jones
terms, w-projection, faceting and uniform weighting:

* records on (the default): every work item from records;
* records off (bullseye_set_visibility_records(0)): every work item prepared in place;
* a 1 MB record budget: the first segments from records, the rest in place, in the same launches;
* records reading the original [T][A][F][S][Ch] Jones table instead of the time-innermost copy
  (bullseye_set_jones_time_major(0)).
"""
import pytest

from bullseye_gb300 import synth
from bullseye_gb300.imaging import run_imaging
from tests.golden.cases import cpu_conv
from tests.test_gpu_parity import gpu_libs, oracle_libs, rel  # noqa: F401

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def problem():
    return synth.small_problem("double", nx=128, n_ant=24, n_times=60, n_chan=3, n_facets=3, jones=True, s=6, os=9,
                               wplanes=8, min_support=5)


_REFS = {}


def _reference(p, oracle):
    if p.precision not in _REFS:
        q = p.astype("double")
        _REFS[p.precision] = run_imaging(oracle, q.with_conv(cpu_conv(q)), "facet_4_cor_corrections", keep_raw=True,
                                         uniform=True)
    return _REFS[p.precision]


@pytest.mark.parametrize("precision", ["double", "single"])
@pytest.mark.parametrize("form", ["records", "in_place", "partial", "jones_original_layout"])
def test_record_forms_match_oracle(precision, form, problem, gpu_libs, oracle_libs):
    from bullseye_gb300.library import check
    p = problem.astype(precision)
    lib = gpu_libs[precision]
    lib.bullseye_set_batched_calls(1)
    lib.bullseye_set_visibility_records(0 if form == "in_place" else 1)
    lib.bullseye_set_record_budget((1 << 20) if form == "partial" else 0)
    lib.bullseye_set_jones_time_major(0 if form == "jones_original_layout" else 1)
    try:
        res = run_imaging(lib, p, "facet_4_cor_corrections", keep_raw=True, uniform=True,
                          norm_bins=(2 * p.conv_support + 1) ** 2)
    finally:
        lib.bullseye_set_visibility_records(1)
        lib.bullseye_set_record_budget(0)
        lib.bullseye_set_jones_time_major(1)
    check(lib)
    ref = _reference(p, oracle_libs["double"])
    tol = 1e-12 if precision == "double" else 1e-5
    assert rel(res.raw_grid, ref.raw_grid) <= tol
    assert rel(res.normalization, ref.normalization) <= (1e-12 if precision == "double" else 1e-6)
    assert rel(res.sampling, ref.sampling) <= tol


def _aa_faceted():
    return synth.small_problem("single", nx=128, n_ant=24, n_times=60, n_chan=3, n_facets=3, jones=True, s=3, os=15)


def _bench_shape():
    # the benchmark's kernel stack and facets (EVLA-27, 16 facets, 64 w planes, os 15, Jones)
    return synth.config2("single", n_times=16, n_chan=8, n_facets=16, nx=1024, cell=5.0, wplanes=64, s=31,
                         min_support=15, os=15, n_src=50)


@pytest.mark.parametrize("shape", ["bench_wproj", "aa_faceted"])
def test_single_precision_records_match_in_place(shape, gpu_libs):
    """The record kernel chooses cells and taps with double-float arithmetic, the in-place prologue
    with FP64: the grids agree to the FP32 accumulation noise (a tap moved by one oversampled step
    in any visibility would show at about 1e-4 of the grid maximum)."""
    from tests.test_gpu_parity import run_gpu
    p = _bench_shape() if shape == "bench_wproj" else _aa_faceted()
    lib = gpu_libs["single"]
    lib.bullseye_set_batched_calls(1)
    out = {}
    for form in ("records", "in_place"):
        lib.bullseye_set_visibility_records(1 if form == "records" else 0)
        try:
            out[form] = run_gpu(lib, p, "facet_4_cor_corrections", keep_raw=True, uniform=True)
        finally:
            lib.bullseye_set_visibility_records(1)
    assert rel(out["records"].raw_grid, out["in_place"].raw_grid) <= 2e-6
    assert rel(out["records"].normalization, out["in_place"].normalization) <= 1e-6
    assert rel(out["records"].sampling, out["in_place"].sampling) <= 2e-6
