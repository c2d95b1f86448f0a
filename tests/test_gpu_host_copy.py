"""Bulk copies of the caller's host buffers and the row staging limit (rows.cu).

The caller's rows, Jones terms and grids in page-locked memory are copied by SM kernels over the
CPU-GPU link (bullseye_set_host_copy(1), the default); with mode 0, or from pageable memory, by
the copy engines.  Every form must give the oracle's grids, sampling function and normalisation
(1e-12 for the 64-bit library, 1e-5 for the 32-bit one) and the same finalized images:

* pinned arrays at offset 0 (16-byte aligned), 8 (4-byte units) and 1 byte (byte copies, and an
  unaligned head and tail) into their allocations, with SM copies and with the copy engines;
* rows of one call split by a small staging limit (bullseye_set_max_stage_bytes) into several
  chunks gridded in one group.
"""
import numpy as np
import pytest

from bullseye_gb300 import synth
from bullseye_gb300.imaging import pinned_host, run_imaging
from tests.golden.cases import cpu_conv
from tests.test_gpu_parity import gpu_libs, oracle_libs, rel  # noqa: F401

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rows_problem():
    p = synth.small_problem("double", nx=128, n_ant=41, n_times=40, n_chan=2, n_facets=2, jones=True, s=4, os=9,
                            wplanes=4, min_support=5)
    return p


_REFS = {}


def _reference(p, oracle):
    if p.precision not in _REFS:
        q = p.astype("double")
        _REFS[p.precision] = run_imaging(oracle, q.with_conv(cpu_conv(q)), "facet_4_cor_corrections", repack=True,
                                         keep_raw=True, uniform=True, do_finalize=True)
    return _REFS[p.precision]


def _tol(precision):
    return 1e-12 if precision == "double" else 1e-5


@pytest.mark.parametrize("precision", ["double", "single"])
@pytest.mark.parametrize("mode", [1, 0])
@pytest.mark.parametrize("offset", [0, 8, 1])
def test_pinned_buffers_match_oracle(precision, mode, offset, rows_problem, gpu_libs, oracle_libs):
    from bullseye_gb300.library import check
    p = rows_problem.astype(precision)
    lib = gpu_libs[precision]
    lib.bullseye_set_host_copy(mode)
    try:
        res = run_imaging(lib, p, "facet_4_cor_corrections", repack=True, keep_raw=True, uniform=True,
                          do_finalize=True, norm_bins=(2 * p.conv_support + 1) ** 2, host_alloc=pinned_host(offset))
    finally:
        lib.bullseye_set_host_copy(1)
    check(lib)
    ref = _reference(p, oracle_libs["double"])
    tol = _tol(precision)
    assert np.max(np.abs(ref.raw_grid)) > 0
    assert rel(res.raw_grid, ref.raw_grid) <= tol
    assert rel(res.sampling, ref.sampling) <= tol
    assert rel(res.normalization, ref.normalization) <= (1e-12 if precision == "double" else 1e-6)
    assert rel(res.image, ref.image) <= tol


@pytest.mark.parametrize("precision", ["double", "single"])
@pytest.mark.parametrize("host", ["pinned", "pageable"])
def test_staging_limit_splits_rows_into_chunks(precision, host, rows_problem, gpu_libs, oracle_libs):
    """A 1 MB staging limit splits the call's 32,800 rows (about 8 MB) into several chunks, each
    sorted and tracked on its own, all gridded after the last one."""
    from bullseye_gb300.library import check
    p = rows_problem.astype(precision)
    lib = gpu_libs[precision]
    lib.bullseye_set_max_stage_bytes(1 << 20)
    try:
        res = run_imaging(lib, p, "facet_4_cor_corrections", repack=True, keep_raw=True, uniform=True,
                          do_finalize=True, norm_bins=(2 * p.conv_support + 1) ** 2,
                          host_alloc=pinned_host() if host == "pinned" else None)
    finally:
        lib.bullseye_set_max_stage_bytes(0)
    check(lib)
    ref = _reference(p, oracle_libs["double"])
    tol = _tol(precision)
    assert rel(res.raw_grid, ref.raw_grid) <= tol
    assert rel(res.sampling, ref.sampling) <= tol
    assert rel(res.image, ref.image) <= tol
