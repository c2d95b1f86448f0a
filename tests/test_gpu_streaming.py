"""Host-input gridding streams its rows: rows are uploaded on a copy stream and sorted by
baseline on the device, in one chunk per call, or, gridded in groups, in chunks gridded while the
next chunk uploads (rows.cu).

* 41 antennas x 80 timesteps = 65,600 cross rows in Measurement Set order
  (time-major); repack_input_data either permutes the caller's arrays (the reference's behaviour,
  the default) or, with bullseye_set_host_repack(0), only fills the baseline starts.  Both must
  match the FP64 oracle to 1e-12 (64-bit library) and 1e-5 (32-bit), with Jones terms and
  uniform weighting, through the batched and the plain kernels, and over two chunked calls
  without a barrier between their gridding calls;
* with host repack off, the caller's arrays are left in place.
"""
import numpy as np
import pytest

from bullseye_gb300 import synth
from bullseye_gb300.imaging import run_imaging
from tests.golden.cases import cpu_conv
from tests.test_gpu_parity import gpu_libs, oracle_libs, rel  # noqa: F401

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def many_rows():
    p = synth.small_problem("double", nx=128, n_ant=41, n_times=80, n_chan=2, n_facets=2, jones=True, s=4, os=9,
                            wplanes=4, min_support=5)
    assert p.rows > 65536
    return p


class _NoHostRepack:
    """The library with bullseye_set_host_repack(0) for the run."""

    def __init__(self, lib):
        self.lib = lib

    def __getattr__(self, k):
        return getattr(self.lib, k)

    def initLibrary(self, st):
        self.lib.bullseye_set_host_repack(0)
        self.lib.initLibrary(st)

    def releaseLibrary(self):
        self.lib.releaseLibrary()
        self.lib.bullseye_set_host_repack(1)


_REFS = {}


def _reference(p, oracle):
    if p.precision not in _REFS:
        q = p.astype("double")
        _REFS[p.precision] = run_imaging(oracle, q.with_conv(cpu_conv(q)), "facet_4_cor_corrections", keep_raw=True,
                                         uniform=True)
    return _REFS[p.precision]


@pytest.mark.parametrize("precision", ["double", "single"])
@pytest.mark.parametrize("host_repack", [True, False])
@pytest.mark.parametrize("form", ["batched", "plain"])
@pytest.mark.parametrize("chunks", [1, 2])
def test_streamed_rows_match_oracle(precision, host_repack, form, chunks, many_rows, gpu_libs, oracle_libs):
    """chunks = 1: one call of 65,600 rows; chunks = 2: two calls."""
    from bullseye_gb300.library import check
    p = many_rows.astype(precision)
    lib = gpu_libs[precision]
    lib.bullseye_set_batched_calls(1 if form == "batched" else 0)
    try:
        res = run_imaging(lib if host_repack else _NoHostRepack(lib), p, "facet_4_cor_corrections", repack=True,
                          keep_raw=True, uniform=True, chunks=chunks, norm_bins=(2 * p.conv_support + 1) ** 2)
    finally:
        lib.bullseye_set_batched_calls(1)
        lib.bullseye_set_host_repack(1)
    check(lib)
    ref = _reference(p, oracle_libs["double"])
    tol = 1e-12 if precision == "double" else 1e-5
    assert rel(res.raw_grid, ref.raw_grid) <= tol
    assert rel(res.normalization, ref.normalization) <= (1e-12 if precision == "double" else 1e-6)
    assert rel(res.sampling, ref.sampling) <= tol


def test_host_repack_off_leaves_caller_arrays(many_rows, gpu_libs):
    import ctypes
    from bullseye_gb300.abi import gridding_parameters_type
    from bullseye_gb300.imaging import baseline_index
    lib = gpu_libs["double"]
    p = many_rows
    a1, a2 = p.antenna1.astype(np.uint32).copy(), p.antenna2.astype(np.uint32).copy()
    uvw = np.ascontiguousarray(p.uvw).copy()
    starts = np.zeros(p.baseline_count + 1, np.uintp)
    st = gridding_parameters_type("double")()
    st.row_count, st.baseline_count, st.antenna_count = p.rows, p.baseline_count, p.n_antennas
    st.channel_count, st.number_of_polarization_terms = p.channels, 4
    P = ctypes.c_void_p
    st.antenna_1_ids, st.antenna_2_ids = a1.ctypes.data_as(P), a2.ctypes.data_as(P)
    st.uvw_coords = uvw.ctypes.data_as(P)
    st.baseline_starting_indexes = starts.ctypes.data_as(P)
    lib.bullseye_set_host_repack(0)
    try:
        lib.repack_input_data(ctypes.byref(st))
    finally:
        lib.bullseye_set_host_repack(1)
    assert np.array_equal(a1, p.antenna1) and np.array_equal(uvw, p.uvw)
    counts = np.bincount(baseline_index(p.antenna1, p.antenna2, p.n_antennas), minlength=p.baseline_count)
    assert np.array_equal(starts, np.concatenate([[0], np.cumsum(counts)]).astype(np.uintp))


@pytest.mark.parametrize("precision", ["double", "single"])
def test_grouped_gridding_matches_oracle(precision, many_rows, gpu_libs, oracle_libs):
    """bullseye_set_grid_groups(2): the two row chunks of one call are gridded as they arrive."""
    from bullseye_gb300.library import check
    p = many_rows.astype(precision)
    lib = gpu_libs[precision]
    lib.bullseye_set_grid_groups(2)
    try:
        res = run_imaging(_NoHostRepack(lib), p, "facet_4_cor_corrections", repack=True, keep_raw=True, uniform=True,
                          norm_bins=(2 * p.conv_support + 1) ** 2)
    finally:
        lib.bullseye_set_grid_groups(1)
        lib.bullseye_set_host_repack(1)
    check(lib)
    ref = _reference(p, oracle_libs["double"])
    tol = 1e-12 if precision == "double" else 1e-5
    assert rel(res.raw_grid, ref.raw_grid) <= tol
    assert rel(res.sampling, ref.sampling) <= tol
