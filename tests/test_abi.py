"""CPU tests of the C-ABI boundary: struct layout, exported symbols, host-only entry points."""
import ctypes
import os
import re

import numpy as np
import pytest

from bullseye_gb300.abi import EXPECTED_OFFSETS, EXPECTED_SIZEOF, REFERENCE_EXPORTS, gridding_parameters_type

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("precision", ["single", "double"])
def test_struct_layout_matches_reference(precision):
    cls = gridding_parameters_type(precision)
    assert ctypes.sizeof(cls) == EXPECTED_SIZEOF[precision]
    for field, off in EXPECTED_OFFSETS[precision].items():
        assert getattr(cls, field).offset == off, field


def declared_symbols():
    text = open(os.path.join(REPO, "include", "bullseye_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\([^;{]*\)\s*;", text)))


@pytest.mark.parametrize("lang", ["c99", "c++17"])
def test_header_compiles_as_plain_c_and_cpp(lang, tmp_path):
    """The boundary header is what a cgo / ctypes / JNI binding includes: it must stand alone in C
    (no C++ types) and in C++, warning-free."""
    import shutil
    import subprocess
    cc = shutil.which("gcc" if lang == "c99" else "g++")
    if cc is None:
        pytest.skip("no host compiler")
    src = tmp_path / ("use.c" if lang == "c99" else "use.cpp")
    # the struct is opaque in the header (callers pass the reference's struct by pointer)
    src.write_text('#include "bullseye_gb300.h"\nint main(void) { gridding_parameters *p = 0; return p != 0; }\n')
    cmd = [cc, "-std=" + lang, "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(REPO, "include"),
           "-c", str(src), "-o", str(tmp_path / "use.o")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_header_declares_every_reference_export():
    syms = declared_symbols()
    for name in REFERENCE_EXPORTS:
        assert name in syms, name


@pytest.mark.parametrize("precision", ["single", "double"])
def test_library_loads_and_exports_header_symbols(precision, built_libraries):
    from bullseye_gb300.build import library_path
    lib = ctypes.CDLL(library_path(precision))
    for name in declared_symbols():
        assert hasattr(lib, name), name
    lib.bullseye_precision_bits.restype = ctypes.c_int
    assert lib.bullseye_precision_bits() == (32 if precision == "single" else 64)


def test_repack_input_data_is_a_stable_baseline_sort(built_libraries):
    """repack_input_data (host-only) against a numpy stable sort by baseline slot."""
    from bullseye_gb300 import synth
    from bullseye_gb300.imaging import baseline_index
    from bullseye_gb300.library import load_library
    lib = load_library("GPU", "double")
    p = synth.small_problem("double", n_ant=6, n_times=7, n_chan=3)
    rng = np.random.default_rng(0)
    perm = rng.permutation(p.rows)  # scramble the rows first
    arrays = dict(vis=p.vis[perm].copy(), uvw=p.uvw[perm].copy(), wt=p.weights[perm].copy(),
                  fl=p.flags[perm].copy(), fr=p.flagged_rows[perm].copy(), spw=p.spw_ids[perm].copy(),
                  a1=p.antenna1[perm].copy(), a2=p.antenna2[perm].copy(), field=p.field_ids[perm].copy(),
                  t=p.timestamp_ids[perm].copy())
    starts = np.zeros(p.baseline_count + 1, np.uintp)
    st = gridding_parameters_type("double")()
    P = ctypes.c_void_p
    st.visibilities = arrays["vis"].ctypes.data_as(P)
    st.uvw_coords = arrays["uvw"].ctypes.data_as(P)
    st.visibility_weights = arrays["wt"].ctypes.data_as(P)
    st.flags = arrays["fl"].ctypes.data_as(P)
    st.flagged_rows = arrays["fr"].ctypes.data_as(P)
    st.spw_index_array = arrays["spw"].ctypes.data_as(P)
    st.antenna_1_ids = arrays["a1"].ctypes.data_as(P)
    st.antenna_2_ids = arrays["a2"].ctypes.data_as(P)
    st.field_array = arrays["field"].ctypes.data_as(P)
    st.timestamp_ids = arrays["t"].ctypes.data_as(P)
    st.should_invert_jones_terms = True
    st.baseline_starting_indexes = starts.ctypes.data_as(P)
    st.row_count = p.rows
    st.baseline_count = p.baseline_count
    st.antenna_count = p.n_antennas
    st.channel_count = p.channels
    st.number_of_polarization_terms = p.n_pol
    lib.repack_input_data(ctypes.byref(st))
    b = baseline_index(p.antenna1[perm], p.antenna2[perm], p.n_antennas)
    order = np.argsort(b, kind="stable")
    np.testing.assert_array_equal(arrays["vis"], p.vis[perm][order])
    np.testing.assert_array_equal(arrays["uvw"], p.uvw[perm][order])
    np.testing.assert_array_equal(arrays["fl"], p.flags[perm][order])
    np.testing.assert_array_equal(arrays["t"], p.timestamp_ids[perm][order])
    counts = np.bincount(b, minlength=p.baseline_count)
    np.testing.assert_array_equal(starts, np.concatenate([[0], np.cumsum(counts)]))


@pytest.mark.parametrize("precision", ["single", "double"])
def test_workspace_size_covers_the_support_aware_schedule(precision, built_libraries):
    """bullseye_facet_4_cor_corrections_ws_bytes (host-only): the compensation grid (32-bit library),
    the facet table and an error word, plus the support-aware form's tables and run schedule, which
    grow by about 33 bytes per (row, channel)."""
    from bullseye_gb300.library import load_library
    lib = load_library("GPU", precision)

    def size(rows, chans=32, nx=512, wplanes=32, support=15):
        st = gridding_parameters_type(precision)()
        st.row_count = rows
        st.channel_count = chans
        st.spw_count = 1
        st.nx = st.ny = nx
        st.num_facet_centres = 2
        st.cube_channel_dim_size = 1
        st.number_of_polarization_terms = st.number_of_polarization_terms_being_gridded = 4
        st.conv_support, st.conv_oversample, st.wplanes = support, 15, wplanes
        st.baseline_count = 0
        return int(lib.bullseye_facet_4_cor_corrections_ws_bytes(ctypes.byref(st)))

    grid_bytes = 2 * 4 * 512 * 512 * 8 if precision == "single" else 0
    small, large = size(1000), size(101000)
    assert small >= grid_bytes
    per_vis = (large - small) / (100000 * 32)
    assert 32.0 <= per_vis <= 34.0, per_vis
    assert size(1000, wplanes=64) > small  # the window table grows with the w planes
