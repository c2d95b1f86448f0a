"""GPU nearest-neighbour sampling counts, bit for bit against the reference and the oracle.

* the fixtures made by the reference's own nearest-neighbour gridder (tests/golden/nn_counts_*.npz):
  a third of the samples sit within 1e-5 pixels of a half-integer, where only the reference's exact
  operation sequence gives the same cell;
* a config-1 sized problem (64 antennas, 120 timesteps, 1024^2) against the oracle restatement.
"""
import ctypes
import os

import numpy as np
import pytest

from tests.golden.nn_cases import FACETS, NX, NY, SF_CH, make_struct

from bullseye_gb300 import synth

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _device_counts(lib, precision, d, faceting, nx, ny, sf_ch, facets, struct_fn):
    import torch
    def same_bits(v):
        v = np.ascontiguousarray(v)
        if v.dtype == np.bool_:
            return v.astype(np.uint8)
        if v.dtype.kind == "u" and v.dtype.itemsize > 1:  # torch lacks most unsigned types
            return v.view({4: np.int32, 8: np.int64}[v.dtype.itemsize])
        return v
    dev = {k: torch.as_tensor(same_bits(v)).cuda() for k, v in d.items()
           if isinstance(v, np.ndarray) and k != "phase_centre"}
    dev["phase_centre"] = d["phase_centre"]
    F = facets if faceting else 1
    counts = torch.zeros((F, sf_ch, ny, nx), dtype=torch.int32, device="cuda")
    ptr = lambda t: ctypes.c_void_p(t.data_ptr()) if hasattr(t, "data_ptr") else None  # noqa: E731
    st = struct_fn(dev, ptr, ctypes.c_void_p(counts.data_ptr()))
    rc = lib.bullseye_sampling_counts_nn(ctypes.byref(st), ctypes.c_void_p(counts.data_ptr()), faceting,
                                         ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0
    return counts.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("precision", ["single", "double"])
@pytest.mark.parametrize("faceting", [0, 1])
def test_counts_match_reference_fixture(precision, faceting, gpu_required, built_libraries):
    from bullseye_gb300.library import check, load_library
    lib = load_library("GPU", precision)
    fx = np.load(os.path.join(HERE, "golden", f"nn_counts_{precision}.npz"))
    d = {k[3:]: fx[k] for k in fx.files if k.startswith("in_")}
    got = _device_counts(lib, precision, d, faceting, NX, NY, SF_CH, FACETS,
                         lambda dev, ptr, buf: make_struct(precision, dev, bool(faceting), ptr, buf))
    check(lib)
    want = fx["counts_facet" if faceting else "counts_grid"]
    assert got.shape == want.shape
    assert np.array_equal(got, want), int(np.abs(got.astype(np.int64) - want).sum())


@pytest.mark.parametrize("precision", ["single", "double"])
def test_counts_match_oracle_config1(precision, gpu_required, built_libraries, oracle_built):
    from bullseye_gb300.abi import complex_dtype, gridding_parameters_type
    from bullseye_gb300.library import check, load_library
    from oracle.harness import load_oracle
    from tests.golden.nn_cases import host_ptr
    p = synth.config1(precision, n_times=60)
    d = dict(uvw=p.uvw, lam=p.wavelengths.reshape(-1), spw=p.spw_ids, field=p.field_ids,
             flagged_rows=p.flagged_rows, enabled=np.ones(p.spws * p.channels, np.bool_),
             sfcgi=np.zeros(p.spws * p.channels, np.uintp), phase_centre=np.asarray(p.phase_centre))

    def struct(arr, ptr, buf):
        st = gridding_parameters_type(precision)()
        st.uvw_coords, st.reference_wavelengths, st.spw_index_array = ptr(arr["uvw"]), ptr(arr["lam"]), ptr(arr["spw"])
        st.field_array, st.flagged_rows, st.enabled_channels = ptr(arr["field"]), ptr(arr["flagged_rows"]), ptr(arr["enabled"])
        st.sampling_function_channel_grid_indicies = ptr(arr["sfcgi"])
        st.sampling_function_buffer = buf
        st.sampling_function_channel_count = 1
        st.row_count, st.channel_count, st.spw_count = p.rows, p.channels, p.spws
        st.nx, st.ny = p.nx, p.ny
        st.cell_size_x, st.cell_size_y = p.cell_x, p.cell_y
        st.num_facet_centres = 1
        st.phase_centre_ra, st.phase_centre_dec = p.phase_centre
        st.conv_support, st.conv_oversample = 0, 1
        return st

    lib = load_library("GPU", precision)
    got = _device_counts(lib, precision, d, 0, p.nx, p.ny, 1, 1, struct)
    check(lib)
    orc = load_oracle(precision)
    buf = np.zeros((1, 1, p.ny, p.nx), complex_dtype(precision))
    st = struct(d, host_ptr, host_ptr(buf))
    orc.oracle_sampling_counts_nn(ctypes.byref(st), 0)
    want = buf.real.astype(np.uint32)
    assert int(want.sum()) > 100000
    assert np.array_equal(got, want)
