"""Device-side errors and argument rejection of the device-pointer gridding entries.

bullseye_facet_4_cor_corrections_noalloc and bullseye_facet_4_cor_corrections_ws queue their work
without synchronising, so an error found by a kernel (a singular Jones matrix, which is zeroed as
the reference's jones_2x2.h invert_all does before it throws, or an id out of range) is written to
the call's error word; bullseye_facet_4_cor_corrections_status reads it back and reports it through
bullseye_last_error.  A call whose arguments are rejected must leave the caller's arrays untouched
(the entries invert jones_terms in place only once every check has passed).  The workspace entry
runs persistent per-class launches, so it is not bound by the 2^31 CTAs of the plain kernel.
"""
import ctypes

import numpy as np
import pytest

from bullseye_gb300 import synth
from tests.test_zz_no_alloc import _device_struct, _rel

pytestmark = pytest.mark.gpu


def _problem(**kw):
    args = dict(nx=96, n_ant=6, n_times=6, n_chan=2, n_facets=2, jones=True, s=4, os=9, wplanes=4, min_support=5)
    args.update(kw)
    return synth.small_problem("single", **args)


def _workspace(lib, st, torch):
    nbytes = int(lib.bullseye_facet_4_cor_corrections_ws_bytes(ctypes.byref(st)))
    ws = torch.empty(nbytes + 256, dtype=torch.uint8, device="cuda")
    return ws, (ws.data_ptr() + 255) // 256 * 256, nbytes


@pytest.mark.parametrize("entry", ["noalloc", "ws"])
def test_singular_jones_is_reported_by_status(entry, gpu_required, built_libraries):
    import torch
    from bullseye_gb300.library import ImagingError, check, load_library
    torch.cuda.set_device(0)
    lib = load_library("GPU", "single")
    check(lib)
    p = _problem()
    p.jones[1, 2, 0, 0, 1, :] = 0  # one singular matrix
    keep = []
    st, arrs = _device_struct(p, torch, keep)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ws = None
    if entry == "noalloc":
        rc = lib.bullseye_facet_4_cor_corrections_noalloc(ctypes.byref(st), stream)
        ws_ptr = None
    else:
        ws, ws_ptr, nbytes = _workspace(lib, st, torch)
        rc = lib.bullseye_facet_4_cor_corrections_ws(ctypes.byref(st), ctypes.c_void_p(ws_ptr), nbytes, stream)
    assert rc == 0
    status = lib.bullseye_facet_4_cor_corrections_status(ctypes.byref(st), ws_ptr and ctypes.c_void_p(ws_ptr), stream)
    assert status == 4  # BZ_ERR_SINGULAR_JONES
    with pytest.raises(ImagingError, match="singular"):
        check(lib)
    # the word was cleared: a second query reports nothing
    assert lib.bullseye_facet_4_cor_corrections_status(ctypes.byref(st), ws_ptr and ctypes.c_void_p(ws_ptr), stream) == 0
    check(lib)
    # the singular matrix was zeroed, the others inverted in place
    J = arrs["jones"].cpu().numpy()
    assert np.all(J[1, 2, 0, 0, 1] == 0)
    m = p.jones[0, 0, 0, 0, 0].reshape(2, 2).astype(np.complex128)
    assert np.allclose(J[0, 0, 0, 0, 0].reshape(2, 2), np.linalg.inv(m), rtol=1e-4, atol=1e-5)
    del ws


def test_clean_call_reports_no_device_error(gpu_required, built_libraries):
    import torch
    from bullseye_gb300.library import check, load_library
    torch.cuda.set_device(0)
    lib = load_library("GPU", "single")
    keep = []
    st, _ = _device_struct(_problem(), torch, keep)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.bullseye_facet_4_cor_corrections_noalloc(ctypes.byref(st), stream) == 0
    assert lib.bullseye_facet_4_cor_corrections_status(None, None, stream) == 0
    check(lib)


def test_rejected_call_leaves_jones_untouched(gpu_required, built_libraries):
    """A workspace that is too small, and a grid beyond the fixed scratch, are rejected before any
    work is queued: the caller's Jones terms are not inverted."""
    import torch
    from bullseye_gb300.library import ImagingError, check, load_library
    torch.cuda.set_device(0)
    lib = load_library("GPU", "single")
    keep = []
    p = _problem()
    st, arrs = _device_struct(p, torch, keep)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ws, ws_ptr, nbytes = _workspace(lib, st, torch)
    rc = lib.bullseye_facet_4_cor_corrections_ws(ctypes.byref(st), ctypes.c_void_p(ws_ptr), nbytes - 256, stream)
    assert rc == 2
    with pytest.raises(ImagingError, match="workspace"):
        check(lib)
    st.nx = st.ny = 2048  # beyond the allocation-free scratch
    assert lib.bullseye_facet_4_cor_corrections_noalloc(ctypes.byref(st), stream) == 5
    with pytest.raises(ImagingError, match="scratch"):
        check(lib)
    torch.cuda.synchronize()
    assert np.array_equal(arrs["jones"].cpu().numpy(), p.jones)


def test_workspace_entry_takes_more_than_2e31_work_items(gpu_required, built_libraries):
    """8 facets x 2^25 baseline slots x 8 channels = 2^31 (facet, track, channel) items: more than one
    plain launch takes, accepted by the workspace entry's persistent launches.  The rows sit in the
    first slots (the rest are empty), and the grids match the same rows with the usual slot count."""
    import torch
    from bullseye_gb300.library import check, load_library
    torch.cuda.set_device(0)
    lib = load_library("GPU", "single")
    p = _problem(n_facets=8, n_chan=8, n_times=4)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    keep = []
    grids = []
    for slots in (None, 1 << 25):
        st, arrs = _device_struct(p, torch, keep)
        if slots:
            starts = arrs["starts"].cpu().numpy()
            big = np.full(slots + 1, starts[-1], np.int64)
            big[:starts.size] = starts
            arrs["big_starts"] = torch.as_tensor(big, device="cuda")
            st.baseline_starting_indexes = ctypes.c_void_p(arrs["big_starts"].data_ptr())
            st.baseline_count = slots
            assert 8 * slots * 8 > 0x7FFFFFFF
        ws, ws_ptr, nbytes = _workspace(lib, st, torch)
        rc = lib.bullseye_facet_4_cor_corrections_ws(ctypes.byref(st), ctypes.c_void_p(ws_ptr), nbytes, stream)
        check(lib)
        assert rc == 0
        assert lib.bullseye_facet_4_cor_corrections_status(ctypes.byref(st), ctypes.c_void_p(ws_ptr), stream) == 0
        grids.append(arrs["grid"].cpu().numpy())
        del ws
        torch.cuda.empty_cache()
    assert np.max(np.abs(grids[0])) > 0
    assert _rel(grids[1], grids[0]) <= 1e-6
