"""Tap-index flips of the reference's single-precision arithmetic (config 3, the 80 km precision
workload), counted with the oracle's cell choices.

The reference's 32-bit library forms the pixel coordinates, the footprint corner and the tap
offsets in float (convolution_policies.h:70-118 under FE_DOWNWARD); its 64-bit library in double.
On 4096^2 facets of 0.25 arcsec the coordinates reach about 2000 pixels, where a float resolves
2.4e-4 pixel, so the two choose different taps for a fraction of the samples.  The oracle records
every (facet, row, channel)'s corner and tap offsets in both precisions on the same input values
(the single-precision arrays, widened for the 64-bit run, as the precision report does); the 32-bit
drop-in chooses them in FP64 (or double-float), so its choices are the 64-bit ones and these flips
are the reference's, not its.  The FP64 rejections also pin bullseye_gb300.geometry.offgrid_pairs.
"""
import ctypes

import numpy as np

from bullseye_gb300 import synth
from bullseye_gb300.geometry import offgrid_pairs
from bullseye_gb300.imaging import run_imaging


def _taps(lib, p):
    F = max(1, p.n_facets)
    log = np.full(F * p.rows * p.channels * 4, -2, np.int64)
    lib.oracle_record_taps.restype = None
    lib.oracle_record_taps.argtypes = [ctypes.c_void_p, ctypes.c_size_t]
    lib.oracle_record_taps(log.ctypes.data_as(ctypes.c_void_p), log.size)
    try:
        run_imaging(lib, p, "facet_single_pol")
    finally:
        lib.oracle_record_taps(None, 0)
    return log.reshape(F, p.rows, p.channels, 4)


def test_reference_fp32_tap_flips_on_the_80km_workload(oracle_built):
    from oracle.harness import load_oracle
    p32 = synth.config3("single")
    p64 = p32.astype("double")
    t32 = _taps(load_oracle("single"), p32)
    t64 = _taps(load_oracle("double"), p64)
    assert (t64 != -2).all() and (t32 != -2).all()  # every sample visited
    acc64 = t64[..., 0] >= 0
    # off-grid samples: the 64-bit reference's rejections are the geometry module's count
    assert np.array_equal((~acc64).sum(axis=(1, 2)), offgrid_pairs(p64))
    corner = (t32[..., :2] != t64[..., :2]).any(-1) & acc64
    tap = (t32[..., 2:] != t64[..., 2:]).any(-1) & acc64 & ~corner
    n = acc64.sum(axis=(1, 2))
    per_facet = [{"accepted": int(n[f]), "corner_flips": int(corner[f].sum()), "tap_flips": int(tap[f].sum())}
                 for f in range(t64.shape[0])]
    print("fp32 reference against fp64 reference, per facet:", per_facet)
    # the float choice moves a footprint or a tap offset for a few percent of the samples at most
    assert all(r["tap_flips"] + r["corner_flips"] < 0.05 * r["accepted"] for r in per_facet)
    assert sum(r["tap_flips"] for r in per_facet) > 0
