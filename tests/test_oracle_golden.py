"""Pin the oracle (the C restatement of the reference CPU library) to the reference's own outputs.

The fixtures in tests/golden were produced by the reference CPU imaging library compiled from its
sources (tests/golden/make_golden.py).  Non-faceted modes must agree bit for bit; faceted modes
agree to FP64 rounding (the reference evaluates its phase under FE_DOWNWARD, where the compiler's
choice of operation order changes the last bits) and, in single precision, to the accuracy of the
reference's float phase argument.
"""
import numpy as np
import pytest

from tests.golden.cases import CASES, PRECISIONS, cpu_conv, load_case

from bullseye_gb300.imaging import run_imaging

FACET_TOL = {"double": 1e-13, "single": 5e-5}


def _rel(a, b):
    s = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / s) if s else float(np.max(np.abs(a - b)))


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_reference_fixture(name, precision, oracle_built):
    from oracle.harness import load_oracle
    call, _, rkw = CASES[name]
    p, out = load_case(name, precision)
    lib = load_oracle(precision)
    res = run_imaging(lib, p.with_conv(cpu_conv(p)), call, keep_raw=True, **rkw)
    assert lib.oracle_last_error() == 0
    faceted = call.startswith("facet")
    tol = FACET_TOL[precision] if faceted else 0.0
    pairs = [("raw_grid", res.raw_grid), ("grid", res.grid), ("normalization", res.normalization),
             ("sampling", res.sampling), ("image", res.image), ("psf", res.psf)]
    for key, got in pairs:
        if key not in out:
            assert got is None
            continue
        ref = out[key]
        assert got.shape == ref.shape, key
        if tol == 0.0 or key in ("normalization", "sampling", "psf"):
            np.testing.assert_array_equal(got, ref, err_msg=f"{name}/{precision}/{key}")
        else:
            assert _rel(got, ref) <= tol, f"{name}/{precision}/{key}: {_rel(got, ref)}"
