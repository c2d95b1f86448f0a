"""Integer sampling counts (nearest-neighbour policy): oracle against the reference, bit for bit.

tests/golden/nn_counts_<precision>.npz comes from the reference's own gridder instantiated with its
nearest-neighbour convolution policy (oracle/ref_nn_harness.cpp, tests/golden/make_nn_counts.py).
The oracle's restatement must reproduce every count exactly, in both precisions and modes; the GPU
library is checked against the same fixtures in tests/test_gpu_nn_counts.py.
"""
import ctypes
import os

import numpy as np
import pytest

from tests.golden.nn_cases import FACETS, NX, NY, SF_CH, host_ptr, make_inputs, make_struct

from bullseye_gb300.abi import complex_dtype

HERE = os.path.dirname(os.path.abspath(__file__))


def fixture(precision):
    return np.load(os.path.join(HERE, "golden", f"nn_counts_{precision}.npz"))


def inputs_from(fx):
    return {k[3:]: fx[k] for k in fx.files if k.startswith("in_")}


@pytest.mark.parametrize("precision", ["single", "double"])
def test_fixture_inputs_are_reproducible(precision):
    """The generator is deterministic, so the fixture's inputs can be regenerated anywhere."""
    fx = fixture(precision)
    d = make_inputs(precision)
    for k, v in inputs_from(fx).items():
        assert np.array_equal(d[k], v), k


@pytest.mark.parametrize("precision", ["single", "double"])
@pytest.mark.parametrize("faceting", [0, 1])
def test_oracle_counts_match_reference(precision, faceting, oracle_built):
    from oracle.harness import load_oracle
    fx = fixture(precision)
    d = inputs_from(fx)
    lib = load_oracle(precision)
    F = FACETS if faceting else 1
    buf = np.zeros((F, SF_CH, NY, NX), complex_dtype(precision))
    st = make_struct(precision, d, bool(faceting), host_ptr, host_ptr(buf))
    lib.oracle_sampling_counts_nn(ctypes.byref(st), faceting)
    want = fx["counts_facet" if faceting else "counts_grid"]
    assert np.all(buf.imag == 0)
    assert np.array_equal(buf.real.astype(np.uint32), want)
