"""bullseye_gb300.geometry.offgrid_pairs against the oracle's own acceptance test.

With an all-ones AA kernel, unit weights and nothing flagged, every (row, channel) sample that the
reference accepts into a facet adds exactly W x W to that facet's FP64 normalisation sum
(bullseye/mo/cpu_algorithm/templated_gridder.h:97), so the oracle's sums count its accepted
samples; the rest are the off-grid samples the reference drops without a count.
"""
import numpy as np
import pytest

from bullseye_gb300 import synth
from bullseye_gb300.geometry import offgrid_pairs
from bullseye_gb300.imaging import run_imaging


@pytest.fixture(scope="module")
def oracle64(oracle_built):
    from oracle.harness import load_oracle
    return load_oracle("double")


@pytest.mark.parametrize("cell", [60.0, 240.0])
def test_offgrid_counts_match_the_oracle(cell, oracle64):
    p = synth.small_problem("double", nx=96, n_ant=10, n_times=20, n_chan=3, n_facets=3, cell=cell, s=3, os=15,
                            flag_fraction=0.0)
    p.conv = np.ones_like(p.conv)
    p.weights = np.ones_like(p.weights)
    p.flags = np.zeros_like(p.flags)
    p.flagged_rows = np.zeros_like(p.flagged_rows)
    res = run_imaging(oracle64, p, "facet_4_cor")
    W = 2 * p.conv_support + 1
    accepted = np.rint(res.normalization[:, 0, 0] / (W * W)).astype(np.int64)
    assert np.allclose(res.normalization[:, 0, 0], accepted * W * W)
    expected = p.rows * p.channels - accepted
    got = offgrid_pairs(p)
    assert np.array_equal(got, expected), (got, expected)
    if cell == 240.0:
        assert got.sum() > 0  # the long baselines leave the grid
