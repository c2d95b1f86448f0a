"""Prediction (degridding as a forward operator) through the C-ABI: bullseye_predict.

* against the FP64 restatement oracle/predict.py (pinned to the reference's prototype degridder,
  tests/test_predict_oracle.py): model images with a gridding-correction taper, transformed with the
  inverse of finalize's shifts and degridded with Jones terms and the facet phase applied forward,
  in the normalised (sum of taps) and the unnormalised form, faceted and not, AA and w-projection;
  1e-12 relative in the 64-bit library, 1e-5 in the 32-bit one;
* against the reference's prototype degridder itself (tests/golden/notebook_degrid.npz, from the
  model grid, normalised);
* the unnormalised prediction without Jones terms from a grid is the adjoint of gridding with unit
  weights (bullseye_grid_adjoint), and its Jones form is J_p X J_q^H of the per-facet predictions.
"""
import os

import numpy as np
import pytest

from bullseye_gb300 import synth
from oracle.predict import model_grids, predict as oracle_predict

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def _problem(precision, wplanes, facets=2):
    return synth.small_problem(precision, nx=80, ny=72, n_ant=6, n_times=8, n_chan=2, n_facets=facets, jones=facets > 0,
                               s=4, os=9, wplanes=wplanes, min_support=5 if wplanes > 1 else None, seed=5)


def _rand_model(shape, seed):
    rng = np.random.default_rng(seed)
    return rng.normal(size=shape) + 1j * rng.normal(size=shape)


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("precision", ["double", "single"])
@pytest.mark.parametrize("wplanes", [1, 4])
@pytest.mark.parametrize("faceting", [True, False])
@pytest.mark.parametrize("normalise", [False, True])
def test_predict_matches_oracle(precision, wplanes, faceting, normalise, gpu_required, built_libraries):
    import torch
    from bullseye_gb300.autograd import FacetGeometry, predict
    torch.cuda.set_device(0)
    p = _problem(precision, wplanes, facets=2 if faceting else 0)
    geom = FacetGeometry.from_problem(p)
    ct = torch.complex64 if precision == "single" else torch.complex128
    images = _rand_model(geom.grid_shape, 7)
    # a positive taper in [0.5, 1.5] (a kernel's own correction falls to 1e-5 or crosses zero at the
    # field edge, which would make random images ill-conditioned for a relative comparison)
    rng = np.random.default_rng(2)
    tx, ty = 0.5 + rng.uniform(0, 1, p.nx), 0.5 + rng.uniform(0, 1, p.ny)
    taper = (torch.as_tensor(tx, device="cuda"), torch.as_tensor(ty, device="cuda"))
    J = torch.as_tensor(p.jones, device="cuda").to(ct).contiguous() if p.jones is not None else None
    got = predict(geom, torch.as_tensor(images, device="cuda").to(ct).contiguous(), J, faceting=faceting,
                  normalise=normalise, taper=taper)
    inv = np.argsort(geom.order)
    got = got.cpu().numpy()[inv]
    # the oracle sees the library's inputs at the library's precision, widened
    q = p.astype("double")
    want = oracle_predict(q, model_grids(images.astype(np.complex64 if precision == "single" else np.complex128),
                                         tx, ty), faceting=faceting, normalise=normalise)
    assert np.max(np.abs(want)) > 0
    tol = 1e-12 if precision == "double" else 1e-5
    assert _rel(got, want) <= tol


@pytest.mark.parametrize("precision", ["double", "single"])
def test_predict_from_grid_matches_notebook_degridder(precision, gpu_required, built_libraries):
    import torch
    from bullseye_gb300.autograd import FacetGeometry, predict
    from tests.test_predict_oracle import notebook_problem
    d = np.load(os.path.join(HERE, "golden", "notebook_degrid.npz"))
    p = notebook_problem(d).astype(precision)
    geom = FacetGeometry.from_problem(p)
    ct = torch.complex64 if precision == "single" else torch.complex128
    scales = np.array([1.0, 2.0, -0.5, 3.0])
    grids = np.stack([d["model"].T * s for s in scales])[None, None]
    got = predict(geom, torch.as_tensor(grids, device="cuda").to(ct).contiguous(), None, faceting=False,
                  normalise=True, from_grid=True).cpu().numpy()[np.argsort(geom.order)]
    n_in = int(d["interior_rows"])
    tol = 1e-12 if precision == "double" else 1e-5
    for k, s in enumerate(scales):
        assert _rel(got[:n_in, 0, k], d["vis"][:n_in] * s) <= tol, k


@pytest.mark.parametrize("wplanes", [1, 4])
def test_unnormalised_prediction_is_the_adjoint_with_unit_weights(wplanes, gpu_required, built_libraries):
    import torch
    from bullseye_gb300.autograd import FacetGeometry, grid_adjoint, predict
    p = _problem("double", wplanes, facets=2)
    p.jones = None
    p.weights = np.ones_like(p.weights)
    p.flags = np.zeros_like(p.flags)
    p.flagged_rows = np.zeros_like(p.flagged_rows)  # the adjoint skips flagged rows, prediction does not
    geom = FacetGeometry.from_problem(p)
    G = torch.as_tensor(_rand_model(geom.grid_shape, 3), device="cuda").contiguous()
    pv = predict(geom, G, None, faceting=True, from_grid=True)
    V0 = torch.zeros((p.rows, p.channels, 4), dtype=torch.complex128, device="cuda")
    gv, _ = grid_adjoint(geom, V0, None, G)
    assert _rel(pv.cpu().numpy(), gv.cpu().numpy()) <= 1e-14


def test_jones_are_applied_forward_per_facet(gpu_required, built_libraries):
    """With Jones terms, the prediction is sum_f J_p,f X_f J_q,f^H of the per-facet predictions X_f."""
    import torch
    from dataclasses import replace
    from bullseye_gb300.autograd import FacetGeometry, predict
    p = _problem("double", 4, facets=2)
    geom = FacetGeometry.from_problem(p)
    G = _rand_model(geom.grid_shape, 11)
    J = torch.as_tensor(p.jones, device="cuda").contiguous()
    full = predict(geom, torch.as_tensor(G, device="cuda").contiguous(), J, from_grid=True).cpu().numpy()
    want = np.zeros_like(full)
    o = geom.order
    t, a1, a2 = p.timestamp_ids[o].astype(np.int64), p.antenna1[o].astype(np.int64), p.antenna2[o].astype(np.int64)
    for f in range(2):
        pf = replace(p, facet_centres=p.facet_centres[f:f + 1], jones=None)
        gf = FacetGeometry.from_problem(pf)
        X = predict(gf, torch.as_tensor(G[f:f + 1], device="cuda").contiguous(), None, from_grid=True).cpu().numpy()
        for c in range(p.channels):
            Jp = p.jones[t, a1, f, 0, c].reshape(-1, 2, 2)
            Jq = p.jones[t, a2, f, 0, c].reshape(-1, 2, 2)
            want[:, c] += (Jp @ X[:, c].reshape(-1, 2, 2) @ np.conj(np.transpose(Jq, (0, 2, 1)))).reshape(-1, 4)
    assert _rel(full, want) <= 1e-12


def test_predict_rejects_bad_arguments(gpu_required, built_libraries):
    import ctypes
    from bullseye_gb300.abi import gridding_parameters_type
    from bullseye_gb300.library import ImagingError, check, load_library
    lib = load_library("GPU", "double")
    st = gridding_parameters_type("double")()
    buf = ctypes.c_void_p(256)
    assert lib.bullseye_predict(None, buf, None, None, 1, 0, buf, None, 0, None) == 2
    assert lib.bullseye_predict(ctypes.byref(st), buf, None, None, 1, 0, buf, None, 0, None) == 2
    with pytest.raises(ImagingError):
        check(lib)
