"""Pin the prediction restatement (oracle/predict.py) to the reference's prototype degridder.

tests/golden/notebook_degrid.npz holds what writing_and_wiki/notebooks/Resampling.ipynb cell 17
computes on seeded inputs (the sum of grid x tap over the footprint divided by the sum of the taps).
The restatement, in its normalised form and fed the notebook's model grid, must reproduce it.  The
notebook picks the footprint with round-to-nearest, which is the reference gridder's w-projection
rule (its AA rule rounds down), so the problem is a two-plane w stack holding the notebook's filter
in both planes with rows at w = 0.  The notebook indexes its grid [u][v] and places pixel u at
column u; the gridder's grids are [v][u], pixel u at u + N/2, with the v axis negated by the
cell-size sign.  The notebook and the gridder accept different footprints at the grid edge, so the
fixture's last rows are not compared.
"""
import os

import numpy as np

from bullseye_gb300 import synth
from oracle.predict import model_grids, predict

HERE = os.path.dirname(os.path.abspath(__file__))


def notebook_problem(d, precision="double"):
    suv, aa = d["scaled_uv"], d["aa"]
    S, OS = int(d["support"]), int(d["oversample"])
    N = d["model"].shape[0]
    rows = suv.shape[0]
    cell = 30.0
    arcsec = float(np.float32(np.pi / 180.0 / 3600.0))
    u_scale = N * cell * arcsec
    uvw = np.zeros((rows, 3))
    uvw[:, 0] = (suv[:, 0] - N // 2) / u_scale
    uvw[:, 1] = (suv[:, 1] - N // 2) / -u_scale
    p = synth.small_problem(precision, nx=N, n_ant=2, n_times=1, n_chan=1, s=S, os=OS, wplanes=2, seed=3)
    p.uvw = uvw
    p.vis = np.zeros((rows, 1, 4), np.complex128)
    p.weights = np.ones((rows, 1, 4))
    p.flags = np.zeros((rows, 1, 4), bool)
    p.flagged_rows = np.zeros(rows, bool)
    p.field_ids = np.zeros(rows, np.uint32)
    p.spw_ids = np.zeros(rows, np.uint32)
    p.antenna1 = np.zeros(rows, np.uint32)
    p.antenna2 = np.ones(rows, np.uint32)
    p.timestamp_ids = np.zeros(rows, np.uintp)
    p.wavelengths = np.ones((1, 1))
    p.cell_x = p.cell_y = cell
    p.conv = np.stack([aa, aa]).astype(np.complex128)
    p.wmax = 1.0
    p.facet_centres = None
    p.jones = None
    return p


def test_normalised_prediction_matches_notebook_degridder():
    d = np.load(os.path.join(HERE, "golden", "notebook_degrid.npz"))
    p = notebook_problem(d)
    scales = np.array([1.0, 2.0, -0.5, 3.0])
    grids = np.stack([d["model"].T * s for s in scales])[None, None]  # [1][1][4][v][u]
    vis = predict(p, grids, faceting=False, normalise=True)
    n_in = int(d["interior_rows"])
    ref = d["vis"]
    for k, s in enumerate(scales):
        got, want = vis[:n_in, 0, k], ref[:n_in] * s
        assert np.max(np.abs(got - want)) <= 1e-12 * np.max(np.abs(want)), k


def test_model_grid_is_the_inverse_of_finalize():
    """finalize's image = fftshift(ifft2(ifftshift(grid))) unnormalised; model_grids inverts it up to
    the pixel count, for even and odd sizes."""
    rng = np.random.default_rng(1)
    for ny, nx in ((16, 16), (15, 21)):
        g = rng.normal(size=(ny, nx)) + 1j * rng.normal(size=(ny, nx))
        img = np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(g)), axes=(-2, -1)) * (nx * ny)
        back = model_grids(img) / (nx * ny)
        assert np.max(np.abs(back - g)) <= 1e-12 * np.max(np.abs(g))
