"""The adjoint (degridding) kernel and the differentiable gridding function.

* dot-product identity Re<R, G(V)> = Re<A(R), V> for every four-correlation gridding mode (Jones
  correction, faceting only, no faceting), AA and w-projection kernels, both precisions;
* finite differences of a real loss of the grids with respect to visibilities and Jones terms
  (central differences, eps = 1e-3, 200 coordinates, agreement to 1e-4 of the largest gradient);
* the single-precision gradients against the double-precision ones;
* the reference's own degridder (the prototype of writing_and_wiki/notebooks/Resampling.ipynb,
  cell 17, run as written into tests/golden/notebook_degrid.npz): with unit weights, no faceting
  and the model grid as grad_grid, the adjoint divided by the tap sum reproduces it.
"""
import ctypes
import os

import numpy as np
import pytest

from bullseye_gb300 import synth
from bullseye_gb300.imaging import run_imaging

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _problem(precision, wplanes=4, facets=3, jones=True):
    return synth.small_problem(precision, nx=96, n_ant=7, n_times=10, n_chan=3, n_facets=facets, jones=jones, s=4,
                               os=9, wplanes=wplanes, min_support=5 if wplanes > 1 else None, seed=21)


def _ctype(precision):
    import torch
    return torch.complex64 if precision == "single" else torch.complex128


def _rand(torch, shape, dtype, seed):
    g = torch.Generator(device="cpu").manual_seed(seed)
    re = torch.randn(shape, generator=g, dtype=torch.float64)
    im = torch.randn(shape, generator=g, dtype=torch.float64)
    return torch.complex(re, im).to(dtype).cuda()


@pytest.mark.parametrize("precision", ["double", "single"])
@pytest.mark.parametrize("wplanes", [1, 4])
def test_dot_product_jones(precision, wplanes, gpu_required, built_libraries):
    import torch
    from bullseye_gb300.autograd import FacetGeometry, facet_grid, grid_adjoint
    p = _problem(precision, wplanes)
    geom = FacetGeometry.from_problem(p)
    ct = _ctype(precision)
    V = torch.as_tensor(p.vis[geom.order]).cuda().to(ct).contiguous()
    J = torch.as_tensor(p.jones).cuda().to(ct).contiguous()
    G, _ = facet_grid(geom, V, J)
    R = _rand(torch, geom.grid_shape, ct, 3)
    gv, _ = grid_adjoint(geom, V, J, R)
    lhs = float((R.conj() * G).real.double().sum())
    rhs = float((gv.conj() * V).real.double().sum())
    tol = 1e-11 if precision == "double" else 2e-5
    assert abs(lhs - rhs) <= tol * max(abs(lhs), 1e-30), (lhs, rhs)


@pytest.mark.parametrize("precision", ["double", "single"])
@pytest.mark.parametrize("call,facets,wplanes", [("facet_4_cor", 3, 4), ("facet_4_cor", 2, 1),
                                                 ("grid_4_cor", 0, 4), ("grid_4_cor", 0, 1)])
def test_dot_product_without_jones(precision, call, facets, wplanes, gpu_required, built_libraries):
    """Forward through the library's regular entry point (host buffers), adjoint through the C-ABI."""
    import torch
    from bullseye_gb300.autograd import FacetGeometry, grid_adjoint
    from bullseye_gb300.library import check, load_library
    torch.cuda.set_device(0)
    p = _problem(precision, wplanes, facets=facets, jones=False)
    lib = load_library("GPU", precision)
    res = run_imaging(lib, p, call, keep_raw=True)
    check(lib)
    geom = FacetGeometry.from_problem(p)
    ct = _ctype(precision)
    G = torch.as_tensor(res.raw_grid).cuda().to(ct).reshape(geom.grid_shape)
    V = torch.as_tensor(p.vis[geom.order]).cuda().to(ct).contiguous()
    R = _rand(torch, geom.grid_shape, ct, 4)
    gv, gj = grid_adjoint(geom, V, None, R, faceting=call.startswith("facet"))
    assert gj is None
    lhs = float((R.conj() * G).real.double().sum())
    rhs = float((gv.conj() * V).real.double().sum())
    tol = 1e-11 if precision == "double" else 2e-5
    assert abs(lhs - rhs) <= tol * max(abs(lhs), 1e-30), (lhs, rhs)


def test_finite_differences(gpu_required, built_libraries):
    """L = Re<C, G> + 1/2 sum r |G|^2; 100 visibility and 100 Jones coordinates, real or imaginary part."""
    import torch
    from bullseye_gb300.autograd import FacetGeometry, facet_grid
    p = _problem("double", 4)
    geom = FacetGeometry.from_problem(p)
    V0 = torch.as_tensor(p.vis[geom.order]).cuda().contiguous()
    J0 = torch.as_tensor(p.jones).cuda().contiguous()
    C = _rand(torch, geom.grid_shape, torch.complex128, 5)
    gen = torch.Generator(device="cpu").manual_seed(6)
    r = (torch.rand(geom.grid_shape, generator=gen, dtype=torch.float64) * 1e-3).cuda()

    def loss(V, J):
        G, _ = facet_grid(geom, V, J)
        return (C.conj() * G).real.sum() + 0.5 * (r * G.abs() ** 2).sum()

    V = V0.clone().requires_grad_(True)
    J = J0.clone().requires_grad_(True)
    loss(V, J).backward()
    gV, gJ = V.grad.detach(), J.grad.detach()
    assert torch.isfinite(gV.abs()).all() and torch.isfinite(gJ.abs()).all()
    eps = 1e-3
    rng = np.random.default_rng(7)
    cases = []
    # coordinates whose gradient is not structurally zero (flagged data have none)
    vi = torch.nonzero(gV.abs().reshape(-1) > 0).reshape(-1).cpu().numpy()
    ji = torch.nonzero(gJ.abs().reshape(-1) > 0).reshape(-1).cpu().numpy()
    assert vi.size >= 100 and ji.size >= 100
    for idx in rng.choice(vi, 100, replace=False):
        cases.append(("V", int(idx), int(rng.integers(2))))
    for idx in rng.choice(ji, 100, replace=False):
        cases.append(("J", int(idx), int(rng.integers(2))))
    worst = {"V": 0.0, "J": 0.0}
    scale = {"V": float(gV.abs().max()), "J": float(gJ.abs().max())}
    with torch.no_grad():
        for which, idx, part in cases:
            step = eps if part == 0 else 1j * eps
            Vp, Vm, Jp, Jm = V0.clone(), V0.clone(), J0.clone(), J0.clone()
            if which == "V":
                Vp.view(-1)[idx] += step
                Vm.view(-1)[idx] -= step
                g = gV.reshape(-1)[idx]
            else:
                Jp.view(-1)[idx] += step
                Jm.view(-1)[idx] -= step
                g = gJ.reshape(-1)[idx]
            fd = (float(loss(Vp, Jp)) - float(loss(Vm, Jm))) / (2 * eps)
            an = float(g.real if part == 0 else g.imag)
            worst[which] = max(worst[which], abs(fd - an) / scale[which])
    assert worst["V"] <= 1e-4 and worst["J"] <= 1e-4, worst


@pytest.mark.parametrize("wplanes", [1, 4])
def test_single_matches_double(wplanes, gpu_required, built_libraries):
    import torch
    from bullseye_gb300.autograd import FacetGeometry, grid_adjoint
    out = {}
    # the double problem is the single one widened, so both select the same cells and taps (a
    # coordinate rounded to float can cross a cell boundary, which moves that visibility's gradient)
    ps = _problem("single", wplanes)
    for prec in ("double", "single"):
        p = ps.astype(prec)
        geom = FacetGeometry.from_problem(p)
        ct = _ctype(prec)
        V = torch.as_tensor(p.vis[geom.order]).cuda().to(ct).contiguous()
        J = torch.as_tensor(p.jones).cuda().to(ct).contiguous()
        R = _rand(torch, geom.grid_shape, ct, 8)
        gv, gj = grid_adjoint(geom, V, J, R)
        out[prec] = (gv.to(torch.complex128).cpu().numpy(), gj.to(torch.complex128).cpu().numpy())
    for k in range(2):
        a, b = out["single"][k], out["double"][k]
        err = np.max(np.abs(a - b)) / np.max(np.abs(b))
        assert err <= 1e-5, (k, err)


@pytest.mark.parametrize("precision", ["double", "single"])
def test_matches_notebook_degridder(precision, gpu_required, built_libraries):
    """The reference prototype degridder: V = sum G tap / sum tap at round(u) - SUPPORT + conv.

    The library's w-projection path picks the footprint with round-to-nearest like the notebook;
    the AA path rounds down, as the reference CPU library does, so the comparison uses a
    two-plane w stack whose planes both hold the notebook's filter and rows with w = 0.  The
    library places pixel coordinate u at grid column u + N/2 and stores grids [v][u] (the notebook
    indexes [u][v]), and its v axis is negated by the cell-size sign.  The notebook and the library
    accept different footprints at the grid edge (the notebook skips round(u) + W >= N and wraps
    negative cells; the library skips footprints that leave [0, N - 2)); the fixture's last rows sit
    there and are not compared.
    """
    import torch
    from bullseye_gb300.abi import complex_dtype, real_dtype
    from bullseye_gb300.autograd import FacetGeometry, grid_adjoint
    d = np.load(os.path.join(HERE, "golden", "notebook_degrid.npz"))
    model, suv, aa, ref = d["model"], d["scaled_uv"], d["aa"], d["vis"]
    S, OS = int(d["support"]), int(d["oversample"])
    n_in = int(d["interior_rows"])
    N = model.shape[0]
    rows = suv.shape[0]
    rd, cd = real_dtype(precision), complex_dtype(precision)
    cell = 30.0
    arcsec = float(np.float32(np.pi / 180.0 / 3600.0))
    u_scale = N * np.float64(np.asarray(cell, rd)) * arcsec
    v_scale = -u_scale
    uvw = np.zeros((rows, 3))
    uvw[:, 0] = (suv[:, 0] - N // 2) / u_scale
    uvw[:, 1] = (suv[:, 1] - N // 2) / v_scale
    p = synth.small_problem(precision, nx=N, n_ant=2, n_times=1, n_chan=1, s=S, os=OS, wplanes=2, seed=3)
    K = aa.shape[0]
    p.uvw = uvw.astype(rd)
    p.vis = np.zeros((rows, 1, 4), cd)
    p.weights = np.ones((rows, 1, 4), rd)
    p.flags = np.zeros((rows, 1, 4), bool)
    p.flagged_rows = np.zeros(rows, bool)
    p.field_ids = np.zeros(rows, np.uint32)
    p.spw_ids = np.zeros(rows, np.uint32)
    p.antenna1 = np.zeros(rows, np.uint32)
    p.antenna2 = np.ones(rows, np.uint32)
    p.timestamp_ids = np.zeros(rows, np.uintp)
    p.wavelengths = np.ones((1, 1), rd)
    p.cell_x = p.cell_y = cell
    p.conv = np.stack([aa, aa]).astype(cd)
    assert p.conv.shape == (2, K)
    p.wmax = 1.0
    p.facet_centres = None
    p.jones = None
    geom = FacetGeometry.from_problem(p)
    ct = _ctype(precision)
    scales = np.array([1.0, 2.0, -0.5, 3.0])
    grid = np.stack([model.T * s for s in scales])[None, None].astype(cd)  # [1][1][4][v][u]
    V = torch.zeros((rows, 1, 4), dtype=ct, device="cuda")
    num, _ = grid_adjoint(geom, V, None, torch.as_tensor(grid).cuda(), faceting=False)
    den, _ = grid_adjoint(geom, V, None, torch.ones(geom.grid_shape, dtype=ct, device="cuda"), faceting=False)
    inv = np.argsort(geom.order)
    num = num.cpu().numpy()[inv][:, 0, :]
    den = den.cpu().numpy()[inv][:, 0, 0].real
    assert np.all(den[:n_in] > 0)
    tol = 1e-12 if precision == "double" else 1e-5
    for k, s in enumerate(scales):
        got = num[:n_in, k] / den[:n_in]
        want = ref[:n_in] * s
        err = np.max(np.abs(got - want)) / np.max(np.abs(want))
        assert err <= tol, (k, err)


def test_rejects_bad_arguments(gpu_required, built_libraries):
    from bullseye_gb300.abi import gridding_parameters_type
    from bullseye_gb300.library import load_library
    for prec in ("single", "double"):
        lib = load_library("GPU", prec)
        st = gridding_parameters_type(prec)()
        buf = ctypes.c_void_p(1)
        assert lib.bullseye_grid_adjoint(None, buf, buf, None, 1, None) == 2
        assert lib.bullseye_grid_adjoint(ctypes.byref(st), buf, buf, None, 1, None) == 2
        assert lib.bullseye_grid_adjoint(ctypes.byref(st), None, buf, None, 1, None) == 2
