"""Golden-vector cases: inputs are seeded synthetic problems, outputs come from the reference's
own CPU imaging library built from source (oracle/_ref, see make_golden.py).

Each case records the ABI call, the problem generator arguments and the run options.  Inputs and
outputs are stored together in ``<name>_<precision>.npz`` so the check does not depend on the
platform's libm reproducing the generator bit for bit.
"""
from __future__ import annotations

import dataclasses
import os

import numpy as np

from bullseye_gb300.imaging import GriddingProblem

HERE = os.path.dirname(os.path.abspath(__file__))

CASES = {
    # name: (abi call, small_problem kwargs, run_imaging kwargs)
    "grid_single_aa": ("grid_single_pol", dict(nx=48, n_ant=6, n_times=8, n_chan=2, kernel="sinc"), dict()),
    "grid_duel_aa": ("grid_duel_pol", dict(nx=48, n_ant=6, n_times=8, n_chan=2), dict()),
    "grid_4cor_uniform": ("grid_4_cor", dict(nx=48, ny=40, n_ant=6, n_times=8, n_chan=2),
                          dict(uniform=True, psf=True, do_finalize=True)),
    "facet_4cor": ("facet_4_cor", dict(nx=48, n_ant=6, n_times=8, n_chan=2, n_facets=3), dict(do_finalize=True)),
    "facet_jones": ("facet_4_cor_corrections", dict(nx=48, n_ant=6, n_times=8, n_chan=2, n_facets=2, jones=True),
                    dict(uniform=True)),
    "grid_4cor_wproj": ("grid_4_cor", dict(nx=64, n_ant=6, n_times=8, n_chan=2, s=4, os=7, wplanes=4,
                                           min_support=5), dict(psf=True, do_finalize=True)),
    "facet_single_wproj": ("facet_single_pol", dict(nx=64, n_ant=6, n_times=8, n_chan=2, s=4, os=7, wplanes=4,
                                                    n_facets=2, min_support=5), dict(uniform=True)),
    "facet_jones_wproj": ("facet_4_cor_corrections", dict(nx=64, n_ant=5, n_times=6, n_chan=2, s=3, os=5,
                                                          wplanes=3, n_facets=2, jones=True), dict()),
    "odd_grid_finalize": ("grid_4_cor", dict(nx=45, ny=39, n_ant=5, n_times=6, n_chan=1),
                          dict(psf=True, do_finalize=True)),
}

PRECISIONS = ("double", "single")


def case_path(name: str, precision: str) -> str:
    return os.path.join(HERE, f"{name}_{precision}.npz")


_ARRAYS = ("vis", "uvw", "wavelengths", "weights", "flags", "flagged_rows", "field_ids", "spw_ids", "antenna1",
           "antenna2", "timestamp_ids", "conv", "facet_centres", "jones", "enabled_channels", "channel_grid_index",
           "sampling_channel_grid_index")


def problem_to_arrays(p: GriddingProblem) -> dict:
    out = {}
    for f in dataclasses.fields(p):
        v = getattr(p, f.name)
        if f.name in _ARRAYS:
            if v is not None:
                out["in_" + f.name] = np.asarray(v)
        elif f.name == "phase_centre":
            out["in_phase_centre"] = np.asarray(v, dtype=np.float64)
        else:
            out["in_" + f.name] = np.asarray(v)
    return out


def problem_from_arrays(d) -> GriddingProblem:
    kw = {}
    for f in dataclasses.fields(GriddingProblem):
        key = "in_" + f.name
        if key not in d:
            kw[f.name] = None
            continue
        v = d[key]
        if f.name in _ARRAYS:
            kw[f.name] = np.array(v)
        elif f.name == "phase_centre":
            kw[f.name] = tuple(float(x) for x in v)
        elif f.name == "precision":
            kw[f.name] = str(v)
        elif v.dtype.kind == "f":
            kw[f.name] = float(v)
        else:
            kw[f.name] = int(v)
    return GriddingProblem(**kw)


def load_case(name: str, precision: str):
    d = np.load(case_path(name, precision), allow_pickle=False)
    return problem_from_arrays(d), {k[4:]: d[k] for k in d.files if k.startswith("out_")}


def cpu_conv(p: GriddingProblem) -> np.ndarray:
    """The kernel table the CPU ABI expects: the 2-D w stack (outer products of the separable
    1-D stack, computed in float64 then rounded) when w-projection is on, else the 1-D AA table."""
    from bullseye_gb300.filters import outer_stack
    if p.wplanes > 1:
        st = outer_stack(p.conv.astype(np.complex128))
        return st.astype(p.conv.dtype)
    return p.conv
