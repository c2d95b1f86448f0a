"""ctypes mirror of the ``gridding_parameters`` struct and the imaging-library exports.

The struct is the single argument of every imaging-library entry point.  Its field order,
types and meaning follow the reference exactly, because the drop-in library must accept the
struct that bullseye's pipeliner fills:

* C++ definition: bullseye/mo/cpu_gpu_common/gridding_parameters.h:44-109
* ctypes mirror used by the pipeliner: bullseye/mo/gridding_parameters.py:44-112
* precision typedefs: bullseye/mo/cpu_gpu_common/base_types.h:41-59 (single precision keeps
  ``normalization_base_type`` as double)

Layout (x86-64 and aarch64 LP64 agree): 392 bytes in single precision, 408 in double.
"""
from __future__ import annotations

import ctypes
from ctypes import c_bool, c_double, c_float, c_size_t, c_uint, c_void_p

import numpy as np

PRECISIONS = ("single", "double")

#: Exported entry points of the reference imaging libraries
#: (bullseye/mo/cpu_gpu_common/wrapper.h:41-61).  All take ``gridding_parameters&`` except
#: the two walltime getters, ``gridding_barrier`` and ``releaseLibrary``.
REFERENCE_EXPORTS = (
    "get_gridding_walltime", "get_inversion_walltime", "gridding_barrier", "initLibrary",
    "releaseLibrary", "weight_uniformly", "normalize", "repack_input_data", "finalize",
    "finalize_psf", "grid_single_pol", "facet_single_pol", "grid_duel_pol", "facet_duel_pol",
    "grid_4_cor", "facet_4_cor", "facet_4_cor_corrections", "grid_sampling_function",
    "facet_sampling_function",
)

_STRUCTS: dict[str, type] = {}


def _fields(real):
    return [
        ("visibilities", c_void_p),
        ("uvw_coords", c_void_p),
        ("reference_wavelengths", c_void_p),
        ("visibility_weights", c_void_p),
        ("flags", c_void_p),
        ("flagged_rows", c_void_p),
        ("field_array", c_void_p),
        ("spw_index_array", c_void_p),
        ("imaging_field", c_uint),
        ("baseline_count", c_size_t),
        ("row_count", c_size_t),
        ("chunk_max_row_count", c_size_t),
        ("channel_count", c_size_t),
        ("number_of_polarization_terms", c_size_t),
        ("number_of_polarization_terms_being_gridded", c_size_t),
        ("spw_count", c_size_t),
        ("no_timestamps_read", c_size_t),
        ("nx", c_size_t),
        ("ny", c_size_t),
        ("cell_size_x", real),
        ("cell_size_y", real),
        ("conv", c_void_p),
        ("conv_support", c_size_t),
        ("conv_oversample", c_size_t),
        ("polarization_index", c_size_t),
        ("second_polarization_index", c_size_t),
        ("output_buffer", c_void_p),
        ("phase_centre_ra", real),
        ("phase_centre_dec", real),
        ("facet_centres", c_void_p),
        ("num_facet_centres", c_size_t),
        ("jones_terms", c_void_p),
        ("should_invert_jones_terms", c_bool),
        ("antenna_1_ids", c_void_p),
        ("antenna_2_ids", c_void_p),
        ("timestamp_ids", c_void_p),
        ("antenna_count", c_size_t),
        ("enabled_channels", c_void_p),
        ("channel_grid_indicies", c_void_p),
        ("cube_channel_dim_size", c_size_t),
        ("should_grid_sampling_function", c_bool),
        ("sampling_function_buffer", c_void_p),
        ("sampling_function_channel_grid_indicies", c_void_p),
        ("sampling_function_channel_count", c_size_t),
        ("is_final_data_chunk", c_bool),
        ("wplanes", c_size_t),
        ("wmax_est", real),
        ("baseline_starting_indexes", c_void_p),
        ("antenna_jones_starting_indexes", c_void_p),
        ("jones_time_indicies_per_antenna", c_void_p),
        ("normalization_terms", c_void_p),
    ]


def gridding_parameters_type(precision: str) -> type:
    """Return the ctypes ``Structure`` class for ``precision`` ('single' or 'double')."""
    if precision not in PRECISIONS:
        raise ValueError(f"precision must be one of {PRECISIONS}, got {precision!r}")
    if precision not in _STRUCTS:
        real = c_float if precision == "single" else c_double
        cls = type(f"gridding_parameters_{precision}", (ctypes.Structure,), {"_fields_": _fields(real)})
        _STRUCTS[precision] = cls
    return _STRUCTS[precision]


def real_dtype(precision: str):
    """numpy dtype of visibility, uvw, wavelength, weight, convolution and grid reals."""
    return np.float32 if precision == "single" else np.float64


def complex_dtype(precision: str):
    return np.complex64 if precision == "single" else np.complex128


EXPECTED_SIZEOF = {"single": 392, "double": 408}
#: Field offsets measured on the reference build (probe recorded in the survey of the
#: reference); the C++ header of the drop-in static_asserts the same numbers.
EXPECTED_OFFSETS = {
    "single": {"cell_size_x": 152, "conv": 160, "phase_centre_ra": 208, "wmax_est": 352,
               "normalization_terms": 384},
    "double": {"conv": 168, "phase_centre_ra": 216, "wmax_est": 368, "normalization_terms": 400},
}


def bind_exports(lib, extra_double=(), extra_int=()):
    """Set ctypes restypes/argtypes for the reference exports on a loaded library handle."""
    for name in REFERENCE_EXPORTS:
        fn = getattr(lib, name)
        if name in ("get_gridding_walltime", "get_inversion_walltime") or name in extra_double:
            fn.restype = c_double
            fn.argtypes = []
        elif name in ("gridding_barrier", "releaseLibrary"):
            fn.restype = None
            fn.argtypes = []
        else:
            fn.restype = None
            fn.argtypes = [c_void_p]
    return lib


class BullseyeFacet(ctypes.Structure):
    """One facet of an uneven layout for ``bullseye_grid_batched_facets`` (include/bullseye_gb300.h):
    centre and cell sizes in arcsec, grid size, and the complex-element offset of its
    [cube][4][ny][nx] block in the caller's grid buffer."""
    _fields_ = [("ra", c_double), ("dec", c_double), ("cell_x", c_double), ("cell_y", c_double),
                ("nx", c_size_t), ("ny", c_size_t), ("grid_offset", c_size_t)]
