"""Loader for the GB300 imaging libraries (the drop-in for ``libgpu_imaging{32,64}.so``).

``load_library('GPU', precision)`` mirrors the reference's loader
(bullseye/mo/library_loader.py:42-59): it returns a ``ctypes.pydll`` handle whose functions take
a ``ctypes.byref(gridding_parameters)``.  Only the 'GPU' architecture exists here; the libraries
are the in-tree builds under ``bullseye_gb300/lib``.  There is no CPU fallback: when the CUDA
library is missing this raises.

The returned handle has restypes/argtypes set for the 19 reference exports and for the
extensions declared in ``include/bullseye_gb300.h``, plus :func:`check` which raises
:class:`ImagingError` with the library's sticky error message.
"""
from __future__ import annotations

import ctypes
import os

from .abi import PRECISIONS, bind_exports

HERE = os.path.dirname(os.path.abspath(__file__))
LIBDIR = os.path.join(HERE, "lib")


class ImagingError(RuntimeError):
    pass


def library_path(precision: str) -> str:
    if precision not in PRECISIONS:
        raise ValueError(f"precision must be one of {PRECISIONS}")
    return os.path.join(LIBDIR, "libgpu_imaging%s.so" % ("32" if precision == "single" else "64"))


_CACHE: dict = {}

EXTENSIONS = {
    "bullseye_last_error": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t]),
    "bullseye_clear_error": (None, []),
    "bullseye_precision_bits": (ctypes.c_int, []),
    "bullseye_set_compensated": (None, [ctypes.c_int]),
    "bullseye_set_device_inputs": (None, [ctypes.c_int]),
    "bullseye_get_stream": (ctypes.c_void_p, []),
    "bullseye_kernel_launches": (ctypes.c_longlong, []),
    "bullseye_gridder_kernel_ms": (ctypes.c_double, [ctypes.c_int, ctypes.POINTER(ctypes.c_longlong)]),
    "bullseye_fp32_fma_tflops": (ctypes.c_double, [ctypes.c_int]),
    "bullseye_facet_4_cor_corrections_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "bullseye_grid_batched": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "bullseye_grid_adjoint": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                             ctypes.c_int, ctypes.c_void_p]),
    "bullseye_sampling_counts_nn": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "bullseye_set_batched_profiling": (None, [ctypes.c_int]),
    "bullseye_batched_profile": (ctypes.c_int, [ctypes.c_void_p] * 6 + [ctypes.c_int]),
    "bullseye_batched_plane_classes": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "bullseye_selftest_bounded_wait": (ctypes.c_int, []),
    "bullseye_set_batched_calls": (None, [ctypes.c_int]),
    "bullseye_set_tracing": (None, [ctypes.c_int]),
    "bullseye_finalize_stokes": (None, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "bullseye_trace_report": (ctypes.c_size_t, [ctypes.c_char_p, ctypes.c_size_t]),
    "bullseye_grid_batched_facets": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    "bullseye_facet_4_cor_corrections_ws_bytes": (ctypes.c_size_t, [ctypes.c_void_p]),
    "bullseye_facet_4_cor_corrections_ws": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                                           ctypes.c_void_p]),
    "bullseye_facet_4_cor_corrections_status": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "bullseye_predict_ws_bytes": (ctypes.c_size_t, [ctypes.c_void_p]),
    "bullseye_predict": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "bullseye_trim_memory": (None, []),
    "bullseye_set_host_repack": (None, [ctypes.c_int]),
    "bullseye_set_grid_groups": (None, [ctypes.c_int]),
    "bullseye_set_host_copy": (None, [ctypes.c_int]),
    "bullseye_set_max_stage_bytes": (None, [ctypes.c_size_t]),
    "bullseye_set_visibility_records": (None, [ctypes.c_int]),
    "bullseye_set_record_budget": (None, [ctypes.c_size_t]),
    "bullseye_set_jones_time_major": (None, [ctypes.c_int]),
    "bullseye_reset_counters": (None, []),
    "bullseye_zero_grids": (None, []),
    "bullseye_set_gridding_correction": (None, [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t]),
}


def load_library(architecture: str = "GPU", precision: str = "single"):
    """Load (once per process) the imaging library for ``precision``."""
    if architecture != "GPU":
        raise ValueError("only the 'GPU' architecture is provided by bullseye_gb300")
    key = precision
    if key in _CACHE:
        return _CACHE[key]
    path = library_path(precision)
    if not os.path.exists(path):
        raise ImagingError(f"{path} is not built: run bullseye_gb300.build.build() (nvcc, sm_103a)")
    lib = ctypes.PyDLL(path, mode=getattr(os, "RTLD_LOCAL", 0))
    bind_exports(lib)
    for name, (res, args) in EXTENSIONS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _CACHE[key] = lib
    return lib


def last_error(lib) -> tuple[int, str]:
    buf = ctypes.create_string_buffer(1024)
    code = lib.bullseye_last_error(buf, len(buf))
    return code, buf.value.decode(errors="replace")


def check(lib) -> None:
    """Raise :class:`ImagingError` if the library recorded an error (and clear it)."""
    code, msg = last_error(lib)
    if code:
        lib.bullseye_clear_error()
        raise ImagingError(f"imaging library error {code}: {msg}")
