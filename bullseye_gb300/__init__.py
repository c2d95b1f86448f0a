"""GB300-native drop-in for bullseye's facet-imaging hot path.

The product is the pair of CUDA shared libraries ``libgpu_imaging32.so`` /
``libgpu_imaging64.so`` (built by :func:`bullseye_gb300.build.build`), which export the C-ABI of
the reference's GPU imaging libraries (bullseye/mo/cpu_gpu_common/wrapper.h:41-61) plus the
extended entry points declared in ``include/bullseye_gb300.h``.  This package holds the host
side around them: the ctypes ABI mirror (:mod:`.abi`), the library loader (:mod:`.library`), the
pipeliner-style call sequence (:mod:`.imaging`), kernel tables (:mod:`.filters`) and synthetic
workloads (:mod:`.synth`).
"""
__all__ = ["abi", "imaging", "filters", "synth"]
