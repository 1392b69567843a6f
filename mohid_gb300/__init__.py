"""GB300-native MOHID Water tracer advection-diffusion step.

The package is the host side of libmohid_ad.so (CUDA, sm_103a), whose C-ABI
(include/mohid_ad.h) is the drop-in boundary for ModuleAdvectionDiffusion's
AdvectionDiffusion call and for the legacy CUDA Thomas binding.
"""
__version__ = "0.1.0"
