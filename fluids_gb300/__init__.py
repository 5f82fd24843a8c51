"""fluids_gb300 -- GB300-native (sm_103a) SPH particle pipeline of paivett/fluids.

The compute path is libsph_gb300.so (CUDA kernels + the C ABI of include/sph_capi.h), built
in-tree by ``build()``.  This package is the host-side mirror of the reference's solver
interface over that ABI; it has no CPU fallback.
"""
from . import build as _build_mod
from .capi import (SPH_MODE_COMPAT, SPH_MODE_PHYSICS, SPH_NEIGH_LIST, SPH_NEIGH_SCAN, SPH_PCISPH, SPH_WCSPH,
                   Context, SphError, SphParams, default_params, make_params)


def build(force=False, verbose=False):
    """Compiles libsph_gb300.so for sm_103a (nvcc) if any source changed; returns its path."""
    return _build_mod.build(force=force, verbose=verbose)


def build_driver(force=False):
    """Compiles the headless C++ driver (driver/sph_driver.cpp) against the library."""
    return _build_mod.build_driver(force=force)


def cuda_available():
    from . import capi
    return capi.cuda_available()


__all__ = ["build", "build_driver", "cuda_available", "Context", "SphError", "SphParams", "default_params", "make_params",
           "SPH_WCSPH", "SPH_PCISPH", "SPH_MODE_COMPAT", "SPH_MODE_PHYSICS", "SPH_NEIGH_SCAN", "SPH_NEIGH_LIST"]
