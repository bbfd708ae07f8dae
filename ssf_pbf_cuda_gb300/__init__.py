"""ssf_pbf_cuda_gb300 — GB300-native Position-Based-Fluids solver step.

The product is ``libpbf103.so`` (CUDA for sm_103a behind the C ABI of
``include/pbf103.h``); this package builds it and mirrors the reference
simulator's solver interface in Python (``api``).  The library loads lazily
on first use and raises if it has not been built: there is no CPU path.
"""
from ._lib import (PBF_FLAG_COLLISION_LIMIT, PBF_FLAG_NONFINITE, PBF_TENSILE_OFF, PBF_TENSILE_REFERENCE,
                   PBF_TENSILE_TEXTBOOK, PBF_VORTICITY_OFF, PBF_VORTICITY_REFERENCE, PBF_VORTICITY_TEXTBOOK,
                   PbfError, load)
from .api import (Batch, Boundary, PbfParticle, Server, calc_grid_size, config_params, default_params,
                  one_step, one_step_external, resolve_grid, scene_bytes)

__all__ = [
    "Batch", "Boundary", "PbfParticle", "Server", "PbfError", "calc_grid_size", "config_params",
    "default_params", "one_step", "one_step_external", "resolve_grid", "scene_bytes", "load",
    "PBF_FLAG_COLLISION_LIMIT", "PBF_FLAG_NONFINITE", "PBF_TENSILE_OFF", "PBF_TENSILE_REFERENCE",
    "PBF_TENSILE_TEXTBOOK", "PBF_VORTICITY_OFF", "PBF_VORTICITY_REFERENCE", "PBF_VORTICITY_TEXTBOOK",
]
