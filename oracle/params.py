"""Solver parameters for the oracle without the CUDA library — TEST
INFRASTRUCTURE AND CPU BASELINE ONLY.

The CPU reference arm of the benchmark must not load the product library,
so it builds its parameter sets here: the reference's pbf_parameter /
pbf_external fields (src/pbf/pbf_type.h:49-72) with the benchmark
configuration's values, and the hash grid from calcGridSize
(src/pbf/pbf_type.cpp:141-162) as the oracle's C restates it
(ora_calc_grid_size).  The keys are those the oracle's make_params reads.
"""
from __future__ import annotations

from . import oracle as O

# s_corr forms, XSPH and vorticity forms (the oracle's numbering)
TENSILE_REFERENCE, TENSILE_TEXTBOOK, TENSILE_OFF = 0, 1, 2
XSPH_OFF, XSPH_WALK, XSPH_LIST = 0, 1, 2
VORTICITY_OFF, VORTICITY_REFERENCE, VORTICITY_TEXTBOOK = 0, 1, 2


def base_params(**overrides) -> dict:
    """h = 0.1 m, spacing 0.05 m, rest density 1000, mass rho0 s^3, dt 1/120,
    CFM eps 600, gravity -9.8, 30 neighbour slots (29 usable), the
    reference's s_corr, XSPH and vorticity off."""
    p = {
        "stable_density": 1000.0, "stable_distance": 0.05, "particle_mass": 0.125, "smoothing_length": 0.1,
        "time_step": 1.0 / 120.0, "relaxation": 600.0, "xsph_parameter": 0.01, "vc_parameter": 0.0005,
        "body_force": [0.0, -9.8, 0.0], "max_pair_particle_num": 30, "tensile_mode": TENSILE_REFERENCE,
        "scorr_k": 0.1, "scorr_n": 4, "scorr_dq": 0.2, "xsph_mode": XSPH_OFF, "vorticity_mode": VORTICITY_OFF,
        "max_collision_passes": 64, "cell_width": 0.0, "grid_size": [0, 0, 0],
    }
    p.update(overrides)
    p["cell_width"] = p["cell_width"] or p["smoothing_length"]
    return p


def config_params(**overrides) -> dict:
    """The benchmark workloads' physics: textbook s_corr k 0.1, n 4, dq 0.2h;
    XSPH c 0.01 and textbook vorticity eps 0.0005 over the neighbour list."""
    p = base_params(tensile_mode=TENSILE_TEXTBOOK, xsph_mode=XSPH_LIST, vorticity_mode=VORTICITY_TEXTBOOK)
    p.update(overrides)
    return p


def scene_params(sc, base: dict | None = None) -> dict:
    """A scene's parameters with its grid: calcGridSize for cells of 2h over
    the scene's domain (the scene may fix its own grid)."""
    p = dict(base or config_params())
    if getattr(sc, "grid", None) is not None:
        p["grid_size"] = [int(t) for t in sc.grid]
    if not all(p["grid_size"]):
        p["grid_size"] = list(O.calc_grid_size(2.0 * p["cell_width"], sc.domain_end))
    return p
