"""Headless counterparts of the reference's scene simulators
(yodaplusplus/ssf_pbf_cuda, src/simulator/**, driven by src/main.cpp's
loop): the same initial conditions, parameters, boundaries, emitter rule and
solver calls, on a particle handle resident on the GPU.  The originals hand
the solver a GL-mapped vertex buffer as the positions each step; here the
handle keeps its own device arrays, and ``SsfRenderer.render_particles``
draws them when a frame is wanted.

The interface follows pbf_base_sim and the simulators
(src/simulator/pbf_base_sim.h:6-30, src/simulator/dam/pbf_dam_sim.h:12-14):
``simulate_one_step``, ``particles_num``, ``particles_position`` (sorted
order, as the reference's), ``global_domain``, ``elapsed_step``,
``elapsed_seconds``, ``time_step``.
"""
from __future__ import annotations

import numpy as np

from . import api

f32 = np.float32


def init_params(space: float, time_step: float, relaxation_numerator: float) -> dict:
    """pbf_parameter as the init conditions set it (pbf_dam_init_cond.cpp:13-21,
    pbf_sphere_init_cond.cpp:13-21): mass from the volume in double,
    h = 1.4f * space, relaxation = k / space^2 (1/m^2), XSPH 0.1 and
    vorticity 0.005 (both inactive in the reference's step), gravity."""
    s = f32(space)
    mass = f32(np.float64(s) ** 3 * f32(1.0e3))
    return api.default_params(
        stable_density=1.0e3, stable_distance=float(s), particle_mass=float(mass),
        smoothing_length=float(f32(1.4) * s), time_step=float(f32(time_step)),
        relaxation=float(f32(relaxation_numerator) / (s * s)), xsph_parameter=float(f32(0.1)),
        vc_parameter=float(f32(0.005)), body_force=[0.0, -9.8, 0.0], cell_width=0.0)


class _Sim:
    iterations = 3  # one_step(..., 3) in both simulators

    def __init__(self, params: dict, capacity: int, domain, device: int):
        self.params = params
        self.domain = (tuple(float(t) for t in domain[0]), tuple(float(t) for t in domain[1]))
        self.particle = api.PbfParticle(params, capacity, self.domain[1], device)
        self.elapsed_step = 0

    @property
    def particles_num(self) -> int:
        return self.particle.num

    def particles_position(self) -> np.ndarray:
        """Positions in the solver's sorted order (getParticlesPosition)."""
        return self.particle.get_particles()[0]

    @property
    def global_domain(self) -> tuple:
        return self.domain

    @property
    def time_step(self) -> float:
        return self.params["time_step"]

    @property
    def elapsed_seconds(self) -> float:
        return self.elapsed_step * self.time_step


class DamSim(_Sim):
    """pbf_dam_sim (src/simulator/dam/pbf_dam_sim.cpp:10-67) with
    pbf_dam_init_cond (pbf_dam_init_cond.cpp:7-25, 59-63): a block
    cartesian_volume((2.25,)*3, (5.65,)*3, space) at rest in the domain
    [1, 10]^3 of 40,000 slots, dt 0.015, stepped by the overload without a
    boundary argument (the fixed sphere (3, 3, 3), r = 3), 3 iterations.
    main.cpp's alternative scene uses space 0.16 (src/main.cpp:83)."""

    def __init__(self, space: float = 0.16, device: int = 0, capacity: int = 40000):
        super().__init__(init_params(space, 0.015, 1.0), capacity, ((1.0,) * 3, (10.0,) * 3), device)
        block = api.arrangement("volume", origin=(2.25,) * 3, end=(5.65,) * 3, space=self.params["stable_distance"])
        self.particle.generate(block)

    def simulate_one_step(self, stream=None):
        api.one_step(self.particle, None, self.domain, self.iterations, stream)
        self.elapsed_step += 1


class SphereSim(_Sim):
    """pbf_sphere_sim (src/simulator/sphere/pbf_sphere_sim.cpp:271-397) with
    pbf_sphere_init_cond (pbf_sphere_init_cond.cpp:7-25, 74-80): an empty
    domain [0.05, 7]^3 of 60,000 slots inside the sphere (3, 3, 3), r = 3,
    filled by a jet on the plane x = 1.25 ((y, z) in [3.5, 4.5] x [2.5, 3.5],
    velocity (2.8, 0, 0)): once at set-up, then on every 8th step while fewer
    than 80% of the slots are used (decided on the device); dt 0.007,
    3 iterations.  src/main.cpp:82 runs it with space 0.1."""

    def __init__(self, space: float = 0.1, device: int = 0, capacity: int = 60000):
        super().__init__(init_params(space, 0.007, 2.0), capacity, ((0.05,) * 3, (7.0,) * 3), device)
        self.boundary = api.Boundary(inner_spheres=[(3.0, 3.0, 3.0, 3.0)])
        jet = api.arrangement("rectangle", axis="x", axis_value=1.25, origin=(3.5, 2.5), end=(4.5, 3.5),
                              space=self.params["stable_distance"])
        self.jet = api.Emitter(arrangement=jet, velocity=(2.8, 0.0, 0.0), device=device)
        self.particle.emit(self.jet, 1.0)  # the set-up add (pbf_sphere_sim.cpp:327-333) always fits
        self._count = 0

    def simulate_one_step(self, stream=None):
        # pbf_sphere_sim.cpp:355-397: the step counter, the jet rule, one_step
        self._count += 1
        if self._count % 8 == 0:
            self.particle.emit(self.jet, 0.8, stream)
        api.one_step(self.particle, self.boundary, self.domain, self.iterations, stream)
        self.elapsed_step += 1


SCENES = {"sphere": SphereSim, "dam": DamSim}
