"""Host-side mirror of the reference's solver interface (fluid/simulation/fluidsimulation.h:23-92)
over the C ABI: same method names, argument meaning and error behaviour (a failing call
raises, as CLError::check throws in opencl/clerror.cpp:15-19).

    sim = create_simulation(PhysicsSettings(...), SimulationSettings(...))   # factory,
    sim.set_rect_limits(2, 1, 1)                                              # fluidsimulationfactory.h
    sim.add_volume(BoxVolume(size, center))
    sim.add_boundary(FishTank(2, 1, 1), "container")
    sim.simulate()
"""
from dataclasses import dataclass, field

import numpy as np

from . import capi
from .scenes import BoxVolume


@dataclass
class PhysicsSettings:
    """settings/physicssettings.h"""
    rest_density: float = 1000.0
    k_viscosity: float = 0.00001
    gravity: float = 9.8
    gas_stiffness: float = 750.0
    surface_tension: float = 0.001


@dataclass
class SimulationSettings:
    """settings/simulationsettings.h (+ the GB300 build's mode and tuning fields)"""
    time_step: float = 0.0012
    max_vel: float = 10.0
    fluid_particle_radius: float = 0.008
    fluid_support_radius: float = 0.032
    pcisph_max_iterations: int = 7
    pcisph_error_ratio: float = 0.01
    sim_method: str = "WCSPH"              # "WCSPH" | "PCISPH"
    mode: int = capi.SPH_MODE_COMPAT
    extra: dict = field(default_factory=dict)   # any other sph_params field


def to_params(ps, ss):
    method = capi.SPH_PCISPH if ss.sim_method.upper() == "PCISPH" else capi.SPH_WCSPH
    p = capi.default_params(method)
    p.mode = ss.mode
    p.time_step = ss.time_step
    p.max_vel = ss.max_vel
    p.particle_radius = ss.fluid_particle_radius
    p.support_radius = ss.fluid_support_radius
    p.pcisph_max_iterations = ss.pcisph_max_iterations
    p.pcisph_error_ratio = ss.pcisph_error_ratio
    p.rest_density = ps.rest_density
    p.k_viscosity = ps.k_viscosity
    p.gravity = ps.gravity
    p.gas_stiffness = ps.gas_stiffness
    p.surface_tension = ps.surface_tension
    for k, v in ss.extra.items():
        setattr(p, k, v)
    return p


class FluidSimulation:
    """Base class of both solvers (fluidsimulation.h:23-92)."""

    def __init__(self, physics, simulation, params=None):
        self._params = params if params is not None else to_params(physics, simulation)
        self._ctx = capi.Context(self._params)
        self._bodies = []
        self._particle_radius = self._params.particle_radius

    # --- FluidSimulation interface ---------------------------------------------------
    def simulate(self, steps=1):
        """Advances the solver ``steps`` time steps (fluidsimulation.h:36)."""
        self._ctx.simulate(steps)

    def reset(self, physics, simulation):
        """Resets to the initial volumes with new settings (fluidsimulation.h:47-48)."""
        self._params = to_params(physics, simulation)
        self._particle_radius = self._params.particle_radius
        self._ctx.reset(self._params)

    def particle_count(self):
        return self._ctx.particle_count()

    def add_boundary(self, boundary, boundary_id, can_move=False):
        """Samples ``boundary`` (FishTank, Cube or any object with surface_sampling(spacing)
        and a RigidBody pose) at the particle spacing (fluidsimulation.h:66-68)."""
        pts = boundary.surface_sampling(2.0 * self._particle_radius)
        self._ctx.add_boundary(pts, can_move=can_move, rot3x4=boundary.rot3x4(), lin=boundary.lin4(),
                               ang=boundary.ang4(), mass=boundary.mass)
        self._bodies.append((boundary_id, boundary))

    def set_rect_limits(self, width, height, depth):
        self._ctx.set_rect_limits(width, height, depth)

    def boundary_particle_count(self):
        return self._ctx.boundary_particle_count()

    def add_volume(self, volume, velocities=None):
        """Adds a fluid volume (fluidsimulation.h:91): a BoxVolume, or an (n, 4) array."""
        pts = volume.particles(self._particle_radius) if isinstance(volume, BoxVolume) else capi.f4(volume)
        self._ctx.add_volume(pts, velocities)

    # --- GB300 extras ----------------------------------------------------------------
    @property
    def context(self):
        return self._ctx

    def positions(self):
        return self._ctx.get("POS").reshape(-1, 4)

    def velocities(self):
        return self._ctx.get("VEL").reshape(-1, 4)

    def particle_ids(self):
        return self._ctx.get("ID")

    def body_forces(self):
        return self._ctx.body_forces(len(self._bodies))

    def stats(self):
        return self._ctx.stats()

    def check_device(self):
        """Raises if the device status word reports NaN or a timed-out wait."""
        f = self._ctx.device_flags(clear=True)
        if f & capi.FLAGS["TIMEOUT"]:
            raise capi.SphError(6, "a bounded device wait timed out")
        if f & capi.FLAGS["NAN"]:
            raise capi.SphError(5, "non-finite particle state")
        return f

    def close(self):
        self._ctx.close()


class WCSPHSimulation(FluidSimulation):
    """fluid/simulation/wcsphsimluation.h"""


class PCISPHSimulation(FluidSimulation):
    """fluid/simulation/pcisphsimluation.h"""

    def iterations(self):
        return int(self._ctx.get("PCI_ITERS")[0])


def create_simulation(physics, simulation):
    """FluidSimulationFactory::build_simulation (fluidsimulationfactory.h:13-40)."""
    m = simulation.sim_method.upper()
    if m == "WCSPH":
        return WCSPHSimulation(physics, simulation)
    if m == "PCISPH":
        return PCISPHSimulation(physics, simulation)
    raise capi.SphError(1, "Unknown simulation method!")


def positions_by_id(sim):
    """Positions ordered by particle id (the reference keeps no ids; the GB300 build carries
    one so results can be compared across steps)."""
    p = sim.positions()
    ids = sim.particle_ids()
    out = np.empty_like(p)
    out[ids] = p
    return out
