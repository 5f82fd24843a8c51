"""Long rollouts: trajectories of FP32 GPU and FP64 CPU diverge chaotically, so the
comparison is statistical -- mean density error, kinetic and potential energy and the
centre of mass of the GPU solver against the FP64 oracle of the same PHYSICS step, after
hundreds of steps of a dam break (WCSPH) and of a PCISPH block."""
import numpy as np
import pytest

from fluids_gb300 import capi, workloads
from parity_util import make_pair

pytestmark = pytest.mark.gpu


def _stats_close(g, o, steps, dens_tol=2e-2):
    msg = "after %d steps: gpu %s oracle %s" % (steps, g, o)
    assert abs(g["kinetic"] - o["kinetic"]) <= 2e-2 * abs(o["kinetic"]) + 1e-9, msg
    assert abs(g["potential"] - o["potential"]) <= 1e-3 * abs(o["potential"]), msg
    for a in ("com_x", "com_y", "com_z"):
        assert abs(g[a] - o[a]) <= 1e-3, msg
    assert abs(g["mean_abs_density_error"] - o["mean_abs_density_error"]) <= \
        dens_tol * o["mean_abs_density_error"] + 1e-4, msg
    assert abs(g["mean_compression"] - o["mean_compression"]) <= 0.1 * o["mean_compression"] + 1e-4, msg


def test_wcsph_dam_break_rollout_statistics(gpu_lib):
    dx, container, steps = 0.015, (1.0, 1.0, 0.6), 400
    fluid = workloads.dam_break(20, 40, 20, dx, container, seed=3)
    params = workloads.wcsph_params(dx, 2e-4, capi.SPH_MODE_PHYSICS)
    bodies = [workloads._tank(container, dx)]
    ctx, orc = make_pair(params, fluid, bodies, container, precision=1)
    ctx.simulate(steps)
    orc.step(steps)
    g, o = ctx.stats(), orc.stats()
    assert ctx.device_flags() & (capi.FLAGS["NAN"] | capi.FLAGS["TIMEOUT"]) == 0
    assert o["kinetic"] > 0
    _stats_close(g, o, steps)


def test_pcisph_block_rollout_statistics(gpu_lib):
    dx, container, steps = 0.02, (1.0, 1.0, 0.6), 150
    fluid = workloads.dam_break(14, 28, 14, dx, container, seed=4)
    params = capi.make_params(capi.SPH_PCISPH, mode=capi.SPH_MODE_PHYSICS, time_step=5e-4, max_vel=20.0,
                              particle_radius=dx / 2, support_radius=2 * dx, pcisph_min_iterations=3,
                              pcisph_max_iterations=8, pcisph_error_ratio=0.01, k_viscosity=0.1,
                              surface_tension=0.0, relax_on_add=0)
    bodies = [workloads._tank(container, dx)]
    ctx, orc = make_pair(params, fluid, bodies, container, precision=1)
    ctx.simulate(steps)
    orc.step(steps)
    g, o = ctx.stats(), orc.stats()
    assert o["kinetic"] > 0
    _stats_close(g, o, steps)


def test_dam_break_65k_full_length_rollout_statistics(gpu_lib):
    """The plain WCSPH dam break at its full size and length: 65,536 particles on a 32 x 64 x
    32 lattice with FishTank walls, 1000 steps of 2e-4 s (PHYSICS).  The GPU's FP32 run against
    the FP64 oracle of the same step, by the statistics of _stats_close (the oracle's own FP32
    and FP64 runs of this scene differ by 0.16 % in kinetic energy and 2e-4 m in centre of
    mass after 1000 steps)."""
    w = workloads.dam_break_65k(mode=capi.SPH_MODE_PHYSICS)
    ctx, orc = make_pair(w["params"], w["fluid"], w["bodies"], w["container"], precision=1)
    ctx.simulate(1000)
    orc.step(1000)
    g, o = ctx.stats(), orc.stats()
    assert ctx.device_flags() & (capi.FLAGS["NAN"] | capi.FLAGS["TIMEOUT"]) == 0
    assert o["kinetic"] > 100.0   # the block has collapsed and is flowing
    _stats_close(g, o, 1000)


def test_pcisph_cube_full_length_rollout_statistics(gpu_lib):
    """The PCISPH scene at its full size and length: 358,400 particles in two 0.5 x 1.0 x 0.7 m
    blocks around the static rotated cube, 500 steps of 5e-4 s (PHYSICS, 3..8 iterations, 1 %
    tolerance).  The GPU's FP32 run against the FP64 oracle of the same step.  The oracle's own
    FP32 and FP64 runs of this scene differ after 500 steps by 0.07 % in kinetic and 0.06 % in
    potential energy, 0.1 mm in centre of mass and 3.1 % in the mean density error (which
    follows the per-step iteration count of the pressure loop), so that statistic is held to
    6 % here instead of 2 %."""
    w = workloads.pcisph_cube(mode=capi.SPH_MODE_PHYSICS)
    ctx, orc = make_pair(w["params"], w["fluid"], w["bodies"], w["container"], precision=1)
    ctx.simulate(500)
    orc.step(500)
    g, o = ctx.stats(), orc.stats()
    assert ctx.device_flags() & (capi.FLAGS["NAN"] | capi.FLAGS["TIMEOUT"]) == 0
    assert o["kinetic"] > 1000.0   # both blocks have collapsed around the cube
    _stats_close(g, o, 500, dens_tol=6e-2)
