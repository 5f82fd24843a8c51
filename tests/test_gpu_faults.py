"""Failure detection without a GPU fault: faults are made on the host (a NaN written into the
state, a particle put outside the grid, an unreachable PCISPH tolerance, a barrier stall
injected through sph_inject_fault) and the device status word reports each; the context
stays usable afterwards."""
import numpy as np
import pytest

from fluids_gb300 import capi, workloads

pytestmark = pytest.mark.gpu

F = capi.FLAGS


def wcsph_ctx():
    w = workloads.dam_break_65k(steps=10)
    return workloads.build_context(w)


def pcisph_ctx(eta=0.01, max_iter=8):
    dx = 0.015
    from scenes_np import jittered_block
    fluid = jittered_block(12, 12, 12, dx, (-0.09, -0.5 + dx, -0.09), seed=3)
    p = capi.make_params(capi.SPH_PCISPH, mode=capi.SPH_MODE_PHYSICS, time_step=5e-4, max_vel=10.0,
                         particle_radius=dx / 2, support_radius=2 * dx, k_viscosity=0.01, surface_tension=0.0,
                         pcisph_min_iterations=3, pcisph_max_iterations=max_iter, pcisph_error_ratio=eta,
                         relax_on_add=0)
    ctx = capi.Context(p)
    ctx.set_rect_limits(0.5, 1.0, 0.4)
    ctx.add_volume(fluid)
    return ctx


def test_nan_in_the_state_is_flagged(gpu_lib):
    ctx = wcsph_ctx()
    ctx.simulate(2)
    assert ctx.device_flags(clear=True) & F["NAN"] == 0
    good = ctx.get("POS").copy()
    bad = good.copy()
    bad[4 * 100] = np.nan
    ctx.set("POS", bad)
    ctx.simulate(1)
    assert ctx.device_flags(clear=True) & F["NAN"]
    # recovery: the good state back, the flag stays clear
    ctx.set("POS", good)
    ctx.set("VEL", np.zeros_like(good))
    ctx.set("VEL_HALF", np.zeros_like(good))
    ctx.simulate(3)
    assert ctx.device_flags(clear=True) & F["NAN"] == 0
    assert np.isfinite(ctx.get("POS")).all()


def test_particle_outside_the_grid_is_flagged_and_clamped(gpu_lib):
    ctx = wcsph_ctx()
    pos = ctx.get("POS").reshape(-1, 4).copy()
    pos[7, 0] = 40.0          # far outside the container-fitted grid
    ctx.set("POS", pos)
    ctx.simulate(1)
    assert ctx.device_flags(clear=True) & F["ESCAPED"]
    out = ctx.get("POS").reshape(-1, 4)
    assert np.isfinite(out).all() and np.abs(out[:, 0]).max() <= 1.0 + 1e-6   # the box clamp brought it back


def test_unreachable_pcisph_tolerance_is_flagged(gpu_lib):
    ctx = pcisph_ctx(eta=1e-9, max_iter=3)
    ctx.simulate(1)
    assert ctx.device_flags(clear=True) & F["NONCONVERGED"]
    assert int(ctx.get("PCI_ITERS")[0]) == 3


def test_injected_barrier_stall_times_out_and_the_context_recovers(gpu_lib):
    ctx = pcisph_ctx()
    ctx.simulate(2)
    assert ctx.device_flags(clear=True) & F["TIMEOUT"] == 0
    before = ctx.get("POS").copy()
    ctx.inject_fault(capi.SPH_FAULT_BARRIER_STALL)
    ctx.simulate(1)                      # every CTA's bounded wait runs out (about a second)
    flags = ctx.device_flags(clear=True)
    assert flags & F["TIMEOUT"]
    assert np.array_equal(ctx.get("POS"), before)   # the timed-out step did not integrate
    ctx.simulate(3)                      # later steps run normally
    assert ctx.device_flags(clear=True) & F["TIMEOUT"] == 0
    assert not np.array_equal(ctx.get("POS"), before)
    with pytest.raises(capi.SphError):
        wcsph_ctx().inject_fault(capi.SPH_FAULT_BARRIER_STALL)   # WCSPH has no grid barrier


def test_injected_allocation_failure_leaves_the_context_unchanged(gpu_lib):
    """An allocator failure made on the host (the next arena allocation is refused as
    cudaMalloc refuses one): each scene call that must grow the arena returns SPH_E_NOMEM, and
    the context keeps its particles, bodies, container and evolved state, steps on, and grows
    once the allocation is allowed."""
    from scenes_np import jittered_block
    ctx = wcsph_ctx()
    ctx.simulate(3)
    n, nb = ctx.particle_count(), ctx.boundary_particle_count()
    state = {f: ctx.get(f).copy() for f in ("POS", "VEL", "VEL_HALF", "ID")}
    extra = jittered_block(4, 4, 4, 0.015, (0.3, -0.2, 0.0), seed=9)
    wall = np.array([[x, 0.2, z, 1.0] for x in np.arange(-0.1, 0.1, 0.015) for z in np.arange(-0.1, 0.1, 0.015)],
                    np.float32)
    for call in (lambda: ctx.add_volume(extra), lambda: ctx.add_boundary(wall),
                 lambda: ctx.set_rect_limits(2.2, 1.0, 1.0)):
        ctx.inject_fault(capi.SPH_FAULT_ALLOC_FAIL)
        with pytest.raises(capi.SphError) as e:
            call()
        assert e.value.code == capi.SPH_E_NOMEM
        assert ctx.particle_count() == n and ctx.boundary_particle_count() == nb
        for f, a in state.items():
            assert np.array_equal(ctx.get(f), a), f
    ctx.simulate(2)                      # the context steps on
    assert ctx.device_flags(clear=True) & (F["NAN"] | F["TIMEOUT"]) == 0
    assert not np.array_equal(ctx.get("POS"), state["POS"])
    ctx.add_boundary(wall)               # and grows once the allocation is allowed
    assert ctx.boundary_particle_count() == nb + len(wall)
    ctx.inject_fault(capi.SPH_FAULT_ALLOC_FAIL)
    ctx.inject_fault(capi.SPH_FAULT_NONE)   # cancelled: the next growth succeeds
    ctx.add_volume(extra)
    assert ctx.particle_count() == n + len(extra)
    ctx.simulate(2)
    assert np.isfinite(ctx.get("POS")).all()
