"""Edge cases of the step on the GPU: no particles, one particle, counts around a warp and a
sort tile, fluid without boundary, boundary without fluid, a crowded cell over the 50-entry
neighbour cap, and a batched context with an empty scene -- each runs graph-captured steps
without a device flag other than the expected ones, with finite state, and agrees with the
oracle where the oracle runs the same inputs."""
import numpy as np
import pytest

from fluids_gb300 import capi
from oracle import Oracle
from scenes_np import jittered_block

pytestmark = pytest.mark.gpu

BAD = capi.FLAGS["NAN"] | capi.FLAGS["TIMEOUT"]
DX = 0.015


def params(method, **kw):
    base = dict(mode=capi.SPH_MODE_PHYSICS, time_step=2e-4 if method == capi.SPH_WCSPH else 5e-4,
                particle_radius=DX / 2, support_radius=2 * DX, k_viscosity=0.01, surface_tension=0.001,
                relax_on_add=0)
    base.update(kw)
    return capi.make_params(method, **base)


def blob(n, seed=0):
    rng = np.random.default_rng(seed)
    p = np.ones((n, 4), np.float32)
    p[:, :3] = rng.uniform(-0.05, 0.05, (n, 3))
    p[:, 1] -= 0.3
    return p


@pytest.mark.parametrize("method", [capi.SPH_WCSPH, capi.SPH_PCISPH])
@pytest.mark.parametrize("n", [1, 2, 31, 33, 4095, 4097])
def test_small_and_ragged_counts(gpu_lib, method, n):
    ctx = capi.Context(params(method))
    ctx.set_rect_limits(0.5, 1.0, 0.4)
    ctx.add_volume(blob(n, seed=n))
    ctx.simulate(5)
    ctx.synchronize()
    assert ctx.device_flags() & BAD == 0
    pos = ctx.get("POS").reshape(-1, 4)
    assert pos.shape == (n, 4) and np.isfinite(pos).all()
    assert sorted(ctx.get("ID").tolist()) == list(range(n))


def test_context_without_particles_steps_as_a_no_op(gpu_lib):
    ctx = capi.Context(params(capi.SPH_WCSPH))
    ctx.set_rect_limits(0.5, 1.0, 0.4)
    ctx.simulate(3)
    ctx.synchronize()
    assert ctx.particle_count() == 0


def test_boundary_only_and_fluid_only(gpu_lib):
    floor = np.array([[x, -0.5, z, 1.0] for x in np.arange(-0.2, 0.21, DX) for z in np.arange(-0.15, 0.16, DX)],
                     np.float32)
    ctx = capi.Context(params(capi.SPH_WCSPH))
    ctx.set_rect_limits(0.5, 1.0, 0.4)
    ctx.add_boundary(floor)
    ctx.simulate(2)               # boundary only: nothing to step
    ctx.add_volume(jittered_block(8, 8, 8, DX, (-0.06, -0.5 + DX, -0.06), seed=4))
    ctx.simulate(5)
    assert ctx.device_flags() & BAD == 0 and np.isfinite(ctx.get("POS")).all()


def test_crowded_cell_caps_the_lists_like_the_oracle(gpu_lib):
    """80 particles inside one cell: every list is capped at 50 entries in traversal order,
    bit-exact with the oracle (COMPAT stages)."""
    rng = np.random.default_rng(5)
    fluid = np.ones((80, 4), np.float32)
    fluid[:, :3] = rng.uniform(0.0, 0.004, (80, 3))
    fluid[:, 1] -= 0.3
    p = capi.make_params(capi.SPH_WCSPH, mode=capi.SPH_MODE_COMPAT, time_step=2e-4, particle_radius=DX / 2,
                         support_radius=2 * DX, relax_on_add=0, neighbor_mode=capi.SPH_NEIGH_LIST)
    ctx = capi.Context(p)
    ctx.set_rect_limits(0.5, 1.0, 0.4)
    ctx.add_volume(fluid)
    o = Oracle(method=0, mode=0, container=(0.5, 1.0, 0.4), time_step=2e-4, particle_radius=DX / 2,
               support_radius=2 * DX)
    o.set_fluid(fluid)
    for st in ("HASHES", "SORT", "SHUFFLE", "CELL_INTERVALS", "NEIGH_LIST"):
        ctx.stage(st)
        o.stage(st)
    assert (ctx.get("NEIGH_LEN") == 50).all()
    assert np.array_equal(ctx.get("NEIGH_LEN"), o.get("NEIGH_LEN"))
    n = 80
    assert np.array_equal(ctx.get("NEIGH_LIST").reshape(-1, n)[:50], o.get("NEIGH_LIST").reshape(-1, n)[:50])


def test_batched_context_with_an_empty_scene(gpu_lib):
    p = params(capi.SPH_WCSPH)
    f1 = jittered_block(6, 6, 6, DX, (-0.05, -0.5 + DX, -0.05), seed=6)
    descs = (capi.SceneDesc * 3)()
    keep = []
    for k, (fl, cont) in enumerate(((f1, (0.5, 1.0, 0.4)), (None, (0.3, 1.0, 0.3)), (f1, (0.6, 1.0, 0.4)))):
        d = descs[k]
        for a in range(3):
            d.container[a] = cont[a]
        d.k_viscosity, d.gas_stiffness = 0.01, p.gas_stiffness
        if fl is not None:
            a = np.ascontiguousarray(fl)
            keep.append(a)
            d.fluid_pos4, d.n_fluid = a.ctypes.data, len(a)
    h = capi.C.c_void_p()
    capi.check(capi.lib().sph_batch_create(capi.C.byref(p), 3, descs, capi.C.byref(h)))
    L = capi.lib()
    try:
        assert L.sph_batch_scene_count(h) == 3
        capi.check(L.sph_simulate(h, 5), h)
        capi.check(L.sph_synchronize(h), h)
        f = capi.C.c_uint()
        capi.check(L.sph_device_flags(h, capi.C.byref(f), 0), h)
        assert f.value & BAD == 0
    finally:
        L.sph_destroy(h)
