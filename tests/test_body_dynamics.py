"""Two-way rigid-body coupling (sph_set_body_dynamics): the integrator on known motions
(oracle, CPU) and the GPU against the oracle with the fluid pushing the body (-m gpu)."""
import numpy as np
import pytest

from fluids_gb300 import capi, workloads
from fluids_gb300.scenes import Cube, rotation_y
from oracle import Oracle
from parity_util import make_pair
from scenes_np import jittered_block

DX = 0.015
CONTAINER = (0.5, 1.0, 0.4)


def cube_body(side, center, mass, rot=None):
    c = Cube(side, mass=mass, position=center, rotation=rot)
    return c.surface_sampling(DX), c.rot3x4()


def solid_cube_inv_inertia(side, mass):
    return [6.0 / (mass * side * side)] * 3


def far_fluid():
    return jittered_block(4, 4, 4, DX, (0.1, -0.45, 0.1), seed=1)


def oracle_with_body(center, mass=0.2, side=0.06, ang=None, radius=0.0):
    o = Oracle(method=0, mode=1, container=CONTAINER, time_step=2e-4, surface_tension=0.0)
    pts, rot = cube_body(side, center, mass)
    o.add_boundary(pts, can_move=1, rot3x4=rot, ang=ang, mass=mass)
    o.set_body_dynamics(0, True, solid_cube_inv_inertia(side, mass), radius)
    o.set_fluid(far_fluid())
    return o


def test_free_fall_is_semi_implicit_euler():
    o = oracle_with_body((-0.1, 0.2, -0.1))
    n, dt, g = 50, np.float32(2e-4), -9.81
    o.step(n)
    rot, lin, ang = o.body_state(0)
    assert np.allclose(o.get("BODY_FORCE")[:3], 0) and np.allclose(ang, 0)
    assert lin[1] == pytest.approx(n * g * dt, rel=1e-5)
    assert rot[1, 3] == pytest.approx(0.2 + g * dt * dt * n * (n + 1) / 2, abs=1e-6)
    assert rot[0, 3] == pytest.approx(-0.1, abs=1e-7)


def test_spin_turns_about_the_axis_and_stays_orthonormal():
    w = 3.0
    o = oracle_with_body((-0.1, 0.2, -0.1), ang=[0.0, w, 0.0, 0.0])
    n = 400
    o.step(n)
    rot, _, ang = o.body_state(0)
    R = rot[:, :3].astype(np.float64)
    assert np.allclose(R @ R.T, np.eye(3), atol=1e-6)
    th = w * 2e-4 * n
    Ry = np.array([[np.cos(th), 0, np.sin(th)], [0, 1, 0], [-np.sin(th), 0, np.cos(th)]])
    assert np.allclose(R, Ry, atol=1e-4)
    assert ang[1] == pytest.approx(w, rel=1e-6)


def test_container_keeps_the_centre_inside():
    o = oracle_with_body((-0.1, -0.447, -0.1), radius=0.05)
    o.step(300)
    rot, lin, _ = o.body_state(0)
    assert rot[1, 3] == pytest.approx(-0.5 + 0.05, abs=1e-6) and lin[1] == 0.0


def test_dynamics_needs_a_movable_body_with_mass():
    o = Oracle(method=0, mode=1, container=CONTAINER)
    pts, rot = cube_body(0.06, (0, 0, 0), 0.0)
    o.add_boundary(pts, can_move=1, rot3x4=rot, mass=0.0)
    with pytest.raises(ValueError):
        o.set_body_dynamics(0, True, [1, 1, 1], 0.0)


@pytest.mark.gpu
def test_gpu_body_follows_oracle_in_fluid(gpu_lib):
    """A light cube submerged in a fluid block (the fluid inside its volume removed): the
    fluid's pressure pushes it up, gravity pulls it down; the GPU's body trajectory and
    fluid agree with the oracle's."""
    fluid = jittered_block(14, 16, 12, DX, (-0.1, -0.5 + DX, -0.08), seed=2)
    side, mass = 0.06, 0.1
    center = np.array([0.0, -0.5 + DX + 7 * DX, 0.0], np.float32)
    inside = np.all(np.abs(fluid[:, :3] - center) < side / 2 + DX / 2, axis=1)
    fluid = np.ascontiguousarray(fluid[~inside])
    pts, rot = cube_body(side, tuple(center), mass)
    floor = np.array([[x, -0.5, z, 1.0] for x in np.arange(-0.25, 0.26, DX) for z in np.arange(-0.2, 0.21, DX)],
                     np.float32)
    params = workloads.wcsph_params(DX, 2e-4, capi.SPH_MODE_PHYSICS, sigma=0.0)
    bodies = [(floor, None, 0, 0.0), (pts, rot, 1, mass)]
    ctx, orc = make_pair(params, fluid, bodies, CONTAINER)
    ii = solid_cube_inv_inertia(side, mass)
    ctx.set_body_dynamics(1, True, ii, side / 2)
    orc.set_body_dynamics(1, True, ii, side / 2)
    with pytest.raises(capi.SphError):
        ctx.set_body_dynamics(0, True, ii, 0.0)      # static floor
    steps = 60
    ctx.simulate(steps)
    orc.step(steps)
    gr, gl, ga = ctx.body_state(1)
    orr, ol, oa = orc.body_state(1)
    f = orc.get("BODY_FORCE")[4:7]
    assert np.linalg.norm(f) > 0, "the fluid must push the body"
    assert np.abs(gr - orr).max() < 1e-6
    assert np.abs(gl - ol).max() <= 1e-4 * max(np.abs(ol).max(), 1e-3)
    assert np.abs(ga - oa).max() <= 1e-3 * max(np.abs(oa).max(), 1e-3) + 1e-6
    pos = ctx.get("POS").reshape(-1, 4)
    opos = orc.get("POS").reshape(-1, 4)
    assert np.abs(pos[:, :3] - opos[:, :3]).max() < 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [capi.SPH_MODE_COMPAT, capi.SPH_MODE_PHYSICS])
def test_gpu_boundary_force_and_torque_match_oracle(gpu_lib, mode):
    """compute_fluid_force + clsum (kernels/boundary.cl:61-118, boundaryhandler.cpp:296-349)
    in one stage on identical inputs: a movable cube with mass, turned 0.3 rad about y,
    submerged in a fluid block under a hydrostatic pressure field.  The body's summed force
    and torque agree with the oracle's within 1e-5 (the torque relative to the larger of its
    own size and the force times the cube's half side, since a nearly symmetric body has a
    small torque)."""
    fluid = jittered_block(14, 16, 12, DX, (-0.1, -0.5 + DX, -0.08), seed=3)
    side, mass = 0.06, 0.1
    center = np.array([0.0, -0.5 + DX + 7 * DX, 0.0], np.float32)
    inside = np.all(np.abs(fluid[:, :3] - center) < side / 2 + DX, axis=1)
    fluid = np.ascontiguousarray(fluid[~inside])
    c = Cube(side, mass=mass, position=tuple(center), rotation=rotation_y(0.3))
    pts, rot = c.surface_sampling(DX), c.rot3x4()
    params = workloads.wcsph_params(DX, 2e-4, mode, sigma=0.0)
    ctx, orc = make_pair(params, fluid, [(pts, rot, 1, mass)], CONTAINER)
    for s in ("BOUNDARY_SYNC", "HASHES", "SORT", "SHUFFLE", "CELL_INTERVALS"):
        ctx.stage(s)
        orc.stage(s)
    assert np.array_equal(ctx.get("BPOS_SORTED"), orc.get("BPOS_SORTED"))
    assert np.array_equal(ctx.get("CELL_INTERVALS"), orc.get("CELL_INTERVALS"))
    y = ctx.get("POS_SORTED").reshape(-1, 4)[:, 1].astype(np.float64)
    p = (1000.0 * 9.81 * (y.max() + DX - y)).astype(np.float32)
    d = (1000.0 + p / 400.0).astype(np.float32)
    for o in (ctx, orc):
        o.set("DENSITY", d)
        o.set("PRESSURE", p)
        o.stage("BOUNDARY_FORCES")
    f, t = ctx.get("BODY_FORCE")[:3].astype(np.float64), ctx.get("BODY_TORQUE")[:3].astype(np.float64)
    of, ot = orc.get("BODY_FORCE")[:3].astype(np.float64), orc.get("BODY_TORQUE")[:3].astype(np.float64)
    assert np.linalg.norm(of) > 0 and np.linalg.norm(ot) > 0
    assert np.linalg.norm(f - of) <= 1e-5 * np.linalg.norm(of)
    assert np.linalg.norm(t - ot) <= 1e-5 * max(np.linalg.norm(ot), np.linalg.norm(of) * side / 2)
    ctx.close()
