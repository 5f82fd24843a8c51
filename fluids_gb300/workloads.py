"""The benchmark scenes, built from seeded synthetic inputs with the shapes the benchmark
configurations name (no dataset is involved).

    dam_break_65k   WCSPH dam break, 32x64x32 lattice at dx = 0.015 m, 2x1x1 m container
    pcisph_cube     PCISPH double block (2 x 0.5x1.0x0.7 m at dx = 0.0125 m) + rotated 0.3 m cube
    double_dam_4m   WCSPH double dam break, 2 x 128^3 at dx = 0.005 m (4,194,304 particles)

Each returns a dict: params (capi.SphParams), fluid (n, 4), velocities or None, bodies
[(points, rot3x4, can_move, mass)], container (w, h, d), steps, plus descriptive fields.
"""
import numpy as np

from . import capi
from .scenes import BoxVolume, Cube, FishTank, jitter, lattice_block, rotation_y

REST_DENSITY = 1000.0
GAMMA = 7.0


def tait_stiffness(c0, rho0=REST_DENSITY, gamma=GAMMA):
    """Tait EOS stiffness k = rho0 c0^2 / gamma."""
    return rho0 * c0 * c0 / gamma


def wcsph_params(dx, dt, mode=capi.SPH_MODE_PHYSICS, c0=20.0, mu=0.01, sigma=0.001, vmax=10.0, **kw):
    p = capi.make_params(capi.SPH_WCSPH, mode=mode, time_step=dt, max_vel=vmax, particle_radius=dx / 2.0,
                         support_radius=2.0 * dx, rest_density=REST_DENSITY, k_viscosity=mu, gravity=9.81,
                         gas_stiffness=tait_stiffness(c0), surface_tension=sigma)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def _tank(container, dx):
    t = FishTank(*container)
    return (t.surface_sampling(dx), t.rot3x4(), 0, 0.0)


def dam_break(nx, ny, nz, dx, container=(2.0, 1.0, 1.0), seed=0, amp=1e-4):
    """A lattice block resting on the floor against the +x wall (one spacing from each)."""
    W, H, D = container
    lo = (W / 2 - nx * dx, -H / 2 + dx, -(nz - 1) * dx / 2)
    return jitter(lattice_block(nx, ny, nz, dx, lo), amp, seed)


def dam_break_65k(mode=capi.SPH_MODE_PHYSICS, seed=0, steps=1000, **kw):
    dx, container = 0.015, (2.0, 1.0, 1.0)
    fluid = dam_break(32, 64, 32, dx, container, seed)
    return dict(name="wcsph_dam_break_65536", params=wcsph_params(dx, 2e-4, mode, **kw), fluid=fluid,
                velocities=None, bodies=[_tank(container, dx)], container=container, steps=steps, dx=dx)


def double_dam_4m(mode=capi.SPH_MODE_PHYSICS, seed=0, steps=200, n=128, **kw):
    """Two n^3 blocks flush with the floor at x in [-1, -0.36] and [0.36, 1] (n = 128)."""
    dx, container = 0.005, (2.0, 1.0, 1.0)
    W, H, D = container
    a = lattice_block(n, n, n, dx, (-W / 2 + dx, -H / 2 + dx, -(n - 1) * dx / 2))
    b = lattice_block(n, n, n, dx, (W / 2 - n * dx, -H / 2 + dx, -(n - 1) * dx / 2))
    fluid = jitter(np.concatenate([a, b]), 1e-4, seed)
    return dict(name="wcsph_double_dam_break_%d" % len(fluid), params=wcsph_params(dx, 5e-5, mode, **kw),
                fluid=fluid, velocities=None, bodies=[_tank(container, dx)], container=container, steps=steps,
                dx=dx)


def pcisph_cube(mode=capi.SPH_MODE_PHYSICS, seed=0, steps=500, dx=0.0125, **kw):
    """Two 0.5x1.0x0.7 m BoxVolumes centred at x = +-(0.75 - dx), y = dx, z = -0.1 and a static
    0.3 m cube at (0, -0.35, 0) rotated 0.5 rad about y.  BoxVolume puts its first layer on the
    box's lower face, so centres at (+-0.74, 0, -0.1) would put that layer on the floor's
    boundary particles and 0.8 dx from the -x wall's; the blocks are raised one spacing and
    moved in to one spacing from the side walls."""
    container = (2.0, 1.0, 1.0)
    r = dx / 2.0
    cx = 0.75 - dx
    vols = [BoxVolume((0.5, 1.0, 0.7), (cx, dx, -0.1)), BoxVolume((0.5, 1.0, 0.7), (-cx, dx, -0.1))]
    fluid = jitter(np.concatenate([v.particles(r) for v in vols]), 1e-4, seed)
    cube = Cube(0.3, 0.0, (0.0, -0.35, 0.0), rotation_y(0.5))
    p = capi.make_params(capi.SPH_PCISPH, mode=mode, time_step=5e-4, max_vel=20.0, particle_radius=r,
                         support_radius=2.0 * dx, pcisph_min_iterations=3, pcisph_max_iterations=8,
                         pcisph_error_ratio=0.01, rest_density=REST_DENSITY, k_viscosity=1.7, gravity=9.81,
                         surface_tension=1.0, relax_on_add=0)
    for k, v in kw.items():
        setattr(p, k, v)
    bodies = [_tank(container, dx), (cube.surface_sampling(dx), cube.rot3x4(), 0, 0.0)]
    return dict(name="pcisph_double_block_cube_%d" % len(fluid), params=p, fluid=fluid, velocities=None,
                bodies=bodies, container=container, steps=steps, dx=dx)


def pcisph_double_dam_4m(mode=capi.SPH_MODE_PHYSICS, seed=0, steps=200, n=128, dt=2e-4, **kw):
    """The 4,194,304-particle double dam break of double_dam_4m stepped by PCISPH with the
    parameters of pcisph_cube (tolerance 1 %, 3..8 iterations); dt = 2e-4 s is that
    configuration's 5e-4 s scaled by the spacing ratio 0.005 / 0.0125."""
    w = double_dam_4m(mode, seed, steps, n)
    dx = w["dx"]
    p = capi.make_params(capi.SPH_PCISPH, mode=mode, time_step=dt, max_vel=20.0, particle_radius=dx / 2.0,
                         support_radius=2.0 * dx, pcisph_min_iterations=3, pcisph_max_iterations=8,
                         pcisph_error_ratio=0.01, rest_density=REST_DENSITY, k_viscosity=1.7, gravity=9.81,
                         surface_tension=1.0, relax_on_add=0)
    for k, v in kw.items():
        setattr(p, k, v)
    w.update(name="pcisph_double_dam_break_%d" % len(w["fluid"]), params=p)
    return w


def batched_scenes(nscenes=256, seed=0, dx=0.015, nmin=2048, nmax=65536):
    """Independent dam breaks of uneven size: N log-uniform in [nmin, nmax], container
    (a, 1, 1) with a ~ U[1, 3], viscosity log-uniform in [1e-3, 1e-1], c0 ~ U[10, 40] m/s.
    Each block has aspect ~1:2:1 and rests on the floor against the +x wall."""
    rng = np.random.default_rng(seed)
    scenes = []
    for s in range(nscenes):
        n = int(round(np.exp(rng.uniform(np.log(nmin), np.log(nmax)))))
        a = float(rng.uniform(1.0, 3.0))
        mu = float(np.exp(rng.uniform(np.log(1e-3), np.log(1e-1))))
        c0 = float(rng.uniform(10.0, 40.0))
        nx = max(2, int(round((n / 2.0) ** (1.0 / 3.0))))
        ny = max(2, min(64, int(round(n / (nx * nx)))))
        container = (a, 1.0, 1.0)
        fluid = dam_break(nx, ny, nx, dx, container, seed=seed * 100003 + s)
        walls = FishTank(*container).surface_sampling(dx)
        scenes.append(dict(container=container, mu=mu, kgas=tait_stiffness(c0), c0=c0, fluid=fluid,
                           boundary=walls, vel=None))
    return scenes


def batched_params(dx=0.015, dt=2e-4, **kw):
    """Shared parameters of the batched scenes (viscosity and stiffness come per scene)."""
    return wcsph_params(dx, dt, capi.SPH_MODE_PHYSICS, **kw)


def scene_params(shared, scene):
    """The single-scene parameters equal to one scene of a batch."""
    p = capi.SphParams.from_buffer_copy(shared)
    p.k_viscosity = scene["mu"]
    p.gas_stiffness = scene["kgas"]
    return p


def build_scene_context(shared, scene):
    """A plain single-scene context for one scene of a batch."""
    ctx = capi.Context(scene_params(shared, scene))
    ctx.set_rect_limits(*scene["container"])
    ctx.add_boundary(scene["boundary"])
    ctx.add_volume(scene["fluid"], scene.get("vel"))
    return ctx


def build_context(w, params=None):
    """Creates a context and loads a workload: limits, boundaries, then the fluid."""
    ctx = capi.Context(params if params is not None else w["params"])
    ctx.set_rect_limits(*w["container"])
    for pts, rot, mv, mass in w["bodies"]:
        ctx.add_boundary(pts, can_move=mv, rot3x4=rot, mass=mass)
    ctx.add_volume(w["fluid"], w.get("velocities"))
    return ctx


def fourier_velocity(pos, nmodes=8, amp=0.5, seed=0, length=0.48):
    """Divergence-free random Fourier field v(x) = sum_k a_k sin(k.x + phi_k) with every a_k
    perpendicular to k (so div v = 0), |k| uniform in [2 pi / length, 8 pi / length], scaled
    so that the largest particle speed is amp."""
    rng = np.random.default_rng(seed)
    x = np.asarray(pos, dtype=np.float64)[:, :3]
    v = np.zeros_like(x)
    for _ in range(nmodes):
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        k = d * rng.uniform(2 * np.pi / length, 8 * np.pi / length)
        a = rng.normal(size=3)
        a -= d * np.dot(a, d)
        phi = rng.uniform(0, 2 * np.pi)
        v += np.sin(x @ k + phi)[:, None] * a[None, :]
    v *= amp / np.max(np.linalg.norm(v, axis=1))
    out = np.zeros((len(x), 4), np.float32)
    out[:, :3] = v
    return out


def adjoint_block(n_side=32, dx=0.015, seed=0, steps=200, checkpoint_every=20, mu=0.01, c0=20.0):
    """Differentiable WCSPH workload: an n_side^3 lattice block at dx (jitter 1e-4) centred in a
    2x2x2 m container (no boundary particles, no wall contact within the run), a divergence-
    free Fourier initial velocity with 8 modes and amplitude 0.5 m/s, and a seeded target
    cloud (each particle's start plus a 1 cm Gaussian offset and a 1 cm shift in x) for the
    loss mean_i |x_i(T) - y_i|^2.  Surface tension is 0."""
    container = (2.0, 2.0, 2.0)
    lo = -(n_side - 1) * dx / 2
    fluid = jitter(lattice_block(n_side, n_side, n_side, dx, (lo, lo, lo)), 1e-4, seed)
    vel = fourier_velocity(fluid, 8, 0.5, seed + 1, length=n_side * dx)
    rng = np.random.default_rng(seed + 2)
    target = fluid.copy()
    target[:, :3] += rng.normal(scale=0.01, size=(len(fluid), 3)).astype(np.float32)
    target[:, 0] += 0.01
    p = wcsph_params(dx, 2e-4, capi.SPH_MODE_PHYSICS, c0=c0, mu=mu, sigma=0.0)
    return dict(name="wcsph_adjoint_%d" % len(fluid), params=p, fluid=fluid, velocities=vel, target=target,
                bodies=[], container=container, steps=steps, checkpoint_every=checkpoint_every, dx=dx, mu=mu,
                c0=c0, kgas=tait_stiffness(c0))
