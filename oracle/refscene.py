"""The benchmark scenes for bench.py's reference arm, built without the product library --
TEST INFRASTRUCTURE.

The fluid is the benchmark's seeded lattice (the loop order of BoxVolume::particles, y
slowest) with its splitmix64 jitter, restated here in numpy; the container walls come from
the reference's own FishTank::surface_sampling (scene/fishtank.cpp:108-141, compiled by
oracle/build_ref.sh).  tests/test_scene_pinning.py checks that these are bit for bit the
scenes fluids_gb300.workloads builds through the library, so both arms step the same
particles.
"""
import numpy as np

from . import refkernels as rk

GOLDEN = np.uint64(0x9E3779B97F4A7C15)


def jitter(pos4, amp, seed):
    """pos += (2u - 1) amp per x, y, z component in particle order, u the top 24 bits of
    successive splitmix64 outputs from state seed (the library's sph_jitter)."""
    p = np.array(pos4, np.float32, copy=True).reshape(-1, 4)
    m = np.arange(1, 3 * len(p) + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + m * GOLDEN
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    z ^= z >> np.uint64(31)
    u = (z >> np.uint64(40)).astype(np.float32) * np.float32(1.0 / 16777216.0)
    d = (np.float32(2.0) * u - np.float32(1.0)) * np.float32(amp)
    p[:, :3] += d.reshape(-1, 3)
    return p


def lattice_block(nx, ny, nz, dx, lo):
    j, i, k = np.meshgrid(np.arange(ny), np.arange(nx), np.arange(nz), indexing="ij")
    p = np.zeros((nx * ny * nz, 4), np.float32)
    p[:, 0] = lo[0] + i.reshape(-1) * dx
    p[:, 1] = lo[1] + j.reshape(-1) * dx
    p[:, 2] = lo[2] + k.reshape(-1) * dx
    p[:, 3] = 1
    return p


def double_dam_4m(seed=0, n=128):
    """The WCSPH double dam break: two n^3 blocks at dx = 0.005 m flush with the floor at
    x in [-1, -0.36] and [0.36, 1] of a 2 x 1 x 1 m tank, jitter 1e-4 m; dt = 5e-5 s, the
    dam break's fluid constants (c0 = 20 m/s, mu = 0.01, sigma = 0.001, vmax = 10 m/s)."""
    dx, container = 0.005, (2.0, 1.0, 1.0)
    W, H, D = container
    a = lattice_block(n, n, n, dx, (-W / 2 + dx, -H / 2 + dx, -(n - 1) * dx / 2))
    b = lattice_block(n, n, n, dx, (W / 2 - n * dx, -H / 2 + dx, -(n - 1) * dx / 2))
    fluid = jitter(np.concatenate([a, b]), 1e-4, seed)
    walls = rk.scene_fishtank(W, H, D, dx)
    params = dict(time_step=5e-5, max_vel=10.0, k_viscosity=0.01, surface_tension=0.001,
                  gas_stiffness=1000.0 * 20.0 * 20.0 / 7.0, rest_density=1000.0, gravity=9.81,
                  particle_radius=dx / 2.0, support_radius=2.0 * dx)
    return dict(name="wcsph_double_dam_break_%d" % len(fluid), fluid=fluid, walls=walls, container=container,
                dx=dx, params=params)
