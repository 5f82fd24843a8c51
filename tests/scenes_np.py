"""Small seeded particle sets for CPU tests (numpy only, no product library needed)."""
import numpy as np


def jittered_block(nx, ny, nz, dx, lo, amp=1e-4, seed=0):
    """Lattice block of nx*ny*nz particles at spacing dx from corner ``lo``, jittered by
    U(-amp, amp) per component; float32 (N, 4) with w = 1."""
    rng = np.random.default_rng(seed)
    g = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij"), -1).reshape(-1, 3)
    p = np.zeros((len(g), 4), np.float32)
    p[:, :3] = (g * dx + np.asarray(lo)).astype(np.float32)
    p[:, :3] += rng.uniform(-amp, amp, (len(g), 3)).astype(np.float32)
    p[:, 3] = 1
    return p


def floor_patch(x0, x1, z0, z1, y, dx):
    xs = np.arange(x0, x1, dx, dtype=np.float32)
    zs = np.arange(z0, z1, dx, dtype=np.float32)
    return np.array([[x, y, z, 1.0] for x in xs for z in zs], np.float32)


def small_scene(seed=0):
    """About 2k fluid particles resting on a boundary floor inside a 0.5 x 1 x 0.4 m box:
    the block touches the +x and -z container limits so the collision branch runs."""
    dx = 0.015
    fluid = jittered_block(12, 16, 10, dx, (0.25 - 11 * dx, -0.5 + dx, -0.2), seed=seed)
    floor = floor_patch(-0.25, 0.26, -0.2, 0.21, -0.5, dx)
    return dict(fluid=fluid, boundary=floor, container=(0.5, 1.0, 0.4), dx=dx)
