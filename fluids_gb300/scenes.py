"""Scene objects of the reference (fluid volumes and rigid bodies) for the headless driver.

``BoxVolume.particles``, ``FishTank.surface_sampling``, ``Cube.surface_sampling``,
``Sphere.surface_sampling`` and ``Model.surface_sampling`` call the C-ABI samplers that restate
fluid/simulation/boxvolume.cpp:11-40, scene/fishtank.cpp:108-141, scene/cube.cpp:136-171,
scene/sphere.cpp:135-171 and scene/model.cpp:170-214 (the last on the GPU).  ``jitter`` is the seeded splitmix64 jitter of the benchmark
scenes.  The benchmark scenes (dam breaks, the rotated cube) are built by ``make_scene``.
"""
import math

import numpy as np

from . import capi


def _sample(fn, *args):
    n = fn(*args, None, 0)
    if n < 0:
        raise ValueError("bad sampler arguments")
    out = np.zeros((n, 4), np.float32)
    fn(*args, capi.ptr(out), n)
    return out


class BoxVolume:
    """fluid/simulation/boxvolume.h: a box of fluid given by size and centre."""

    def __init__(self, size, center):
        self.size = np.asarray(size, np.float32).reshape(3)
        self.center = np.asarray(center, np.float32).reshape(3)

    def particles(self, particle_radius):
        L = capi.lib()
        s = np.ascontiguousarray(self.size)
        c = np.ascontiguousarray(self.center)
        return _sample(L.sph_scene_box_volume, capi.ptr(s), capi.ptr(c), float(particle_radius))


class RigidBody:
    """Pose, velocity and mass a boundary needs (scene/rigidbody.h without Bullet)."""

    def __init__(self, mass=0.0, position=(0.0, 0.0, 0.0), rotation=None, linear_vel=(0, 0, 0),
                 angular_vel=(0, 0, 0)):
        self.mass = float(mass)
        self.position = np.asarray(position, np.float32).reshape(3)
        self.rotation = np.eye(3, dtype=np.float32) if rotation is None else np.asarray(rotation, np.float32)
        self.linear_vel = np.asarray(linear_vel, np.float32).reshape(3)
        self.angular_vel = np.asarray(angular_vel, np.float32).reshape(3)

    def rot3x4(self):
        m = np.zeros((3, 4), np.float32)
        m[:, :3] = self.rotation
        m[:, 3] = self.position
        return m

    def lin4(self):
        return np.append(self.linear_vel, 0.0).astype(np.float32)

    def ang4(self):
        return np.append(self.angular_vel, 0.0).astype(np.float32)


class FishTank(RigidBody):
    """scene/fishtank.h: open-top rectangular container centred at the origin."""

    def __init__(self, width, height, depth, mass=0.0):
        super().__init__(mass)
        self.width, self.height, self.depth = float(width), float(height), float(depth)

    def surface_sampling(self, spacing):
        return _sample(capi.lib().sph_scene_fishtank, self.width, self.height, self.depth, float(spacing))


class Cube(RigidBody):
    """scene/cube.h: a cube of side ``side``, sampled as a hollow shell in body coordinates."""

    def __init__(self, side, mass=0.0, position=(0, 0, 0), rotation=None):
        super().__init__(mass, position, rotation)
        self.side = float(side)

    def surface_sampling(self, spacing):
        return _sample(capi.lib().sph_scene_cube, self.side, float(spacing))


def load_obj(path):
    """ModelMesh(path) (sph_scene_load_obj): (vertices (n, 3) float32, indices (m,) uint32)."""
    L = capi.lib()
    nv, ni = capi.C.c_int(), capi.C.c_int()
    capi.check(L.sph_scene_load_obj(str(path).encode(), None, 0, None, 0, capi.C.byref(nv), capi.C.byref(ni)))
    v = np.zeros((nv.value, 3), np.float32)
    ix = np.zeros(ni.value, np.uint32)
    capi.check(L.sph_scene_load_obj(str(path).encode(), capi.ptr(v), nv.value, capi.ptr(ix), ni.value,
                                    capi.C.byref(nv), capi.C.byref(ni)))
    return v, ix


def voxelize(vertices3, indices, voxel_size, precision=None):
    """sph_scene_voxelize (GPU): the 8 corners of every voxel the mesh touches, (n, 4)."""
    L = capi.lib()
    v = np.ascontiguousarray(vertices3, np.float32).reshape(-1, 3)
    ix = np.ascontiguousarray(indices, np.uint32).reshape(-1)
    prec = float(voxel_size) / 10.0 if precision is None else float(precision)
    args = (capi.ptr(v), len(v), capi.ptr(ix), len(ix), float(voxel_size), prec)
    n = L.sph_scene_voxelize(*args, None, 0)
    if n < 0:
        raise capi.SphError(-n, "sph_scene_voxelize")
    out = np.zeros((n, 4), np.float32)
    if n:
        capi.check(min(0, L.sph_scene_voxelize(*args, capi.ptr(out), n)))
    return out


def icosphere(radius, level):
    """IcoSphereMesh(radius, level): (vertices (n, 3), indices (m,))."""
    L = capi.lib()
    nv, ni = capi.C.c_int(), capi.C.c_int()
    capi.check(L.sph_scene_icosphere(float(radius), int(level), None, 0, None, 0, capi.C.byref(nv),
                                     capi.C.byref(ni)))
    v = np.zeros((nv.value, 3), np.float32)
    ix = np.zeros(ni.value, np.uint32)
    capi.check(L.sph_scene_icosphere(float(radius), int(level), capi.ptr(v), nv.value, capi.ptr(ix), ni.value,
                                     capi.C.byref(nv), capi.C.byref(ni)))
    return v, ix


class Sphere(RigidBody):
    """scene/sphere.h: a sphere of radius ``radius`` (the scene files' "size"), sampled from a
    level-3 icosphere."""

    def __init__(self, radius, mass=0.0, position=(0, 0, 0)):
        super().__init__(mass, position)
        self.radius = float(radius)

    def surface_sampling(self, spacing):
        return _sample(capi.lib().sph_scene_sphere, self.radius, float(spacing))


class Wall(RigidBody):
    """scene/wall.h: a width x height plane (z = 0 in body coordinates)."""

    def __init__(self, width, height, mass=0.0, position=(0, 0, 0), rotation=None):
        super().__init__(mass, position, rotation)
        self.width, self.height = float(width), float(height)

    def surface_sampling(self, spacing):
        return _sample(capi.lib().sph_scene_wall, self.width, self.height, float(spacing))


class Model(RigidBody):
    """scene/model.h: a triangle mesh read from an OBJ file, sampled by voxelizing it on the
    GPU (voxel size = particle spacing, precision = spacing / 10)."""

    def __init__(self, obj_filename, mass=0.0, position=(0, 0, 0), rotation=None):
        super().__init__(mass, position, rotation)
        self.vertices, self.indices = load_obj(obj_filename)

    def surface_sampling(self, spacing):
        return voxelize(self.vertices, self.indices, float(spacing), float(spacing) / 10.0)


def rotation_y(theta):
    c, s = math.cos(theta), math.sin(theta)
    return np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]], np.float32)


def jitter(pos4, amp, seed):
    p = capi.f4(pos4).copy()
    capi.lib().sph_jitter(capi.ptr(p), len(p), float(amp), int(seed) & 0xFFFFFFFFFFFFFFFF)
    return p


def lattice_block(nx, ny, nz, dx, lo):
    """nx*ny*nz particles at spacing dx from corner lo (loop order y, x, z as BoxVolume)."""
    j, i, k = np.meshgrid(np.arange(ny), np.arange(nx), np.arange(nz), indexing="ij")
    p = np.zeros((nx * ny * nz, 4), np.float32)
    p[:, 0] = (lo[0] + i.reshape(-1) * dx)
    p[:, 1] = (lo[1] + j.reshape(-1) * dx)
    p[:, 2] = (lo[2] + k.reshape(-1) * dx)
    p[:, 3] = 1
    return p
