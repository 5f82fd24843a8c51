"""Argument checks of the C ABI that run before any device work (no GPU needed): the mesh
voxelizer, the screen-space image entry points, checkpoint files and fault injection refuse
bad input with SPH_E_* codes instead of launching."""
import ctypes as C

import numpy as np

from fluids_gb300 import capi


def test_voxelizer_refuses_bad_meshes_before_launch():
    L = capi.lib()
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    ix = np.array([0, 1, 2], np.uint32)
    vx = L.sph_scene_voxelize
    p = capi.ptr
    assert vx(p(tri), 3, p(np.array([0, 1, 3], np.uint32)), 3, 0.25, 0.025, None, 0) == -capi.SPH_E_INVALID
    assert vx(p(tri), 3, p(ix), 2, 0.25, 0.025, None, 0) == -capi.SPH_E_INVALID          # not triangles
    assert vx(p(tri), 3, p(ix), 3, 0.0, 0.0, None, 0) == -capi.SPH_E_INVALID             # voxel size
    assert vx(p(tri), 3, p(ix), 3, 0.25, -1.0, None, 0) == -capi.SPH_E_INVALID           # precision
    assert vx(None, 3, p(ix), 3, 0.25, 0.025, None, 0) == -capi.SPH_E_INVALID
    bad = tri.copy()
    bad[1, 0] = np.inf
    assert vx(p(bad), 3, p(ix), 3, 0.25, 0.025, None, 0) == -capi.SPH_E_INVALID          # non-finite vertex
    # one triangle spanning more than 2^24 voxels: refused on the host
    assert vx(p(tri), 3, p(ix), 3, 1e-4, 1e-5, None, 0) == -capi.SPH_E_OVERFLOW


def test_image_entry_points_refuse_bad_sizes_and_aliasing():
    L = capi.lib()
    buf = C.c_void_p(0x1000)   # never dereferenced: every call below is refused first
    other = C.c_void_p(0x2000)
    assert L.sph_filter_bilateral(buf, other, 0, 10, None) == capi.SPH_E_INVALID
    assert L.sph_filter_bilateral(buf, other, 70000, 2, None) == capi.SPH_E_INVALID     # beyond the grid
    assert L.sph_filter_bilateral(buf, buf, 16, 16, None) == capi.SPH_E_INVALID         # in place
    assert L.sph_filter_bilateral(None, other, 16, 16, None) == capi.SPH_E_INVALID
    assert L.sph_render_smooth(buf, other, 16, 16, -1, None) == capi.SPH_E_INVALID
    assert L.sph_filter_curvature_flow(buf, buf, 16, 16, 1.0, 1.0, None) == capi.SPH_E_INVALID
    ip = (C.c_float * 16)()
    assert L.sph_render_normals(buf, other, 16, 0, ip, None) == capi.SPH_E_INVALID
    assert L.sph_render_normals(buf, other, 16, 16, None, None) == capi.SPH_E_INVALID
    view = capi.make_view(np.eye(4), np.eye(4), 0.1, 100.0, 64, 48)
    assert L.sph_render_depth(None, C.byref(view), buf) == capi.SPH_E_INVALID


def test_state_and_fault_entry_points_refuse_null_contexts():
    L = capi.lib()
    assert L.sph_save_state(None, b"/tmp/x") == capi.SPH_E_INVALID
    assert L.sph_load_state(None, b"/tmp/x") == capi.SPH_E_INVALID
    assert L.sph_inject_fault(None, capi.SPH_FAULT_BARRIER_STALL) == capi.SPH_E_INVALID


def test_scene_builders_refuse_bad_arguments():
    L = capi.lib()
    nv, ni = C.c_int(), C.c_int()
    assert L.sph_scene_icosphere(1.0, 5, None, 0, None, 0, C.byref(nv), C.byref(ni)) == capi.SPH_E_INVALID
    assert L.sph_scene_icosphere(1.0, -1, None, 0, None, 0, C.byref(nv), C.byref(ni)) == capi.SPH_E_INVALID
    assert L.sph_scene_sphere(0.1, 0.0, None, 0) < 0
    assert L.sph_scene_sphere(0.0, 0.01, None, 0) < 0
    assert L.sph_scene_load_obj(None, None, 0, None, 0, C.byref(nv), C.byref(ni)) == capi.SPH_E_INVALID
