"""Mesh and sphere boundary sampling: the OBJ reader (sph_scene_load_obj) and icosphere
against the reference's own ModelMesh / IcoSphereMesh compiled for the CPU (oracle/_ref,
where the reference is mounted), the sphere sampler against the restatement in
oracle/mesh.py, and the GPU voxelizer (sph_scene_voxelize) against the golden output of the
reference's vendored voxelizer (tests/golden/voxel_teapot.npz) -- all bit for bit, the
voxelizer's list in its own order."""
import os

import numpy as np
import pytest

from fluids_gb300 import capi, scenes
from oracle import mesh as omesh
from oracle import refkernels

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "voxel_teapot.npz")
MODELS = os.path.join(refkernels.REFERENCE_ROOT, "data", "models")
needs_ref = pytest.mark.skipif(not (refkernels.available() and os.path.isdir(MODELS)),
                               reason="reference sources not mounted")


@needs_ref
@pytest.mark.parametrize("model", ["teapot", "bunny", "armadillo", "dragon", "dragon_small"])
def test_obj_reader_matches_reference_modelmesh(model):
    path = os.path.join(MODELS, model + ".obj")
    v, ix = scenes.load_obj(path)
    rv, rix = refkernels.load_obj(path)
    assert np.array_equal(v, rv) and np.array_equal(ix, rix)


def test_obj_reader_faces_and_references(tmp_path):
    """Fans of polygons, negative (relative) references, v/t, v//n and v/t/n forms, and one
    vertex per distinct (position, normal) pair."""
    obj = tmp_path / "quad.obj"
    obj.write_text("v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvt 0 0\nvn 0 0 1\nvn 0 0 -1\n"
                   "f 1 2 3 4\n"
                   "f -4/1 -3/1 -2/1\n"
                   "f 1//1 2//1 3//2\n"
                   "f 1/1/1 3/1/1 4/1/1\n")
    v, ix = scenes.load_obj(str(obj))
    tri = v[ix].reshape(-1, 3, 3)
    assert len(tri) == 5
    assert np.array_equal(tri[0], [[0, 0, 0], [1, 0, 0], [1, 1, 0]])
    assert np.array_equal(tri[1], [[0, 0, 0], [1, 1, 0], [0, 1, 0]])
    assert np.array_equal(tri[2], [[0, 0, 0], [1, 0, 0], [1, 1, 0]])
    # (1, no normal), (2, -), (3, -), (4, -), then (1, n1), (2, n1), (3, n2), (3, n1), (4, n1)
    assert len(v) == 9
    assert list(ix[:6]) == [0, 1, 2, 0, 2, 3] and list(ix[6:9]) == [0, 1, 2]
    assert list(ix[9:]) == [4, 5, 6, 4, 7, 8]
    with pytest.raises(capi.SphError):
        scenes.load_obj(str(tmp_path / "missing.obj"))
    bad = tmp_path / "bad.obj"
    bad.write_text("v 0 0 0\nf 1 2 3\n")
    with pytest.raises(capi.SphError):
        scenes.load_obj(str(bad))


def test_icosphere_matches_restatement():
    for level in range(4):
        v, ix = scenes.icosphere(0.1, level)
        ov, oix = omesh.icosphere(0.1, level)
        assert np.array_equal(v, ov) and np.array_equal(ix, oix)
    v, ix = scenes.icosphere(1.0, 3)
    assert len(v) == 1272 and len(ix) == 3840
    assert np.allclose(np.linalg.norm(v, axis=1), 1.0, atol=1e-6)


@needs_ref
def test_icosphere_matches_reference():
    for level in range(4):
        v, ix = scenes.icosphere(0.25, level)
        rv, rix = refkernels.icosphere(0.25, level)
        assert np.array_equal(v, rv) and np.array_equal(ix, rix)


@pytest.mark.parametrize("radius,spacing", [(0.1, 0.015), (0.05, 0.01), (0.3, 0.03)])
def test_sphere_sampling_matches_restatement(radius, spacing):
    got = scenes.Sphere(radius).surface_sampling(spacing)
    want = omesh.sphere_sampling(radius, spacing)
    assert np.array_equal(got, want)
    # the last 1272 particles are the icosphere's vertices, on the sphere
    assert np.allclose(np.linalg.norm(got[-1272:, :3], axis=1), radius, rtol=1e-6)


@needs_ref
def test_voxel_golden_is_the_reference_output():
    g = dict(np.load(GOLDEN))
    v, ix = refkernels.load_obj(os.path.join(MODELS, "teapot.obj"))
    assert np.array_equal(v, g["vertices"]) and np.array_equal(ix, g["indices"])
    out = refkernels.voxelize(g["vertices"], g["indices"], g["spacing"], g["precision"])
    assert np.array_equal(out, g["out"])


def test_voxel_golden_shape():
    """Corners come in groups of 8 around a voxel centre, half a voxel away on every axis."""
    g = dict(np.load(GOLDEN))
    out = g["out"][:, :3].reshape(-1, 8, 3)
    centre = out.mean(axis=1, keepdims=True)
    assert np.allclose(np.abs(out - centre), g["spacing"] / 2, atol=1e-6)


@pytest.mark.gpu
def test_gpu_voxelizer_matches_reference_golden(gpu_lib):
    g = dict(np.load(GOLDEN))
    out = scenes.voxelize(g["vertices"], g["indices"], float(g["spacing"]), float(g["precision"]))
    assert out.shape == g["out"].shape
    bad = np.nonzero(np.any(out != g["out"], axis=1))[0]
    assert len(bad) == 0, "%d of %d particles differ, first %s: %s vs %s" % (
        len(bad), len(out), bad[:4], out[bad[:4]], g["out"][bad[:4]])


@pytest.mark.gpu
def test_gpu_voxelizer_edge_cases(gpu_lib):
    L = capi.lib()
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    ix = np.array([0, 1, 2], np.uint32)
    # a zero-area triangle gives no voxel
    flat = np.array([[0, 0, 0], [1, 0, 0], [2, 0, 0]], np.float32)
    assert len(scenes.voxelize(flat, ix, 0.1)) == 0
    # one triangle: every output voxel touches it, corners in groups of 8
    out = scenes.voxelize(tri, ix, 0.25)
    assert len(out) > 0 and len(out) % 8 == 0
    # count-only call, then a too-small buffer writes nothing
    n = L.sph_scene_voxelize(capi.ptr(tri), 3, capi.ptr(ix), 3, 0.25, 0.025, None, 0)
    assert n == len(out)
    buf = np.full((n, 4), 7.0, np.float32)
    assert L.sph_scene_voxelize(capi.ptr(tri), 3, capi.ptr(ix), 3, 0.25, 0.025, capi.ptr(buf), n - 1) == n
    assert (buf == 7.0).all()
    # bad arguments and a triangle spanning more than 2^24 voxels are refused before launch
    bad_ix = np.array([0, 1, 5], np.uint32)
    assert L.sph_scene_voxelize(capi.ptr(tri), 3, capi.ptr(bad_ix), 3, 0.25, 0.025, None, 0) == -capi.SPH_E_INVALID
    assert L.sph_scene_voxelize(capi.ptr(tri), 3, capi.ptr(ix), 2, 0.25, 0.025, None, 0) == -capi.SPH_E_INVALID
    assert L.sph_scene_voxelize(capi.ptr(tri), 3, capi.ptr(ix), 3, 0.0, 0.0, None, 0) == -capi.SPH_E_INVALID
    assert L.sph_scene_voxelize(capi.ptr(tri), 3, capi.ptr(ix), 3, 1e-4, 1e-5, None, 0) == -capi.SPH_E_OVERFLOW


def test_wall_sampling_matches_restatement():
    """Wall::surface_sampling (scene/wall.cpp:142-152): x outer, y inner, float steps."""
    from fluids_gb300.scenes import Wall
    for w, h, s in ((0.5, 0.3, 0.015), (1.0, 0.2, 0.03), (0.0, 0.1, 0.02)):
        got = Wall(w, h).surface_sampling(s)
        want = []
        x = -np.float32(w) / np.float32(2)
        while x <= np.float32(w) / np.float32(2):
            y = -np.float32(h) / np.float32(2)
            while y <= np.float32(h) / np.float32(2):
                want.append((x, y, 0.0, 1.0))
                y = np.float32(y + np.float32(s))
            x = np.float32(x + np.float32(s))
        assert np.array_equal(got, np.array(want, np.float32).reshape(-1, 4))
