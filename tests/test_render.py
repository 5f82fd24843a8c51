"""Screen-space fluid surface (fluids_gb300/csrc/sph_render.cu) against the restatement in
oracle/render.py and the golden images of tests/golden/render_small.npz (depth and normals
from the restatement; bilateral, two blur iterations and curvature flow from the reference's
own kernels/bilateral.cl and kernels/curvatureflow.cl compiled for the CPU).

Tolerances: the depth and normals images bit for bit (the kernels round every operation
like the restatement); the filters within 2e-6 of the depth scale for the bilateral filter
(exp differs in its last bits) and 1e-5 relative to each pixel's magnitude for the curvature
flow (pow(d, 1.5) likewise)."""
import os

import numpy as np
import pytest

from fluids_gb300 import capi
from oracle import refkernels
from oracle import render as orender

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "render_small.npz")


def golden():
    return dict(np.load(GOLDEN))


def assert_curvature(name, got, want):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    err = np.abs(got - want) / np.maximum(np.abs(want), 1.0)
    assert np.isfinite(got).all() == np.isfinite(want).all(), name
    assert err.max() <= 1e-5, "%s: max rel err %.3g at %s" % (name, err.max(), np.unravel_index(err.argmax(), err.shape))


def assert_bilateral(name, got, want):
    err = np.abs(np.asarray(got, np.float64) - want).max()
    assert err <= 2e-6, "%s: max err %.3g" % (name, err)


def describe_mismatch(got, want):
    bad = got != want
    if not bad.any():
        return "equal"
    idx = np.argwhere(bad)[:5]
    return "%d of %d differ, first %s: %s vs %s, max |diff| %.3g" % (
        bad.sum(), bad.size, idx.tolist(), got[bad][:5], want[bad][:5], np.nanmax(np.abs(got - want)))


# ---- the restatement (CPU) ------------------------------------------------------------

def test_restatement_reproduces_golden():
    g = golden()
    d = orender.splat_depth(g["pos"], g["modelview"], g["projection"], g["point_radius"], g["point_scale"],
                            int(g["width"]), int(g["height"]))
    assert np.array_equal(d, g["depth"]), describe_mismatch(d, g["depth"])
    assert_bilateral("bilateral", orender.bilateral(g["depth"]), g["bilateral"])
    s = g["depth"]
    for _ in range(4):
        s = orender.bilateral(s)
    assert_bilateral("smooth2", s, g["smooth2"])
    ip = g["inv_projection"]
    assert_curvature("curvature", orender.curvature_flow(g["depth"], ip[0, 0], ip[1, 1]), g["curvature"])
    n = orender.depth_normals(g["smooth2"], ip)
    assert np.array_equal(n, g["normals"]), describe_mismatch(n, g["normals"])


@pytest.mark.skipif(not refkernels.available(), reason="reference kernels not available")
def test_filter_restatement_matches_reference_kernels():
    rng = np.random.default_rng(7)
    img = np.zeros((40, 56), np.float32)
    img[5:33, 8:50] = 0.6 + 0.01 * rng.random((28, 42)).astype(np.float32)
    img[12:18, 20:30] = 0.62                  # a step inside the 0.015 gate
    img[20:24, 30:34] = 0.7                   # a step outside it
    img[0:3, 0:4] = 0.5                       # touching the clamped edge
    assert_bilateral("bilateral", orender.bilateral(img), refkernels.bilateral_filter(img))
    for ipx, ipy in ((-0.55, -0.41), (0.9, 0.7)):
        assert_curvature("curvature", orender.curvature_flow(img, ipx, ipy), refkernels.curvature_flow(img, ipx, ipy))


def test_single_sprite_is_a_disc_at_the_sphere_depth():
    w, h = 96, 96
    pr = orender.perspective(45.0, 1.0, 0.5, 30.0)
    mv = np.eye(4, dtype=np.float32)
    pos = np.array([[0.0, 0.0, -3.0, 0.0]], np.float32)
    radius, scale = 1.0, w * np.tan(np.radians(22.5))
    d = orender.splat_depth(pos, mv, pr, radius, scale, w, h)
    size = radius * scale / 3.0
    area = (d != 0).sum()
    assert abs(area - np.pi * (size / 2) ** 2) < 0.1 * area
    # the centre fragment lies on the sphere at eye z = -3 + radius; the depth uses the
    # transposed projection (sphere_pos_eye * pr_matrix)
    z = np.float64(-3.0 + radius)
    nd = (pr[0, 2] * 0 + pr[2, 2] * z + pr[3, 2]) / (pr[2, 3] * z + pr[3, 3])
    assert abs(d[h // 2, w // 2] - nd) < 2e-3


def test_nearer_sprite_wins_and_ties_keep_the_first():
    w, h = 48, 48
    pr = orender.perspective(45.0, 1.0, 0.5, 30.0)
    mv = np.eye(4, dtype=np.float32)
    far = np.array([[0.0, 0.0, -4.0, 0.0]], np.float32)
    near = np.array([[0.0, 0.0, -3.0, 0.0]], np.float32)
    args = (mv, pr, 0.3, w * np.tan(np.radians(22.5)), w, h)
    a = orender.splat_depth(np.concatenate([far, near]), *args)
    b = orender.splat_depth(np.concatenate([near, far]), *args)
    n = orender.splat_depth(near, *args)
    assert np.array_equal(a, b)
    assert a[h // 2, w // 2] == n[h // 2, w // 2]
    twice = orender.splat_depth(np.concatenate([near, near]), *args)
    assert np.array_equal(twice, n)


def test_filters_leave_empty_pixels_empty():
    img = np.zeros((16, 16), np.float32)
    img[4:8, 4:8] = 0.5
    out = orender.bilateral(img)
    assert (out[img == 0] == 0).all()
    # a flat patch is a fixed point of the bilateral filter
    assert np.allclose(out[img != 0], 0.5, atol=1e-7)


# ---- the CUDA kernels (GPU) -------------------------------------------------------------

def _context(pos4):
    p = capi.make_params(0, mode=capi.SPH_MODE_COMPAT, relax_on_add=0, neighbor_mode=capi.SPH_NEIGH_LIST)
    ctx = capi.Context(p)
    ctx.set_rect_limits(1.0, 1.0, 1.0)
    ctx.add_volume(pos4)
    return ctx


@pytest.mark.gpu
def test_gpu_depth_matches_restatement(gpu_lib):
    import torch
    g = golden()
    w, h = int(g["width"]), int(g["height"])
    ctx = _context(g["pos"])
    pos = ctx.get("POS").reshape(-1, 4)
    view = capi.make_view(g["modelview"], g["projection"], g["point_radius"], g["point_scale"], w, h)
    img = torch.full((h, w), 7.0, dtype=torch.float32, device="cuda")
    ctx.render_depth(view, img.data_ptr())
    ctx.synchronize()
    got = img.cpu().numpy()
    want = orender.splat_depth(pos, g["modelview"], g["projection"], g["point_radius"], g["point_scale"], w, h)
    if np.array_equal(pos, g["pos"]):
        assert np.array_equal(want, g["depth"])
    assert np.array_equal(got, want), describe_mismatch(got, want)
    # a second, larger image reallocates the depth-test scratch
    view2 = capi.make_view(g["modelview"], g["projection"], g["point_radius"], g["point_scale"], 2 * w, 2 * h)
    img2 = torch.empty((2 * h, 2 * w), dtype=torch.float32, device="cuda")
    ctx.render_depth(view2, img2.data_ptr())
    ctx.synchronize()
    want2 = orender.splat_depth(pos, g["modelview"], g["projection"], g["point_radius"], g["point_scale"], 2 * w,
                                2 * h)
    got2 = img2.cpu().numpy()
    assert np.array_equal(got2, want2), describe_mismatch(got2, want2)


@pytest.mark.gpu
def test_gpu_filters_match_reference_golden(gpu_lib):
    import torch
    g = golden()
    w, h = int(g["width"]), int(g["height"])
    src = torch.from_numpy(g["depth"]).cuda()
    out = torch.empty_like(src)
    capi.filter_bilateral(src.data_ptr(), out.data_ptr(), w, h)
    torch.cuda.synchronize()
    assert_bilateral("bilateral", out.cpu().numpy(), g["bilateral"])
    work = src.clone()
    tmp = torch.empty_like(src)
    capi.render_smooth(work.data_ptr(), tmp.data_ptr(), w, h, 2)
    torch.cuda.synchronize()
    assert_bilateral("smooth2", work.cpu().numpy(), g["smooth2"])
    ip = g["inv_projection"]
    capi.filter_curvature_flow(src.data_ptr(), out.data_ptr(), w, h, ip[0, 0], ip[1, 1])
    torch.cuda.synchronize()
    assert_curvature("curvature", out.cpu().numpy(), g["curvature"])
    with pytest.raises(capi.SphError):
        capi.filter_bilateral(src.data_ptr(), src.data_ptr(), w, h)


@pytest.mark.gpu
def test_gpu_normals_match_restatement(gpu_lib):
    import torch
    g = golden()
    w, h = int(g["width"]), int(g["height"])
    src = torch.from_numpy(g["smooth2"]).cuda()
    nrm = torch.full((h, w, 4), 9.0, dtype=torch.float32, device="cuda")
    capi.render_normals(src.data_ptr(), nrm.data_ptr(), w, h, g["inv_projection"])
    torch.cuda.synchronize()
    got = nrm.cpu().numpy()
    assert np.array_equal(got, g["normals"]), describe_mismatch(got, g["normals"])


@pytest.mark.gpu
def test_gpu_renderer_stage_sequence(gpu_lib):
    """SSpaceFluidRenderer.render: depth, two blur iterations and normals on the context's
    stream reproduce the golden blurred depth; the normals follow the restatement."""
    import torch
    from fluids_gb300 import render
    g = golden()
    w, h = int(g["width"]), int(g["height"])
    ctx = _context(g["pos"])
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    cam = render.Camera(w, h)
    assert np.array_equal(cam.projection(), g["projection"])
    r = render.SSpaceFluidRenderer(w, h, filter_iterations=2, point_radius=float(g["point_radius"]))
    depth, normals = r.render(ctx, cam, g["modelview"], stream.cuda_stream)
    torch.cuda.synchronize()
    assert_bilateral("blurred depth", depth.cpu().numpy(), g["smooth2"])
    want = orender.depth_normals(depth.cpu().numpy(), g["inv_projection"])
    got = normals.cpu().numpy()
    assert np.array_equal(got, want), describe_mismatch(got, want)


def shade_inputs(g):
    h, w = int(g["height"]), int(g["width"])
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float32)
    bkg = np.stack([xx / w, yy / h, 0.5 + 0.0 * xx, np.ones_like(xx)], -1).astype(np.float32)
    S = 8
    t = np.linspace(0.0, 1.0, S, dtype=np.float32)
    cube = np.zeros((6, S, S, 4), np.float32)
    for f in range(6):
        cube[f, ..., 0] = 0.1 * f + t[None, :] * 0.3
        cube[f, ..., 1] = t[:, None] * 0.5
        cube[f, ..., 2] = 1.0 - 0.1 * f
        cube[f, ..., 3] = 1.0
    return bkg, cube


def test_shade_restatement_properties():
    g = golden()
    bkg, cube = shade_inputs(g)
    col = orender.shade(g["smooth2"], g["normals"], bkg, cube, g["modelview"], g["inv_projection"])
    fluid = g["smooth2"] > 0
    assert np.array_equal(col[~fluid][:, :3], bkg[~fluid][:, :3]) and (col[..., 3] == 1).all()
    assert np.isfinite(col[fluid]).all()
    plain = orender.shade(g["smooth2"], g["normals"], None, None, g["modelview"], g["inv_projection"])
    assert (plain[~fluid][:, :3] == 0).all()
    # the cube-map face table: axis directions land on their own face's centre texels
    for f, d in enumerate(([1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1])):
        got = orender._cube(cube, np.array([d], np.float32))[0]
        assert np.allclose(got, cube[f].mean(axis=(0, 1)), atol=1e-6)


@pytest.mark.gpu
def test_gpu_shade_matches_restatement(gpu_lib):
    """final_stage.frag on the GPU against the restatement: every operation rounds the same
    way except powf (specular and Fresnel), so colours agree within 2e-5."""
    import torch
    g = golden()
    w, h = int(g["width"]), int(g["height"])
    bkg, cube = shade_inputs(g)
    d = torch.from_numpy(g["smooth2"]).cuda()
    n = torch.from_numpy(g["normals"]).cuda()
    b = torch.from_numpy(bkg).cuda()
    cm = torch.from_numpy(cube).cuda()
    out = torch.full((h, w, 4), 5.0, dtype=torch.float32, device="cuda")
    capi.render_shade(d.data_ptr(), n.data_ptr(), b.data_ptr(), cm.data_ptr(), cube.shape[1], w, h, g["modelview"],
                      g["inv_projection"], out.data_ptr())
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    want = orender.shade(g["smooth2"], g["normals"], bkg, cube, g["modelview"], g["inv_projection"])
    err = np.abs(got.astype(np.float64) - want).max()
    assert err <= 2e-5, "max colour error %.3g" % err
    # no background and no cube map: black behind, no reflection
    capi.render_shade(d.data_ptr(), n.data_ptr(), 0, 0, 0, w, h, g["modelview"], g["inv_projection"],
                      out.data_ptr())
    torch.cuda.synchronize()
    want = orender.shade(g["smooth2"], g["normals"], None, None, g["modelview"], g["inv_projection"])
    assert np.abs(out.cpu().numpy().astype(np.float64) - want).max() <= 2e-5


@pytest.mark.gpu
def test_gpu_render_frame_equals_the_stage_sequence(gpu_lib):
    """sph_render_frame (host image) equals depth -> 2 blur iterations -> normals -> shade
    called one by one (no background, no cube map), up to the last bits of the inverse
    projection (inverted in C there, by numpy here)."""
    import torch
    from fluids_gb300 import render
    g = golden()
    w, h = int(g["width"]), int(g["height"])
    ctx = _context(g["pos"])
    view = capi.make_view(g["modelview"], g["projection"], g["point_radius"], g["point_scale"], w, h)
    frame = ctx.render_frame(view, 2)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    cam = render.Camera(w, h)
    r = render.SSpaceFluidRenderer(w, h, filter_iterations=2, point_radius=float(g["point_radius"]))
    r.render(ctx, cam, g["modelview"], stream.cuda_stream)
    col = r.shade(cam, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    ref = col.cpu().numpy()
    assert np.abs(frame.astype(np.float64) - ref).max() <= 1e-4
    assert np.array_equal(frame[..., 3], ref[..., 3]) and frame[..., :3].max() > 0


LIGHTS = [((-1.0, -1.0, -1.0), (1.0, 1.0, 1.0, 1.0)), ((0.5, -1.0, 0.2), (0.4, 0.3, 0.2, 1.0))]


def test_particles_restatement_properties():
    w = h = 64
    pr = orender.perspective(45.0, 1.0, 0.5, 30.0)
    mv = np.eye(4, dtype=np.float32)
    near = np.array([[0.0, 0.0, -3.0, 1.0]], np.float32)
    far = np.array([[0.0, 0.0, -4.0, 1.0]], np.float32)
    args = (mv, pr, 0.5, w * np.tan(np.radians(22.5)), w, h, LIGHTS)
    a = orender.particles_image(np.concatenate([far, near]), *args)
    b = orender.particles_image(np.concatenate([near, far]), *args)
    n = orender.particles_image(near, *args)
    assert np.array_equal(a, b) and np.array_equal(a[h // 2, w // 2], n[h // 2, w // 2])
    assert (a >= 0).all() and (a <= 1).all() and (a[..., 3] == 1).all()
    assert a[..., :3].max() > 0 and (a[0, 0, :3] == 0).all()


@pytest.mark.gpu
def test_gpu_particles_match_restatement(gpu_lib):
    """The particle render method: depth test, winners and lighting bit for bit."""
    import torch
    g = golden()
    w, h = int(g["width"]), int(g["height"])
    ctx = _context(g["pos"])
    pos = ctx.get("POS").reshape(-1, 4)
    view = capi.make_view(g["modelview"], g["projection"], g["point_radius"] * 0.5, g["point_scale"], w, h)
    img = torch.full((h, w, 4), 3.0, dtype=torch.float32, device="cuda")
    ctx.render_particles(view, LIGHTS, img.data_ptr())
    ctx.synchronize()
    got = img.cpu().numpy()
    want = orender.particles_image(pos, g["modelview"], g["projection"], g["point_radius"] * 0.5, g["point_scale"],
                                   w, h, LIGHTS)
    assert np.array_equal(got, want), describe_mismatch(got, want)
    frame = ctx.render_frame(view, method=capi.SPH_RENDER_PARTICLES, lights=LIGHTS)
    assert np.array_equal(frame, want)
