"""Host side of the screen-space fluid surface: the camera of scene/camera.cpp and the stage
sequence of SSpaceFluidRenderer (fluid/render/sspacefluidrenderer.cpp), over the C ABI of
include/sph_capi.h (sph_render_depth, sph_render_smooth, sph_render_normals,
sph_render_shade).  Images are device tensors (torch is only the allocator here); the
background the scene would draw behind the fluid and the skybox cube map are caller images.
"""
import math

import numpy as np

from . import capi


def perspective(fov_deg, aspect, near, far):
    """QMatrix4x4::perspective as Camera::set_perspective uses it (scene/camera.cpp:32-36),
    in mathematical (row, column) layout."""
    f = 1.0 / math.tan(math.radians(fov_deg) / 2.0)
    m = np.zeros((4, 4), np.float64)
    m[0, 0] = f / aspect
    m[1, 1] = f
    m[2, 2] = -(far + near) / (far - near)
    m[2, 3] = -2.0 * far * near / (far - near)
    m[3, 2] = -1.0
    return m.astype(np.float32)


def look_at(eye, center, up):
    """QMatrix4x4::lookAt: world to eye coordinates, in mathematical layout."""
    eye, center, up = (np.asarray(a, np.float64) for a in (eye, center, up))
    f = center - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -f
    m[:3, 3] = -m[:3, :3] @ eye
    return m.astype(np.float32)


def _rotation(angle_deg, axis):
    """QMatrix4x4::rotate's matrix for a unit axis (mathematical layout)."""
    a = math.radians(angle_deg)
    c, s = math.cos(a), math.sin(a)
    x, y, z = axis
    m = np.eye(4)
    m[:3, :3] = [[c + x * x * (1 - c), x * y * (1 - c) - z * s, x * z * (1 - c) + y * s],
                 [y * x * (1 - c) + z * s, c + y * y * (1 - c), y * z * (1 - c) - x * s],
                 [z * x * (1 - c) - y * s, z * y * (1 - c) + x * s, c + z * z * (1 - c)]]
    return m


class Camera:
    """The reference's default camera: perspective fov 45 degrees, near 0.5, far 30, aspect =
    width / height (gui/glwidget.cpp:82-88) and the view transformation translate(0, 0, -zoom)
    . rotate(roll about x) . rotate(pitch about y) with zoom 4, roll 45, pitch 0
    (scene/camera.cpp:4-21)."""

    def __init__(self, width, height, fov=45.0, near=0.5, far=30.0, zoom=4.0, roll=45.0, pitch=0.0):
        self.width, self.height = int(width), int(height)
        self.fov, self.near, self.far = float(fov), float(near), float(far)
        self.zoom, self.roll, self.pitch = float(zoom), float(roll), float(pitch)

    def transformation(self):
        """Camera::transformation(): the fluid's modelview (scene/fluid.cpp:55-60, fluid at
        the origin)."""
        t = np.eye(4)
        t[2, 3] = -self.zoom
        return (t @ _rotation(self.roll, (1, 0, 0)) @ _rotation(self.pitch, (0, 1, 0))).astype(np.float32)

    def projection(self):
        return perspective(self.fov, self.width / max(self.height, 1), self.near, self.far)

    def point_scale(self):
        """The depth stage's point_scale uniform (sspacefluidrenderer.cpp:366)."""
        return self.width * math.tan(math.radians(self.fov) * 0.5)


class SSpaceFluidRenderer:
    """Depth, blur and normals stages of SSpaceFluidRenderer::render (:35-53) for one
    context.  filter_iterations: the blur stage runs the bilateral filter twice per
    iteration (:388-407).  point_radius: the depth stage's sprite radius (0.0625 in the
    reference, :365)."""

    def __init__(self, width, height, filter_iterations=2, point_radius=0.125 * 0.5):
        import torch
        self.width, self.height = int(width), int(height)
        self.filter_iterations = int(filter_iterations)
        self.point_radius = float(point_radius)
        dev = torch.device("cuda", torch.cuda.current_device())
        self.depth = torch.zeros((self.height, self.width), dtype=torch.float32, device=dev)
        self.blurred = torch.zeros_like(self.depth)
        self.normals = torch.zeros((self.height, self.width, 4), dtype=torch.float32, device=dev)
        self.color = torch.zeros((self.height, self.width, 4), dtype=torch.float32, device=dev)
        self._mv = None

    def render(self, ctx, camera, mv_matrix, stream=None):
        """Renders ctx's fluid particles; returns (depth after the blur stage, normals).
        stream: the integer cudaStream_t the context runs on (Context.set_stream); all
        stages are then queued on it.  With None the host waits for the depth stage and the
        filters run on the default stream."""
        pr = camera.projection()
        view = capi.make_view(mv_matrix, pr, self.point_radius, camera.point_scale(), self.width, self.height)
        ctx.render_depth(view, self.depth.data_ptr())
        if stream is None:
            ctx.synchronize()
        s = int(stream or 0)
        capi.render_smooth(self.depth.data_ptr(), self.blurred.data_ptr(), self.width, self.height,
                           self.filter_iterations, s)
        capi.render_normals(self.depth.data_ptr(), self.normals.data_ptr(), self.width, self.height,
                            np.linalg.inv(pr.astype(np.float64)).astype(np.float32), s)
        self._mv = np.asarray(mv_matrix, np.float32)
        return self.depth, self.normals

    def shade(self, camera, background=None, cube_map=None, stream=None):
        """_render_final_stage (final_stage.frag) after render(): the fluid's colour as an
        (h, w, 4) device image.  background: (h, w, 4) float32 device tensor or None;
        cube_map: (6, S, S, 4) float32 device tensor (faces +x, -x, +y, -y, +z, -z) or None."""
        if self._mv is None:
            raise RuntimeError("shade() needs render() first")
        pr = camera.projection()
        ipr = np.linalg.inv(pr.astype(np.float64)).astype(np.float32)
        bg = 0 if background is None else background.data_ptr()
        cube, size = (0, 0) if cube_map is None else (cube_map.data_ptr(), int(cube_map.shape[1]))
        capi.render_shade(self.depth.data_ptr(), self.normals.data_ptr(), bg, cube, size, self.width, self.height,
                          self._mv, ipr, self.color.data_ptr(), int(stream or 0))
        return self.color
