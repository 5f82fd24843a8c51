"""CPU restatement of the reference's screen-space fluid surface -- TEST INFRASTRUCTURE (the
checker of fluids_gb300/csrc/sph_render.cu; nothing in the product imports it).

  splat_depth      shaders/sspace_fluid_rendering/depth_stage.vert:15-24 and depth_stage.frag:52-85
                   drawn as GL_POINTS in particle order with GL_LESS against a depth buffer
                   cleared to 1 (fluid/render/sspacefluidrenderer.cpp:353-386); no background
                   depth texture (fragments at normalised depth >= 1 are dropped)
  bilateral        kernels/bilateral.cl:5-47
  curvature_flow   kernels/curvatureflow.cl:54-129
  depth_normals    shaders/sspace_fluid_rendering/normals_stage.frag:108-144, sampling texel
                   centres with the coordinates clamped to the image
  shade            shaders/sspace_fluid_rendering/final_stage.frag:25-74, offset reads bilinear
                   (GL_LINEAR, clamped), the cube map by the OpenGL face table

Images are (height, width) float32 arrays, row 0 at the bottom (window coordinates).
Matrices are 4x4 in mathematical (row, column) layout.  splat_depth and depth_normals do
every multiply and add in float32 in the order the CUDA kernels do (the kernels are built
without FMA contraction), so the two agree bit for bit; the filters call exp and pow,
whose last bit the CUDA versions are free to differ in.  The filter restatements are pinned
against the reference's own kernels compiled for the CPU (oracle/_ref).
"""
import numpy as np

F = np.float32


def _mv(m, v):
    """m @ v for a 4x4 float32 matrix and four float32 arrays, summed left to right."""
    return [((m[r, 0] * v[0] + m[r, 1] * v[1]) + m[r, 2] * v[2]) + m[r, 3] * v[3] for r in range(4)]


def splat_depth(pos4, modelview, projection, point_radius, point_scale, width, height):
    """NDC depth of the nearest sphere-sprite fragment per pixel, 0 where none."""
    mv = np.asarray(modelview, F).reshape(4, 4)
    pr = np.asarray(projection, F).reshape(4, 4)
    rad, scale = F(point_radius), F(point_scale)
    zbuf = np.full((height, width), np.inf, F)
    depth = np.zeros((height, width), F)
    pos4 = np.asarray(pos4, F).reshape(-1, 4)
    one = F(1.0)
    for p in pos4:
        e = _mv(mv, [p[0], p[1], p[2], one])
        c = _mv(pr, e)
        if not (c[3] > 0) or abs(c[0]) > c[3] or abs(c[1]) > c[3] or abs(c[2]) > c[3]:
            continue
        dist = np.sqrt((e[0] * e[0] + e[1] * e[1]) + e[2] * e[2])
        size = max(rad * (scale / dist), one)
        wx = ((c[0] / c[3] + one) * F(0.5)) * F(width)
        wy = ((c[1] / c[3] + one) * F(0.5)) * F(height)
        x0, x1 = max(0, int(np.floor(wx - F(0.5) * size))), min(width - 1, int(np.ceil(wx + F(0.5) * size)))
        y0, y1 = max(0, int(np.floor(wy - F(0.5) * size))), min(height - 1, int(np.ceil(wy + F(0.5) * size)))
        if x0 > x1 or y0 > y1:
            continue
        px = np.arange(x0, x1 + 1, dtype=F)[None, :]
        py = np.arange(y0, y1 + 1, dtype=F)[:, None]
        nx = (F(2.0) * ((px + F(0.5)) - wx)) / size + np.zeros_like(py)
        ny = (F(-2.0) * ((py + F(0.5)) - wy)) / size + np.zeros_like(px)
        mag = nx * nx + ny * ny
        inside = mag <= one
        with np.errstate(invalid="ignore", divide="ignore"):
            nz = np.sqrt(one - mag)
            nl = np.sqrt((nx * nx + ny * ny) + nz * nz)
            nx, ny, nz = nx / nl, ny / nl, nz / nl
            s0, s1, s2 = e[0] + nx * rad, e[1] + ny * rad, e[2] + nz * rad
            # sphere_pos_eye * pr_matrix: the vector on the left, so columns 2 and 3
            cz = ((s0 * pr[0, 2] + s1 * pr[1, 2]) + s2 * pr[2, 2]) + one * pr[3, 2]
            cw = ((s0 * pr[0, 3] + s1 * pr[1, 3]) + s2 * pr[2, 3]) + one * pr[3, 3]
            nd = cz / cw
            lin = (nd + one) * F(0.5)
        keep = inside & (lin < one)
        lin = np.maximum(lin, F(0.0))
        zb = zbuf[y0:y1 + 1, x0:x1 + 1]
        win = keep & (lin < zb)
        zb[win] = lin[win]
        depth[y0:y1 + 1, x0:x1 + 1][win] = nd[win]
    return depth


def _shift(img, dx, dy):
    """img sampled at (x + dx, y + dy) with coordinates clamped to the image."""
    h, w = img.shape
    xs = np.clip(np.arange(w) + dx, 0, w - 1)
    ys = np.clip(np.arange(h) + dy, 0, h - 1)
    return img[np.ix_(ys, xs)]


def bilateral(depth):
    depth = np.asarray(depth, F)
    s = np.zeros_like(depth)
    ws = np.zeros_like(depth)
    for dx in range(-4, 4):
        for dy in range(-4, 4):
            smp = _shift(depth, dx, dy)
            r = np.sqrt(F(dx * dx + dy * dy)) * F(0.0001)
            w = np.exp(-r * r).astype(F)
            ok = np.abs(smp - depth) < F(0.015)
            s = np.where(ok, s + smp * w, s)
            ws = np.where(ok, ws + w, ws)
    with np.errstate(invalid="ignore", divide="ignore"):
        return np.where(depth > 0, s / ws, F(0.0)).astype(F)


def curvature_flow(depth, inv_proj_x, inv_proj_y):
    z = np.asarray(depth, F)
    h, w = z.shape
    xp, xn, yp, yn = _shift(z, 1, 0), _shift(z, -1, 0), _shift(z, 0, 1), _shift(z, 0, -1)
    zdx = np.where((xp == 0) | (xn == 0), F(0), F(0.5) * (xp - xn))
    zdy = np.where((yp == 0) | (yn == 0), F(0), F(0.5) * (yp - yn))
    zdx2 = (xp + xn) - F(2.0) * z
    zdy2 = (yp + yn) - F(2.0) * z
    zdxy = (((_shift(z, 1, 1) + _shift(z, -1, -1)) - _shift(z, 1, -1)) - _shift(z, -1, 1)) / F(4.0)
    cx = F(2.0) / (F(w) * -F(inv_proj_x))
    cy = F(2.0) / (F(h) * -F(inv_proj_y))
    d = (cy * cy * zdx * zdx + cx * cx * zdy * zdy) + cx * cx * cy * cy * z * z
    ddx = (cy * cy * F(2.0) * zdx * zdx2 + cx * cx * F(2.0) * zdy * zdxy) + cx * cx * cy * cy * F(2.0) * z * zdx
    ddy = (cy * cy * F(2.0) * zdx * zdxy + cx * cx * F(2.0) * zdy * zdy2) + cx * cx * cy * cy * F(2.0) * z * zdy
    ex = F(0.5) * zdx * ddx - zdx2 * d
    ey = F(0.5) * zdy * ddy - zdy2 * d
    with np.errstate(invalid="ignore", divide="ignore", over="ignore"):
        hm = F(0.5) * ((cy * ex + cx * ey) / np.power(d, F(1.5)))
        out = z + hm * F(0.00055) * (F(1.0) + (np.abs(zdx) + np.abs(zdy)) * F(1000.0))
    return np.where(z > 0, out, F(0.0)).astype(F)


def depth_normals(depth, inv_projection):
    """(height, width, 4) view-space normals (x, y, z, 1); zeros where depth <= 0."""
    z = np.asarray(depth, F)
    h, w = z.shape
    ip = np.asarray(inv_projection, F).reshape(4, 4)
    one, two = F(1.0), F(2.0)
    tx, ty = one / F(w), one / F(h)
    u = ((np.arange(w, dtype=F) + F(0.5)) * tx)[None, :] + np.zeros((h, 1), F)
    v = ((np.arange(h, dtype=F) + F(0.5)) * ty)[:, None] + np.zeros((1, w), F)

    def eye(uu, vv, dd):
        e = _mv(ip, [uu * two - one, vv * two - one, dd, np.ones_like(dd)])
        return [e[0] / e[3], e[1] / e[3], e[2] / e[3]]

    with np.errstate(invalid="ignore", divide="ignore"):
        p = eye(u, v, z)
        a = eye(u + tx, v, _shift(z, 1, 0))
        b = eye(u - tx, v, _shift(z, -1, 0))
        ddx = [a[k] - p[k] for k in range(3)]
        b = [p[k] - b[k] for k in range(3)]
        sw = np.abs(ddx[2]) > np.abs(b[2])
        ddx = [np.where(sw, b[k], ddx[k]) for k in range(3)]
        a = eye(u, v + ty, _shift(z, 0, 1))
        b = eye(u, v - ty, _shift(z, 0, -1))
        ddy = [a[k] - p[k] for k in range(3)]
        b = [p[k] - b[k] for k in range(3)]
        sw = np.abs(ddy[2]) > np.abs(b[2])
        ddy = [np.where(sw, b[k], ddy[k]) for k in range(3)]
        cx = ddx[1] * ddy[2] - ddx[2] * ddy[1]
        cy = ddx[2] * ddy[0] - ddx[0] * ddy[2]
        cz = ddx[0] * ddy[1] - ddx[1] * ddy[0]
        ln = np.sqrt((cx * cx + cy * cy) + cz * cz)
        out = np.stack([cx / ln, cy / ln, cz / ln, np.ones_like(cx)], axis=-1)
    return np.where((z > 0)[..., None], out, F(0.0)).astype(F)


def perspective(fov_deg, aspect, near, far):
    """QMatrix4x4::perspective (gluPerspective) in mathematical layout."""
    f = 1.0 / np.tan(np.radians(fov_deg) / 2.0)
    m = np.zeros((4, 4), np.float64)
    m[0, 0] = f / aspect
    m[1, 1] = f
    m[2, 2] = -(far + near) / (far - near)
    m[2, 3] = -2.0 * far * near / (far - near)
    m[3, 2] = -1.0
    return m.astype(F)


def look_at(eye, center, up):
    """QMatrix4x4::lookAt (gluLookAt) in mathematical layout."""
    eye, center, up = (np.asarray(a, np.float64) for a in (eye, center, up))
    f = center - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -f
    m[:3, 3] = -m[:3, :3] @ eye
    return m.astype(F)


def _bilinear(img, u, v):
    """GL_LINEAR read at normalised (u, v) with coordinates clamped to the edge texels;
    img is (h, w) or (h, w, c)."""
    h, w = img.shape[:2]
    px = u * F(w) - F(0.5)
    py = v * F(h) - F(0.5)
    bx, by = np.floor(px), np.floor(py)
    fx, fy = px - bx, py - by
    x0 = np.clip(bx.astype(np.int64), 0, w - 1)
    x1 = np.clip(bx.astype(np.int64) + 1, 0, w - 1)
    y0 = np.clip(by.astype(np.int64), 0, h - 1)
    y1 = np.clip(by.astype(np.int64) + 1, 0, h - 1)
    if img.ndim == 3:
        fx, fy = fx[..., None], fy[..., None]

    def lerp(a, b, t):
        return a * (F(1) - t) + b * t

    return lerp(lerp(img[y0, x0], img[y0, x1], fx), lerp(img[y1, x0], img[y1, x1], fx), fy)


def _cube(cube, r):
    """GL cube-map read: major-axis face (+x, -x, +y, -y, +z, -z), the face's (s, t) by the
    OpenGL face table, bilinear within the face.  cube: (6, S, S, 4); r: (..., 3)."""
    rx, ry, rz = r[..., 0], r[..., 1], r[..., 2]
    ax, ay, az = np.abs(rx), np.abs(ry), np.abs(rz)
    xm = (ax >= ay) & (ax >= az)
    ym = ~xm & (ay >= az)
    face = np.where(xm, np.where(rx >= 0, 0, 1), np.where(ym, np.where(ry >= 0, 2, 3), np.where(rz >= 0, 4, 5)))
    ma = np.where(xm, ax, np.where(ym, ay, az))
    sc = np.where(xm, np.where(rx >= 0, -rz, rz), np.where(ym, rx, np.where(rz >= 0, rx, -rx)))
    tc = np.where(xm, -ry, np.where(ym, np.where(ry >= 0, rz, -rz), -ry))
    s = (sc / ma + F(1)) * F(0.5)
    t = (tc / ma + F(1)) * F(0.5)
    out = np.zeros(r.shape[:-1] + (4,), F)
    for f in range(6):
        m = face == f
        if m.any():
            out[m] = _bilinear(cube[f], s[m], t[m])
    return out


def shade(depth, normals, background, cube, modelview, inv_projection):
    """final_stage.frag over a (h, w) blurred depth and (h, w, 4) normals; background
    (h, w, 4) or None (black), cube (6, S, S, 4) or None (black).  Returns (h, w, 4)."""
    z = np.asarray(depth, F)
    h, w = z.shape
    n = np.asarray(normals, F)
    bkg = np.zeros((h, w, 4), F) if background is None else np.asarray(background, F)
    mv = np.asarray(modelview, F).reshape(4, 4)
    ip = np.asarray(inv_projection, F).reshape(4, 4)
    one = F(1)
    u = ((np.arange(w, dtype=F) + F(0.5)) * (one / F(w)))[None, :] + np.zeros((h, 1), F)
    v = ((np.arange(h, dtype=F) + F(0.5)) * (one / F(h)))[:, None] + np.zeros((1, w), F)

    def norm3(x, y, zz):
        ln = np.sqrt((x * x + y * y) + zz * zz)
        return x / ln, y / ln, zz / ln

    with np.errstate(invalid="ignore", divide="ignore", over="ignore"):
        ix, iy, iz = norm3(*(np.full((h, w), mv[k, 0] * F(0.7) + mv[k, 1] * F(1.0), F) for k in range(3)))
        e = _mv(ip, [u * F(2) - one, v * F(2) - one, z, np.ones_like(z)])
        p = [e[0] / e[3], e[1] / e[3], e[2] / e[3]]
        vx, vy, vz = norm3(-p[0], -p[1], -p[2])
        hx, hy, hz = norm3(ix + vx, iy + vy, iz + vz)
        nx, ny, nz = n[..., 0], n[..., 1], n[..., 2]
        spec = np.power(np.maximum(F(0), (hx * nx + hy * ny) + hz * nz), F(50))
        ndv = (nx * vx + ny * vy) + nz * vz
        fres = F(0.1) + (one - F(0.1)) * np.power(one - ndv, F(5))
        ndi = (nx * -vx + ny * -vy) + nz * -vz
        rx, ry, rz = norm3(-vx - (F(2) * ndi) * nx, -vy - (F(2) * ndi) * ny, -vz - (F(2) * ndi) * nz)
        refl = np.zeros((h, w, 4), F) if cube is None else _cube(np.asarray(cube, F), np.stack([rx, ry, rz], -1))
        au = u + nx * F(0.010)
        av = v + ny * F(0.010)
        off = _bilinear(z, au, av) <= 0
        au = np.where(off, u, au)
        av = np.where(off, v, av)
        refr = _bilinear(bkg, au, av)
        t = one - fres
        att = np.array([0.2, 0.2, 0.5], F)
        col = [(att[c] * (one - F(0.7)) + (t * refr[..., c]) * F(0.7) + spec * F(0.5)) + refl[..., c] * fres
               for c in range(3)]
        out = np.stack(col + [np.ones_like(z)], -1).astype(F)
    back = np.concatenate([bkg[..., :3], np.ones((h, w, 1), F)], -1)
    return np.where((z > 0)[..., None], out, back).astype(F)


def particles_image(pos4, modelview, projection, point_radius, point_scale, width, height, lights):
    """ParticlesRenderer (shaders/particles.vert/.frag): sphere sprites depth-tested at their
    centre's window depth, lit by directional lights [(direction, diffuse rgba)].  Returns
    (height, width, 4), (0, 0, 0, 1) where no sprite is, colours clamped to [0, 1]."""
    mv = np.asarray(modelview, F).reshape(4, 4)
    pr = np.asarray(projection, F).reshape(4, 4)
    rad, scale = F(point_radius), F(point_scale)
    best = np.full((height, width), np.inf, F)
    owner = np.full((height, width), -1, np.int64)
    sprites = {}
    one = F(1.0)
    for i, p in enumerate(np.asarray(pos4, F).reshape(-1, 4)):
        e = _mv(mv, [p[0], p[1], p[2], one])
        c = _mv(pr, e)
        if not (c[3] > 0) or abs(c[0]) > c[3] or abs(c[1]) > c[3] or abs(c[2]) > c[3]:
            continue
        dist = np.sqrt((e[0] * e[0] + e[1] * e[1]) + e[2] * e[2])
        size = max(rad * (scale / dist), one)
        wx = ((c[0] / c[3] + one) * F(0.5)) * F(width)
        wy = ((c[1] / c[3] + one) * F(0.5)) * F(height)
        z = max((c[2] / c[3] + one) * F(0.5), F(0))
        if not z < one:
            continue
        sprites[i] = (wx, wy, size)
        x0, x1 = max(0, int(np.floor(wx - F(0.5) * size))), min(width - 1, int(np.ceil(wx + F(0.5) * size)))
        y0, y1 = max(0, int(np.floor(wy - F(0.5) * size))), min(height - 1, int(np.ceil(wy + F(0.5) * size)))
        if x0 > x1 or y0 > y1:
            continue
        px = np.arange(x0, x1 + 1, dtype=F)[None, :]
        py = np.arange(y0, y1 + 1, dtype=F)[:, None]
        nx = (F(2.0) * ((px + F(0.5)) - wx)) / size + np.zeros_like(py)
        ny = (F(2.0) * ((py + F(0.5)) - wy)) / size + np.zeros_like(px)
        inside = (nx * nx + ny * ny) <= one
        b = best[y0:y1 + 1, x0:x1 + 1]
        win = inside & (z < b)
        b[win] = z
        owner[y0:y1 + 1, x0:x1 + 1][win] = i
    out = np.zeros((height, width, 4), F)
    out[..., 3] = 1
    vc = np.array([89.0 / 256.0, 152.0 / 256.0, 255.0 / 256.0, 1.0], F)
    for y, x in zip(*np.nonzero(owner >= 0)):
        wx, wy, size = sprites[int(owner[y, x])]
        nx = (F(2.0) * ((F(x) + F(0.5)) - wx)) / size
        ny = (F(2.0) * ((F(y) + F(0.5)) - wy)) / size
        nz = np.sqrt(one - (nx * nx + ny * ny))
        acc = np.array([0, 0, 0, 1], F)
        for d, col in lights:
            d = np.asarray(d, F)
            ln = np.sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2])
            dx, dy, dz = -(d[0] / ln), -(d[1] / ln), -(d[2] / ln)
            dd = max(F(0), (nx * dx + ny * dy) + nz * dz)
            acc = (acc + (np.asarray(col, F) * vc) * dd).astype(F)
        out[y, x] = np.clip(acc, 0, 1)
    return out
