/*
 * sph_render.cu -- the screen-space fluid surface of the reference's renderer as CUDA
 * kernels writing device images (no graphics API): particle depth sprites, the two
 * smoothing filters, and view-space normals.
 *
 *   k_splat_*        shaders/sspace_fluid_rendering/depth_stage.vert and .frag: each particle
 *                    is a point sprite of gl_PointSize = point_radius * point_scale / |p_eye|;
 *                    a fragment inside the sprite's disc lies on the sphere of radius
 *                    point_radius around the particle; its normalised depth is written where
 *                    it is the nearest (GL_LESS on (z_ndc + 1) / 2, the lowest particle index
 *                    winning a tie as the first primitive does), 0 elsewhere.  The fragment
 *                    shader's depth uses `sphere_pos_eye * pr_matrix` (vector on the left:
 *                    the transpose of the projection), kept as written.  No background
 *                    texture: fragments beyond the far plane are dropped.
 *   k_bilateral      kernels/bilateral.cl (window -4..3 in x and y, depth gate 0.015).
 *   k_curvature_flow kernels/curvatureflow.cl (one explicit step of the mean-curvature flow).
 *   k_depth_normals  shaders/sspace_fluid_rendering/normals_stage.frag: eye-space positions
 *                    from the inverse projection, one-sided differences with the smaller
 *                    depth jump, normal = normalize(ddx x ddy).
 *   k_shade          shaders/sspace_fluid_rendering/final_stage.frag: the fluid's colour over
 *                    a background image with a cube map for reflections, into an RGBA image.
 *   k_particle_*     shaders/particles.vert and .frag (the "particles" render method): the
 *                    same sprites depth-tested at their centres and lit by directional lights.
 * Images are row-major, row 0 at the bottom (window coordinates), single-channel float
 * (depth) or float4 (normals); reads outside the image clamp to the edge.
 */
#include <cmath>
#include <cstring>
#include <utility>

#include "sph_ctx.cuh"

namespace sph {
namespace {

struct View {
    float mv[16], pr[16];   /* column-major 4x4, as GL uniforms */
    float radius, scale;
    int w, h;
};

__device__ __forceinline__ void mat_vec(const float* m, const float v[4], float o[4]) {
    for (int r = 0; r < 4; ++r) o[r] = m[r] * v[0] + m[4 + r] * v[1] + m[8 + r] * v[2] + m[12 + r] * v[3];
}

/* A particle's sprite: eye position, window centre and size; false when GL clips it. */
__device__ __forceinline__ bool sprite(const View& v, float4 p, float e[4], float& wx, float& wy, float& size) {
    const float x[4] = {p.x, p.y, p.z, 1.0f};
    mat_vec(v.mv, x, e);
    float c[4];
    mat_vec(v.pr, e, c);
    if (!(c[3] > 0.f) || fabsf(c[0]) > c[3] || fabsf(c[1]) > c[3] || fabsf(c[2]) > c[3]) return false;
    const float dist = sqrtf(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
    size = fmaxf(v.radius * (v.scale / dist), 1.0f);   /* GL's smallest point size */
    wx = (c[0] / c[3] + 1.0f) * 0.5f * (float)v.w;
    wy = (c[1] / c[3] + 1.0f) * 0.5f * (float)v.h;
    return size > 0.f;
}

/* Depth of the sprite fragment at pixel (px, py): false outside the disc or beyond far. */
__device__ __forceinline__ bool fragment(const View& v, const float e[4], float wx, float wy, float size, int px,
                                         int py, float& nd, float& lin) {
    /* gl_PointCoord has its origin at the sprite's upper left; the shader maps it to
       (2s - 1, 1 - 2t) and then negates y, so y grows downwards on the screen */
    float nx = 2.0f * ((float)px + 0.5f - wx) / size;
    float ny = -2.0f * ((float)py + 0.5f - wy) / size;
    const float mag = nx * nx + ny * ny;
    if (mag > 1.0f) return false;
    float nz = sqrtf(1.0f - mag);
    const float nl = sqrtf(nx * nx + ny * ny + nz * nz);
    nx /= nl; ny /= nl; nz /= nl;
    const float s[4] = {e[0] + nx * v.radius, e[1] + ny * v.radius, e[2] + nz * v.radius, 1.0f};
    /* sphere_pos_eye * pr_matrix: component j = dot(s, column j) */
    const float cz = s[0] * v.pr[8] + s[1] * v.pr[9] + s[2] * v.pr[10] + s[3] * v.pr[11];
    const float cw = s[0] * v.pr[12] + s[1] * v.pr[13] + s[2] * v.pr[14] + s[3] * v.pr[15];
    nd = cz / cw;
    lin = (nd + 1.0f) * 0.5f;
    if (!(lin < 1.0f)) return false;   /* background (depth 1) and GL_LESS against the cleared buffer */
    if (lin < 0.0f) lin = 0.0f;
    return true;
}

/* Depth test of every sprite fragment: one 64-bit key per pixel, (normalised depth bits << 32)
 * | particle index, so atomicMin keeps the nearest fragment and, among equal depths, the
 * lowest index (the first primitive GL_LESS lets through).  Depths are >= 0, so their bit
 * patterns order like the values.  A plain read first skips fragments that already lose:
 * keys only decrease, so a stale read can only cost an unneeded atomic. */
/* A lower bound of the normalised depth of every fragment of a sprite, or 0 when none is
 * known.  With the projection's column-2 and column-3 x, y entries zero (any symmetric
 * perspective) the fragment depth (s2 pr10 + pr11) / (s2 pr14 + pr15) depends only on the
 * sphere point's eye z, s2 in [e_z, e_z + r]; away from the pole s2 = -pr15 / pr14 it is
 * monotone there, so its smaller end value bounds every fragment.  A margin of 1e-5 covers the
 * fragments' own rounding. */
__device__ __forceinline__ float depth_floor(const View& v, const float e[4]) {
    const float* m = v.pr;
    if (m[8] != 0.f || m[9] != 0.f || m[12] != 0.f || m[13] != 0.f) return 0.f;
    const float lo = e[2] - 1e-3f * v.radius, hi = e[2] + v.radius * 1.001f;
    if (m[14] != 0.f) {
        const float pole = -m[15] / m[14];
        if (pole >= lo && pole <= hi) return 0.f;
    }
    auto lin = [&](float s2) { return ((s2 * m[10] + m[11]) / (s2 * m[14] + m[15]) + 1.0f) * 0.5f; };
    const float b = fminf(lin(lo), lin(hi)) - 1e-5f;
    return b > 0.f ? b : 0.f;
}

/* Front-to-back processing order: the top 16 bits of the eye distance (sign, exponent and 7
 * mantissa bits: monotone for positive floats), particles behind the eye last.  Any order
 * gives the same image; near sprites first let later ones skip their pixels early. */
__global__ void k_depth_order(View v, int n, const float4* __restrict__ pos, uint32_t* __restrict__ keys,
                              int32_t* __restrict__ vals) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = pos[i];
    const float d = -(v.mv[2] * p.x + v.mv[6] * p.y + v.mv[10] * p.z + v.mv[14]);
    keys[i] = d > 0.f ? __float_as_uint(d) >> 16 : 0xffffu;
    vals[i] = i;
}

__global__ void k_splat_keys(View v, int n, const float4* __restrict__ pos, const int32_t* __restrict__ order,
                             unsigned long long* __restrict__ key) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int i = order[t];
    float e[4], wx, wy, size;
    if (!sprite(v, pos[i], e, wx, wy, size)) return;
    /* a pixel already nearer than this sprite can get is skipped before any fragment arithmetic:
       keys only decrease, so a stale read (even an L1 copy older than other CTAs' atomics)
       only costs the full test */
    const unsigned floor_bits = __float_as_uint(depth_floor(v, e));
    const int x0 = max(0, (int)floorf(wx - 0.5f * size)), x1 = min(v.w - 1, (int)ceilf(wx + 0.5f * size));
    const int y0 = max(0, (int)floorf(wy - 0.5f * size)), y1 = min(v.h - 1, (int)ceilf(wy + 0.5f * size));
    constexpr int kAhead = 8;   /* key loads in flight per thread */
    for (int py = y0; py <= y1; ++py) {
        unsigned long long* row = key + (size_t)py * v.w;
        for (int px0 = x0; px0 <= x1; px0 += kAhead) {
            unsigned long long cur[kAhead];
#pragma unroll
            for (int u = 0; u < kAhead; ++u)
                cur[u] = px0 + u <= x1 ? __ldca(row + px0 + u) : 0ull;   /* L1 copy: stale is still safe */
#pragma unroll
            for (int u = 0; u < kAhead; ++u) {
                const int px = px0 + u;
                if (px > x1 || (unsigned)(cur[u] >> 32) < floor_bits) continue;
                float nd, lin;
                if (!fragment(v, e, wx, wy, size, px, py, nd, lin)) continue;
                const unsigned long long k = ((unsigned long long)__float_as_uint(lin) << 32) | (unsigned)i;
                if (k < cur[u]) atomicMin(row + px, k);
            }
        }
    }
}

/* Per pixel: the winning particle's fragment depth, recomputed with the same arithmetic. */
__global__ void k_splat_resolve(View v, const float4* __restrict__ pos, const unsigned long long* __restrict__ key,
                                float* __restrict__ depth) {
    const int px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y * blockDim.y + threadIdx.y;
    if (px >= v.w || py >= v.h) return;
    const size_t k = (size_t)py * v.w + px;
    const unsigned long long kk = key[k];
    float out = 0.0f;
    if (kk != ~0ull) {
        float e[4], wx, wy, size, nd, lin;
        if (sprite(v, pos[(unsigned)kk], e, wx, wy, size) && fragment(v, e, wx, wy, size, px, py, nd, lin)) out = nd;
    }
    depth[k] = out;
}

/* shaders/particles.vert and particles.frag (ParticlesRenderer, fluid/render/
 * particlesrenderer.cpp:40-88): the same sphere sprites, but the fragment shader writes no
 * depth, so every fragment of a sprite is depth-tested at its centre's window depth
 * (z_ndc + 1) / 2; the lowest index wins a tie as with the depth stage. */
__device__ __forceinline__ bool particle_depth(const View& v, const float e[4], float& z) {
    float c[4];
    mat_vec(v.pr, e, c);
    z = (c[2] / c[3] + 1.0f) * 0.5f;
    if (z < 0.0f) z = 0.0f;
    return z < 1.0f;
}

__global__ void k_particle_keys(View v, int n, const float4* __restrict__ pos, const int32_t* __restrict__ order,
                                unsigned long long* __restrict__ key) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int i = order[t];
    float e[4], wx, wy, size, z;
    if (!sprite(v, pos[i], e, wx, wy, size) || !particle_depth(v, e, z)) return;
    const unsigned zb = __float_as_uint(z);
    const unsigned long long k = ((unsigned long long)zb << 32) | (unsigned)i;
    const int x0 = max(0, (int)floorf(wx - 0.5f * size)), x1 = min(v.w - 1, (int)ceilf(wx + 0.5f * size));
    const int y0 = max(0, (int)floorf(wy - 0.5f * size)), y1 = min(v.h - 1, (int)ceilf(wy + 0.5f * size));
    for (int py = y0; py <= y1; ++py) {
        unsigned long long* row = key + (size_t)py * v.w;
        for (int px = x0; px <= x1; ++px) {
            const unsigned long long cur = __ldca(row + px);
            if (k >= cur) continue;   /* a nearer (or equal, lower-index) fragment is there */
            const float nx = 2.0f * ((float)px + 0.5f - wx) / size;
            const float ny = 2.0f * ((float)py + 0.5f - wy) / size;
            if (nx * nx + ny * ny > 1.0f) continue;
            atomicMin(row + px, k);
        }
    }
}

struct Lights {
    int count;
    float dir[8][3];
    float diffuse[8][4];
};

/* Per pixel: the winning sprite's normal from the point coordinate, n = (2s - 1, 1 - 2t,
 * sqrt(1 - |n.xy|^2)), lit by each directional light: diffuse * vertex colour (89, 152, 255)
 * / 256 * max(0, n . -normalize(direction)), summed onto (0, 0, 0, 1) and clamped to [0, 1]
 * as a fixed-point framebuffer stores it; (0, 0, 0, 1) where no sprite is. */
__global__ void k_particle_shade(View v, const float4* __restrict__ pos, const unsigned long long* __restrict__ key,
                                 Lights L, float4* __restrict__ out) {
    const int px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y * blockDim.y + threadIdx.y;
    if (px >= v.w || py >= v.h) return;
    const size_t k = (size_t)py * v.w + px;
    const unsigned long long kk = key[k];
    float4 col = make_float4(0.f, 0.f, 0.f, 1.f);
    float e[4], wx, wy, size;
    if (kk != ~0ull && sprite(v, pos[(unsigned)kk], e, wx, wy, size)) {
        const float nx = 2.0f * ((float)px + 0.5f - wx) / size;
        const float ny = 2.0f * ((float)py + 0.5f - wy) / size;
        const float nz = sqrtf(1.0f - (nx * nx + ny * ny));
        const float vc[4] = {89.0f / 256.0f, 152.0f / 256.0f, 255.0f / 256.0f, 1.0f};
        float acc[4] = {0.f, 0.f, 0.f, 1.f};
        for (int l = 0; l < L.count; ++l) {
            float dx = L.dir[l][0], dy = L.dir[l][1], dz = L.dir[l][2];
            const float len = sqrtf((dx * dx + dy * dy) + dz * dz);
            dx = -(dx / len); dy = -(dy / len); dz = -(dz / len);
            const float d = fmaxf(0.0f, (nx * dx + ny * dy) + nz * dz);
            for (int c = 0; c < 4; ++c) acc[c] += (L.diffuse[l][c] * vc[c]) * d;
        }
        col = make_float4(fminf(fmaxf(acc[0], 0.f), 1.f), fminf(fmaxf(acc[1], 0.f), 1.f),
                          fminf(fmaxf(acc[2], 0.f), 1.f), fminf(fmaxf(acc[3], 0.f), 1.f));
    }
    out[k] = col;
}

__global__ void k_splat_clear(size_t npix, unsigned long long* __restrict__ key) {
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < npix) key[k] = ~0ull;
}

__device__ __forceinline__ float texel(const float* img, int w, int h, int x, int y) {
    x = x < 0 ? 0 : (x >= w ? w - 1 : x);
    y = y < 0 ? 0 : (y >= h ? h - 1 : y);
    return img[(size_t)y * w + x];
}

/* kernels/bilateral.cl */
__global__ void k_bilateral(const float* __restrict__ in, float* __restrict__ out, int w, int h) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    const float depth = texel(in, w, h, x, y);
    float o = 0.0f;
    if (depth > 0.0f) {
        float sum = 0.0f, wsum = 0.0f;
        for (int dx = -4; dx < 4; ++dx)
            for (int dy = -4; dy < 4; ++dy) {
                const float s = texel(in, w, h, x + dx, y + dy);
                if (fabsf(s - depth) < 0.015f) {
                    const float fx = (float)dx, fy = (float)dy;
                    const float r = sqrtf(fx * fx + fy * fy) * 0.0001f;
                    const float wt = expf(-r * r);
                    sum += s * wt;
                    wsum += wt;
                }
            }
        o = sum / wsum;
    }
    out[(size_t)y * w + x] = o;
}

/* kernels/curvatureflow.cl */
__global__ void k_curvature_flow(const float* __restrict__ in, float* __restrict__ out, int w, int h, float ipx,
                                 float ipy) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    const float depth = texel(in, w, h, x, y);
    float o = 0.0f;
    if (depth > 0.0f) {
        const float dt = 0.00055f, dzt = 1000.0f;
        const float zc = depth;
        const float zdxp = texel(in, w, h, x + 1, y), zdxn = texel(in, w, h, x - 1, y);
        float zdx = 0.5f * (zdxp - zdxn);
        zdx = (zdxp == 0.0f || zdxn == 0.0f) ? 0.0f : zdx;
        const float zdyp = texel(in, w, h, x, y + 1), zdyn = texel(in, w, h, x, y - 1);
        float zdy = 0.5f * (zdyp - zdyn);
        zdy = (zdyp == 0.0f || zdyn == 0.0f) ? 0.0f : zdy;
        const float zdx2 = zdxp + zdxn - 2.0f * zc;
        const float zdy2 = zdyp + zdyn - 2.0f * zc;
        const float zdxpyp = texel(in, w, h, x + 1, y + 1), zdxnyn = texel(in, w, h, x - 1, y - 1);
        const float zdxpyn = texel(in, w, h, x + 1, y - 1), zdxnyp = texel(in, w, h, x - 1, y + 1);
        const float zdxy = (zdxpyp + zdxnyn - zdxpyn - zdxnyp) / 4.0f;
        const float cx = 2.0f / ((float)w * -ipx);
        const float cy = 2.0f / ((float)h * -ipy);
        const float d = cy * cy * zdx * zdx + cx * cx * zdy * zdy + cx * cx * cy * cy * zc * zc;
        const float ddx = cy * cy * 2.0f * zdx * zdx2 + cx * cx * 2.0f * zdy * zdxy + cx * cx * cy * cy * 2.0f * zc * zdx;
        const float ddy = cy * cy * 2.0f * zdx * zdxy + cx * cx * 2.0f * zdy * zdy2 + cx * cx * cy * cy * 2.0f * zc * zdy;
        const float ex = 0.5f * zdx * ddx - zdx2 * d;
        const float ey = 0.5f * zdy * ddy - zdy2 * d;
        const float hm = 0.5f * ((cy * ex + cx * ey) / powf(d, 1.5f));
        o = depth + hm * dt * (1.0f + (fabsf(zdx) + fabsf(zdy)) * dzt);
    }
    out[(size_t)y * w + x] = o;
}

struct Inv {
    float m[16];
};

__device__ __forceinline__ void uv_to_eye(const Inv& ip, float u, float v, float depth, float o[3]) {
    const float c[4] = {u * 2.0f - 1.0f, v * 2.0f - 1.0f, depth, 1.0f};
    float e[4];
    mat_vec(ip.m, c, e);
    o[0] = e[0] / e[3];
    o[1] = e[1] / e[3];
    o[2] = e[2] / e[3];
}

/* shaders/sspace_fluid_rendering/normals_stage.frag */
__global__ void k_depth_normals(const float* __restrict__ depth, float4* __restrict__ nrm, int w, int h, Inv ip) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    const float d = texel(depth, w, h, x, y);
    if (d <= 0.0f) {
        nrm[(size_t)y * w + x] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const float tx = 1.0f / (float)w, ty = 1.0f / (float)h;
    const float u = ((float)x + 0.5f) * tx, v = ((float)y + 0.5f) * ty;
    float p[3], a[3], b[3], ddx[3], ddy[3];
    uv_to_eye(ip, u, v, d, p);
    uv_to_eye(ip, u + tx, v, texel(depth, w, h, x + 1, y), a);
    uv_to_eye(ip, u - tx, v, texel(depth, w, h, x - 1, y), b);
    for (int k = 0; k < 3; ++k) {
        ddx[k] = a[k] - p[k];
        b[k] = -b[k] + p[k];
    }
    if (fabsf(ddx[2]) > fabsf(b[2]))
        for (int k = 0; k < 3; ++k) ddx[k] = b[k];
    uv_to_eye(ip, u, v + ty, texel(depth, w, h, x, y + 1), a);
    uv_to_eye(ip, u, v - ty, texel(depth, w, h, x, y - 1), b);
    for (int k = 0; k < 3; ++k) {
        ddy[k] = a[k] - p[k];
        b[k] = -b[k] + p[k];
    }
    if (fabsf(ddy[2]) > fabsf(b[2]))
        for (int k = 0; k < 3; ++k) ddy[k] = b[k];
    float cx = ddx[1] * ddy[2] - ddx[2] * ddy[1];
    float cy = ddx[2] * ddy[0] - ddx[0] * ddy[2];
    float cz = ddx[0] * ddy[1] - ddx[1] * ddy[0];
    const float l = sqrtf(cx * cx + cy * cy + cz * cz);
    nrm[(size_t)y * w + x] = make_float4(cx / l, cy / l, cz / l, 1.0f);
}

/* Bilinear read of a single-channel or float4 image at normalised coordinates (u, v) with
 * texel centres at (i + 0.5) / w, coordinates clamped to the edge texels (GL_LINEAR). */
__device__ __forceinline__ void bilinear_at(float u, float v, int w, int h, int& x0, int& y0, int& x1, int& y1,
                                            float& fx, float& fy) {
    const float px = u * (float)w - 0.5f, py = v * (float)h - 0.5f;
    const float bx = floorf(px), by = floorf(py);
    fx = px - bx;
    fy = py - by;
    x0 = (int)bx; y0 = (int)by;
    x1 = x0 + 1; y1 = y0 + 1;
    x0 = x0 < 0 ? 0 : (x0 >= w ? w - 1 : x0); x1 = x1 < 0 ? 0 : (x1 >= w ? w - 1 : x1);
    y0 = y0 < 0 ? 0 : (y0 >= h ? h - 1 : y0); y1 = y1 < 0 ? 0 : (y1 >= h ? h - 1 : y1);
}

__device__ __forceinline__ float lerp1(float a, float b, float t) { return a * (1.0f - t) + b * t; }

__device__ float sample1(const float* img, int w, int h, float u, float v) {
    int x0, y0, x1, y1;
    float fx, fy;
    bilinear_at(u, v, w, h, x0, y0, x1, y1, fx, fy);
    const float a = lerp1(img[(size_t)y0 * w + x0], img[(size_t)y0 * w + x1], fx);
    const float b = lerp1(img[(size_t)y1 * w + x0], img[(size_t)y1 * w + x1], fx);
    return lerp1(a, b, fy);
}

__device__ float4 sample4(const float4* img, int w, int h, float u, float v) {
    int x0, y0, x1, y1;
    float fx, fy;
    bilinear_at(u, v, w, h, x0, y0, x1, y1, fx, fy);
    const float4 p = img[(size_t)y0 * w + x0], q = img[(size_t)y0 * w + x1];
    const float4 r = img[(size_t)y1 * w + x0], t = img[(size_t)y1 * w + x1];
    return make_float4(lerp1(lerp1(p.x, q.x, fx), lerp1(r.x, t.x, fx), fy),
                       lerp1(lerp1(p.y, q.y, fx), lerp1(r.y, t.y, fx), fy),
                       lerp1(lerp1(p.z, q.z, fx), lerp1(r.z, t.z, fx), fy),
                       lerp1(lerp1(p.w, q.w, fx), lerp1(r.w, t.w, fx), fy));
}

/* GL cube-map lookup: the face of the major axis (+x, -x, +y, -y, +z, -z) and its (s, t) by
 * the OpenGL face table, then a bilinear read of that face (S x S float4 texels). */
__device__ float4 sample_cube(const float4* cube, int S, float rx, float ry, float rz) {
    const float ax = fabsf(rx), ay = fabsf(ry), az = fabsf(rz);
    int face;
    float sc, tc, ma;
    if (ax >= ay && ax >= az) {
        face = rx >= 0.f ? 0 : 1; ma = ax; sc = rx >= 0.f ? -rz : rz; tc = -ry;
    } else if (ay >= az) {
        face = ry >= 0.f ? 2 : 3; ma = ay; sc = rx; tc = ry >= 0.f ? rz : -rz;
    } else {
        face = rz >= 0.f ? 4 : 5; ma = az; sc = rz >= 0.f ? rx : -rx; tc = -ry;
    }
    const float s = (sc / ma + 1.0f) * 0.5f, t = (tc / ma + 1.0f) * 0.5f;
    return sample4(cube + (size_t)face * S * S, S, S, s, t);
}

struct Shade {
    float mv[16], ip[16];
};

__device__ __forceinline__ void norm3(float& x, float& y, float& z) {
    const float l = sqrtf((x * x + y * y) + z * z);
    x /= l; y /= l; z /= l;
}

/* shaders/sspace_fluid_rendering/final_stage.frag: Blinn-Phong specular, Fresnel (Schlick,
 * r0 = 0.1), cube-map reflection, background refraction offset by the normal, fixed
 * attenuation colour; background where depth <= 0.  Light direction mv * (0.7, 1, 0, 0). */
__global__ void k_shade(const float* __restrict__ depth, const float4* __restrict__ nrm,
                        const float4* __restrict__ bkg, const float4* __restrict__ cube, int S, int w, int h,
                        Shade sh, float4* __restrict__ out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    const size_t k = (size_t)y * w + x;
    const float u = ((float)x + 0.5f) * (1.0f / (float)w), v = ((float)y + 0.5f) * (1.0f / (float)h);
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    const float d = depth[k];
    const float4 nn = nrm[k];
    const float4 bg = bkg ? bkg[k] : zero;
    if (d <= 0.0f) {
        out[k] = make_float4(bg.x, bg.y, bg.z, 1.0f);
        return;
    }
    const float* m = sh.mv;
    float ix = m[0] * 0.7f + m[4] * 1.0f, iy = m[1] * 0.7f + m[5] * 1.0f, iz = m[2] * 0.7f + m[6] * 1.0f;
    float p[3];
    Inv ip;
    for (int q = 0; q < 16; ++q) ip.m[q] = sh.ip[q];
    uv_to_eye(ip, u, v, d, p);
    norm3(ix, iy, iz);
    float vx = -p[0], vy = -p[1], vz = -p[2];
    norm3(vx, vy, vz);
    float hx = ix + vx, hy = iy + vy, hz = iz + vz;
    norm3(hx, hy, hz);
    const float ndh = (hx * nn.x + hy * nn.y) + hz * nn.z;
    const float spec = powf(fmaxf(0.0f, ndh), 50.0f);
    const float ndv = (nn.x * vx + nn.y * vy) + nn.z * vz;
    const float fres = 0.1f + (1.0f - 0.1f) * powf(1.0f - ndv, 5.0f);
    /* reflect(-viewer, normal) = -v - 2 dot(n, -v) n */
    const float ndi = (nn.x * -vx + nn.y * -vy) + nn.z * -vz;
    float rx = -vx - (2.0f * ndi) * nn.x, ry = -vy - (2.0f * ndi) * nn.y, rz = -vz - (2.0f * ndi) * nn.z;
    norm3(rx, ry, rz);
    const float4 refl = cube ? sample_cube(cube, S, rx, ry, rz) : zero;
    float au = u + nn.x * 0.010f, av = v + nn.y * 0.010f;
    if (sample1(depth, w, h, au, av) <= 0.0f) {
        au = u;
        av = v;
    }
    const float4 refr = bkg ? sample4(bkg, w, h, au, av) : zero;
    const float t = 1.0f - fres;
    const float fx = 0.2f * (1.0f - 0.7f) + (t * refr.x) * 0.7f;
    const float fy = 0.2f * (1.0f - 0.7f) + (t * refr.y) * 0.7f;
    const float fz = 0.5f * (1.0f - 0.7f) + (t * refr.z) * 0.7f;
    out[k] = make_float4((fx + spec * 0.5f) + refl.x * fres, (fy + spec * 0.5f) + refl.y * fres,
                         (fz + spec * 0.5f) + refl.z * fres, 1.0f);
}

inline dim3 grid2(int w, int h, dim3 b) { return dim3((w + b.x - 1) / b.x, (h + b.y - 1) / b.y); }

/* sizes the 16 x 16 pixel grids can cover */
inline bool image_ok(int w, int h) {
    return w > 0 && h > 0 && w <= 65536 && h <= 65536 && (long long)w * h <= (1LL << 28);
}

}  // namespace
}  // namespace sph

extern "C" {

/* Checks the view, allocates the depth-test keys and the particle-order buffers, clears the
 * keys and sorts the particles front to back; the caller splats and resolves. */
static int splat_prepare(sph_ctx* x, const sph_view* view, sph::View& v, unsigned long long*& key,
                         const int32_t*& sorted) {
    if (!sph::image_ok(view->width, view->height))
        return sph_ctx_fail(x, SPH_E_INVALID, "render: width and height must be 1..65536 (at most 2^28 pixels)");
    if (!(view->point_radius > 0.f) || !(view->point_scale > 0.f))
        return sph_ctx_fail(x, SPH_E_INVALID, "render: point_radius and point_scale must be > 0");
    if (!x->has_state || x->N <= 0) return sph_ctx_fail(x, SPH_E_STATE, "render: no particles added");
    const size_t npix = (size_t)view->width * view->height;
    /* keys, order, their sort ping-pong copies and the sort's workspace, all the context's own */
    const size_t nsort = 16 * (size_t)x->N + sph::sort_workspace_bytes(x->N, 16);
    if (x->render_sort_bytes < nsort) {
        cudaStreamSynchronize(x->stream);
        cudaFree(x->render_sort);
        x->render_sort = nullptr;
        x->render_sort_bytes = 0;
        if (cudaMalloc(&x->render_sort, nsort) != cudaSuccess) {
            cudaGetLastError();
            return sph_ctx_fail(x, SPH_E_NOMEM, "render: particle order buffers");
        }
        x->render_sort_bytes = nsort;
    }
    if (x->render_pixels < npix) {
        cudaStreamSynchronize(x->stream);
        cudaFree(x->render_buf);
        x->render_buf = nullptr;
        x->render_pixels = 0;
        if (cudaMalloc(&x->render_buf, 8 * npix) != cudaSuccess) {
            cudaGetLastError();
            return sph_ctx_fail(x, SPH_E_NOMEM, "render: depth-test buffers");
        }
        x->render_pixels = npix;
    }
    std::memcpy(v.mv, view->modelview, sizeof v.mv);
    std::memcpy(v.pr, view->projection, sizeof v.pr);
    v.radius = view->point_radius;
    v.scale = view->point_scale;
    v.w = view->width;
    v.h = view->height;
    key = reinterpret_cast<unsigned long long*>(x->render_buf);
    const cudaStream_t s = x->stream;
    const int bs = 256, n = x->N;
    sph::k_splat_clear<<<(unsigned)((npix + bs - 1) / bs), bs, 0, s>>>(npix, key);
    uint32_t* okeys = reinterpret_cast<uint32_t*>(x->render_sort);
    int32_t* order = reinterpret_cast<int32_t*>(okeys + n);
    uint32_t* okeys_alt = reinterpret_cast<uint32_t*>(order + n);
    int32_t* order_alt = reinterpret_cast<int32_t*>(okeys_alt + n);
    void* ws = order_alt + n;
    sph::k_depth_order<<<(n + bs - 1) / bs, bs, 0, s>>>(v, n, x->b.pos, okeys, order);
    uint32_t* ks;
    int32_t* so;
    sph::sort_pairs(s, okeys, order, okeys_alt, order_alt, n, 16, ws, x->b.flags, x->num_sms, &ks, &so);
    sorted = so;
    return SPH_OK;
}

int sph_render_depth(sph_ctx* x, const sph_view* view, float* d_depth) {
    if (!x || !view || !d_depth) return SPH_E_INVALID;
    sph::View v;
    unsigned long long* key;
    const int32_t* sorted;
    const int rc = splat_prepare(x, view, v, key, sorted);
    if (rc != SPH_OK) return rc;
    const cudaStream_t s = x->stream;
    const int bs = 256, n = x->N;
    const dim3 b2(16, 16);
    sph::k_splat_keys<<<(n + bs - 1) / bs, bs, 0, s>>>(v, n, x->b.pos, sorted, key);
    sph::k_splat_resolve<<<sph::grid2(v.w, v.h, b2), b2, 0, s>>>(v, x->b.pos, key, d_depth);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return sph_ctx_fail(x, SPH_E_CUDA, std::string("render launch: ") + cudaGetErrorString(e));
    return SPH_OK;
}

int sph_render_particles(sph_ctx* x, const sph_view* view, const sph_light* lights, int nlights, float* d_rgba) {
    if (!x || !view || !d_rgba || nlights < 0 || nlights > 8 || (nlights > 0 && !lights)) return SPH_E_INVALID;
    sph::Lights L{};
    L.count = nlights;
    for (int l = 0; l < nlights; ++l) {
        for (int k = 0; k < 3; ++k) L.dir[l][k] = lights[l].direction[k];
        for (int k = 0; k < 4; ++k) L.diffuse[l][k] = lights[l].diffuse[k];
    }
    sph::View v;
    unsigned long long* key;
    const int32_t* sorted;
    const int rc = splat_prepare(x, view, v, key, sorted);
    if (rc != SPH_OK) return rc;
    const cudaStream_t s = x->stream;
    const int bs = 256, n = x->N;
    const dim3 b2(16, 16);
    sph::k_particle_keys<<<(n + bs - 1) / bs, bs, 0, s>>>(v, n, x->b.pos, sorted, key);
    sph::k_particle_shade<<<sph::grid2(v.w, v.h, b2), b2, 0, s>>>(v, x->b.pos, key, L,
                                                                   reinterpret_cast<float4*>(d_rgba));
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return sph_ctx_fail(x, SPH_E_CUDA, std::string("render launch: ") + cudaGetErrorString(e));
    return SPH_OK;
}

int sph_filter_bilateral(const float* d_in, float* d_out, int width, int height, void* stream) {
    if (!d_in || !d_out || !sph::image_ok(width, height) || d_in == d_out) return SPH_E_INVALID;
    const dim3 b(16, 16);
    sph::k_bilateral<<<sph::grid2(width, height, b), b, 0, (cudaStream_t)stream>>>(d_in, d_out, width, height);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_E_CUDA;
}

int sph_render_smooth(float* d_depth, float* d_tmp, int width, int height, int iterations, void* stream) {
    if (!d_depth || !d_tmp || !sph::image_ok(width, height) || iterations < 0 || d_depth == d_tmp)
        return SPH_E_INVALID;
    const dim3 b(16, 16);
    const cudaStream_t s = (cudaStream_t)stream;
    for (int it = 0; it < iterations; ++it) {
        sph::k_bilateral<<<sph::grid2(width, height, b), b, 0, s>>>(d_depth, d_tmp, width, height);
        sph::k_bilateral<<<sph::grid2(width, height, b), b, 0, s>>>(d_tmp, d_depth, width, height);
    }
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_E_CUDA;
}

int sph_filter_curvature_flow(const float* d_in, float* d_out, int width, int height, float inv_proj_x,
                              float inv_proj_y, void* stream) {
    if (!d_in || !d_out || !sph::image_ok(width, height) || d_in == d_out) return SPH_E_INVALID;
    const dim3 b(16, 16);
    sph::k_curvature_flow<<<sph::grid2(width, height, b), b, 0, (cudaStream_t)stream>>>(d_in, d_out, width, height,
                                                                                         inv_proj_x, inv_proj_y);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_E_CUDA;
}

int sph_render_normals(const float* d_depth, float* d_normals4, int width, int height, const float inv_projection[16],
                       void* stream) {
    if (!d_depth || !d_normals4 || !inv_projection || !sph::image_ok(width, height)) return SPH_E_INVALID;
    sph::Inv ip;
    std::memcpy(ip.m, inv_projection, sizeof ip.m);
    const dim3 b(16, 16);
    sph::k_depth_normals<<<sph::grid2(width, height, b), b, 0, (cudaStream_t)stream>>>(
        d_depth, reinterpret_cast<float4*>(d_normals4), width, height, ip);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_E_CUDA;
}

/* 4x4 inverse (column-major in and out) by Gauss-Jordan elimination in double. */
static bool invert4(const float* a, float* out) {
    double m[4][8];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            m[r][c] = a[c * 4 + r];
            m[r][c + 4] = r == c ? 1.0 : 0.0;
        }
    for (int c = 0; c < 4; ++c) {
        int p = c;
        for (int r = c + 1; r < 4; ++r)
            if (std::fabs(m[r][c]) > std::fabs(m[p][c])) p = r;
        if (std::fabs(m[p][c]) < 1e-300) return false;
        if (p != c)
            for (int k = 0; k < 8; ++k) std::swap(m[p][k], m[c][k]);
        const double d = m[c][c];
        for (int k = 0; k < 8; ++k) m[c][k] /= d;
        for (int r = 0; r < 4; ++r)
            if (r != c) {
                const double f = m[r][c];
                for (int k = 0; k < 8; ++k) m[r][k] -= f * m[c][k];
            }
    }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) out[c * 4 + r] = (float)m[r][c + 4];
    return true;
}

int sph_render_frame(sph_ctx* x, const sph_view* view, int method, int filter_iterations, const sph_light* lights,
                     int nlights, float* rgba_host) {
    if (!x || !view || !rgba_host || filter_iterations < 0 ||
        (method != SPH_RENDER_SCREEN_SPACE && method != SPH_RENDER_PARTICLES))
        return SPH_E_INVALID;
    if (!sph::image_ok(view->width, view->height))
        return sph_ctx_fail(x, SPH_E_INVALID, "render: width and height must be 1..65536 (at most 2^28 pixels)");
    float ip[16];
    if (!invert4(view->projection, ip)) return sph_ctx_fail(x, SPH_E_INVALID, "render: singular projection");
    const int w = view->width, h = view->height;
    const size_t npix = (size_t)w * h;
    if (x->frame_pixels < npix) {
        cudaStreamSynchronize(x->stream);
        cudaFree(x->frame_buf);
        x->frame_buf = nullptr;
        x->frame_pixels = 0;
        if (cudaMalloc(&x->frame_buf, 40 * npix) != cudaSuccess) {
            cudaGetLastError();
            return sph_ctx_fail(x, SPH_E_NOMEM, "render: frame images");
        }
        x->frame_pixels = npix;
    }
    float* depth = static_cast<float*>(x->frame_buf);
    float* tmp = depth + npix;
    float* normals = tmp + npix;
    float* color = normals + 4 * npix;
    void* s = x->stream;
    int rc;
    if (method == SPH_RENDER_PARTICLES) {
        rc = sph_render_particles(x, view, lights, nlights, color);
    } else {
        rc = sph_render_depth(x, view, depth);
        if (rc == SPH_OK) rc = sph_render_smooth(depth, tmp, w, h, filter_iterations, s);
        if (rc == SPH_OK) rc = sph_render_normals(depth, normals, w, h, ip, s);
        if (rc == SPH_OK)
            rc = sph_render_shade(depth, normals, nullptr, nullptr, 0, w, h, view->modelview, ip, color, s);
    }
    if (rc != SPH_OK) return sph_ctx_fail(x, rc, "render: frame stages");
    if (cudaMemcpyAsync(rgba_host, color, 16 * npix, cudaMemcpyDeviceToHost, x->stream) != cudaSuccess ||
        cudaStreamSynchronize(x->stream) != cudaSuccess) {
        cudaGetLastError();
        return sph_ctx_fail(x, SPH_E_CUDA, "render: frame copy");
    }
    return SPH_OK;
}

int sph_render_shade(const float* d_depth, const float* d_normals4, const float* d_background4,
                     const float* d_cube4, int cube_size, int width, int height, const float modelview[16],
                     const float inv_projection[16], float* d_rgba, void* stream) {
    if (!d_depth || !d_normals4 || !d_rgba || !modelview || !inv_projection || !sph::image_ok(width, height))
        return SPH_E_INVALID;
    if (d_cube4 && (cube_size <= 0 || cube_size > 16384)) return SPH_E_INVALID;
    sph::Shade sh;
    std::memcpy(sh.mv, modelview, sizeof sh.mv);
    std::memcpy(sh.ip, inv_projection, sizeof sh.ip);
    const dim3 b(16, 16);
    sph::k_shade<<<sph::grid2(width, height, b), b, 0, (cudaStream_t)stream>>>(
        d_depth, reinterpret_cast<const float4*>(d_normals4), reinterpret_cast<const float4*>(d_background4),
        reinterpret_cast<const float4*>(d_cube4), cube_size, width, height, sh, reinterpret_cast<float4*>(d_rgba));
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_E_CUDA;
}

}  // extern "C"
