/*
 * sph_boundary.cu -- boundary-particle coupling (kernels/boundary.cl) and device statistics.
 *
 *   k_bnd_transform  transform_particles (boundary.cl:33-59): x = R x_raw + c, boundary
 *                    velocity v = v_lin + w*(x - c) componentwise in COMPAT (the kernel
 *                    text), w x (x - c) in PHYSICS (P6).  Uncontracted arithmetic, so the
 *                    positions (and the Morton keys built from them) equal the oracle's.
 *   k_bnd_phi        compute_boundary_phi (boundary.cl:4-31): Psi_b = rho0 / (W_sum w) / coeff
 *                    over the particles of the same body.  The reference loops over every
 *                    particle of the body (O(n^2)); here the sorted boundary cell table gives
 *                    the same set (r^2 < h^2) in O(n), summed in cell order.
 *   k_bnd_forces     compute_fluid_force (boundary.cl:61-118) + clsum (clreduce.h:74-86): the
 *                    pressure force of the fluid on each particle of a body with mass > 0 and
 *                    its torque about the body centre, one record per boundary particle;
 *   k_body_sum       the per-body sums of those records (one block per body, a fixed
 *                    strided order and a fixed tree), so a body's force -- and the motion of a
 *                    dynamic body -- is the same on every run (no host read per body as in
 *                    boundaryhandler.cpp:338-346).
 *   k_stats          density error, kinetic/potential energy and centre of mass.
 */
#include "sph_kernels.cuh"

namespace sph {

__global__ void k_bnd_transform(int nb, const float4* __restrict__ raw, const int32_t* __restrict__ body,
                                const float* __restrict__ xf, const int32_t* __restrict__ range, int compat,
                                int only_movable, float4* __restrict__ pos, float4* __restrict__ vel) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    const int bi = body[i];
    if (only_movable && range[4 * bi + 2] == 0) return;
    const float* t = xf + 20 * bi;
    const float4 r = raw[i];
    /* dot(m_k, p) over (x, y, z, w) with m_k.w = 0: ((a+b)+c)+0 */
    const float px = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(t[0], r.x), __fmul_rn(t[1], r.y)), __fmul_rn(t[2], r.z)), 0.f);
    const float py = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(t[4], r.x), __fmul_rn(t[5], r.y)), __fmul_rn(t[6], r.z)), 0.f);
    const float pz = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(t[8], r.x), __fmul_rn(t[9], r.y)), __fmul_rn(t[10], r.z)), 0.f);
    const float x = __fadd_rn(px, t[3]), y = __fadd_rn(py, t[7]), z = __fadd_rn(pz, t[11]);
    pos[i] = make_float4(x, y, z, 1.f);
    const float rx = __fsub_rn(x, t[3]), ry = __fsub_rn(y, t[7]), rz = __fsub_rn(z, t[11]);
    const float ax = t[16], ay = t[17], az = t[18];
    float vx, vy, vz;
    if (compat) {
        vx = __fadd_rn(t[12], __fmul_rn(ax, rx));
        vy = __fadd_rn(t[13], __fmul_rn(ay, ry));
        vz = __fadd_rn(t[14], __fmul_rn(az, rz));
    } else {
        vx = t[12] + (ay * rz - az * ry);
        vy = t[13] + (az * rx - ax * rz);
        vz = t[14] + (ax * ry - ay * rx);
    }
    vel[i] = make_float4(vx, vy, vz, 0.f);
}

__global__ void k_bnd_phi(Const c, int nb, const float4* __restrict__ bpos_s, const int32_t* __restrict__ body_s,
                          const int2* __restrict__ btab, const int32_t* __restrict__ bmask_s, float phi_coeff,
                          float* __restrict__ bphi_s, float* __restrict__ bphi, const SceneDev* __restrict__ scenes,
                          const int32_t* __restrict__ scene_of) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    const float4 pi = bpos_s[i];
    const int bi = body_s[i];
    const float H = c.h_def, HH = H * H;
    Const cu = c;
    cu.cap = 0x7fffffff;
    cu.h2_list = HH;
    /* batched contexts: one boundary body per scene (scene_of = body ids), binned on that
     * scene's grid; a single-scene context passes no scene_of */
    btab += scene_setup(cu, scenes, scene_of, i);
    float del = 0.f;
    scan_neighbors<true>(cu, pi.x, pi.y, pi.z, btab, bpos_s, [&](int j, float4, float dx, float dy, float dz) {
        if (__ldg(&body_s[j]) == bi) {
            const float r2 = r2_exact(dx, dy, dz);
            if (c.monaghan) {   /* W_DEFAULT(r^2, h) with the Monaghan kernels (boundary.cl:26) */
                del += w_monaghan(r2, H, H);
            } else {
                const float t = HH - r2;
                del += (t * t) * t;
            }
        }
    });
    const float phi = (c.rho0 / (del * c.boundary_eval)) / phi_coeff;
    bphi_s[i] = phi;
    bphi[bmask_s[i]] = phi;
}

__global__ void k_bnd_forces(Const c, int nb, const float4* __restrict__ bpos, const float* __restrict__ bphi,
                             const int32_t* __restrict__ body, const int32_t* __restrict__ range,
                             const float* __restrict__ xf, const float4* __restrict__ spos,
                             const float* __restrict__ dens, const float* __restrict__ pres,
                             const int2* __restrict__ tab, float4* __restrict__ bft) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < nb;
    int bi = -1;
    float fx = 0.f, fy = 0.f, fz = 0.f, tx = 0.f, ty = 0.f, tz = 0.f;
    if (live) {
        bi = body[i];
        if (range[4 * bi + 3] == 0) bi = -1;
    }
    if (bi >= 0) {
        const float4 pi = bpos[i];
        const float H = c.h_def;
        int cx, cy, cz;
        cell_of(c, pi.x, pi.y, pi.z, cx, cy, cz);
        int cnt = 0;
        for (int o = 0; cnt < c.cap && o < 27; ++o) {
            int ox, oy, oz;
            neigh_offset(o, ox, oy, oz);
            long long id;
            if (!neigh_cell(c, cx + ox, cy + oy, cz + oz, id)) continue;
            const int2 rg = tab[id];
            for (int j = rg.x; cnt < c.cap && j < rg.y; ++j) {
                const float4 pj = spos[j];
                const float rx = pj.x - pi.x, ry = pj.y - pi.y, rz = pj.z - pi.z;
                const float rn = sqrtf(rx * rx + ry * ry + rz * rz);
                if (rn < H) {
                    const float dj = dens[j];
                    const float C = pres[j] / (dj * dj);
                    ++cnt;
                    const float s = c.bforce_spiky / rn, t = (H - rn) * (H - rn);
                    fx += (((rx * s) * t) * 2.0f) * C;
                    fy += (((ry * s) * t) * 2.0f) * C;
                    fz += (((rz * s) * t) * 2.0f) * C;
                }
            }
        }
        const float k = c.mass * bphi[i];
        fx *= k; fy *= k; fz *= k;
        const float* t = xf + 20 * bi;
        const float ex = pi.x - t[3], ey = pi.y - t[7], ez = pi.z - t[11];
        tx = ey * fz - ez * fy;
        ty = ez * fx - ex * fz;
        tz = ex * fy - ey * fx;
    }
    if (live) {
        bft[2 * (size_t)i] = make_float4(fx, fy, fz, 0.f);
        bft[2 * (size_t)i + 1] = make_float4(tx, ty, tz, 0.f);
    }
}

/* One block per body: thread t sums records origin + t, origin + t + 256, ... in order, then
 * a fixed tree over the 256 partial sums. */
__global__ void __launch_bounds__(256) k_body_sum(const int32_t* __restrict__ range, const float4* __restrict__ bft,
                                                  float4* __restrict__ body_force, float4* __restrict__ body_torque) {
    __shared__ float part[6][256];
    const int b = blockIdx.x, t = threadIdx.x;
    const int origin = range[4 * b], count = range[4 * b + 1];
    float a[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (range[4 * b + 3] != 0)
        for (int k = t; k < count; k += 256) {
            const float4 f = bft[2 * (size_t)(origin + k)], q = bft[2 * (size_t)(origin + k) + 1];
            a[0] += f.x; a[1] += f.y; a[2] += f.z;
            a[3] += q.x; a[4] += q.y; a[5] += q.z;
        }
#pragma unroll
    for (int k = 0; k < 6; ++k) part[k][t] = a[k];
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (t < w)
#pragma unroll
            for (int k = 0; k < 6; ++k) part[k][t] += part[k][t + w];
        __syncthreads();
    }
    if (t == 0) {
        body_force[b] = make_float4(part[0][0], part[1][0], part[2][0], 0.f);
        body_torque[b] = make_float4(part[3][0], part[4][0], part[5][0], 0.f);
    }
}

/* stats[0..7]: sum max(e,0), sum |e|, max e (as ordered bits), KE, PE, sum x, y, z */
__global__ void k_stats(Const c, const float* __restrict__ dens, const float4* __restrict__ pos,
                        const float4* __restrict__ vel, double* __restrict__ out) {
    double a[7] = {0, 0, 0, 0, 0, 0, 0};
    float mx = -3.0e38f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < c.n; i += gridDim.x * blockDim.x) {
        const float e = (dens[i] - c.rho0) / c.rho0;
        a[0] += e > 0.f ? e : 0.f;
        a[1] += fabsf(e);
        mx = fmaxf(mx, e);
        const float4 p = pos[i], v = vel[i];
        a[2] += 0.5 * (double)c.mass * (double)(v.x * v.x + v.y * v.y + v.z * v.z);
        a[3] += (double)c.mass * (double)(-c.g) * (double)p.y;
        a[4] += p.x; a[5] += p.y; a[6] += p.z;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int k = 0; k < 7; ++k) a[k] += __shfl_xor_sync(0xffffffffu, a[k], o);
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&out[0], a[0]);
        atomicAdd(&out[1], a[1]);
        atomicAdd(&out[3], a[2]);
        atomicAdd(&out[4], a[3]);
        atomicAdd(&out[5], a[4]);
        atomicAdd(&out[6], a[5]);
        atomicAdd(&out[7], a[6]);
        /* order-preserving map of the float max into an unsigned slot (out[2] bits) */
        unsigned u = __float_as_uint(mx);
        u = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
        atomicMax(reinterpret_cast<unsigned long long*>(&out[2]), (unsigned long long)u);
    }
}

/* Per-scene version of k_stats for batched contexts: out[8 * scene + k], same layout.
 * Scenes are contiguous ranges, so a warp almost always belongs to one scene and reduces
 * with shuffles before one atomic per quantity. */
__global__ void k_scene_stats(Const c, const float* __restrict__ dens, const float4* __restrict__ pos,
                              const float4* __restrict__ vel, const int32_t* __restrict__ scene_of,
                              double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < c.n;
    const int s = live ? scene_of[i] : -1;
    double a[7] = {0, 0, 0, 0, 0, 0, 0};
    float mx = -3.0e38f;
    if (live) {
        const float e = (dens[i] - c.rho0) / c.rho0;
        a[0] = e > 0.f ? e : 0.f;
        a[1] = fabsf(e);
        mx = e;
        const float4 p = pos[i], v = vel[i];
        a[2] = 0.5 * (double)c.mass * (double)(v.x * v.x + v.y * v.y + v.z * v.z);
        a[3] = (double)c.mass * (double)(-c.g) * (double)p.y;
        a[4] = p.x; a[5] = p.y; a[6] = p.z;
    }
    const int s0 = __shfl_sync(0xffffffffu, s, 0);
    const bool uniform = __all_sync(0xffffffffu, s == s0);
    if (uniform) {
        if (s0 < 0) return;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
            for (int k = 0; k < 7; ++k) a[k] += __shfl_xor_sync(0xffffffffu, a[k], o);
            mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        }
        if ((threadIdx.x & 31) != 0) return;
    } else if (s < 0) {
        return;
    }
    double* o = out + 8 * (size_t)(uniform ? s0 : s);
    atomicAdd(&o[0], a[0]);
    atomicAdd(&o[1], a[1]);
    atomicAdd(&o[3], a[2]);
    atomicAdd(&o[4], a[3]);
    atomicAdd(&o[5], a[4]);
    atomicAdd(&o[6], a[5]);
    atomicAdd(&o[7], a[6]);
    unsigned u = __float_as_uint(mx);
    u = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
    atomicMax(reinterpret_cast<unsigned long long*>(&o[2]), (unsigned long long)u);
}

void launch_scene_stats(cudaStream_t s, const Const& c, const Bufs& b, double* out, int nscenes) {
    cudaMemsetAsync(out, 0, 8 * sizeof(double) * nscenes, s);
    if (c.n <= 0) return;
    k_scene_stats<<<(c.n + 255) / 256, 256, 0, s>>>(c, b.density, b.pos, b.vel, b.scene_of, out);
}

static inline int nblk(int n, int bs) { return (n + bs - 1) / bs; }

void launch_bnd_transform(cudaStream_t s, const Bufs& b, int nbodies, int nb, bool compat, bool only_movable,
                          int bs) {
    if (nb <= 0 || nbodies <= 0) return;
    k_bnd_transform<<<nblk(nb, bs), bs, 0, s>>>(nb, b.braw, b.bbody, b.body_xf, b.body_range, compat ? 1 : 0,
                                                only_movable ? 1 : 0, b.bpos, b.bvel);
}
void launch_bnd_phi(cudaStream_t s, const Const& c, const Bufs& b, float phi_coeff, int bs) {
    if (c.nb <= 0) return;
    k_bnd_phi<<<nblk(c.nb, bs), bs, 0, s>>>(c, c.nb, b.bpos_s, b.bbody_s, b.btab, b.bmask_sorted, phi_coeff,
                                            b.bphi_s, b.bphi, b.scenes, b.scene_of ? b.bbody_s : nullptr);
}
/* bnear[cell] = 1 for the 27 cells around each sorted boundary particle's cell (the cells
 * whose particles can have a boundary neighbour); concurrent stores all write 1. */
__global__ void k_bnd_near(Const c0, int nb, const float4* __restrict__ bpos_s, uint8_t* __restrict__ near,
                           const SceneDev* __restrict__ scenes, const int32_t* __restrict__ scene_of) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    Const c = c0;
    const long long base = scene_setup(c, scenes, scene_of, i);
    const float4 p = bpos_s[i];
    int cx, cy, cz;
    cell_of(c, p.x, p.y, p.z, cx, cy, cz);
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                long long id;
                if (neigh_cell(c, cx + dx, cy + dy, cz + dz, id)) near[base + id] = 1;
            }
}

void launch_bnd_near(cudaStream_t s, const Const& c, const Bufs& b, int nb, int bs) {
    cudaMemsetAsync(b.bnear, 0, (size_t)c.ncells, s);
    if (nb <= 0) return;
    k_bnd_near<<<nblk(nb, bs), bs, 0, s>>>(c, nb, b.bpos_s, b.bnear, b.scenes, b.scene_of ? b.bbody_s : nullptr);
}

/* One step of a dynamic body (semi-implicit Euler, the default of the reference's rigid-body
 * engine without collisions): v += dt (F / m + g), x += dt v; w += dt R I^-1 R^T tau; the
 * orientation turns by |w| dt about w (Rodrigues) and is re-orthonormalised; with a radius
 * r > 0 the centre is kept r inside the container (the velocity into the wall is dropped).
 * The force and torque are the fluid's (k_bnd_forces, boundaryhandler.cpp:296-349). */
__device__ __forceinline__ void body_step(float* t, const float* d, float4 F, float4 T, float g, float dt,
                                          float lx, float ly, float lz) {
    const float m = d[1];
    const float ax = F.x / m, ay = F.y / m + g, az = F.z / m;
    t[12] = t[12] + dt * ax;
    t[13] = t[13] + dt * ay;
    t[14] = t[14] + dt * az;
    t[3] = t[3] + dt * t[12];
    t[7] = t[7] + dt * t[13];
    t[11] = t[11] + dt * t[14];
    float r[9] = {t[0], t[1], t[2], t[4], t[5], t[6], t[8], t[9], t[10]};
    float y[3];
    for (int k = 0; k < 3; ++k) y[k] = (r[k] * T.x + r[3 + k] * T.y + r[6 + k] * T.z) * d[2 + k];
    for (int i = 0; i < 3; ++i) t[16 + i] = t[16 + i] + dt * (r[3 * i] * y[0] + r[3 * i + 1] * y[1] + r[3 * i + 2] * y[2]);
    const float wx = t[16], wy = t[17], wz = t[18];
    const float wn = sqrtf(wx * wx + wy * wy + wz * wz);
    const float th = wn * dt;
    if (th > 0.f) {
        const float kx = wx / wn, ky = wy / wn, kz = wz / wn;
        const float cs = cosf(th), sn = sinf(th), C = 1.0f - cs;
        const float q[9] = {cs + kx * kx * C, kx * ky * C - kz * sn, kx * kz * C + ky * sn,
                            ky * kx * C + kz * sn, cs + ky * ky * C, ky * kz * C - kx * sn,
                            kz * kx * C - ky * sn, kz * ky * C + kx * sn, cs + kz * kz * C};
        float n[9];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) n[3 * i + j] = q[3 * i] * r[j] + q[3 * i + 1] * r[3 + j] + q[3 * i + 2] * r[6 + j];
        const float l0 = sqrtf(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        for (int j = 0; j < 3; ++j) n[j] /= l0;
        const float p = n[3] * n[0] + n[4] * n[1] + n[5] * n[2];
        for (int j = 0; j < 3; ++j) n[3 + j] -= p * n[j];
        const float l1 = sqrtf(n[3] * n[3] + n[4] * n[4] + n[5] * n[5]);
        for (int j = 0; j < 3; ++j) n[3 + j] /= l1;
        n[6] = n[1] * n[5] - n[2] * n[4];
        n[7] = n[2] * n[3] - n[0] * n[5];
        n[8] = n[0] * n[4] - n[1] * n[3];
        t[0] = n[0]; t[1] = n[1]; t[2] = n[2];
        t[4] = n[3]; t[5] = n[4]; t[6] = n[5];
        t[8] = n[6]; t[9] = n[7]; t[10] = n[8];
    }
    const float rad = d[5];
    if (rad > 0.f) {
        const float lo[3] = {-lx / 2.0f + rad, -ly / 2.0f + rad, -lz / 2.0f + rad};
        const float hi[3] = {lx / 2.0f - rad, 10.0f - rad, lz / 2.0f - rad};
        const int ci[3] = {3, 7, 11};
        for (int a = 0; a < 3; ++a) {
            if (t[ci[a]] < lo[a]) {
                t[ci[a]] = lo[a];
                if (t[12 + a] < 0.f) t[12 + a] = 0.f;
            } else if (t[ci[a]] > hi[a]) {
                t[ci[a]] = hi[a];
                if (t[12 + a] > 0.f) t[12 + a] = 0.f;
            }
        }
    }
}

__global__ void k_body_integrate(Const c, int nbodies, float* __restrict__ xf, const float* __restrict__ dyn,
                                 const float4* __restrict__ force, const float4* __restrict__ torque) {
    for (int k = threadIdx.x; k < nbodies; k += blockDim.x) {
        const float* d = dyn + 8 * k;
        if (d[0] == 0.f) continue;
        body_step(xf + 20 * k, d, force[k], torque[k], c.g, c.dt, c.lim_x, c.lim_y, c.lim_z);
    }
}

void launch_body_integrate(cudaStream_t s, const Const& c, const Bufs& b, int nbodies) {
    if (nbodies <= 0) return;
    k_body_integrate<<<1, 32, 0, s>>>(c, nbodies, b.body_xf, b.body_dyn, b.body_force, b.body_torque);
}

void launch_bnd_forces(cudaStream_t s, const Const& c, const Bufs& b, int nbodies, int bs) {
    if (c.nb <= 0 || nbodies <= 0) return;
    k_bnd_forces<<<nblk(c.nb, bs), bs, 0, s>>>(c, c.nb, b.bpos, b.bphi, b.bbody, b.body_range, b.body_xf, b.pos_s,
                                               b.density, b.pressure, b.tab, b.bft);
    k_body_sum<<<nbodies, 256, 0, s>>>(b.body_range, b.bft, b.body_force, b.body_torque);
}
void launch_stats(cudaStream_t s, const Const& c, const Bufs& b) {
    cudaMemsetAsync(b.stats, 0, 8 * sizeof(double), s);
    if (c.n <= 0) return;
    int g = nblk(c.n, 256);
    if (g > 1024) g = 1024;
    k_stats<<<g, 256, 0, s>>>(c, b.density, b.pos, b.vel, b.stats);
}

}  // namespace sph
