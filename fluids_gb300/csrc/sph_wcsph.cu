/*
 * sph_wcsph.cu -- WCSPH neighbour passes.
 *
 *   k_wc_density  compute_density_pressure (kernels/wcsph.cl:32-79): rho from fluid and
 *                 boundary (Psi-weighted) poly6 sums, Tait pressure max(0, k((rho/rho0)^7-1)).
 *                 COMPAT evaluates poly6 at r as the kernel text does; PHYSICS at r^2 (P1).
 *   k_normals     compute_normals (kernels/normals.cl:23-70), shared with PCISPH.
 *   k_wc_forces   compute_acceleration (kernels/wcsph.cl:81-173): boundary pressure, fluid
 *                 pressure, viscosity and Akinci surface tension, gravity; PHYSICS carries
 *                 the mass factors of kernels/pcisph.cl:216-219 (P3).  With FUSE the
 *                 leapfrog integration of predict_vel_n_pos (kernels/wcsph.cl:176-224) runs
 *                 as the epilogue, so the acceleration never round-trips through HBM.
 * One thread per particle in Morton order: the 32 particles of a warp share most of their
 * 27 neighbour cells, so neighbour positions come from L1/L2 rather than HBM.
 */
#include "sph_kernels.cuh"

namespace sph {

template <bool COMPAT, bool LIST>
__global__ void __launch_bounds__(256) k_wc_density(Const c, Neigh<LIST> fl, Neigh<LIST> bl,
                                                    const float* __restrict__ bphi_s, float* __restrict__ dens,
                                                    float* __restrict__ pres) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const float4 pi = __ldg(&fl.npos[i]);
    const float hh = c.h * c.h;
    float di = 0.f;
    fl.visit(c, i, pi.x, pi.y, pi.z, [&](int, float4, float dx, float dy, float dz) {
        const float r2 = dx * dx + dy * dy + dz * dz;
        const float t = hh - (COMPAT ? sqrtf(r2) : r2);
        di += (t * t) * t;
    });
    di *= c.poly6_eval * c.mass;
    float bdi = 0.f;
    if (c.nb > 0) {
        bl.visit(c, i, pi.x, pi.y, pi.z, [&](int j, float4, float dx, float dy, float dz) {
            const float r2 = dx * dx + dy * dy + dz * dz;
            const float t = hh - (COMPAT ? sqrtf(r2) : r2);
            bdi += ((t * t) * t) * __ldg(&bphi_s[j]);
        });
    }
    di += c.poly6_eval * bdi;
    dens[i] = di;
    const float pv = c.kgas * (pown7(di / c.rho0) - 1.0f);
    pres[i] = (0.f < pv) ? pv : 0.f;
}

template <bool LIST>
__global__ void __launch_bounds__(256) k_normals(Const c, Neigh<LIST> fl, const float* __restrict__ dens,
                                                 float4* __restrict__ normal) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const float4 pi = __ldg(&fl.npos[i]);
    const float H = c.h_def, HH = H * H;
    float nx = 0.f, ny = 0.f, nz = 0.f;
    fl.visit(c, i, pi.x, pi.y, pi.z, [&](int j, float4, float dx, float dy, float dz) {
        const float t = HH - (dx * dx + dy * dy + dz * dz);
        const float s = t * t;
        const float dj = __ldg(&dens[j]);
        nx += (dx * s) / dj;
        ny += (dy * s) / dj;
        nz += (dz * s) / dj;
    });
    const float k = c.poly6_grad;
    normal[i] = make_float4(((k * nx) * c.mass_def) * H, ((k * ny) * c.mass_def) * H, ((k * nz) * c.mass_def) * H,
                            0.f);
}

/* predict_vel_n_pos (kernels/wcsph.cl:176-224) for one particle. */
__device__ __forceinline__ void wc_integrate_one(const Const& c, float4 p, float4 vh, float ax, float ay, float az,
                                                 float4& po, float4& vo, float4& vho, bool& bad) {
    const float dt = c.dt, vm = c.vmax;
    vh.x += dt * ax;
    vh.y += dt * ay;
    vh.z += dt * az;
    p.x += dt * clampf(vh.x + dt * ax, -vm, vm);
    p.y += dt * clampf(vh.y + dt * ay, -vm, vm);
    p.z += dt * clampf(vh.z + dt * az, -vm, vm);
    const float vn = len3(vh.x, vh.y, vh.z);
    float cx = clampf(p.x, (-c.lim_x) / 2.0f, c.lim_x / 2.0f);
    float cy = clampf(p.y, (-c.lim_y) / 2.0f, 10.0f);
    float cz = clampf(p.z, (-c.lim_z) / 2.0f, c.lim_z / 2.0f);
    const float ex = cx - p.x, ey = cy - p.y, ez = cz - p.z;
    const float d = len3(ex, ey, ez);
    if (d > 0.f && vn > 0.f) {
        float sx = signf(ex), sy = signf(ey), sz = signf(ez);
        const float sl = len3(sx, sy, sz);
        sx /= sl; sy /= sl; sz /= sl;
        const float rest = (1.0f * d) / (dt * vn);
        const float k = (1.0f + rest) * (vh.x * sx + vh.y * sy + vh.z * sz);
        vh.x -= k * sx;
        vh.y -= k * sy;
        vh.z -= k * sz;
        p.x = cx; p.y = cy; p.z = cz;
    }
    const float vx = vh.x + (dt * ax) * 0.5f, vy = vh.y + (dt * ay) * 0.5f, vz = vh.z + (dt * az) * 0.5f;
    po = make_float4(p.x, p.y, p.z, 1.f);
    vho = make_float4(clampf(vh.x, -vm, vm), clampf(vh.y, -vm, vm), clampf(vh.z, -vm, vm), 0.f);
    vo = make_float4(clampf(vx, -vm, vm), clampf(vy, -vm, vm), clampf(vz, -vm, vm), 0.f);
    bad = !(isfinite(p.x) && isfinite(p.y) && isfinite(p.z) && isfinite(vx) && isfinite(vy) && isfinite(vz));
}

template <bool COMPAT, bool LIST, bool FUSE, bool WRITE_ACC, bool ST>
__global__ void __launch_bounds__(256) k_wc_forces(Const c, Neigh<LIST> fl, Neigh<LIST> bl, Bufs b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const float4 pi = __ldg(&b.pos_s[i]);
    const float4 vi = __ldg(&b.vel_s[i]);
    const float di = __ldg(&b.density[i]), p_i = __ldg(&b.pressure[i]);
    const float C = p_i / (di * di);
    const float h = c.h, sg = c.spiky_grad;
    float bax = 0.f, bay = 0.f, baz = 0.f;
    if (c.nb > 0) {
        bl.visit(c, i, pi.x, pi.y, pi.z, [&](int j, float4, float dx, float dy, float dz) {
            const float rn = sqrtf(dx * dx + dy * dy + dz * dz);
            const float phi = -__ldg(&b.bphi_s[j]);
            const float s = sg / rn, t = (h - rn) * (h - rn);
            bax += ((((phi * dx) * s) * t) * 2.0f) * C;
            bay += ((((phi * dy) * s) * t) * 2.0f) * C;
            baz += ((((phi * dz) * s) * t) * 2.0f) * C;
        });
    }
    float4 ni = make_float4(0.f, 0.f, 0.f, 0.f);
    if (ST) ni = __ldg(&b.normal[i]);
    float pax = 0.f, pay = 0.f, paz = 0.f, vax = 0.f, vay = 0.f, vaz = 0.f;
    float cux = 0.f, cuy = 0.f, cuz = 0.f, cox = 0.f, coy = 0.f, coz = 0.f;
    const float rmin = c.rmin_wc;
    fl.visit(c, i, pi.x, pi.y, pi.z, [&](int j, float4, float dx, float dy, float dz) {
        const float dj = __ldg(&b.density[j]);
        const float rn = sqrtf(dx * dx + dy * dy + dz * dz);
        if (di > 0.f && dj > 0.f && rn > rmin) {
            const float pj = __ldg(&b.pressure[j]);
            const float4 vj = __ldg(&b.vel_s[j]);
            const float s = sg / rn, t = (h - rn) * (h - rn), q = C + pj / (dj * dj);
            pax += ((dx * s) * t) * q;
            pay += ((dy * s) * t) * q;
            paz += ((dz * s) * t) * q;
            const float w = h - rn;
            vax += ((vj.x - vi.x) * w) / dj;
            vay += ((vj.y - vi.y) * w) / dj;
            vaz += ((vj.z - vi.z) * w) / dj;
            if (ST) {
                const float4 nj = __ldg(&b.normal[j]);
                const float K = st_corr(c.rho0, di, dj);
                cux += (ni.x - nj.x) * K;
                cuy += (ni.y - nj.y) * K;
                cuz += (ni.z - nj.z) * K;
                const float sk = st_kernel(rn, h, c.st_term);
                cox += ((dx / rn) * sk) * K;
                coy += ((dy / rn) * sk) * K;
                coz += ((dz / rn) * sk) * K;
            }
        }
    });
    const float m = c.mass;
    pax *= -m; pay *= -m; paz *= -m;
    const float vs = COMPAT ? (c.visc_lapl * c.mu) : (c.visc_lapl * c.mu) * (m / di);
    vax *= vs; vay *= vs; vaz *= vs;
    float ax = pax + vax + bax, ay = c.g + pay + vay + bay, az = paz + vaz + baz;
    if (ST) {
        const float cs = COMPAT ? c.st_main : c.st_main * m;
        const float ns = -c.sigma;
        ax = ((((ns * (cux + cox * cs)) + pax) + vax) + bax);
        ay = (((c.g + ns * (cuy + coy * cs)) + pay) + vay) + bay;
        az = ((((ns * (cuz + coz * cs)) + paz) + vaz) + baz);
    }
    if (WRITE_ACC) b.accel[i] = make_float4(ax, ay, az, 0.f);
    if (FUSE) {
        float4 po, vo, vho;
        bool bad;
        wc_integrate_one(c, pi, __ldg(&b.vhalf_s[i]), ax, ay, az, po, vo, vho, bad);
        b.pos[i] = po;
        b.vel[i] = vo;
        b.vhalf[i] = vho;
        b.ids[i] = __ldg(&b.ids_s[i]);
        if (bad) atomicOr(b.flags, kFlagNan);
    }
}

__global__ void __launch_bounds__(256) k_wc_integrate(Const c, Bufs b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const float4 a = __ldg(&b.accel[i]);
    float4 po, vo, vho;
    bool bad;
    wc_integrate_one(c, __ldg(&b.pos_s[i]), __ldg(&b.vhalf_s[i]), a.x, a.y, a.z, po, vo, vho, bad);
    b.pos[i] = po;
    b.vel[i] = vo;
    b.vhalf[i] = vho;
    b.ids[i] = __ldg(&b.ids_s[i]);
    if (bad) atomicOr(b.flags, kFlagNan);
}

static inline int nblk(int n, int bs) { return (n + bs - 1) / bs; }

template <bool LIST>
static Neigh<LIST> fluid_src(const Bufs& b) {
    return Neigh<LIST>{b.tab, b.nlist, b.nlen, b.pos_s};
}
template <bool LIST>
static Neigh<LIST> bnd_src(const Bufs& b) {
    return Neigh<LIST>{b.btab, b.sblist, b.sblen, b.bpos_s};
}

void launch_wc_density(cudaStream_t s, const Const& c, const Bufs& b, bool lists, int bs) {
    if (c.n <= 0) return;
    const int g = nblk(c.n, bs);
    if (c.compat) {
        if (lists) k_wc_density<true, true><<<g, bs, 0, s>>>(c, fluid_src<true>(b), bnd_src<true>(b), b.bphi_s, b.density, b.pressure);
        else k_wc_density<true, false><<<g, bs, 0, s>>>(c, fluid_src<false>(b), bnd_src<false>(b), b.bphi_s, b.density, b.pressure);
    } else {
        if (lists) k_wc_density<false, true><<<g, bs, 0, s>>>(c, fluid_src<true>(b), bnd_src<true>(b), b.bphi_s, b.density, b.pressure);
        else k_wc_density<false, false><<<g, bs, 0, s>>>(c, fluid_src<false>(b), bnd_src<false>(b), b.bphi_s, b.density, b.pressure);
    }
}

void launch_normals(cudaStream_t s, const Const& c, const Bufs& b, bool lists, int bs) {
    if (c.n <= 0) return;
    const int g = nblk(c.n, bs);
    if (lists) k_normals<true><<<g, bs, 0, s>>>(c, fluid_src<true>(b), b.density, b.normal);
    else k_normals<false><<<g, bs, 0, s>>>(c, fluid_src<false>(b), b.density, b.normal);
}

template <bool COMPAT, bool LIST>
static void forces_dispatch(cudaStream_t s, const Const& c, const Bufs& b, bool fuse, bool write_acc, int bs) {
    const int g = nblk(c.n, bs);
    const bool st = c.sigma != 0.f;
    auto fs = fluid_src<LIST>(b);
    auto bsrc = bnd_src<LIST>(b);
#define SPH_WCF(F, W, S) k_wc_forces<COMPAT, LIST, F, W, S><<<g, bs, 0, s>>>(c, fs, bsrc, b)
    if (fuse) {
        if (write_acc) { if (st) SPH_WCF(true, true, true); else SPH_WCF(true, true, false); }
        else { if (st) SPH_WCF(true, false, true); else SPH_WCF(true, false, false); }
    } else {
        if (st) SPH_WCF(false, true, true); else SPH_WCF(false, true, false);
    }
#undef SPH_WCF
}

void launch_wc_forces(cudaStream_t s, const Const& c, const Bufs& b, bool lists, bool fuse_integrate,
                      bool write_acc, int bs) {
    if (c.n <= 0) return;
    if (c.compat) {
        if (lists) forces_dispatch<true, true>(s, c, b, fuse_integrate, write_acc, bs);
        else forces_dispatch<true, false>(s, c, b, fuse_integrate, write_acc, bs);
    } else {
        if (lists) forces_dispatch<false, true>(s, c, b, fuse_integrate, write_acc, bs);
        else forces_dispatch<false, false>(s, c, b, fuse_integrate, write_acc, bs);
    }
}

void launch_wc_integrate(cudaStream_t s, const Const& c, const Bufs& b, int bs) {
    if (c.n <= 0) return;
    k_wc_integrate<<<nblk(c.n, bs), bs, 0, s>>>(c, b);
}

}  // namespace sph
