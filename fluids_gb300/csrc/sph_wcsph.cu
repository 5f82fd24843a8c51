/*
 * sph_wcsph.cu -- WCSPH neighbour passes.
 *
 *   k_wc_density  compute_density_pressure (kernels/wcsph.cl:32-79): rho from fluid and
 *                 boundary (Psi-weighted) poly6 sums, Tait pressure max(0, k((rho/rho0)^7-1)).
 *                 COMPAT evaluates poly6 at r as the kernel text does; PHYSICS at r^2 (P1).
 *                 Also writes aux = (p/rho^2, 1/rho, rho, p) so the later passes divide by
 *                 nothing inside their neighbour loops.
 *   k_normals     compute_normals (kernels/normals.cl:23-70), shared with PCISPH.
 *   k_wc_forces   compute_acceleration (kernels/wcsph.cl:81-173): boundary pressure, fluid
 *                 pressure, viscosity and Akinci surface tension, gravity; PHYSICS carries
 *                 the mass factors of kernels/pcisph.cl:216-219 (P3).  With FUSE the
 *                 leapfrog integration of predict_vel_n_pos (kernels/wcsph.cl:176-224) runs
 *                 as the epilogue, so the acceleration never round-trips through HBM.
 * One thread per particle in Morton order: the 32 particles of a warp share most of their
 * 27 neighbour cells, so neighbour data comes from L1/L2 rather than HBM.  Inside the
 * neighbour loops 1/r comes from rsqrtf and 1/rho_j from aux or the correctly rounded
 * reciprocal of the density (FP32 results differ from the
 * reference's IEEE divisions by a few ulp, inside the parity tolerance).
 */
#include "sph_kernels.cuh"

namespace sph {

__device__ __forceinline__ float4 make_aux(float d, float p) {
    return make_float4(p / (d * d), 1.0f / d, d, p);
}

/* W_DEFAULT(r_norm, support_radius) of compute_density_pressure (wcsph.cl:61-62,70-71):
 * PHYSICS (h^2 - r^2)^3; COMPAT the kernel text's (h^2 - r)^3, or with the Monaghan kernels
 * w_monaghan(r, h). */
template <bool COMPAT>
__device__ __forceinline__ float w_default(const Const& c, float r2, float hh) {
    if constexpr (COMPAT) {
        if (c.monaghan) return w_monaghan(sqrtf(r2), c.h, c.h_def);
        const float t = hh - sqrtf(r2);
        return (t * t) * t;
    }
    const float t = hh - r2;
    return (t * t) * t;
}

template <bool COMPAT, bool LIST, bool BATCH>
__global__ void __launch_bounds__(256) k_wc_density(Const c0, Neigh<LIST, COMPAT> fl0, Neigh<LIST, COMPAT> bl0,
                                                    const float* __restrict__ bphi_s, float* __restrict__ dens,
                                                    float* __restrict__ pres, float4* __restrict__ aux,
                                                    const SceneDev* __restrict__ scenes,
                                                    const SceneTile* __restrict__ tiles, unsigned* next) {
  for_each_particle<BATCH>(c0, tiles, scenes, next, [&](const Const& c, long long base, int i) {
    Neigh<LIST, COMPAT> fl = fl0, bl = bl0;
    fl.tab += base;
    bl.tab += base;
    const float4 pi = __ldg(&fl.npos[i]);
    const float hh = c.h * c.h;
    float di = 0.f;
    fl.visit(c, i, pi.x, pi.y, pi.z, [&](int, float4, float dx, float dy, float dz) {
        const float r2 = dx * dx + dy * dy + dz * dz;
        di += w_default<COMPAT>(c, r2, hh);
    });
    di *= c.poly6_eval * c.mass;
    float bdi = 0.f;
    if (c.nb > 0) {
        bl.visit(c, i, pi.x, pi.y, pi.z, [&](int j, float4, float dx, float dy, float dz) {
            const float r2 = dx * dx + dy * dy + dz * dz;
            bdi += w_default<COMPAT>(c, r2, hh) * __ldg(&bphi_s[j]);
        });
    }
    di += c.poly6_eval * bdi;
    dens[i] = di;
    const float pv = c.kgas * (pown7(di / c.rho0) - 1.0f);
    const float p = (0.f < pv) ? pv : 0.f;
    pres[i] = p;
    aux[i] = make_aux(di, p);
  });
}

/* compute_neigh_list (kernels/grid.cl:145-182, fluid and boundary) fused with
 * compute_density_pressure: the density sums run over exactly the pairs written to the
 * lists, in list order, so the step needs no separate density pass. */
/* 8 blocks/SM holds the builder at 32 registers, with its candidate loop written two
 * candidates a trip: measured on GB300 at 4M, 1.028 ms against 1.036 ms for the compiler's
 * unrolling by 2 at 6 blocks/SM (36 registers; 1.045 vs 1.052 ms at 8 blocks/SM) and 1.040
 * ms at 4 blocks/SM; unrolling by 1, 3 or 4 was 4-10 % slower; 3 % fewer warp
 * instructions (2.466e8 vs 2.544e8 at 1M). */
#ifndef SPH_LISTS_MIN_BLOCKS
#define SPH_LISTS_MIN_BLOCKS 8
#endif
/* REMAP (the adjoint's tape, which keeps particles in id order): the list of sorted particle
 * i is written as row remap[i] with entries remap[j], and its density, pressure and aux go to
 * remap[i]; the visits, their order and the arithmetic are those of the plain builder. */
/* PCI (PHYSICS PCISPH): the fused density is compute_initial_density (pcisph.cl:33-102) over
 * the same pairs instead -- rho = w (m_def sum W + sum Psi W) with h_def and the PCISPH
 * normaliser, pressure 0 (pcisphsimluation.cpp:118), aux = (0, 1/rho, rho, 0) -- so the
 * PCISPH step needs no separate initial-density pass. */
template <bool COMPAT, bool BATCH, bool REMAP = false, bool PCI = false>
__global__ void __launch_bounds__(256, SPH_LISTS_MIN_BLOCKS) k_lists_density(Const c0, const float4* __restrict__ spos,
                                                       const int2* __restrict__ tab0,
                                                       const float4* __restrict__ bpos_s,
                                                       const int2* __restrict__ btab0,
                                                       const float* __restrict__ bphi_s, int* __restrict__ nlist,
                                                       int* __restrict__ nlen, int* __restrict__ sblist,
                                                       int* __restrict__ sblen, float* __restrict__ dens,
                                                       float* __restrict__ pres, float4* __restrict__ aux,
                                                       const SceneDev* __restrict__ scenes,
                                                       const SceneTile* __restrict__ tiles, unsigned* next,
                                                       const int32_t* __restrict__ remap = nullptr,
                                                       unsigned* __restrict__ flags = nullptr,
                                                       const uint8_t* __restrict__ bnear = nullptr,
                                                       const int32_t* __restrict__ noff = nullptr,
                                                       float4* __restrict__ prho = nullptr) {
  for_each_particle<BATCH>(c0, tiles, scenes, next, [&](const Const& c, long long base, int i) {
    const int2* __restrict__ ftab = tab0 + base;
    const int2* __restrict__ fbtab = btab0 + base;
    const float4 pi = spos[i];
    const float hh = PCI ? c.h_def * c.h_def : c.h * c.h;
    const int row = REMAP ? __ldg(&remap[i]) : i;
    int cx, cy, cz;
    cell_of(c, pi.x, pi.y, pi.z, cx, cy, cz);
    float di = 0.f;
    char* const lrow = reinterpret_cast<char*>(nlist + row);
    const unsigned n4 = 4u * (unsigned)c.n;
    const int k = build_scan(c, pi.x, pi.y, pi.z, cx, cy, cz, ftab, spos, BATCH ? nullptr : noff,
                             [&](bool hit, int j, float r2, int slot) {
        if (hit) *list_slot(lrow, slot, n4) = REMAP ? __ldg(&remap[j]) : j;
        if (COMPAT && c.monaghan) {
            if (hit) di += w_monaghan(sqrtf(r2), c.h, c.h_def);
        } else {
            const float t = hit ? hh - (COMPAT ? sqrtf(r2) : r2) : 0.f;
            di += (t * t) * t;
        }
    });
    nlen[row] = k;
    if (k >= c.cap && REMAP) atomicOr(flags, kFlagOverflow);
    if (!PCI) di *= c.poly6_eval * c.mass;
    int kb = 0;
    float bdi = 0.f;
    /* the boundary scan only where a boundary particle is binned in one of the 27 cells
     * (bnear, PHYSICS grid); every other particle's boundary list is empty */
    const bool scan_b = c.wrap || bnear == nullptr || bnear[base + cell_lin(c, cx, cy, cz)] != 0;
    if (c.nb > 0 && !REMAP && scan_b) {
        char* const brow = reinterpret_cast<char*>(sblist + i);
        kb = build_scan(c, pi.x, pi.y, pi.z, cx, cy, cz, fbtab, bpos_s, BATCH ? nullptr : noff,
                        [&](bool hit, int j, float r2, int slot) {
            if (hit) *list_slot(brow, slot, n4) = j;
            float w = 0.f;
            if (hit) w = __ldg(&bphi_s[j]);
            if (COMPAT && c.monaghan) {
                if (hit) bdi += w_monaghan(sqrtf(r2), c.h, c.h_def) * w;
            } else {
                const float t = hit ? hh - (COMPAT ? sqrtf(r2) : r2) : 0.f;
                bdi += ((t * t) * t) * w;
            }
        });
    }
    if (!REMAP) sblen[i] = kb;
    if (PCI) {
        const float d = c.default_eval * ((di * c.mass_def) + bdi);
        dens[row] = d;
        if (prho) prho[row] = make_float4(pi.x, pi.y, pi.z, d);
        pres[row] = 0.f;
        aux[row] = make_float4(0.f, 1.0f / d, d, 0.f);
        return;
    }
    di += c.poly6_eval * bdi;
    dens[row] = di;
    if (prho) prho[row] = make_float4(pi.x, pi.y, pi.z, di);   /* the normal pass's neighbour records */
    const float pv = c.kgas * (pown7(di / c.rho0) - 1.0f);
    const float p = (0.f < pv) ? pv : 0.f;
    pres[row] = p;
    aux[row] = make_aux(di, p);
  });
}

/* aux from the density / pressure fields (used when those fields were set from outside). */
__global__ void __launch_bounds__(256) k_aux(int n, const float* __restrict__ dens, const float* __restrict__ pres,
                                             float4* __restrict__ aux) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    aux[i] = make_aux(dens[i], pres[i]);
}

/* the normal walk's depth: measured on GB300 at 4M with the (x, y, z, rho) records, 0.225 ms
 * two deep against 0.240 three deep, 0.232 four deep, and with the predicated last batch
 * 0.235 two deep and 0.255 four deep */
#ifndef SPH_NORMALS_WALK
#define SPH_NORMALS_WALK 2
#endif
#ifndef SPH_NORMALS_PRED
#define SPH_NORMALS_PRED 0
#endif
/* MON: compute_normals with the Monaghan kernels, GRAD_W_DEFAULT(r, r.r, h) / rho_j
 * (normals.cl:66; the kernel text passes r^2 where the function takes |r|). */
template <bool LIST, bool EXACT, bool BATCH, bool MON = false, bool PRHO = false>
__global__ void __launch_bounds__(256) k_normals(Const c0, Neigh<LIST, EXACT> fl0, const float4* __restrict__ aux,
                                                 const float* __restrict__ dens, float4* __restrict__ normal,
                                                 const SceneDev* __restrict__ scenes,
                                                 const SceneTile* __restrict__ tiles, unsigned* next,
                                                 const float4* __restrict__ vel_s = nullptr,
                                                 float4* __restrict__ nrec = nullptr) {
  for_each_particle<BATCH>(c0, tiles, scenes, next, [&](const Const& c, long long base, int i) {
    Neigh<LIST, EXACT> fl = fl0;
    fl.tab += base;
    const float4 pi = __ldg(&fl.npos[i]);
    const float H = c.h_def, HH = H * H;
    float nx = 0.f, ny = 0.f, nz = 0.f;
    /* two entries deep with the next two loaded during the visits */
    fl.template visit<true, SPH_NORMALS_WALK, SPH_NORMALS_PRED != 0>(c, i, pi.x, pi.y, pi.z,
                                                                     [&](int j, float4 q, float dx, float dy, float dz) {
        /* 1/rho_j: PRHO, from the w of the neighbour record the walk loaded with its position
         * (npos = prho); otherwise from the dense density array (8 particles per 32-byte
         * sector instead of 2 for aux; the pass is bound by L1 throughput); __frcp_rn is the
         * correctly rounded reciprocal, the value aux holds */
        const float inv_rho = __frcp_rn(PRHO ? q.w : __ldg(&dens[j]));
        if constexpr (MON) {
            float gx, gy, gz;
            grad_w_monaghan(dx, dy, dz, dx * dx + dy * dy + dz * dz, H, H, gx, gy, gz);
            const float dj = __ldg(&dens[j]);
            nx += gx / dj;
            ny += gy / dj;
            nz += gz / dj;
        } else {
            const float t = HH - (dx * dx + dy * dy + dz * dz);
            const float k = (t * t) * inv_rho;
            nx += dx * k;
            ny += dy * k;
            nz += dz * k;
        }
    });
    const float k = (c.poly6_grad * c.mass_def) * H;
    const float4 nv = make_float4(nx * k, ny * k, nz * k, 0.f);
    normal[i] = nv;
    if (nrec != nullptr) {
        const float4 v = __ldg(&vel_s[i]), a = __ldg(&aux[i]);
        nrec[2 * (size_t)i] = make_float4(v.x, v.y, v.z, a.x);
        nrec[2 * (size_t)i + 1] = make_float4(nv.x, nv.y, nv.z, a.y);
    }
  });
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

/* the single-scene force walk's depth: measured on GB300 at 4M, 0.600 ms four deep at 4
 * blocks/SM (64 registers) against 0.707 six deep (spills), and at 3 blocks/SM 0.689, 0.671
 * and 0.663 ms four, six and eight deep */
#ifndef SPH_FORCES_WALK
#define SPH_FORCES_WALK 4
#endif
#ifndef SPH_FORCES_MIN_BLOCKS
#define SPH_FORCES_MIN_BLOCKS 4
#endif
/* PACK (fused step with lists and surface tension): each neighbour's velocity, p/rho^2,
 * normal and 1/rho come from nrec as two adjacent float4 (one 32-byte sector) instead of
 * three separate loads; rho_j = 1/(1/rho_j) enters only the symmetrised surface-tension
 * factor 2 rho0 / (rho_i + rho_j) = 2 rho0 R_j / (rho_i R_j + 1). */
template <bool COMPAT, bool LIST, bool FUSE, bool WRITE_ACC, bool ST, bool BATCH, bool PACK = false>
__global__ void __launch_bounds__(256, SPH_FORCES_MIN_BLOCKS) k_wc_forces(Const c0, Neigh<LIST, COMPAT> fl0, Neigh<LIST, COMPAT> bl0, Bufs b) {
  for_each_particle<BATCH>(c0, b.tiles, b.scenes, b.tile_next + 3, [&](const Const& c, long long base, int i) {
    Neigh<LIST, COMPAT> fl = fl0, bl = bl0;
    fl.tab += base;
    bl.tab += base;
    const float4 pi = __ldg(&b.pos_s[i]);
    const float4 vi = __ldg(&b.vel_s[i]);
    const float4 ai = __ldg(&b.aux[i]);
    const float C = ai.x, di = ai.z;
    const float h = c.h, sg = c.spiky_grad;
    float bax = 0.f, bay = 0.f, baz = 0.f;
    auto boundary_pairs = [&]() {
        if (c.nb <= 0) return;
        const float c2 = 2.0f * C * sg;
        bl.visit(c, i, pi.x, pi.y, pi.z, [&](int j, float4, float dx, float dy, float dz) {
            const float r2 = dx * dx + dy * dy + dz * dz;
            const float irn = rsqrtf(r2);
            const float w = h - r2 * irn;
            const float k = -__ldg(&b.bphi_s[j]) * (irn * (w * w)) * c2;
            bax += dx * k;
            bay += dy * k;
            baz += dz * k;
        });
    };
    if (BATCH) boundary_pairs();
    float4 ni = make_float4(0.f, 0.f, 0.f, 0.f);
    if (ST) ni = __ldg(&b.normal[i]);
    float pax = 0.f, pay = 0.f, paz = 0.f, vax = 0.f, vay = 0.f, vaz = 0.f;
    float cux = 0.f, cuy = 0.f, cuz = 0.f, cox = 0.f, coy = 0.f, coz = 0.f;
    const float rmin2 = c.rmin2_wc, two_rho0 = 2.0f * c.rho0;
    /* the list walk SPH_FORCES_WALK (four) entries deep with the next entries loaded during
     * the visits and a predicated last batch, single-scene; the batched kernel walks two deep
     * with a serial tail (measured faster there) */
    fl.template visit<true, BATCH ? 2 : SPH_FORCES_WALK, !BATCH>(c, i, pi.x, pi.y, pi.z,
                                                                 [&](int j, float4, float dx, float dy, float dz) {
        const float r2 = dx * dx + dy * dy + dz * dz;
        /* loaded ahead of the guard so that the list loop can issue them early */
        float4 aj, vj, nj = make_float4(0.f, 0.f, 0.f, 0.f);
        if constexpr (PACK) {
            vj = __ldg(&b.nrec[2 * (size_t)j]);
            nj = __ldg(&b.nrec[2 * (size_t)j + 1]);
            aj = make_float4(vj.w, nj.w, 1.0f, 0.f);   /* (C_j, R_j, -, -); the guard uses R_j > 0 */
        } else {
            aj = __ldg(&b.aux[j]);
            vj = __ldg(&b.vel_s[j]);
            if (ST) nj = __ldg(&b.normal[j]);
        }
        const bool pos_j = PACK ? aj.y > 0.f : aj.z > 0.f;
        if (di > 0.f && pos_j && r2 > rmin2) {
            const float irn = rsqrtf(r2);
            const float rn = r2 * irn;
            const float w = h - rn;
            const float q = (sg * irn) * (w * w) * (C + aj.x);
            pax += dx * q;
            pay += dy * q;
            paz += dz * q;
            const float vw = w * aj.y;
            vax += (vj.x - vi.x) * vw;
            vay += (vj.y - vi.y) * vw;
            vaz += (vj.z - vi.z) * vw;
            if (ST) {
                const float K = PACK ? __fdividef(two_rho0 * aj.y, di * aj.y + 1.0f) : __fdividef(two_rho0, di + aj.z);
                cux += (ni.x - nj.x) * K;
                cuy += (ni.y - nj.y) * K;
                cuz += (ni.z - nj.z) * K;
                /* selects in the single-scene kernel (0.666 -> 0.636 ms), branches in the batched one */
                const float ck = (BATCH ? st_kernel(rn, h, c.st_term) : st_kernel_sel(rn, h, c.st_term)) * K * irn;
                cox += dx * ck;
                coy += dy * ck;
                coz += dz * ck;
            }
        }
    });
    /* single scene: the boundary pairs after the fluid pairs, so that their sums are not live
     * during the fluid walk (each term keeps its own accumulator, so the result is the same);
     * the batched kernel measured faster with them first (2.46 vs 2.59 ms per batched step) */
    if (!BATCH) boundary_pairs();
    const float m = c.mass;
    pax *= -m; pay *= -m; paz *= -m;
    const float vs = COMPAT ? (c.visc_lapl * c.mu) : (c.visc_lapl * c.mu) * (m * ai.y);
    vax *= vs; vay *= vs; vaz *= vs;
    float ax = pax + vax + bax, ay = c.g + pay + vay + bay, az = paz + vaz + baz;
    if (ST) {
        const float cs = COMPAT ? c.st_main : c.st_main * m;
        const float ns = -c.sigma;
        ax = (((ns * (cux + cox * cs)) + pax) + vax) + bax;
        ay = (((c.g + ns * (cuy + coy * cs)) + pay) + vay) + bay;
        az = (((ns * (cuz + coz * cs)) + paz) + vaz) + baz;
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
  });
}

__global__ void __launch_bounds__(256) k_wc_integrate(Const c0, Bufs b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c0.n) return;
    Const c = c0;
    scene_setup(c, b.scenes, b.scene_of, i);
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
/* grid of a launch: one particle per thread, or the persistent tile grid of a batched context */
template <bool BATCH>
static inline int grid_for(const Const& c, int bs) {
    if constexpr (BATCH) return c.tile_blocks > 0 ? c.tile_blocks : 1;
    return c.blocks > 0 ? c.blocks : nblk(c.n, bs);
}
/* a batched pass's tile counter, zeroed on the stream before its launch (slot: 0 density,
 * 1 list build, 2 normals, 3 forces) */
static unsigned* tile_counter(cudaStream_t s, const Bufs& b, int slot, bool batched) {
    if (!batched) return nullptr;
    cudaMemsetAsync(b.tile_next + slot, 0, sizeof(unsigned), s);
    return b.tile_next + slot;
}

template <bool LIST, bool EXACT>
static Neigh<LIST, EXACT> fluid_src(const Bufs& b) {
    return Neigh<LIST, EXACT>{b.tab, b.nlist, b.nlen, b.pos_s};
}
template <bool LIST, bool EXACT>
static Neigh<LIST, EXACT> bnd_src(const Bufs& b) {
    return Neigh<LIST, EXACT>{b.btab, b.sblist, b.sblen, b.bpos_s};
}

template <bool COMPAT, bool LIST, bool BATCH>
static void density_launch(cudaStream_t s, const Const& c, const Bufs& b, int bs) {
    unsigned* next = tile_counter(s, b, 0, BATCH);
    k_wc_density<COMPAT, LIST, BATCH><<<grid_for<BATCH>(c, bs), bs, 0, s>>>(c, fluid_src<LIST, COMPAT>(b),
                                                                   bnd_src<LIST, COMPAT>(b), b.bphi_s, b.density,
                                                                   b.pressure, b.aux, b.scenes, b.tiles, next);
}

/* Batched contexts exist only in PHYSICS mode, so the scene lookup is compiled for that mode alone. */
template <bool COMPAT, bool LIST>
static void density_dispatch(cudaStream_t s, const Const& c, const Bufs& b, int bs) {
    if constexpr (!COMPAT) {
        if (c.batched) { density_launch<false, LIST, true>(s, c, b, bs); return; }
    }
    density_launch<COMPAT, LIST, false>(s, c, b, bs);
}

void launch_wc_density(cudaStream_t s, const Const& c, const Bufs& b, bool lists, int bs) {
    if (c.n <= 0) return;
    if (c.compat) {
        if (lists) density_dispatch<true, true>(s, c, b, bs);
        else density_dispatch<true, false>(s, c, b, bs);
    } else {
        if (lists) density_dispatch<false, true>(s, c, b, bs);
        else density_dispatch<false, false>(s, c, b, bs);
    }
}

template <bool COMPAT, bool BATCH>
static void lists_density_launch(cudaStream_t s, const Const& c, const Bufs& b, int bs) {
    unsigned* next = tile_counter(s, b, 1, BATCH);
    k_lists_density<COMPAT, BATCH><<<grid_for<BATCH>(c, bs), bs, 0, s>>>(c, b.pos_s, b.tab, b.bpos_s, b.btab,
                                                                b.bphi_s, b.nlist, b.nlen, b.sblist, b.sblen,
                                                                b.density, b.pressure, b.aux, b.scenes, b.tiles,
                                                                next, nullptr, nullptr, b.bnear, b.noff, b.prho);
}

void launch_lists_density_pci(cudaStream_t s, const Const& c, const Bufs& b, int bs) {
    if (c.n <= 0) return;
    k_lists_density<false, false, false, true><<<nblk(c.n, bs), bs, 0, s>>>(
        c, b.pos_s, b.tab, b.bpos_s, b.btab, b.bphi_s, b.nlist, b.nlen, b.sblist, b.sblen, b.density, b.pressure,
        b.aux, b.scenes, b.tiles, nullptr, nullptr, nullptr, b.bnear, b.noff, b.prho);
}
void launch_lists_density_remap(cudaStream_t s, const Const& c, const Bufs& b, const int32_t* remap, int bs) {
    if (c.n <= 0) return;
    k_lists_density<false, false, true><<<nblk(c.n, bs), bs, 0, s>>>(
        c, b.pos_s, b.tab, b.bpos_s, b.btab, b.bphi_s, b.nlist, b.nlen, b.sblist, b.sblen, b.density, b.pressure,
        b.aux, b.scenes, b.tiles, nullptr, remap, b.flags);
}

void launch_lists_density(cudaStream_t s, const Const& c, const Bufs& b, int bs) {
    if (c.n <= 0) return;
    if (c.compat) lists_density_launch<true, false>(s, c, b, bs);
    else if (c.batched) lists_density_launch<false, true>(s, c, b, bs);
    else lists_density_launch<false, false>(s, c, b, bs);
}

void launch_aux(cudaStream_t s, const Const& c, const Bufs& b, int bs) {
    if (c.n <= 0) return;
    k_aux<<<nblk(c.n, bs), bs, 0, s>>>(c.n, b.density, b.pressure, b.aux);
}

void launch_normals(cudaStream_t s, const Const& c, const Bufs& b, bool lists, int bs, bool pack, bool prho) {
    if (c.n <= 0) return;
    const int g = nblk(c.n, bs), gt = grid_for<true>(c, bs);
    float4* nrec = pack ? b.nrec : nullptr;
    unsigned* next = tile_counter(s, b, 2, c.batched != 0);
    if (c.monaghan) {   /* COMPAT only */
        if (lists)
            k_normals<true, true, false, true><<<g, bs, 0, s>>>(c, fluid_src<true, true>(b), b.aux, b.density,
                                                                b.normal, b.scenes, b.tiles, next, b.vel_s, nrec);
        else
            k_normals<false, true, false, true><<<g, bs, 0, s>>>(c, fluid_src<false, true>(b), b.aux, b.density,
                                                                 b.normal, b.scenes, b.tiles, next);
        return;
    }
    if (lists) {
        auto fl = fluid_src<true, true>(b);
        if (prho) fl.npos = b.prho;
        if (c.batched) {
            if (prho)
                k_normals<true, true, true, false, true><<<gt, bs, 0, s>>>(c, fl, b.aux, b.density, b.normal,
                                                                         b.scenes, b.tiles, next, b.vel_s, nrec);
            else
                k_normals<true, true, true><<<gt, bs, 0, s>>>(c, fl, b.aux, b.density, b.normal, b.scenes, b.tiles,
                                                              next, b.vel_s, nrec);
        } else {
            if (prho)
                k_normals<true, true, false, false, true><<<g, bs, 0, s>>>(c, fl, b.aux, b.density, b.normal,
                                                                          b.scenes, b.tiles, next, b.vel_s, nrec);
            else
                k_normals<true, true, false><<<g, bs, 0, s>>>(c, fl, b.aux, b.density, b.normal, b.scenes, b.tiles,
                                                              next, b.vel_s, nrec);
        }
    } else if (c.compat) {
        k_normals<false, true, false><<<g, bs, 0, s>>>(c, fluid_src<false, true>(b), b.aux, b.density, b.normal,
                                                       b.scenes, b.tiles, next);
    } else if (c.batched) {
        k_normals<false, false, true><<<gt, bs, 0, s>>>(c, fluid_src<false, false>(b), b.aux, b.density, b.normal,
                                                        b.scenes, b.tiles, next);
    } else {
        k_normals<false, false, false><<<g, bs, 0, s>>>(c, fluid_src<false, false>(b), b.aux, b.density, b.normal,
                                                        b.scenes, b.tiles, next);
    }
}

template <bool COMPAT, bool LIST, bool BATCH>
static void forces_launch(cudaStream_t s, const Const& c, const Bufs& b, bool fuse, bool write_acc, int bs,
                          bool pack) {
    const int g = grid_for<BATCH>(c, bs);
    tile_counter(s, b, 3, BATCH);
    const bool st = c.sigma != 0.f;
    auto fs = fluid_src<LIST, COMPAT>(b);
    auto bsrc = bnd_src<LIST, COMPAT>(b);
    if constexpr (LIST) {
        if (pack && st && fuse && !write_acc) {
            k_wc_forces<COMPAT, LIST, true, false, true, BATCH, true><<<g, bs, 0, s>>>(c, fs, bsrc, b);
            return;
        }
    }
#define SPH_WCF(F, W, S) k_wc_forces<COMPAT, LIST, F, W, S, BATCH><<<g, bs, 0, s>>>(c, fs, bsrc, b)
    if (fuse) {
        if (write_acc) { if (st) SPH_WCF(true, true, true); else SPH_WCF(true, true, false); }
        else { if (st) SPH_WCF(true, false, true); else SPH_WCF(true, false, false); }
    } else {
        if (st) SPH_WCF(false, true, true); else SPH_WCF(false, true, false);
    }
#undef SPH_WCF
}

template <bool COMPAT, bool LIST>
static void forces_dispatch(cudaStream_t s, const Const& c, const Bufs& b, bool fuse, bool write_acc, int bs,
                            bool pack) {
    if constexpr (!COMPAT) {
        if (c.batched) { forces_launch<false, LIST, true>(s, c, b, fuse, write_acc, bs, pack); return; }
    }
    forces_launch<COMPAT, LIST, false>(s, c, b, fuse, write_acc, bs, pack);
}

void launch_wc_forces(cudaStream_t s, const Const& c, const Bufs& b, bool lists, bool fuse_integrate,
                      bool write_acc, int bs, bool pack) {
    if (c.n <= 0) return;
    if (c.compat) {
        if (lists) forces_dispatch<true, true>(s, c, b, fuse_integrate, write_acc, bs, pack);
        else forces_dispatch<true, false>(s, c, b, fuse_integrate, write_acc, bs, pack);
    } else {
        if (lists) forces_dispatch<false, true>(s, c, b, fuse_integrate, write_acc, bs, pack);
        else forces_dispatch<false, false>(s, c, b, fuse_integrate, write_acc, bs, pack);
    }
}

void launch_wc_integrate(cudaStream_t s, const Const& c, const Bufs& b, int bs) {
    if (c.n <= 0) return;
    k_wc_integrate<<<nblk(c.n, bs), bs, 0, s>>>(c, b);
}

}  // namespace sph
