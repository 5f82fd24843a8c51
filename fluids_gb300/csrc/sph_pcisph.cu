/*
 * sph_pcisph.cu -- PCISPH passes (kernels/pcisph.cl) over the materialised neighbour lists.
 *
 *   k_pci_init_density  fill p = 0 (pcisphsimluation.cpp:118) + compute_initial_density
 *                       (pcisph.cl:33-102)
 *   k_pci_init_forces   fill F_p = 0 (pcisphsimluation.cpp:126) + compute_initial_forces
 *                       (pcisph.cl:134-222): viscosity + Akinci surface tension
 *   k_pci_loop          the whole predict-correct loop of pcisphsimluation.cpp:129-148 in ONE
 *                       persistent cooperative kernel: predict_pos (pcisph.cl:302-344),
 *                       update_pressure (:349-418) with a fused block max of the density
 *                       error (replacing clmax, clreduce.h:54-62, and its blocking read per
 *                       iteration), compute_pressure_force (:420-504).  The stop test runs on
 *                       the device after a grid barrier, so no host round trip per iteration.
 *                       Optionally the final predict_vel_n_pos (:240-284) is fused after it.
 *   k_pci_integrate     predict_vel_n_pos (pcisph.cl:240-284)
 * The grid barrier spins on a generation counter with a bounded poll count (2^24 polls of at
 * least 64 ns); on timeout the kernel sets SPH_FLAG_TIMEOUT and every CTA returns (the launch
 * is cooperative, so all CTAs are co-resident and the wait ends in practice).  The test of
 * that path injects a stall from the host (sph_inject_fault) instead of faulting anything.
 */
#include "sph_kernels.cuh"

namespace sph {

namespace {
constexpr long long kBarrierSpinLimit = 1LL << 24;

/* Grid-wide barrier: bar[0] = arrivals, bar[1] = generation.  Returns false on timeout.
 * extra > 0 (an injected stall) waits for arrivals that never come, so every CTA's bounded
 * wait runs out. */
__device__ __forceinline__ bool grid_barrier(unsigned* bar, unsigned* flags, unsigned extra) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* vgen = bar + 1;
        const unsigned gen = *vgen;
        __threadfence();
        const unsigned arrived = atomicAdd(bar, 1u);
        int ok = 1;
        if (arrived == gridDim.x - 1 + extra) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            long long spins = 0;
            while (*vgen == gen) {
                if (++spins > kBarrierSpinLimit) {
                    atomicOr(flags, kFlagTimeout);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

__device__ __forceinline__ float block_max(float v) {
    __shared__ float s_w[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) s_w[w] = v;
    __syncthreads();
    if (w == 0) {
        v = lane < (int)(blockDim.x >> 5) ? s_w[lane] : 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    }
    return v;
}

/* container clamp of both PCISPH integrators */
__device__ __forceinline__ void pci_advance(const Const& c, float4 p, float4 v, float4 fo, float4 fp, float& px,
                                            float& py, float& pz, float& vx, float& vy, float& vz, float& cx,
                                            float& cy, float& cz, float& d, float& vn) {
    const float md = c.mass_def, dt = c.dt, vm = c.vmax;
    const float ax = (fp.x + fo.x) / md, ay = c.g + (fp.y + fo.y) / md, az = (fp.z + fo.z) / md;
    vx = v.x + clampf(ax * dt, -vm, vm);
    vy = v.y + clampf(ay * dt, -vm, vm);
    vz = v.z + clampf(az * dt, -vm, vm);
    px = p.x + vx * dt;
    py = p.y + vy * dt;
    pz = p.z + vz * dt;
    vn = len3(vx, vy, vz);
    cx = clampf(px, (-c.lim_x) / 2.0f, c.lim_x / 2.0f);
    cy = clampf(py, (-c.lim_y) / 2.0f, 10.0f);
    cz = clampf(pz, (-c.lim_z) / 2.0f, c.lim_z / 2.0f);
    d = len3(cx - px, cy - py, cz - pz);
}

__device__ __forceinline__ void pci_predict_one(const Const& c, const Bufs& b, int i) {
    float px, py, pz, vx, vy, vz, cx, cy, cz, d, vn;
    pci_advance(c, __ldg(&b.pos_s[i]), __ldg(&b.vel_s[i]), b.f_other[i], b.f_press[i], px, py, pz, vx, vy, vz, cx,
                cy, cz, d, vn);
    if (d > 0.f && vn > 0.f) { px = cx; py = cy; pz = cz; }
    b.pos_pred[i] = make_float4(px, py, pz, 1.f);
}

__device__ __forceinline__ void pci_integrate_one(const Const& c, const Bufs& b, int i) {
    float px, py, pz, vx, vy, vz, cx, cy, cz, d, vn;
    pci_advance(c, __ldg(&b.pos_s[i]), __ldg(&b.vel_s[i]), b.f_other[i], b.f_press[i], px, py, pz, vx, vy, vz, cx,
                cy, cz, d, vn);
    if (d > 0.f && vn > 0.f) {
        float sx = signf(cx - px), sy = signf(cy - py), sz = signf(cz - pz);
        const float sl = len3(sx, sy, sz);
        sx /= sl; sy /= sl; sz /= sl;
        const float rest = d / (c.dt * vn);
        const float k = (1.0f + rest) * (vx * sx + vy * sy + vz * sz);
        vx -= k * sx; vy -= k * sy; vz -= k * sz;
        px = cx; py = cy; pz = cz;
    }
    b.pos[i] = make_float4(px, py, pz, 1.f);
    b.vel[i] = make_float4(vx, vy, vz, 0.f);
    b.ids[i] = b.ids_s[i];
    const bool bad = !(isfinite(px) && isfinite(py) && isfinite(pz) && isfinite(vx) && isfinite(vy) && isfinite(vz));
    if (bad) atomicOr(b.flags, kFlagNan);
}

/* update_pressure for one particle: predicted density from the fixed lists at x*.  The
 * list is walked two entries deep with the next two entries loaded during the current two
 * visits (the sum keeps list order).  x* is written by this kernel, so it is read with plain loads.
 * The updated pressure's p / rho^2 (the initial density, as compute_pressure_force uses it)
 * goes to pci_c for the force phase: the same IEEE quotient the force phase would form per
 * pair, formed once per particle. */
/* Visits list entries [0, len) of row e (stride n) in list order, loading the data of D
 * entries (load(j)) before their D visits and the next D entries' indices during them: the
 * walks of the loop are bound by the latency of these dependent loads.  Four deep, measured
 * on GB300: the 4M PCISPH step 6.35 ms against 7.20 ms two deep (the 358k step 0.620 against
 * 0.618 ms); three deep 6.58 ms. */
#ifndef SPH_PCI_WALK_DEPTH
#define SPH_PCI_WALK_DEPTH 4
#endif
template <int D, class L, class V>
__device__ __forceinline__ void walk_list(const int* __restrict__ e, size_t n, int len, int self, L&& load,
                                          V&& visit) {
    /* batches of D entries; a last, partial batch loads its missing entries as the particle
     * itself (a valid index) and does not visit them */
    int jn[D];
#pragma unroll
    for (int u = 0; u < D; ++u) jn[u] = u < len ? __ldg(e + u * n) : self;
#pragma unroll 1
    for (int k = 0; k < len; k += D) {
        decltype(load(0)) q[D];
#pragma unroll
        for (int u = 0; u < D; ++u) q[u] = load(jn[u]);
        e += D * n;
#pragma unroll
        for (int u = 0; u < D; ++u) jn[u] = k + D + u < len ? __ldg(e + u * n) : self;
#pragma unroll
        for (int u = 0; u < D; ++u)
            if (k + u < len) visit(q[u]);
    }
}
template <bool COMPAT>
__device__ __forceinline__ float pci_update_one(const Const& c, const Bufs& b, int i) {
    const float4 pi = b.pos_pred[i];
    const float H = c.h_def, HH = H * H;
    const size_t n = (size_t)c.n;
    float pd = 0.f, pdb = 0.f;
    const int len = __ldg(&b.nlen[i]);
    const int* __restrict__ e = b.nlist + i;
    /* every product and sum rounded on its own, in the kernel's order (r^2 as dot(r, r),
     * pown(h^2 - r^2, 3), the sum in list order): the result does not depend on how the
     * compiler would contract them */
    auto visit = [&](float4 pj) {
        const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
        const float r2 = r2_exact(dx, dy, dz);
        /* the range test as a select: a rejected pair adds +0 */
        if (COMPAT && c.monaghan) {
            pd += w_monaghan(r2, H, H);   /* W_DEFAULT(r^2, h), Monaghan kernels (pcisph.cl:396) */
        } else {
            const float t = (COMPAT || r2 < HH) ? HH - r2 : 0.f;
            pd = __fadd_rn(pd, __fmul_rn(__fmul_rn(t, t), t));
        }
    };
    walk_list<SPH_PCI_WALK_DEPTH>(e, n, len, i, [&](int j) { return b.pos_pred[j]; }, visit);
    pd *= c.default_eval * c.mass_def;
    const int blen = __ldg(&b.sblen[i]);
    for (int k = 0; k < blen; ++k) {
        const int j = __ldg(&b.sblist[k * n + i]);
        const float4 pj = __ldg(&b.bpos_s[j]);
        const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
        const float r2 = r2_exact(dx, dy, dz);
        if (COMPAT && c.monaghan) {
            pdb += w_monaghan(r2, H, H) * __ldg(&b.bphi_s[j]);
        } else if (COMPAT || r2 < HH) {
            const float t = HH - r2;
            pdb = __fadd_rn(pdb, __fmul_rn(__fmul_rn(__fmul_rn(t, t), t), __ldg(&b.bphi_s[j])));
        }
    }
    pdb *= c.default_eval;
    const float e0 = pd + pdb - c.rho0_def;
    const float dv = (0.f < e0) ? e0 : 0.f;
    b.dens_var[i] = dv;
    const float p = __fadd_rn(b.pressure[i], __fmul_rn(dv, c.delta));
    b.pressure[i] = p;
    const float di = __ldg(&b.density[i]);
    const float q = p / (di * di);
    b.pci_c[i] = q;
    const float4 ps = __ldg(&b.pos_s[i]);
    b.pci_pc[i] = make_float4(ps.x, ps.y, ps.z, q);   /* one record per neighbour for the force phase */
    return dv;
}

/* compute_pressure_force for one particle (initial density, updated pressure):
 * (p_i / rho_i^2 + p_j / rho_j^2) per pair with the quotients of pci_c; each neighbour's
 * position and quotient come as one record from pci_pc (both written by the update phase
 * of this kernel, so plain loads). */
template <bool MON = false>
__device__ __forceinline__ void pci_pressure_force_one(const Const& c, const Bufs& b, int i) {
    const float4 pi = __ldg(&b.pos_s[i]);
    const float H = c.h_def;
    const size_t n = (size_t)c.n;
    const float C = b.pci_c[i];
    float fx = 0.f, fy = 0.f, fz = 0.f, gx = 0.f, gy = 0.f, gz = 0.f;
    const int len = __ldg(&b.nlen[i]);
    const int* __restrict__ e = b.nlist + i;
    auto visit = [&](float4 pj, float cj) {
        const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
        const float r2 = dx * dx + dy * dy + dz * dz;
        if constexpr (MON) {   /* GRAD_W_PRESSURE(r, l, h) with the Monaghan kernels (pcisph.cl:482) */
            const float l = sqrtf(r2);
            if (l >= 1e-5f) {
                float gx, gy, gz;
                grad_w_monaghan(dx, dy, dz, l, H, H, gx, gy, gz);
                const float q = C + cj;
                fx += q * gx;
                fy += q * gy;
                fz += q * gz;
            }
            return;
        }
        const float il0 = rsqrtf(r2), l0 = r2 * il0;
        /* the distance guard as selects: a rejected pair (the particle itself) adds zeros */
        const bool ok = l0 >= 1e-5f;
        const float il = ok ? il0 : 0.f, l = ok ? l0 : H;
        const float q = C + cj;
        const float t = (H - l) * (H - l);
        fx += q * ((dx * il) * t);
        fy += q * ((dy * il) * t);
        fz += q * ((dz * il) * t);
    };
    walk_list<SPH_PCI_WALK_DEPTH>(e, n, len, i, [&](int j) { return b.pci_pc[j]; },
                                  [&](const float4& v) { visit(v, v.w); });
    const float sf = (-(c.mass_def * c.mass_def)) * c.spiky_grad;
    fx *= sf; fy *= sf; fz *= sf;
    const int blen = __ldg(&b.sblen[i]);
    for (int k = 0; k < blen; ++k) {
        const int j = __ldg(&b.sblist[k * n + i]);
        const float4 pj = __ldg(&b.bpos_s[j]);
        const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
        const float l = sqrtf(dx * dx + dy * dy + dz * dz);
        const float q = __ldg(&b.bphi_s[j]) * (2.0f * C);
        if constexpr (MON) {
            float wx, wy, wz;
            grad_w_monaghan(dx, dy, dz, l, H, H, wx, wy, wz);
            gx += q * wx;
            gy += q * wy;
            gz += q * wz;
            continue;
        }
        const float il = 1.0f / l, t = (H - l) * (H - l);
        gx += q * ((dx * il) * t);
        gy += q * ((dy * il) * t);
        gz += q * ((dz * il) * t);
    }
    const float sb = (-c.mass_def) * c.spiky_grad;
    b.f_press[i] = make_float4(fx + gx * sb, fy + gy * sb, fz + gz * sb, 0.f);
}
}  // namespace

template <bool COMPAT>
__global__ void __launch_bounds__(256) k_pci_init_density(Const c, Bufs b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    b.pressure[i] = 0.f;
    const float4 pi = __ldg(&b.pos_s[i]);
    const float H = c.h_def, HH = H * H;
    float di = 0.f, bdi = 0.f;
    list_neighbors<2, true>(i, c.n, b.nlist, __ldg(&b.nlen[i]), b.pos_s, pi.x, pi.y, pi.z,
                   [&](int, float4, float dx, float dy, float dz) {
                       const float r2 = dx * dx + dy * dy + dz * dz;
                       if (COMPAT && c.monaghan) {   /* W_DEFAULT(r^2, h), Monaghan (pcisph.cl:81) */
                           di += w_monaghan(r2, H, H);
                       } else {
                           const float t = HH - r2;
                           di += (t * t) * t;
                       }
                   });
    list_neighbors(i, c.n, b.sblist, __ldg(&b.sblen[i]), b.bpos_s, pi.x, pi.y, pi.z,
                   [&](int j, float4, float dx, float dy, float dz) {
                       const float r2 = dx * dx + dy * dy + dz * dz;
                       if (COMPAT && c.monaghan) {
                           bdi += w_monaghan(r2, H, H) * __ldg(&b.bphi_s[j]);
                       } else {
                           const float t = HH - r2;
                           bdi += ((t * t) * t) * __ldg(&b.bphi_s[j]);
                       }
                   });
    const float d = c.default_eval * ((di * c.mass_def) + bdi);
    b.density[i] = d;
    b.aux[i] = make_float4(0.f, 1.0f / d, d, 0.f);
}

/* PACK (surface tension on, the normal pass wrote nrec): each neighbour's velocity, normal
 * and 1/rho come from nrec as two adjacent float4 (one 32-byte sector) instead of three
 * loads, and the pair terms use the forms of the WCSPH force pass: 1/r from rsqrtf,
 * (h - r) / rho_j as (h - r) * (1/rho_j), and 2 rho0 / (rho_i + rho_j) as
 * 2 rho0 R_j / (rho_i R_j + 1) with a fast division (FP32 results within a few ulp of the
 * IEEE forms).  Without PACK the pair terms are the kernel text's IEEE divisions. */
/* MON: LAPL_W_VISCOSITY(r, h) with the Monaghan kernels (pcisph.cl:208) instead of h - r. */
/* the walk two deep with the next entries loaded during the visits and a predicated last
 * batch: 4M 0.587 -> 0.557 ms, 358k 0.074 -> 0.066 ms against four deep without them */
#ifndef SPH_PCI_INIT_U
#define SPH_PCI_INIT_U 2
#endif
#ifndef SPH_PCI_INIT_PIPE
#define SPH_PCI_INIT_PIPE 1
#endif
template <bool PACK, bool MON = false>
__global__ void __launch_bounds__(256) k_pci_init_forces(Const c, Bufs b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    b.f_press[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 pi = __ldg(&b.pos_s[i]), vi = __ldg(&b.vel_s[i]), ni = __ldg(&b.normal[i]);
    const float di = __ldg(&b.density[i]);
    const float H = c.h_def;
    const float two_rho0 = 2.0f * c.rho0_def;
    float vx = 0.f, vy = 0.f, vz = 0.f, ux = 0.f, uy = 0.f, uz = 0.f, ox = 0.f, oy = 0.f, oz = 0.f;
    list_neighbors<SPH_PCI_INIT_U, SPH_PCI_INIT_PIPE, SPH_PCI_INIT_PIPE>(i, c.n, b.nlist, __ldg(&b.nlen[i]), b.pos_s,
                                                                       pi.x, pi.y, pi.z,
                   [&](int j, float4, float dx, float dy, float dz) {
                       float4 vj, nj;
                       float rn, inv, w, K;
                       const float r2 = dx * dx + dy * dy + dz * dz;
                       if constexpr (PACK) {
                           vj = __ldg(&b.nrec[2 * (size_t)j]);
                           nj = __ldg(&b.nrec[2 * (size_t)j + 1]);
                           const float Rj = nj.w;
                           inv = r2 > 0.f ? rsqrtf(r2) : 0.f;
                           rn = r2 * inv;
                           if constexpr (MON) rn = sqrtf(r2);
                           w = (MON ? lapl_w_monaghan(rn, H, H) : H - rn) * Rj;
                           K = __fdividef(two_rho0 * Rj, di * Rj + 1.0f);
                       } else {
                           vj = __ldg(&b.vel_s[j]);
                           nj = __ldg(&b.normal[j]);
                           const float dj = __ldg(&b.density[j]);
                           rn = sqrtf(r2);
                           w = (MON ? lapl_w_monaghan(rn, H, H) : H - rn) / dj;
                           K = st_corr(c.rho0_def, di, dj);
                           inv = rn > 0.f ? 1.0f / rn : 0.f;
                       }
                       vx += (vj.x - vi.x) * w;
                       vy += (vj.y - vi.y) * w;
                       vz += (vj.z - vi.z) * w;
                       ux += (ni.x - nj.x) * K;
                       uy += (ni.y - nj.y) * K;
                       uz += (ni.z - nj.z) * K;
                       const float sk = st_kernel_sel(rn, H, c.st_term);
                       ox += ((dx * inv) * sk) * K;
                       oy += ((dy * inv) * sk) * K;
                       oz += ((dz * inv) * sk) * K;
                   });
    const float md = c.mass_def;
    const float vsc = (c.mu * (md * md)) * (c.visc_lapl / di);
    const float csc = md * c.st_main;
    const float tsc = (-c.sigma) * md;
    b.f_other[i] = make_float4(vx * vsc + tsc * (ux + ox * csc), vy * vsc + tsc * (uy + oy * csc),
                               vz * vsc + tsc * (uz + oz * csc), 0.f);
}

/* 5 blocks/SM (at most 51 registers, a few bytes of spill): 6.7 ms per 4M-particle step vs
 * 7.2 ms at the unbounded 60 registers (4 blocks/SM), measured on GB300. */
#ifndef SPH_PCI_LOOP_MIN_BLOCKS
#define SPH_PCI_LOOP_MIN_BLOCKS 5
#endif
/* the loop's own block size, whatever the context's: measured on GB300, 256 threads at 5
 * blocks/SM 0.623 ms per 358k step and 6.35 ms per 4M step, against 0.651 / 6.79 ms with
 * 512 x 2, 0.648 / 6.77 ms with 1024 x 1 and 0.659 / 6.80 ms with 256 x 4 */
#ifndef SPH_PCI_LOOP_THREADS
#define SPH_PCI_LOOP_THREADS 256
#endif
constexpr int kLoopThreads = SPH_PCI_LOOP_THREADS;
template <bool COMPAT, bool FUSE_INTEGRATE>
__global__ void __launch_bounds__(kLoopThreads, SPH_PCI_LOOP_MIN_BLOCKS) k_pci_loop(Const c, Bufs b, int min_iter, int max_iter) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int stride = gridDim.x * blockDim.x;
    const int n = c.n;
    int it = 1;
    for (; it <= max_iter; ++it) {
        for (int i = tid; i < n; i += stride) pci_predict_one(c, b, i);
        if (!grid_barrier(b.barrier, b.flags, (unsigned)c.barrier_extra)) return;
        float lmax = 0.f;
        for (int i = tid; i < n; i += stride) lmax = fmaxf(lmax, pci_update_one<COMPAT>(c, b, i));
        lmax = block_max(lmax);
        if (threadIdx.x == 0) atomicMax(reinterpret_cast<unsigned*>(&b.pci_maxerr[it - 1]), __float_as_uint(lmax));
        if (!grid_barrier(b.barrier, b.flags, (unsigned)c.barrier_extra)) return;
        const float mx = *reinterpret_cast<volatile float*>(&b.pci_maxerr[it - 1]);
        if (COMPAT && c.monaghan) {
            for (int i = tid; i < n; i += stride) pci_pressure_force_one<true>(c, b, i);
        } else {
            for (int i = tid; i < n; i += stride) pci_pressure_force_one(c, b, i);
        }
        bool stop = false;
        if (it >= min_iter) {
            const float crit = COMPAT ? (mx - c.rho0) / c.rho0 : mx / c.rho0;
            stop = crit < c.pci_eta;
        }
        if (stop) break;
    }
    if (tid == 0) {
        b.pci_iters[0] = it > max_iter ? max_iter : it;
        if (it > max_iter && !COMPAT) atomicOr(b.flags, kFlagNonconverged);
    }
    if (FUSE_INTEGRATE) {
        for (int i = tid; i < n; i += stride) pci_integrate_one(c, b, i);
    }
}

__global__ void __launch_bounds__(256) k_pci_integrate(Const c, Bufs b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    pci_integrate_one(c, b, i);
}

/* The loop's three passes as separate launches, for stage-by-stage parity on fields set
 * from outside: the same per-particle functions as k_pci_loop. */
__global__ void __launch_bounds__(256) k_pci_predict(Const c, Bufs b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < c.n) pci_predict_one(c, b, i);
}

template <bool COMPAT>
__global__ void __launch_bounds__(256) k_pci_update_pressure(Const c, Bufs b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < c.n) pci_update_one<COMPAT>(c, b, i);
}

/* p / rho^2 of every particle from the pressure and density fields as they stand (the
 * update pass forms it as a by-product in the loop). */
__global__ void __launch_bounds__(256) k_pci_quotient(Const c, Bufs b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const float di = b.density[i];
    const float q = b.pressure[i] / (di * di);
    b.pci_c[i] = q;
    const float4 ps = __ldg(&b.pos_s[i]);
    b.pci_pc[i] = make_float4(ps.x, ps.y, ps.z, q);
}

__global__ void __launch_bounds__(256) k_pci_pressure_force(Const c, Bufs b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    if (c.monaghan) pci_pressure_force_one<true>(c, b, i);
    else pci_pressure_force_one(c, b, i);
}

static inline int nblk(int n, int bs) { return (n + bs - 1) / bs; }

void launch_pci_predict(cudaStream_t s, const Const& c, const Bufs& b, int bs) {
    if (c.n <= 0) return;
    k_pci_predict<<<nblk(c.n, bs), bs, 0, s>>>(c, b);
}
void launch_pci_update_pressure(cudaStream_t s, const Const& c, const Bufs& b, int bs) {
    if (c.n <= 0) return;
    if (c.compat) k_pci_update_pressure<true><<<nblk(c.n, bs), bs, 0, s>>>(c, b);
    else k_pci_update_pressure<false><<<nblk(c.n, bs), bs, 0, s>>>(c, b);
}
void launch_pci_pressure_force(cudaStream_t s, const Const& c, const Bufs& b, int bs) {
    if (c.n <= 0) return;
    k_pci_quotient<<<nblk(c.n, bs), bs, 0, s>>>(c, b);
    k_pci_pressure_force<<<nblk(c.n, bs), bs, 0, s>>>(c, b);
}

void launch_pci_init_density(cudaStream_t s, const Const& c, const Bufs& b, int bs) {
    if (c.n <= 0) return;
    if (c.compat) k_pci_init_density<true><<<nblk(c.n, bs), bs, 0, s>>>(c, b);
    else k_pci_init_density<false><<<nblk(c.n, bs), bs, 0, s>>>(c, b);
}
void launch_pci_init_forces(cudaStream_t s, const Const& c, const Bufs& b, int bs, bool pack) {
    if (c.n <= 0) return;
    if (c.monaghan) {
        if (pack) k_pci_init_forces<true, true><<<nblk(c.n, bs), bs, 0, s>>>(c, b);
        else k_pci_init_forces<false, true><<<nblk(c.n, bs), bs, 0, s>>>(c, b);
        return;
    }
    if (pack) k_pci_init_forces<true><<<nblk(c.n, bs), bs, 0, s>>>(c, b);
    else k_pci_init_forces<false><<<nblk(c.n, bs), bs, 0, s>>>(c, b);
}

static void* loop_fn(bool compat, bool fuse) {
    if (compat) return fuse ? (void*)k_pci_loop<true, true> : (void*)k_pci_loop<true, false>;
    return fuse ? (void*)k_pci_loop<false, true> : (void*)k_pci_loop<false, false>;
}

int pci_loop_blocks(int num_sms, int bs) {
    (void)bs;   /* the loop runs with its own block size */
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pci_loop<false, true>, kLoopThreads, 0);
    int per_sm2 = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm2, k_pci_loop<true, false>, kLoopThreads, 0);
    per_sm = per_sm < per_sm2 ? per_sm : per_sm2;
    if (per_sm < 1) per_sm = 1;
    return per_sm * num_sms;
}

cudaError_t launch_pci_loop(cudaStream_t s, const Const& c, const Bufs& b, int min_iter, int max_iter, int blocks,
                            int bs, bool fuse) {
    if (c.n <= 0) return cudaSuccess;
    (void)bs;
    int need = nblk(c.n, kLoopThreads);
    if (blocks > need) blocks = need;
    if (blocks < 1) blocks = 1;
    Const cc = c;
    Bufs bb = b;
    int mi = min_iter, ma = max_iter;
    void* args[] = {&cc, &bb, &mi, &ma};
    return cudaLaunchCooperativeKernel(loop_fn(c.compat != 0, fuse), dim3(blocks), dim3(kLoopThreads), args, 0, s);
}

void launch_pci_integrate(cudaStream_t s, const Const& c, const Bufs& b, int bs) {
    if (c.n <= 0) return;
    k_pci_integrate<<<nblk(c.n, bs), bs, 0, s>>>(c, b);
}

}  // namespace sph
