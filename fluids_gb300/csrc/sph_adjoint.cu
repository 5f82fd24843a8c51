/*
 * sph_adjoint.cu -- differentiable WCSPH (PHYSICS mode): gradients of a loss on the final
 * particle state with respect to the viscosity mu, the Tait stiffness k (and so c0, with
 * k = rho0 c0^2 / 7) and the initial positions and velocities.
 *
 * The reference has no gradients; the forward step here is its WCSPH step
 * (WCSPHSimulation::simulate, fluid/simulation/wcsphsimluation.cpp:40-106, with the PHYSICS
 * corrections) run by the same kernels as the plain solver, with one difference of
 * bookkeeping: the state stays in particle-id order.  Each step bins and sorts a copy of
 * the positions as usual, and the list builder writes every neighbour list, density and
 * pressure under the particle's id (k_lists_density<..., REMAP>), so the list order and
 * the arithmetic are the plain solver's and the force/integrate kernel is the plain one.
 *
 * Reverse mode, per step (state x, v, u = half-step velocity; a = acceleration):
 *   integrate   u' = u + dt a,  x' = x + dt clamp(u' + dt a),  v' = clamp(u' + dt a / 2)
 *   forces      a_i = g + sum_j P_ij + V_ij over the step's (fixed) list, with
 *               P_ij = -m sg (h - r)^2 / r (C_i + C_j) d_ij,  C = p / rho^2,
 *               V_ij = K R_i R_j (h - r)(v_j - v_i),  R = 1 / rho,  K = visc_lapl mu m
 *   density     rho_i = poly6 m sum_j (h^2 - r^2)^3,  p = max(0, k((rho/rho0)^7 - 1))
 * Every pair term is antisymmetric in (i, j) and the lists are symmetric (r^2 < h^2 is the
 * same test both ways, as long as no list reached the cap), so each backward pass is a
 * gather over particle i's own list with D = lambda_a_i - lambda_a_j: deterministic, no
 * atomics.  A list at the cap raises SPH_FLAG_OVERFLOW: its truncation breaks the symmetry.
 *
 * Non-smooth points (documented subgradients): the Tait clamp max(0, .) has derivative 0
 * where the pressure is clamped; each velocity clamp has derivative 1 strictly inside
 * (-vmax, vmax) and 0 outside; the container reflection is not differentiated (the
 * gradient passes as if no wall were there).  A clamp or reflection that was active in a
 * taped step raises SPH_FLAG_NONSMOOTH, so a caller knows the gradient crossed one.
 *
 * Memory: checkpoints of (x, v, u) every `checkpoint_every` steps; the backward pass
 * recomputes one segment at a time from its checkpoint and tapes that segment's states,
 * lists, aux (C, 1/rho, rho, p) and accelerations, then walks it backwards.
 */
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "sph_ctx.cuh"

namespace sph {
namespace {

constexpr unsigned kFlagNonsmooth = 32u;

__device__ __forceinline__ bool inside(float x, float vm) { return x > -vm && x < vm; }

__global__ void k_adj_init(int n, float4* __restrict__ x, float4* __restrict__ v, float4* __restrict__ u) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 p = x[i], w = v[i];
    p.w = 1.f;
    w.w = 0.f;
    x[i] = p;
    v[i] = w;
    u[i] = w;
}

__global__ void k_adj_gather(int n, const int32_t* __restrict__ perm, const float4* __restrict__ x,
                             float4* __restrict__ xs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    xs[i] = __ldg(&x[__ldg(&perm[i])]);
}

__global__ void k_adj_iota(int n, int32_t* __restrict__ ids) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) ids[i] = i;
}

/* Backward of the leapfrog update (wc_integrate_one in sph_wcsph.cu, kernels/wcsph.cl:176-224):
 * from the adjoints of (x', v', u') to lambda_a and lambda_u; lambda_x passes through. */
__global__ void k_adj_integrate_bwd(Const c, int n, const float4* __restrict__ x, const float4* __restrict__ u,
                                    const float4* __restrict__ a, const float4* __restrict__ lx1,
                                    const float4* __restrict__ lv1, const float4* __restrict__ lu1,
                                    float4* __restrict__ la, float4* __restrict__ lu0, unsigned* __restrict__ flags) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float dt = c.dt, vm = c.vmax;
    const float4 ui = u[i], ai = a[i], xi = x[i];
    const float vhx = ui.x + dt * ai.x, vhy = ui.y + dt * ai.y, vhz = ui.z + dt * ai.z;
    const float prx = vhx + dt * ai.x, pry = vhy + dt * ai.y, prz = vhz + dt * ai.z;
    /* replay the wall test of the forward step to report a reflection */
    const float px = xi.x + dt * clampf(prx, -vm, vm), py = xi.y + dt * clampf(pry, -vm, vm),
                pz = xi.z + dt * clampf(prz, -vm, vm);
    const float ex = clampf(px, (-c.lim_x) / 2.0f, c.lim_x / 2.0f) - px;
    const float ey = clampf(py, (-c.lim_y) / 2.0f, 10.0f) - py;
    const float ez = clampf(pz, (-c.lim_z) / 2.0f, c.lim_z / 2.0f) - pz;
    const bool reflect = len3(ex, ey, ez) > 0.f && len3(vhx, vhy, vhz) > 0.f;
    const float h = 0.5f * dt;
    const float ovx = vhx + (dt * ai.x) * 0.5f, ovy = vhy + (dt * ai.y) * 0.5f, ovz = vhz + (dt * ai.z) * 0.5f;
    const bool mpx = inside(prx, vm), mpy = inside(pry, vm), mpz = inside(prz, vm);
    const bool mvx = inside(ovx, vm), mvy = inside(ovy, vm), mvz = inside(ovz, vm);
    const bool mux = inside(vhx, vm), muy = inside(vhy, vm), muz = inside(vhz, vm);
    if (reflect || !(mpx && mpy && mpz && mvx && mvy && mvz && mux && muy && muz)) atomicOr(flags, kFlagNonsmooth);
    const float4 gx = lx1[i], gv = lv1[i], gu = lu1[i];
    const float fpx = mpx ? 1.f : 0.f, fpy = mpy ? 1.f : 0.f, fpz = mpz ? 1.f : 0.f;
    const float fvx = mvx ? 1.f : 0.f, fvy = mvy ? 1.f : 0.f, fvz = mvz ? 1.f : 0.f;
    const float fux = mux ? 1.f : 0.f, fuy = muy ? 1.f : 0.f, fuz = muz ? 1.f : 0.f;
    const float gvhx = dt * fpx * gx.x + fvx * gv.x + fux * gu.x;
    const float gvhy = dt * fpy * gx.y + fvy * gv.y + fuy * gu.y;
    const float gvhz = dt * fpz * gx.z + fvz * gv.z + fuz * gu.z;
    la[i] = make_float4(dt * gvhx + dt * dt * fpx * gx.x + h * fvx * gv.x,
                        dt * gvhy + dt * dt * fpy * gx.y + h * fvy * gv.y,
                        dt * gvhz + dt * dt * fpz * gx.z + h * fvz * gv.z, 0.f);
    lu0[i] = make_float4(gvhx, gvhy, gvhz, 0.f);
}

/* Backward of the pressure and viscosity sums (k_wc_forces, PHYSICS, no surface tension,
 * no boundary): lambda_rho (through C and R), the direct position adjoint, the velocity
 * adjoint, and each particle's share of dL/dmu and dL/dk (added to per-particle doubles). */
__global__ void __launch_bounds__(256) k_adj_forces_bwd(Const c, int n, const float4* __restrict__ x,
                                                        const float4* __restrict__ v,
                                                        const float4* __restrict__ aux,
                                                        const float4* __restrict__ la, const int* __restrict__ list,
                                                        const int* __restrict__ len, float* __restrict__ lrho,
                                                        float4* __restrict__ lxf, float4* __restrict__ lv,
                                                        double* __restrict__ gmu, double* __restrict__ gk) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 pi = __ldg(&x[i]), vi = __ldg(&v[i]), ai = __ldg(&aux[i]), A = __ldg(&la[i]);
    const float Ci = ai.x, Ri = ai.y, rho = ai.z, p = ai.w;
    const float h = c.h, m = c.mass, sg = c.spiky_grad, rmin2 = c.rmin2_wc;
    const float K = c.visc_lapl * c.mu * m;
    const float coefP = -m * sg;
    float lC = 0.f, lR = 0.f;
    float gxx = 0.f, gxy = 0.f, gxz = 0.f, lvx = 0.f, lvy = 0.f, lvz = 0.f;
    float smx = 0.f, smy = 0.f, smz = 0.f;
    if (rho > 0.f) {
        list_neighbors(i, n, list, __ldg(&len[i]), x, pi.x, pi.y, pi.z,
                       [&](int j, float4, float dx, float dy, float dz) {
            const float4 aj = __ldg(&aux[j]);
            const float4 B = __ldg(&la[j]);
            const float4 vj = __ldg(&v[j]);
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (aj.z > 0.f && r2 > rmin2) {
                const float r = sqrtf(r2), ir = 1.0f / r;
                const float w = h - r;
                const float Dx = A.x - B.x, Dy = A.y - B.y, Dz = A.z - B.z;
                const float dD = dx * Dx + dy * Dy + dz * Dz;
                /* pressure: phi(d) = (h - r)^2 / r * d, J^T D = s D + s' (d.D) d / r */
                const float s = w * w * ir;
                const float sp = -w * (h + r) * ir * ir;
                lC += coefP * s * dD;
                const float cs = coefP * (Ci + aj.x);
                const float t = sp * dD * ir;
                gxx += cs * (s * Dx + t * dx);
                gxy += cs * (s * Dy + t * dy);
                gxz += cs * (s * Dz + t * dz);
                /* viscosity */
                const float dvx = vj.x - vi.x, dvy = vj.y - vi.y, dvz = vj.z - vi.z;
                const float dvD = dvx * Dx + dvy * Dy + dvz * Dz;
                const float RR = Ri * aj.y;
                lR += K * aj.y * w * dvD;
                lvx -= K * RR * w * Dx;
                lvy -= K * RR * w * Dy;
                lvz -= K * RR * w * Dz;
                const float q = -K * RR * dvD * ir;
                gxx += q * dx;
                gxy += q * dy;
                gxz += q * dz;
                const float wr = w * aj.y;
                smx += wr * dvx;
                smy += wr * dvy;
                smz += wr * dvz;
            }
        });
    }
    float lr = 0.f, gki = 0.f;
    if (rho > 0.f) {
        const float q = rho / c.rho0;
        const float q6 = ((((q * q) * q) * q) * q) * q;
        const float q7m1 = pown7(q) - 1.0f;   /* the forward pass's EOS, same rounding */
        const float pv = c.kgas * q7m1;
        const bool act = pv > 0.f;
        const float dp = act ? 7.0f * c.kgas * q6 / c.rho0 : 0.f;
        const float dpk = act ? q7m1 : 0.f;
        const float ir2 = 1.0f / (rho * rho);
        lr = lC * (dp * ir2 - 2.0f * p * ir2 / rho) - lR * ir2;
        gki = lC * dpk * ir2;
    }
    lrho[i] = lr;
    lxf[i] = make_float4(gxx, gxy, gxz, 0.f);
    lv[i] = make_float4(lvx, lvy, lvz, 0.f);
    gmu[i] += (double)(c.visc_lapl * m * Ri * (smx * A.x + smy * A.y + smz * A.z));
    gk[i] += (double)gki;
}

/* Backward of the density sum: lambda_x += sum_j -6 poly6 m (h^2 - r^2)^2 (lrho_i + lrho_j) d. */
__global__ void __launch_bounds__(256) k_adj_density_bwd(Const c, int n, const float4* __restrict__ x,
                                                         const float* __restrict__ lrho,
                                                         const int* __restrict__ list,
                                                         const int* __restrict__ len,
                                                         const float4* __restrict__ lx1,
                                                         const float4* __restrict__ lxf,
                                                         float4* __restrict__ lx0) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 pi = __ldg(&x[i]);
    const float li = __ldg(&lrho[i]);
    const float hh = c.h * c.h, k6 = -6.0f * c.poly6_eval * c.mass;
    float gx = 0.f, gy = 0.f, gz = 0.f;
    list_neighbors(i, n, list, __ldg(&len[i]), x, pi.x, pi.y, pi.z, [&](int j, float4, float dx, float dy, float dz) {
        const float t = hh - r2_exact(dx, dy, dz);
        const float q = k6 * (t * t) * (li + __ldg(&lrho[j]));
        gx += q * dx;
        gy += q * dy;
        gz += q * dz;
    });
    const float4 a = lx1[i], b = lxf[i];
    lx0[i] = make_float4(a.x + b.x + gx, a.y + b.y + gy, a.z + b.z + gz, 0.f);
}

__global__ void k_adj_finish(int n, const float4* __restrict__ lv, const float4* __restrict__ lu,
                             float4* __restrict__ gv0) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 a = lv[i], b = lu[i];
    gv0[i] = make_float4(a.x + b.x, a.y + b.y, a.z + b.z, 0.f);
}

__global__ void k_adj_clear_w(int n, float4* __restrict__ g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) g[i].w = 0.f;
}

/* Fixed-order sum of per-particle doubles (one block): the same result on every run. */
__global__ void __launch_bounds__(1024) k_adj_reduce(int n, const double* __restrict__ a,
                                                     const double* __restrict__ b, double* __restrict__ out) {
    __shared__ double sa[1024], sb[1024];
    double xa = 0.0, xb = 0.0;
    for (int i = threadIdx.x; i < n; i += 1024) {
        xa += a[i];
        xb += b[i];
    }
    sa[threadIdx.x] = xa;
    sb[threadIdx.x] = xb;
    __syncthreads();
    for (int s = 512; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
            sa[threadIdx.x] += sa[threadIdx.x + s];
            sb[threadIdx.x] += sb[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = sa[0];
        out[1] = sb[0];
    }
}

inline int blocks(int n, int bs) { return (n + bs - 1) / bs; }

}  // namespace
}  // namespace sph

struct sph_adj {
    sph_ctx* ctx = nullptr;
    int steps = 0, every = 0, nck = 0, N = 0;
    size_t cap = 0;
    std::string err;
    char* arena = nullptr;
    Const c{};
    bool forward_done = false;
    float mu = 0.f, kgas = 0.f;
    /* checkpoints and the tape of one segment */
    float4 *ckx = nullptr, *ckv = nullptr, *cku = nullptr;
    float4 *tx = nullptr, *tv = nullptr, *tu = nullptr, *taux = nullptr, *ta = nullptr;
    int32_t *tlist = nullptr, *tlen = nullptr;
    /* binning scratch */
    float4* pos_s = nullptr;
    float *dens = nullptr, *pres = nullptr;
    uint32_t *keys = nullptr, *keys_alt = nullptr;
    int32_t *mask = nullptr, *mask_alt = nullptr, *cell_prev = nullptr, *iota = nullptr, *ids = nullptr;
    int2* tab = nullptr;
    void* sort_ws = nullptr;
    /* adjoints */
    float4 *lx[2] = {nullptr, nullptr}, *lv[2] = {nullptr, nullptr}, *lu[2] = {nullptr, nullptr};
    float4 *la = nullptr, *lxf = nullptr, *gv0 = nullptr;
    float* lrho = nullptr;
    double *gmu = nullptr, *gk = nullptr, *gsum = nullptr;
    unsigned* flags = nullptr;
};

namespace {

int afail(sph_adj* a, int code, const std::string& msg) {
    a->err = msg;
    return code;
}
#define ADJ_CUDA(a, call)                                                              \
    do {                                                                               \
        cudaError_t _e = (call);                                                       \
        if (_e != cudaSuccess) return afail(a, SPH_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
    } while (0)

struct ACarver {
    size_t off = 0;
    char* base = nullptr;
    template <class T>
    T* take(size_t count) {
        off = (off + 255) & ~size_t(255);
        T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
        off += count * sizeof(T) + 16;
        return p;
    }
};

void carve(sph_adj* a, ACarver& cv) {
    const size_t n = (size_t)a->N, S = (size_t)a->every, nck = (size_t)a->nck;
    a->ckx = cv.take<float4>(nck * n); a->ckv = cv.take<float4>(nck * n); a->cku = cv.take<float4>(nck * n);
    a->tx = cv.take<float4>((S + 1) * n); a->tv = cv.take<float4>((S + 1) * n); a->tu = cv.take<float4>((S + 1) * n);
    a->taux = cv.take<float4>(S * n); a->ta = cv.take<float4>(S * n);
    a->tlist = cv.take<int32_t>(S * a->cap * n); a->tlen = cv.take<int32_t>(S * n);
    a->pos_s = cv.take<float4>(n);
    a->dens = cv.take<float>(n); a->pres = cv.take<float>(n);
    a->keys = cv.take<uint32_t>(n); a->keys_alt = cv.take<uint32_t>(n);
    a->mask = cv.take<int32_t>(n); a->mask_alt = cv.take<int32_t>(n);
    a->cell_prev = cv.take<int32_t>(n);
    a->iota = cv.take<int32_t>(n); a->ids = cv.take<int32_t>(n);
    a->tab = cv.take<int2>((size_t)a->c.ncells);
    a->sort_ws = cv.take<char>(sph::sort_workspace_bytes((int)n, a->c.key_bits));
    for (int k = 0; k < 2; ++k) {
        a->lx[k] = cv.take<float4>(n); a->lv[k] = cv.take<float4>(n); a->lu[k] = cv.take<float4>(n);
    }
    a->la = cv.take<float4>(n); a->lxf = cv.take<float4>(n); a->gv0 = cv.take<float4>(n);
    a->lrho = cv.take<float>(n);
    a->gmu = cv.take<double>(n); a->gk = cv.take<double>(n); a->gsum = cv.take<double>(2);
    a->flags = cv.take<unsigned>(4);
}

/* One forward step in id order: bin + sort a copy, lists/density under the ids, then the
 * plain force + integrate kernel on the id-ordered state. */
int adj_step(sph_adj* a, const float4* x, const float4* v, const float4* u, float4* xn, float4* vn, float4* un,
             float4* aux, float4* acc, int32_t* list, int32_t* len) {
    sph_ctx* ctx = a->ctx;
    const cudaStream_t s = ctx->stream;
    const int n = a->N, bs = ctx->bs;
    const Const& c = a->c;
    sph::launch_hashes(s, c, x, n, a->keys, a->mask, a->tab, a->cell_prev, a->flags, bs, ctx->b.scenes, nullptr);
    uint32_t* ks = nullptr;
    int32_t* ms = nullptr;
    sph::sort_pairs(s, a->keys, a->mask, a->keys_alt, a->mask_alt, n, c.key_bits, a->sort_ws, a->flags, ctx->num_sms,
                    &ks, &ms);
    sph::k_adj_gather<<<sph::blocks(n, bs), bs, 0, s>>>(n, ms, x, a->pos_s);
    sph::launch_cell_ranges(s, c, a->pos_s, ks, n, a->tab, a->cell_prev, a->flags, bs, ctx->b.scenes, nullptr);
    Bufs lb{};
    lb.pos_s = a->pos_s;
    lb.tab = a->tab;
    lb.nlist = list;
    lb.nlen = len;
    lb.density = a->dens;
    lb.pressure = a->pres;
    lb.aux = aux;
    lb.scenes = ctx->b.scenes;
    lb.flags = a->flags;
    sph::launch_lists_density_remap(s, c, lb, ms, bs);
    Bufs fb{};
    fb.pos_s = const_cast<float4*>(x);
    fb.vel_s = const_cast<float4*>(v);
    fb.vhalf_s = const_cast<float4*>(u);
    fb.aux = aux;
    fb.nlist = list;
    fb.nlen = len;
    fb.tab = a->tab;
    fb.pos = xn;
    fb.vel = vn;
    fb.vhalf = un;
    fb.accel = acc;
    fb.ids_s = a->iota;
    fb.ids = a->ids;
    fb.scenes = ctx->b.scenes;
    fb.flags = a->flags;
    sph::launch_wc_forces(s, c, fb, true, true, true, bs);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return afail(a, SPH_E_CUDA, std::string("adjoint forward launch: ") + cudaGetErrorString(e));
    return SPH_OK;
}

int copy_state(sph_adj* a, float4* dx, float4* dv, float4* du, const float4* sx, const float4* sv, const float4* su) {
    const size_t b = 16 * (size_t)a->N;
    const cudaStream_t s = a->ctx->stream;
    ADJ_CUDA(a, cudaMemcpyAsync(dx, sx, b, cudaMemcpyDeviceToDevice, s));
    ADJ_CUDA(a, cudaMemcpyAsync(dv, sv, b, cudaMemcpyDeviceToDevice, s));
    ADJ_CUDA(a, cudaMemcpyAsync(du, su, b, cudaMemcpyDeviceToDevice, s));
    return SPH_OK;
}

}  // namespace

extern "C" {

int sph_adj_create(sph_ctx* ctx, int steps, int checkpoint_every, sph_adj** out) {
    if (!out) return SPH_E_INVALID;
    *out = nullptr;
    if (!ctx) return SPH_E_INVALID;
    if (steps <= 0 || checkpoint_every <= 0)
        return sph_ctx_fail(ctx, SPH_E_INVALID, "adjoint: steps and checkpoint_every must be positive");
    if (ctx->p.method != SPH_WCSPH || ctx->p.mode != SPH_MODE_PHYSICS)
        return sph_ctx_fail(ctx, SPH_E_INVALID, "adjoint: needs a WCSPH context in PHYSICS mode");
    if (!ctx->scene_in.empty()) return sph_ctx_fail(ctx, SPH_E_INVALID, "adjoint: not available on a batched context");
    if (ctx->NB > 0) return sph_ctx_fail(ctx, SPH_E_INVALID, "adjoint: boundary particles are not supported");
    if (ctx->p.surface_tension != 0.f) return sph_ctx_fail(ctx, SPH_E_INVALID, "adjoint: needs surface_tension = 0");
    if (ctx->N <= 0) return sph_ctx_fail(ctx, SPH_E_STATE, "adjoint: the context holds no fluid particles");
    sph_adj* a = new sph_adj();
    a->ctx = ctx;
    a->steps = steps;
    a->every = checkpoint_every < steps ? checkpoint_every : steps;
    a->nck = (steps + a->every - 1) / a->every;
    a->N = ctx->N;
    a->cap = (size_t)ctx->c.cap;
    a->c = ctx->c;
    ACarver probe;
    carve(a, probe);
    cudaError_t e = cudaMalloc(&a->arena, probe.off);
    if (e != cudaSuccess) {
        delete a;
        cudaGetLastError();
        return sph_ctx_fail(ctx, SPH_E_NOMEM, "adjoint: device allocation of the tape failed");
    }
    ACarver cv;
    cv.base = a->arena;
    carve(a, cv);
    const cudaStream_t s = ctx->stream;
    cudaMemsetAsync(a->tab, 0, sizeof(int2) * (size_t)a->c.ncells, s);
    cudaMemsetAsync(a->cell_prev, 0xff, 4 * (size_t)a->N, s);
    cudaMemsetAsync(a->flags, 0, 16, s);
    sph::k_adj_iota<<<sph::blocks(a->N, 256), 256, 0, s>>>(a->N, a->iota);
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        cudaFree(a->arena);
        delete a;
        return sph_ctx_fail(ctx, SPH_E_CUDA, std::string("adjoint setup: ") + cudaGetErrorString(e));
    }
    *out = a;
    return SPH_OK;
}

int sph_adj_destroy(sph_adj* a) {
    if (!a) return SPH_OK;
    /* cudaFree waits for the work that uses the arena; the context is not touched, so the
     * handle may outlive its context (no other call may) */
    cudaFree(a->arena);
    delete a;
    return SPH_OK;
}

const char* sph_adj_last_error(const sph_adj* a) { return a ? a->err.c_str() : "null adjoint handle"; }

int sph_adj_forward(sph_adj* a, const float* x0_4, const float* v0_4, float mu, float gas_stiffness, float* xT_4,
                    float* vT_4) {
    if (!a || !x0_4 || !v0_4) return SPH_E_INVALID;
    if (!(mu >= 0.f) || !(gas_stiffness >= 0.f)) return afail(a, SPH_E_INVALID, "adjoint: mu and k must be >= 0");
    const cudaStream_t s = a->ctx->stream;
    const int n = a->N, bs = a->ctx->bs;
    const size_t bytes = 16 * (size_t)n;
    a->c = a->ctx->c;
    a->c.mu = mu;
    a->c.kgas = gas_stiffness;
    a->mu = mu;
    a->kgas = gas_stiffness;
    a->forward_done = false;
    ADJ_CUDA(a, cudaMemsetAsync(a->flags, 0, 16, s));
    /* state ping-pong in tape slots 0 and 1 */
    float4 *x = a->tx, *v = a->tv, *u = a->tu;
    float4 *xn = a->tx + n, *vn = a->tv + n, *un = a->tu + n;
    ADJ_CUDA(a, cudaMemcpyAsync(x, x0_4, bytes, cudaMemcpyDefault, s));
    ADJ_CUDA(a, cudaMemcpyAsync(v, v0_4, bytes, cudaMemcpyDefault, s));
    sph::k_adj_init<<<sph::blocks(n, bs), bs, 0, s>>>(n, x, v, u);
    for (int t = 0; t < a->steps; ++t) {
        if (t % a->every == 0) {
            const size_t o = (size_t)(t / a->every) * n;
            int rc = copy_state(a, a->ckx + o, a->ckv + o, a->cku + o, x, v, u);
            if (rc) return rc;
        }
        int rc = adj_step(a, x, v, u, xn, vn, un, a->taux, a->ta, a->tlist, a->tlen);
        if (rc) return rc;
        std::swap(x, xn);
        std::swap(v, vn);
        std::swap(u, un);
    }
    if (xT_4) ADJ_CUDA(a, cudaMemcpyAsync(xT_4, x, bytes, cudaMemcpyDefault, s));
    if (vT_4) ADJ_CUDA(a, cudaMemcpyAsync(vT_4, v, bytes, cudaMemcpyDefault, s));
    ADJ_CUDA(a, cudaStreamSynchronize(s));
    a->forward_done = true;
    return SPH_OK;
}

int sph_adj_backward(sph_adj* a, const float* gxT_4, const float* gvT_4, float* gx0_4, float* gv0_4, double* g_mu,
                     double* g_stiffness, double* g_c0) {
    if (!a || !gxT_4) return SPH_E_INVALID;
    if (!a->forward_done) return afail(a, SPH_E_STATE, "adjoint: backward needs a forward pass first");
    const cudaStream_t s = a->ctx->stream;
    const int n = a->N, bs = a->ctx->bs;
    const size_t bytes = 16 * (size_t)n;
    int cur = 0;
    ADJ_CUDA(a, cudaMemcpyAsync(a->lx[0], gxT_4, bytes, cudaMemcpyDefault, s));
    if (gvT_4) ADJ_CUDA(a, cudaMemcpyAsync(a->lv[0], gvT_4, bytes, cudaMemcpyDefault, s));
    else ADJ_CUDA(a, cudaMemsetAsync(a->lv[0], 0, bytes, s));
    ADJ_CUDA(a, cudaMemsetAsync(a->lu[0], 0, bytes, s));
    sph::k_adj_clear_w<<<sph::blocks(n, bs), bs, 0, s>>>(n, a->lx[0]);
    sph::k_adj_clear_w<<<sph::blocks(n, bs), bs, 0, s>>>(n, a->lv[0]);
    ADJ_CUDA(a, cudaMemsetAsync(a->gmu, 0, 8 * (size_t)n, s));
    ADJ_CUDA(a, cudaMemsetAsync(a->gk, 0, 8 * (size_t)n, s));
    const size_t sn = (size_t)n;
    for (int seg = a->nck - 1; seg >= 0; --seg) {
        const int t0 = seg * a->every;
        const int L = (t0 + a->every <= a->steps ? a->every : a->steps - t0);
        const size_t o = (size_t)seg * sn;
        int rc = copy_state(a, a->tx, a->tv, a->tu, a->ckx + o, a->ckv + o, a->cku + o);
        if (rc) return rc;
        for (int k = 0; k < L; ++k) {
            rc = adj_step(a, a->tx + k * sn, a->tv + k * sn, a->tu + k * sn, a->tx + (k + 1) * sn,
                          a->tv + (k + 1) * sn, a->tu + (k + 1) * sn, a->taux + k * sn, a->ta + k * sn,
                          a->tlist + (size_t)k * a->cap * sn, a->tlen + k * sn);
            if (rc) return rc;
        }
        for (int k = L - 1; k >= 0; --k) {
            const int nx = cur ^ 1;
            const float4* xk = a->tx + k * sn;
            const int32_t* lk = a->tlist + (size_t)k * a->cap * sn;
            const int32_t* nk = a->tlen + k * sn;
            sph::k_adj_integrate_bwd<<<sph::blocks(n, bs), bs, 0, s>>>(a->c, n, xk, a->tu + k * sn, a->ta + k * sn,
                                                                        a->lx[cur], a->lv[cur], a->lu[cur], a->la,
                                                                        a->lu[nx], a->flags);
            sph::k_adj_forces_bwd<<<sph::blocks(n, 256), 256, 0, s>>>(a->c, n, xk, a->tv + k * sn,
                                                                       a->taux + k * sn, a->la, lk, nk, a->lrho,
                                                                       a->lxf, a->lv[nx], a->gmu, a->gk);
            sph::k_adj_density_bwd<<<sph::blocks(n, 256), 256, 0, s>>>(a->c, n, xk, a->lrho, lk, nk, a->lx[cur],
                                                                        a->lxf, a->lx[nx]);
            cur = nx;
        }
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return afail(a, SPH_E_CUDA, std::string("adjoint backward launch: ") + cudaGetErrorString(e));
    }
    sph::k_adj_finish<<<sph::blocks(n, bs), bs, 0, s>>>(n, a->lv[cur], a->lu[cur], a->gv0);
    sph::k_adj_reduce<<<1, 1024, 0, s>>>(n, a->gmu, a->gk, a->gsum);
    if (gx0_4) ADJ_CUDA(a, cudaMemcpyAsync(gx0_4, a->lx[cur], bytes, cudaMemcpyDefault, s));
    if (gv0_4) ADJ_CUDA(a, cudaMemcpyAsync(gv0_4, a->gv0, bytes, cudaMemcpyDefault, s));
    double sums[2] = {0.0, 0.0};
    ADJ_CUDA(a, cudaMemcpyAsync(sums, a->gsum, sizeof sums, cudaMemcpyDeviceToHost, s));
    ADJ_CUDA(a, cudaStreamSynchronize(s));
    if (g_mu) *g_mu = sums[0];
    if (g_stiffness) *g_stiffness = sums[1];
    if (g_c0) {
        /* k = rho0 c0^2 / gamma with gamma = 7: dk/dc0 = 2 rho0 c0 / 7 */
        const double rho0 = (double)a->ctx->p.rest_density;
        const double c0 = std::sqrt((double)a->kgas * 7.0 / rho0);
        *g_c0 = sums[1] * 2.0 * rho0 * c0 / 7.0;
    }
    return SPH_OK;
}

int sph_adj_flags(sph_adj* a, unsigned* flags) {
    if (!a || !flags) return SPH_E_INVALID;
    ADJ_CUDA(a, cudaMemcpyAsync(flags, a->flags, sizeof(unsigned), cudaMemcpyDeviceToHost, a->ctx->stream));
    ADJ_CUDA(a, cudaStreamSynchronize(a->ctx->stream));
    return SPH_OK;
}

int sph_adj_tape_bytes(const sph_adj* a, size_t* bytes) {
    if (!a || !bytes) return SPH_E_INVALID;
    ACarver probe;
    sph_adj tmp = *a;
    carve(&tmp, probe);
    *bytes = probe.off;
    return SPH_OK;
}

}  // extern "C"
