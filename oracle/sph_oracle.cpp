/*
 * sph_oracle.cpp -- CPU oracle of the SPH particle pipeline (TEST INFRASTRUCTURE).
 *
 * Checker only: loaded by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline
 * leg; the CUDA library never links or calls it.
 *
 * Restatement rules (shared with the reference shim, so the float/COMPAT instance can be
 * compared bit for bit with the reference kernels compiled for the CPU):
 *   - OpenCL builtins are restated with IEEE single operations: length/fast_length =
 *     sqrt(x*x+y*y+z*z), normalize/fast_normalize = v / length (zero vector -> zero,
 *     as the OpenCL spec's reference definition says), pown(x,n) = left-to-right
 *     repeated multiplication, clamp = min(max(x,lo),hi), sign as in the spec.
 *   - Division is IEEE (the reference builds with -cl-fast-relaxed-math, whose precision
 *     is implementation-defined; the IEEE restatement is the parity target).
 *   - The w lane of float4 values is 1 for positions and 0 for every other vector, so
 *     it contributes 0 to every dot product and is not carried through the arithmetic.
 *   - A neighbour cell whose linear id falls outside the cell table is read as empty;
 *     the reference reads it unchecked (kernels/grid.cl:165-166).
 *
 * PHYSICS mode fixes (everything else follows the kernel text):
 *   P1 WCSPH density evaluates poly6 at r^2, not r (kernels/wcsph.cl:61-62,70-71
 *      versus kernels/pcisph.cl:80-81).
 *   P2 poly6 normalisation 315/(64 pi h^9) everywhere (mullerconstants.cpp:5 has 365) and
 *      PCISPH mass rho0*dx^3 without the /1.15 compensation (pcisphsimluation.cpp:252).
 *   P3 WCSPH viscosity and cohesion carry the mass factors of kernels/pcisph.cl:216-219
 *      (kernels/wcsph.cl:157,167-169 omit them).
 *   P4 PCISPH stop test maxerr/rho0 < eta (pcisphsimluation.cpp:144 subtracts rho0 from an
 *      error that is already rho*-rho0, so it always stops at the minimum iteration).
 *   P5 PCISPH predicted density counts only pairs with r*^2 < h^2 (kernels/pcisph.cl:394-407
 *      adds negative poly6 values for list pairs that moved apart).
 *   P6 boundary particle velocity uses omega x r (kernels/boundary.cl:58 multiplies
 *      componentwise).
 *   P7 grid fitted to the container with a margin and clamped cell coordinates, instead of
 *      a 5 m cube with wrap-around (grid.h:82-88); neighbour sets are unchanged while the
 *      particles stay inside the reference cube.
 */
#include "sph_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

/* opencl/clcompiler.cpp:50-54: float -D constants are printed std::fixed with 6
 * decimals and parsed back by the OpenCL compiler to the nearest float. */
float round6(float v) {
    char buf[64];
    snprintf(buf, sizeof buf, "%.6f", (double)v);
    return strtof(buf, nullptr);
}

/* kernels/morton.h:37-56 with OpenCL C semantics: a uint shifted by 32 is shifted by
 * 32 mod 32 = 0, and the 64-bit masks are truncated to 32 bits on assignment. */
inline uint32_t split_by_3(uint32_t a) {
    uint32_t x = a & 0x1fffffu;
    x = x & 0x0000ffffu;
    x = (x | (x << 16)) & 0xff0000ffu;
    x = (x | (x << 8)) & 0x0f00f00fu;
    x = (x | (x << 4)) & 0xc30c30c3u;
    x = (x | (x << 2)) & 0x49249249u;
    return x;
}
inline uint32_t morton3(uint32_t x, uint32_t y, uint32_t z) {
    uint32_t hx = split_by_3(x);
    uint32_t hy = split_by_3(y) << 1;
    uint32_t hz = split_by_3(z) << 2;
    return (hx | hy) | hz;
}

/* kernels/grid.h:15-49: own cell first, then the 26 others in this order. */
const int kOff[27][3] = {
    {0, 0, 0},
    {-1, -1, -1}, {-1, -1, 0}, {-1, -1, 1}, {-1, 0, -1}, {-1, 0, 0}, {-1, 0, 1},
    {-1, 1, -1}, {-1, 1, 0}, {-1, 1, 1},
    {0, -1, -1}, {0, -1, 0}, {0, -1, 1}, {0, 0, -1},
    {0, 0, 1}, {0, 1, -1}, {0, 1, 0}, {0, 1, 1},
    {1, -1, -1}, {1, -1, 0}, {1, -1, 1}, {1, 0, -1}, {1, 0, 0}, {1, 0, 1},
    {1, 1, -1}, {1, 1, 0}, {1, 1, 1}};

template <class R> struct V3 { R x, y, z; };
template <class R> inline V3<R> v3(R x, R y, R z) { return V3<R>{x, y, z}; }
template <class R> inline V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> inline V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R> inline V3<R> operator*(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <class R> inline V3<R> operator*(R s, V3<R> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class R> inline V3<R> operator/(V3<R> a, R s) { return {a.x / s, a.y / s, a.z / s}; }
template <class R> inline V3<R>& operator+=(V3<R>& a, V3<R> b) { a = a + b; return a; }
template <class R> inline V3<R>& operator-=(V3<R>& a, V3<R> b) { a = a - b; return a; }
template <class R> inline R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> inline R length(V3<R> a) { return std::sqrt(dot(a, a)); }
template <class R> inline V3<R> normalize(V3<R> a) {
    R l = length(a);
    if (l == R(0)) return a;
    return {a.x / l, a.y / l, a.z / l};
}
template <class R> inline R pown(R x, int n) { R r = x; for (int k = 1; k < n; ++k) r = r * x; return r; }

/* kernels/monaghan_kernels.h:7-47, the Monaghan cubic spline the reference selects when its
 * programs are built without USE_MULLER_KERNELS (kernels/kernels.h:8-37).  M_PI_F, pown and
 * INV as the kernel text has them, left to right; hd = SUPPORT_RADIUS (the -D constant). */
constexpr float kPiF = 3.14159265358979323846f;
template <class R> inline R mon_eval(R hd) { return R(1.0f) / (R(kPiF) * pown(hd, 3)); }
template <class R> inline R mon_grad(R hd) { return R(-3.0f) / (R(kPiF) * pown(hd, 4)); }
template <class R> inline R w_monaghan(R r, R h, R hd) {
    if (r <= h) return mon_eval(hd) * ((R(1.0f) - R(1.5f) * pown(r / h, 2)) + R(0.75f) * pown(r / h, 3));
    if (r <= R(2.0f) * h) return (mon_eval(hd) * R(0.25f)) * pown(R(2.0f) - r / h, 3);
    return R(0);
}
template <class R> inline V3<R> grad_w_monaghan(V3<R> r, R rn, R h, R hd) {
    const R g = mon_grad(hd);
    if (rn <= h) {
        const R c = R(0.75f) * (rn / pown(h, 2));   /* subtracted from every component */
        const R ih = R(1.0f) / h;
        return {(g * r.x) * ih - c, (g * r.y) * ih - c, (g * r.z) * ih - c};
    }
    if (rn <= R(2.0f) * h) {
        const R ir = R(1.0f) / rn, q = pown(R(2.0f) - rn / h, 2);
        return {(((g * r.x) * R(0.25f)) * ir) * q, (((g * r.y) * R(0.25f)) * ir) * q,
                (((g * r.z) * R(0.25f)) * ir) * q};
    }
    return {r.x * R(0), r.y * R(0), r.z * R(0)};
}
template <class R> inline R lapl_w_monaghan(R rn, R h, R hd) {
    const R l = R(3.0f) * mon_grad(hd);
    if (rn <= h) return l * (R(1.0f) / h - R(1.5f) * (rn / pown(h, 2)));
    if (rn <= R(2.0f) * h)
        return l * (((R(1.0f) / (R(0.25f) * rn)) * pown(R(2.0f) - rn / h, 2) - R(1.0f) / rn) +
                    rn / (R(4.0f) * pown(h, 2)));
    return R(0);
}
/* OpenCL C spec: clamp = fmin(fmax(x, lo), hi); max(x, y) = (x < y) ? y : x */
template <class R> inline R clampf(R x, R lo, R hi) { return std::fmin(std::fmax(x, lo), hi); }
template <class R> inline R clmax(R x, R y) { return x < y ? y : x; }
template <class R> inline V3<R> clampv(V3<R> a, R lo, R hi) {
    return {clampf(a.x, lo, hi), clampf(a.y, lo, hi), clampf(a.z, lo, hi)};
}
template <class R> inline R signf(R x) {
    if (x > R(0)) return R(1);
    if (x < R(0)) return R(-1);
    if (x != x) return R(0);
    return x;
}
template <class R> inline V3<R> signv(V3<R> a) { return {signf(a.x), signf(a.y), signf(a.z)}; }
template <class R> inline V3<R> cross(V3<R> a, V3<R> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class R> inline V3<R> ld(const std::vector<R>& a, long long i) {
    return {a[4 * i], a[4 * i + 1], a[4 * i + 2]};
}
template <class R> inline void st(std::vector<R>& a, long long i, V3<R> v, R w) {
    a[4 * i] = v.x; a[4 * i + 1] = v.y; a[4 * i + 2] = v.z; a[4 * i + 3] = w;
}

/* kernels/surface_tension.h:23-50 */
template <class R> inline R st_corr(R rho0, R di, R dj) { return R(2) * rho0 / (di + dj); }
template <class R> inline R st_kernel(R r, R h, R c) {
    if (r <= R(0.5) * h) {
        R t1 = h - r;
        R t2 = (t1 * t1 * t1) * (r * r * r);
        return R(2) * t2 - c;
    } else if (r <= h) {
        R t1 = h - r;
        return (t1 * t1 * t1) * (r * r * r);
    }
    return R(0);
}

struct Body {
    std::vector<float> raw;   /* 4 per particle */
    int count = 0, origin = 0;
    int can_move = 0;
    float rot[12];
    float lin[4], ang[4];
    float mass = 0;
    int dynamic = 0;
    float inv_inertia[3] = {0, 0, 0};
    float radius = 0;
};

struct OracleBase {
    virtual ~OracleBase() {}
    virtual int set_fluid(const float* p, const float* v, int n) = 0;
    virtual int add_boundary(const float* p, int n, int mv, const float* rot, const float* lin,
                             const float* ang, float mass) = 0;
    virtual int run_stage(int s) = 0;
    virtual int step(int n) = 0;
    virtual long long elems(int f) = 0;
    virtual int kind(int f) = 0;
    virtual int get(int f, void* out) = 0;
    virtual int set(int f, const void* in) = 0;
    virtual void derived(OrcDerived* d) = 0;
    virtual void stats(double* out) = 0;
    virtual int set_body_dynamics(int body, int enabled, const float* inv_inertia, float radius) = 0;
    virtual int body_state(int body, float* rot, float* lin, float* ang) = 0;
};

/* Stable LSD radix sort of (uint key, int value) pairs, 8-bit digits, all 32 key bits.
 * Restates the algorithm of the external clogs::Radixsort (clogs 1.5.1) that
 * opencl/algorithms/clsort.h:13-35 calls with maxBits = 0 (full key). */
void radix_sort_pairs(uint32_t* keys, int32_t* vals, int n) {
    if (n <= 1) return;
    std::vector<uint32_t> k2(n);
    std::vector<int32_t> v2(n);
    uint32_t* ks = keys; int32_t* vs = vals;
    uint32_t* kd = k2.data(); int32_t* vd = v2.data();
    for (int pass = 0; pass < 4; ++pass) {
        int shift = 8 * pass;
        size_t cnt[257] = {0};
        for (int i = 0; i < n; ++i) cnt[((ks[i] >> shift) & 255u) + 1]++;
        for (int d = 0; d < 256; ++d) cnt[d + 1] += cnt[d];
        for (int i = 0; i < n; ++i) {
            size_t at = cnt[(ks[i] >> shift) & 255u]++;
            kd[at] = ks[i]; vd[at] = vs[i];
        }
        std::swap(ks, kd); std::swap(vs, vd);
    }
    /* four passes: the result is back in the caller's arrays */
}

template <class R>
struct Oracle : OracleBase {
    OrcConfig cfg;
    int N = 0, NB = 0, cap = 50;
    bool compat;
    bool mon;   /* COMPAT with the Monaghan kernels (OrcConfig::kernels) */
    /* derived constants (reference host code restated) */
    R dt, vmax, rho0, rho0_def, mu, sigma, kgas, g;
    R mass, mass_def, h, h_def, h_list;          /* h_def: SUPPORT_RADIUS -D; h_list: CELL_SIZE -D */
    R poly6_eval, poly6_grad, spiky_grad, visc_lapl, st_main, st_term;
    R default_eval, default_grad, pressure_grad, boundary_eval, delta;
    R bforce_spiky;
    R lim[3];
    /* grid */
    R gorigin[3]; float gorigin_f[3]; R gh; int gn[3]; int gwrap; long long gcells; int key_bits;
    /* fluid state */
    std::vector<R> pos, vel, vel_half, pos_s, vel_s, vel_half_s;
    std::vector<uint32_t> hashes; std::vector<int32_t> mask, ids, ids_s;
    std::vector<int32_t> intervals, nlist, nlen, sblist, sblen;
    std::vector<R> density, pressure, normal, accel, pos_pred, f_other, f_press, dens_var;
    /* boundary */
    std::vector<Body> bodies;
    std::vector<R> bpos, bvel, bphi, bpos_s, bphi_s, body_force, body_torque;
    std::vector<uint32_t> bhashes; std::vector<int32_t> bmask, bintervals;
    int32_t pci_iters = 0; std::vector<R> pci_maxerr;

    explicit Oracle(const OrcConfig& c) : cfg(c) {
        compat = cfg.mode == 0;
        mon = compat && cfg.kernels == 1;
        cap = cfg.neigh_cap > 0 ? cfg.neigh_cap : 50;
        derive();
    }

    /* fluid/simulation/wcsphsimluation.cpp:165-202, pcisphsimluation.cpp:230-255,268-278,
     * mullerconstants.cpp:4-38, boundaryhandler.cpp:144,306-309, grid.cpp:61-68 */
    void derive() {
        const float hf = cfg.support_radius, rf = cfg.particle_radius;
        const float rho0f = cfg.rest_density;
        dt = cfg.time_step; vmax = cfg.max_vel; rho0 = rho0f; mu = cfg.k_viscosity;
        sigma = cfg.surface_tension; kgas = cfg.gas_stiffness; g = -cfg.gravity;
        h = hf;
        lim[0] = cfg.container[0]; lim[1] = cfg.container[1]; lim[2] = cfg.container[2];
        const bool dbl = sizeof(R) == 8;
        if (cfg.method == 0) {
            float mf = rho0f * std::pow(2.0f * rf, 3.0f) / 1.0f;
            mass = dbl ? R(rho0f) * std::pow(R(2) * R(rf), R(3)) : R(mf);
            poly6_eval = dbl ? R(315.0 / (64.0 * M_PI * std::pow((double)hf, 9))) : R(float(315.0 / (64.0 * M_PI * std::pow(hf, 9))));
            poly6_grad = dbl ? R(-945.0 / (32.0 * M_PI * std::pow((double)hf, 9))) : R(float(-945.0 / (32.0 * M_PI * std::pow(hf, 9))));
            spiky_grad = dbl ? R(-45.0 / (M_PI * std::pow((double)hf, 6))) : R(float(-45.0 / (M_PI * std::pow(hf, 6))));
            visc_lapl = dbl ? R(45.0 / (M_PI * std::pow((double)hf, 6))) : R(float(45.0 / (M_PI * std::pow(hf, 6))));
            default_grad = poly6_grad;
            pressure_grad = spiky_grad;
            default_eval = poly6_eval;
            mass_def = dbl ? mass : R(round6(mf));    /* normals.cl PARTICLE_MASS (intended binding) */
            rho0_def = rho0;
        } else {
            float mf = rho0f * std::pow(2.0f * rf, 3.0f) / (compat ? 1.15f : 1.0f);
            mass = dbl ? R(rho0f) * std::pow(R(2) * R(rf), R(3)) / R(compat ? 1.15 : 1.0) : R(mf);
            double e = compat ? 365.0 : 315.0;
            default_eval = dbl ? R(e / (64.0 * M_PI * std::pow((double)hf, 9.0))) : R(float(float(e) / (64.0f * M_PI * std::pow(hf, 9.0f))));
            default_grad = dbl ? R(-945.0 / (32.0 * M_PI * std::pow((double)hf, 9.0))) : R(float(-945.0f / (32.0f * M_PI * std::pow(hf, 9.0f))));
            visc_lapl = dbl ? R(45.0 / (M_PI * std::pow((double)hf, 6.0))) : R(float(45.0f / (M_PI * std::pow(hf, 6.0f))));
            pressure_grad = dbl ? R(-45.0 / (M_PI * std::pow((double)hf, 6.0))) : R(float(-45.0f / (M_PI * std::pow(hf, 6.0f))));
            poly6_eval = default_eval; poly6_grad = default_grad; spiky_grad = pressure_grad;
            mass_def = dbl ? mass : R(round6(mf));
            rho0_def = dbl ? rho0 : R(round6(rho0f));
        }
        st_main = dbl ? R(32.0 / (M_PI * std::pow((double)hf, 9.0))) : R(float(32.0f / (M_PI * std::pow(hf, 9.0f))));
        st_term = dbl ? R(std::pow((double)hf, 6.0) / 64.0) : R(std::pow(hf, 6.0f) / 64.0f);
        h_def = dbl ? h : R(round6(hf));
        h_list = h_def;
        /* boundaryhandler.cpp:144 MullerConstants::default_eval (365); P2: 315 */
        {
            double e = compat ? 365.0 : 315.0;
            boundary_eval = dbl ? R(e / (64.0 * M_PI * std::pow((double)hf, 9.0))) : R(float(float(e) / (64.0f * M_PI * std::pow(hf, 9.0f))));
        }
        bforce_spiky = dbl ? R(-45.0 / (M_PI * std::pow((double)hf, 6))) : R(float(-45.0f / (M_PI * std::pow(hf, 6))));
        /* grid: grid.cpp:61-68 (COMPAT cube); P7 container fit (PHYSICS) */
        gh = h;
        if (compat) {
            float size = cfg.grid_size > 0 ? cfg.grid_size : 5.0f;
            int cps = (int)std::ceil(size / hf);
            for (int a = 0; a < 3; ++a) {
                gorigin_f[a] = -(size / 2.0f);
                gorigin[a] = gorigin_f[a];
                gn[a] = cps;
            }
            gwrap = 1;
            key_bits = 32;
        } else {
            float m = cfg.grid_margin > 0 ? cfg.grid_margin : 2.0f;
            int mx = 1;
            for (int a = 0; a < 3; ++a) {
                float L = cfg.container[a];
                gorigin_f[a] = -(L / 2.0f) - m * hf;
                gorigin[a] = gorigin_f[a];
                gn[a] = (int)std::ceil((L + 2.0f * m * hf) / hf);
                if (gn[a] < 1) gn[a] = 1;
                mx = std::max(mx, gn[a]);
            }
            int b = 0; while ((1 << b) < mx) ++b;
            key_bits = 3 * b;
            gwrap = 0;
        }
        gcells = (long long)gn[0] * gn[1] * gn[2];
        delta = 0;
        if (cfg.method == 1) deduce_delta();
    }

    /* pcisphsimluation.cpp:429-469 */
    void deduce_delta() {
        const float hf = cfg.support_radius, rf = cfg.particle_radius;
        const float spiky = float(pressure_grad), poly = float(default_grad);
        const float mf = float(mass), rhof = cfg.rest_density, dtf = cfg.time_step;
        const float sqr_h = hf * hf;
        float beta = 2.0f * std::pow((dtf * mf) / rhof, 2.0f);
        float value_sum[3] = {0.f, 0.f, 0.f}, spiky_sum[3] = {0.f, 0.f, 0.f};
        float vdv = 0.f;
        for (float x = -hf - rf; x <= hf + rf; x += 2.0f * rf)
            for (float y = -hf - rf; y <= hf + rf; y += 2.0f * rf)
                for (float z = -hf - rf; z <= hf + rf; z += 2.0f * rf) {
                    float r2 = (x * x + y * y + z * z);
                    float rn = std::sqrt(r2);
                    if (r2 < sqr_h) {
                        float sf = spiky * (hf - rn) * (hf - rn) * (1.0 / rn);
                        float f = poly * (sqr_h - r2) * (sqr_h - r2);
                        float sv[3] = {sf * x, sf * y, sf * z};
                        float v[3] = {f * x, f * y, f * z};
                        for (int i = 0; i < 3; i++) {
                            value_sum[i] += v[i];
                            spiky_sum[i] += sv[i];
                            vdv += v[i] * sv[i];
                        }
                    }
                }
        float sds = 0.f;
        for (int i = 0; i < 3; i++) sds += spiky_sum[i] * value_sum[i];
        delta = -1.0f / (beta * (-sds - vdv));
    }

    /* kernels/grid.h:74-91 (COMPAT, wrap) or clamped coordinates (PHYSICS, P7) */
    inline void coords(V3<R> p, int c[3]) const {
        R pv[3] = {p.x, p.y, p.z};
        for (int a = 0; a < 3; ++a) {
            R f = std::floor((pv[a] - gorigin[a]) / gh);
            if (gwrap) {
                if (!(f > R(-1e9) && f < R(1e9))) f = 0;
                int ci = (int)f + gn[a];
                c[a] = ci % gn[a];
            } else {
                if (!(f >= R(0))) c[a] = 0;
                else if (f > R(gn[a] - 1)) c[a] = gn[a] - 1;
                else c[a] = (int)f;
            }
        }
    }
    inline long long cell_id(int x, int y, int z) const {
        return (long long)x + (long long)gn[0] * ((long long)y + (long long)gn[1] * z);
    }
    inline bool cell_ok(int x, int y, int z, long long& id) const {
        if (gwrap) {
            id = cell_id(x, y, z);
            return id >= 0 && id < gcells;
        }
        if (x < 0 || y < 0 || z < 0 || x >= gn[0] || y >= gn[1] || z >= gn[2]) return false;
        id = cell_id(x, y, z);
        return true;
    }

    /* kernels/grid.cl:20-39 */
    void compute_hashes(const std::vector<R>& p, int n, std::vector<uint32_t>& hs, std::vector<int32_t>& mk) {
        hs.resize(n); mk.resize(n);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {
            int c[3];
            coords(ld(p, i), c);
            hs[i] = morton3((uint32_t)c[0], (uint32_t)c[1], (uint32_t)c[2]);
            mk[i] = i;
        }
    }
    /* kernels/grid.cl:60-123 with the zero fill of grid.cpp:41 */
    void compute_intervals(const std::vector<R>& sp, const std::vector<uint32_t>& hs, int n, std::vector<int32_t>& iv) {
        iv.assign(2 * gcells, 0);
        for (int i = 0; i < n; ++i) {
            int c0[3]; coords(ld(sp, i), c0);
            long long id0 = cell_id(c0[0], c0[1], c0[2]);
            if (i == n - 1) {
                iv[2 * id0 + 1] = i + 1;
            } else {
                int c1[3]; coords(ld(sp, i + 1), c1);
                long long id1 = cell_id(c1[0], c1[1], c1[2]);
                if (hs[i] < hs[i + 1]) {
                    iv[2 * id0 + 1] = i + 1;
                    iv[2 * id1] = i + 1;
                }
            }
        }
    }
    /* kernels/grid.cl:145-182 (column-major list, 50-cap, traversal order) */
    void neigh_list(const std::vector<R>& refp, int nref, const std::vector<R>& np,
                    const std::vector<int32_t>& iv, std::vector<int32_t>& list, std::vector<int32_t>& len) {
        list.assign((size_t)cap * std::max(nref, 1), 0);
        len.assign(nref, 0);
        const R h2 = h_list * h_list;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < nref; ++i) {
            V3<R> pi = ld(refp, i);
            int c[3]; coords(pi, c);
            int ll = 0;
            for (int o = 0; ll < cap && o < 27; ++o) {
                long long id;
                if (!cell_ok(c[0] + kOff[o][0], c[1] + kOff[o][1], c[2] + kOff[o][2], id)) continue;
                int s = iv[2 * id], e = iv[2 * id + 1];
                for (int j = s; ll < cap && j < e; ++j) {
                    V3<R> r = pi - ld(np, j);
                    R r2 = dot(r, r);
                    if (r2 < h2) { list[(size_t)ll * nref + i] = j; ++ll; }
                }
            }
            len[i] = ll;
        }
    }
    void gather4(const std::vector<R>& src, const std::vector<int32_t>& mk, std::vector<R>& dst, int n) {
        dst.resize(4 * (size_t)n);
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < 4; ++k) dst[4 * (size_t)i + k] = src[4 * (size_t)mk[i] + k];
    }

    /* kernels/wcsph.cl:32-79 (P1 in PHYSICS) */
    void wc_density() {
        density.assign(N, 0); pressure.assign(N, 0);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < N; ++i) {
            V3<R> pi = ld(pos_s, i);
            R di = 0, bdi = 0;
            for (int k = 0; k < nlen[i]; ++k) {
                int j = nlist[(size_t)k * N + i];
                V3<R> d = pi - ld(pos_s, j);
                R rr = compat ? length(d) : dot(d, d);
                di += mon ? w_monaghan(rr, h, h_def) : pown(pown(h, 2) - rr, 3);
            }
            di *= poly6_eval * mass;
            for (int k = 0; k < sblen[i]; ++k) {
                int j = sblist[(size_t)k * N + i];
                V3<R> d = pi - ld(bpos_s, j);
                R rr = compat ? length(d) : dot(d, d);
                bdi += (mon ? w_monaghan(rr, h, h_def) : pown(pown(h, 2) - rr, 3)) * bphi_s[j];
            }
            di += poly6_eval * bdi;
            density[i] = di;
            pressure[i] = clmax(R(0), kgas * (pown(di / rho0, 7) - R(1)));
        }
    }
    /* kernels/normals.cl:23-70 (constants: WCSPH poly6_grad / PCISPH default_grad) */
    void normals() {
        normal.assign(4 * (size_t)N, 0);
        const R H = h_def;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < N; ++i) {
            V3<R> pi = ld(pos_s, i);
            V3<R> n = v3<R>(0, 0, 0);
            for (int k = 0; k < nlen[i]; ++k) {
                int j = nlist[(size_t)k * N + i];
                V3<R> r = pi - ld(pos_s, j);
                if (mon) {
                    n += grad_w_monaghan(r, dot(r, r), H, H) / density[j];
                    continue;
                }
                R s = pown(pown(H, 2) - dot(r, r), 2);
                n += (r * s) / density[j];
            }
            n = ((default_grad * n) * mass_def) * H;
            st(normal, i, n, R(0));
        }
    }
    /* kernels/wcsph.cl:81-173 (P3 in PHYSICS) */
    void wc_accel() {
        accel.assign(4 * (size_t)N, 0);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < N; ++i) {
            V3<R> pi = ld(pos_s, i);
            V3<R> fco = v3<R>(0, 0, 0), fcu = v3<R>(0, 0, 0), pa = v3<R>(0, 0, 0), va = v3<R>(0, 0, 0);
            R di = density[i], p_i = pressure[i];
            V3<R> vi = ld(vel_s, i), ni = ld(normal, i);
            R C = p_i / pown(di, 2);
            V3<R> bpa = v3<R>(0, 0, 0);
            for (int k = 0; k < sblen[i]; ++k) {
                int j = sblist[(size_t)k * N + i];
                V3<R> r = pi - ld(bpos_s, j);
                R rn = length(r);
                bpa += ((((-bphi_s[j]) * r) * (spiky_grad / rn)) * pown(h - rn, 2)) * R(2) * C;
            }
            for (int k = 0; k < nlen[i]; ++k) {
                int j = nlist[(size_t)k * N + i];
                V3<R> vj = ld(vel_s, j), nj = ld(normal, j);
                R dj = density[j], pj = pressure[j];
                V3<R> r = pi - ld(pos_s, j);
                R rn = length(r);
                if (di > 0 && dj > 0 && (double)rn > 0.00001) {
                    pa += ((r * (spiky_grad / rn)) * pown(h - rn, 2)) * (C + pj / pown(dj, 2));
                    va += ((vj - vi) * (h - rn)) / dj;
                    fcu += (ni - nj) * st_corr(rho0, di, dj);
                    fco += (normalize(r) * st_kernel(rn, h, st_term)) * st_corr(rho0, di, dj);
                }
            }
            pa = pa * (-mass);
            if (compat) {
                va = va * (visc_lapl * mu);
                fco = fco * st_main;
            } else {
                va = va * ((visc_lapl * mu) * (mass / di));
                fco = fco * (st_main * mass);
            }
            V3<R> ast = (-sigma) * (fcu + fco);
            V3<R> a = v3<R>(0, g, 0) + ast + pa + va + bpa;
            st(accel, i, a, R(0));
        }
    }
    /* container clamp used by both integrators: x,z in [-L/2, L/2], y in [-H/2, 10] */
    inline V3<R> clamp_box(V3<R> p) const {
        V3<R> c = p;
        c.z = clampf(p.z, (-lim[2]) / R(2), lim[2] / R(2));
        c.x = clampf(p.x, (-lim[0]) / R(2), lim[0] / R(2));
        c.y = clampf(p.y, (-lim[1]) / R(2), R(10));
        return c;
    }
    /* kernels/wcsph.cl:176-224: sorted inputs -> unsorted buffers */
    void wc_integrate() {
#pragma omp parallel for schedule(static)
        for (int i = 0; i < N; ++i) {
            V3<R> p = ld(pos_s, i), vh = ld(vel_half_s, i), a = ld(accel, i);
            vh += dt * a;
            p += dt * clampv(vh + dt * a, -vmax, vmax);
            R vn = length(vh);
            V3<R> cp = clamp_box(p);
            R d = length(cp - p);
            if (d > 0 && vn > 0) {
                V3<R> nrm = normalize(signv(cp - p));
                R rest = (R(1) * d) / (dt * vn);
                vh -= ((R(1) + rest) * dot(vh, nrm)) * nrm;
                p = cp;
            }
            V3<R> vt = vh + ((dt * a) * R(0.5));
            st(pos, i, p, R(1));
            st(vel_half, i, clampv(vh, -vmax, vmax), R(0));
            st(vel, i, clampv(vt, -vmax, vmax), R(0));
        }
        ids = ids_s;
    }

    /* kernels/pcisph.cl:33-102 */
    void pci_init_density() {
        density.assign(N, 0);
        const R H = h_def;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < N; ++i) {
            V3<R> pi = ld(pos_s, i);
            R di = 0, bdi = 0;
            for (int k = 0; k < nlen[i]; ++k) {
                int j = nlist[(size_t)k * N + i];
                V3<R> r = pi - ld(pos_s, j);
                di += mon ? w_monaghan(dot(r, r), H, H) : pown(pown(H, 2) - dot(r, r), 3);
            }
            for (int k = 0; k < sblen[i]; ++k) {
                int j = sblist[(size_t)k * N + i];
                V3<R> r = pi - ld(bpos_s, j);
                bdi += (mon ? w_monaghan(dot(r, r), H, H) : pown(pown(H, 2) - dot(r, r), 3)) * bphi_s[j];
            }
            density[i] = default_eval * ((di * mass_def) + bdi);
        }
    }
    /* kernels/pcisph.cl:134-222 */
    void pci_init_forces() {
        f_other.assign(4 * (size_t)N, 0);
        const R H = h_def;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < N; ++i) {
            V3<R> pi = ld(pos_s, i), vi = ld(vel_s, i), ni = ld(normal, i);
            R di = density[i];
            V3<R> fv = v3<R>(0, 0, 0), fco = v3<R>(0, 0, 0), fcu = v3<R>(0, 0, 0);
            for (int k = 0; k < nlen[i]; ++k) {
                int j = nlist[(size_t)k * N + i];
                V3<R> pj = ld(pos_s, j), vj = ld(vel_s, j), nj = ld(normal, j);
                R dj = density[j];
                V3<R> r = pi - pj;
                R rn = length(r);
                fv += (vj - vi) * ((mon ? lapl_w_monaghan(rn, H, H) : H - rn) / dj);
                fcu += (ni - nj) * st_corr(rho0_def, di, dj);
                fco += (normalize(r) * st_kernel(rn, H, st_term)) * st_corr(rho0_def, di, dj);
            }
            fv = fv * ((mu * pown(mass_def, 2)) * (visc_lapl / di));
            fco = fco * (mass_def * st_main);
            V3<R> ft = ((-sigma) * mass_def) * (fcu + fco);
            st(f_other, i, fv + ft, R(0));
        }
    }
    /* kernels/pcisph.cl:302-344 */
    void pci_predict() {
#pragma omp parallel for schedule(static)
        for (int i = 0; i < N; ++i) {
            V3<R> p = ld(pos_s, i), v = ld(vel_s, i);
            V3<R> a = v3<R>(0, g, 0) + (ld(f_press, i) + ld(f_other, i)) / mass_def;
            v += clampv(a * dt, -vmax, vmax);
            p += v * dt;
            R vn = length(v);
            V3<R> cp = clamp_box(p);
            R d = length(cp - p);
            if (d > 0 && vn > 0) p = cp;
            st(pos_pred, i, p, R(1));
        }
    }
    /* kernels/pcisph.cl:349-418 (P5 in PHYSICS) */
    void pci_update_pressure() {
        const R H = h_def;
        const R H2 = H * H;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < N; ++i) {
            V3<R> pi = ld(pos_pred, i);
            R pd = 0, pdb = 0;
            for (int k = 0; k < nlen[i]; ++k) {
                int j = nlist[(size_t)k * N + i];
                V3<R> r = pi - ld(pos_pred, j);
                R r2 = dot(r, r);
                if (compat || r2 < H2) pd += mon ? w_monaghan(r2, H, H) : pown(pown(H, 2) - r2, 3);
            }
            pd *= default_eval * mass_def;
            for (int k = 0; k < sblen[i]; ++k) {
                int j = sblist[(size_t)k * N + i];
                V3<R> r = pi - ld(bpos_s, j);
                R r2 = dot(r, r);
                if (compat || r2 < H2) pdb += (mon ? w_monaghan(r2, H, H) : pown(pown(H, 2) - r2, 3)) * bphi_s[j];
            }
            pdb *= default_eval;
            R dv = clmax(R(0), pd + pdb - rho0_def);
            dens_var[i] = dv;
            pressure[i] += dv * delta;
        }
    }
    /* kernels/pcisph.cl:420-504 */
    void pci_pressure_force() {
        const R H = h_def;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < N; ++i) {
            V3<R> pi = ld(pos_s, i);
            V3<R> fp = v3<R>(0, 0, 0), fpb = v3<R>(0, 0, 0);
            R di = density[i], p_i = pressure[i];
            R C = p_i / pown(di, 2);
            for (int k = 0; k < nlen[i]; ++k) {
                int j = nlist[(size_t)k * N + i];
                V3<R> r = pi - ld(pos_s, j);
                R l = length(r);
                if (l >= R(1e-5f))
                    fp += (C + pressure[j] / pown(density[j], 2)) *
                          (mon ? grad_w_monaghan(r, l, H, H) : (r * (R(1) / l)) * pown(H - l, 2));
            }
            fp = fp * ((-pown(mass_def, 2)) * pressure_grad);
            for (int k = 0; k < sblen[i]; ++k) {
                int j = sblist[(size_t)k * N + i];
                V3<R> r = pi - ld(bpos_s, j);
                R l = length(r);
                fpb += (bphi_s[j] * (R(2) * C)) *
                       (mon ? grad_w_monaghan(r, l, H, H) : (r * (R(1) / l)) * pown(H - l, 2));
            }
            fpb = fpb * ((-mass_def) * pressure_grad);
            st(f_press, i, fp + fpb, R(0));
        }
    }
    /* pcisphsimluation.cpp:129-148 (P4 in PHYSICS) */
    void pci_loop(int min_iter, int max_iter) {
        dens_var.assign(N, 0);
        pos_pred.assign(4 * (size_t)N, 0);
        pci_maxerr.clear();
        pci_iters = 0;
        for (int it = 1; it <= max_iter; ++it) {
            pci_predict();
            pci_update_pressure();
            pci_pressure_force();
            pci_iters = it;
            R mx = 0;
            for (int i = 0; i < N; ++i) mx = std::max(mx, dens_var[i]);
            pci_maxerr.push_back(mx);
            if (it >= min_iter) {
                R crit = compat ? (mx - rho0) / rho0 : mx / rho0;
                if (crit < R(cfg.pci_error_ratio)) break;
            }
        }
    }
    /* kernels/pcisph.cl:240-284 */
    void pci_integrate() {
#pragma omp parallel for schedule(static)
        for (int i = 0; i < N; ++i) {
            V3<R> p = ld(pos_s, i), v = ld(vel_s, i);
            V3<R> a = v3<R>(0, g, 0) + (ld(f_press, i) + ld(f_other, i)) / mass_def;
            v += clampv(a * dt, -vmax, vmax);
            p += v * dt;
            R vn = length(v);
            V3<R> cp = clamp_box(p);
            R d = length(cp - p);
            if (d > 0 && vn > 0) {
                V3<R> nrm = normalize(signv(cp - p));
                R rest = d / (dt * vn);
                v -= ((R(1) + rest) * dot(v, nrm)) * nrm;
                p = cp;
            }
            st(pos, i, p, R(1));
            st(vel, i, v, R(0));
        }
        ids = ids_s;
    }

    /* kernels/boundary.cl:4-31 over each body's own particles (boundaryhandler.cpp:238-249).
     * Bodies above kBrute particles are summed over the same pairs (r^2 < h^2 within the
     * body) found through cells of the grid, in cell order, instead of the O(n^2) loop. */
    static constexpr int kBrute = 20000;
    void boundary_phi() {
        const R H = h_def, H2 = pown(H, 2);
        bphi.assign(NB, 0);
        for (auto& b : bodies) {
            if (b.count > kBrute) {
                std::vector<std::pair<long long, int>> cells(b.count);
                for (int ii = 0; ii < b.count; ++ii) {
                    int c[3];
                    coords(ld(bpos, b.origin + ii), c);
                    cells[ii] = {cell_id(c[0], c[1], c[2]), ii};
                }
                std::sort(cells.begin(), cells.end());
#pragma omp parallel for schedule(dynamic, 256)
                for (int ii = 0; ii < b.count; ++ii) {
                    int i = b.origin + ii;
                    V3<R> pi = ld(bpos, i);
                    int c[3];
                    coords(pi, c);
                    R del = 0;
                    for (int o = 0; o < 27; ++o) {
                        long long id;
                        if (!cell_ok(c[0] + kOff[o][0], c[1] + kOff[o][1], c[2] + kOff[o][2], id)) continue;
                        auto lo = std::lower_bound(cells.begin(), cells.end(), std::make_pair(id, -1));
                        for (auto it = lo; it != cells.end() && it->first == id; ++it) {
                            V3<R> r = pi - ld(bpos, b.origin + it->second);
                            R r2 = dot(r, r);
                            if (r2 < H2) del += mon ? w_monaghan(r2, H, H) : pown(pown(H, 2) - r2, 3);
                        }
                    }
                    bphi[i] = (rho0 / (del * boundary_eval)) / R(cfg.phi_coeff);
                }
                continue;
            }
#pragma omp parallel for schedule(static)
            for (int ii = 0; ii < b.count; ++ii) {
                int i = b.origin + ii;
                V3<R> pi = ld(bpos, i);
                R del = 0;
                for (int jj = 0; jj < b.count; ++jj) {
                    V3<R> r = pi - ld(bpos, b.origin + jj);
                    R r2 = dot(r, r);
                    if (r2 < H2) del += mon ? w_monaghan(r2, H, H) : pown(pown(H, 2) - r2, 3);
                }
                bphi[i] = (rho0 / (del * boundary_eval)) / R(cfg.phi_coeff);
            }
        }
    }
    /* kernels/boundary.cl:33-59 (P6 in PHYSICS) */
    void transform_body(Body& b) {
        V3<R> cm = v3<R>(b.rot[3], b.rot[7], b.rot[11]);
        V3<R> lin = v3<R>(b.lin[0], b.lin[1], b.lin[2]), ang = v3<R>(b.ang[0], b.ang[1], b.ang[2]);
        for (int ii = 0; ii < b.count; ++ii) {
            V3<R> r = v3<R>(b.raw[4 * ii], b.raw[4 * ii + 1], b.raw[4 * ii + 2]);
            V3<R> m0 = v3<R>(b.rot[0], b.rot[1], b.rot[2]), m1 = v3<R>(b.rot[4], b.rot[5], b.rot[6]),
                  m2 = v3<R>(b.rot[8], b.rot[9], b.rot[10]);
            V3<R> p = v3<R>(dot(m0, r), dot(m1, r), dot(m2, r)) + cm;
            V3<R> rel = p - cm;
            V3<R> v = compat ? lin + v3<R>(ang.x * rel.x, ang.y * rel.y, ang.z * rel.z) : lin + cross(ang, rel);
            st(bpos, b.origin + ii, p, R(1));
            st(bvel, b.origin + ii, v, R(0));
        }
    }
    /* boundaryhandler.cpp:216-236 */
    void boundary_sort() {
        if (NB == 0) return;
        compute_hashes(bpos, NB, bhashes, bmask);
        radix_sort_pairs(bhashes.data(), bmask.data(), NB);
        gather4(bpos, bmask, bpos_s, NB);
        bphi_s.resize(NB);
        for (int i = 0; i < NB; ++i) bphi_s[i] = bphi[bmask[i]];
        compute_intervals(bpos_s, bhashes, NB, bintervals);
    }
    /* boundaryhandler.cpp:251-294 */
    void boundary_sync(bool all) {
        if (NB == 0) return;
        bool any = all;
        for (auto& b : bodies)
            if (b.can_move || all) { transform_body(b); any = true; }
        if (any || bpos_s.empty()) boundary_sort();
    }
    /* kernels/boundary.cl:61-118 + clsum per body (boundaryhandler.cpp:296-349) */
    void boundary_forces() {
        body_force.assign(4 * bodies.size(), 0);
        body_torque.assign(4 * bodies.size(), 0);
        const R H = h_def;
        for (size_t bi = 0; bi < bodies.size(); ++bi) {
            Body& b = bodies[bi];
            if (!(b.mass > 0)) continue;
            V3<R> cm = v3<R>(b.rot[3], b.rot[7], b.rot[11]);
            V3<R> F = v3<R>(0, 0, 0), T = v3<R>(0, 0, 0);
            for (int ii = 0; ii < b.count; ++ii) {
                int i = b.origin + ii;
                V3<R> pi = ld(bpos, i);
                int c[3]; coords(pi, c);
                V3<R> f = v3<R>(0, 0, 0);
                int cnt = 0;
                for (int o = 0; cnt < cap && o < 27; ++o) {
                    long long id;
                    if (!cell_ok(c[0] + kOff[o][0], c[1] + kOff[o][1], c[2] + kOff[o][2], id)) continue;
                    for (int j = intervals[2 * id]; cnt < cap && j < intervals[2 * id + 1]; ++j) {
                        V3<R> r = ld(pos_s, j) - pi;
                        R rn = length(r);
                        if (rn < H) {
                            R C = pressure[j] / pown(density[j], 2);
                            ++cnt;
                            f += ((((r * (bforce_spiky / rn)) * pown(H - rn, 2)) * R(2)) * C);
                        }
                    }
                }
                f = f * (mass * bphi[i]);
                F += f;
                T += cross(pi - cm, f);
            }
            st(body_force, bi, F, R(0));
            st(body_torque, bi, T, R(0));
        }
    }

    /* Rigid-body step of every dynamic body (the GPU's k_body_integrate, same float
     * operations in the same order): semi-implicit Euler under the fluid force and torque
     * and gravity, orientation turned by |w| dt about w (Rodrigues), re-orthonormalised,
     * centre kept radius inside the container. */
    void integrate_bodies() {
        const float dt = cfg.time_step, g = -cfg.gravity;
        const float lx = cfg.container[0], ly = cfg.container[1], lz = cfg.container[2];
        for (size_t k = 0; k < bodies.size(); ++k) {
            Body& b = bodies[k];
            if (!b.dynamic) continue;
            float F[3], T[3];
            for (int a = 0; a < 3; ++a) { F[a] = float(body_force[4 * k + a]); T[a] = float(body_torque[4 * k + a]); }
            float* t = b.rot;     /* rot3x4 with the centre in t[3], t[7], t[11] */
            float* v = b.lin;
            float* w = b.ang;
            const float m = b.mass;
            const float ax = F[0] / m, ay = F[1] / m + g, az = F[2] / m;
            v[0] = v[0] + dt * ax; v[1] = v[1] + dt * ay; v[2] = v[2] + dt * az;
            t[3] = t[3] + dt * v[0]; t[7] = t[7] + dt * v[1]; t[11] = t[11] + dt * v[2];
            float r[9] = {t[0], t[1], t[2], t[4], t[5], t[6], t[8], t[9], t[10]};
            float y[3];
            for (int q = 0; q < 3; ++q) y[q] = (r[q] * T[0] + r[3 + q] * T[1] + r[6 + q] * T[2]) * b.inv_inertia[q];
            for (int i = 0; i < 3; ++i) w[i] = w[i] + dt * (r[3 * i] * y[0] + r[3 * i + 1] * y[1] + r[3 * i + 2] * y[2]);
            const float wn = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
            const float th = wn * dt;
            if (th > 0.f) {
                const float kx = w[0] / wn, ky = w[1] / wn, kz = w[2] / wn;
                const float cs = std::cos(th), sn = std::sin(th), C = 1.0f - cs;
                const float q[9] = {cs + kx * kx * C, kx * ky * C - kz * sn, kx * kz * C + ky * sn,
                                    ky * kx * C + kz * sn, cs + ky * ky * C, ky * kz * C - kx * sn,
                                    kz * kx * C - ky * sn, kz * ky * C + kx * sn, cs + kz * kz * C};
                float n[9];
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) n[3 * i + j] = q[3 * i] * r[j] + q[3 * i + 1] * r[3 + j] + q[3 * i + 2] * r[6 + j];
                const float l0 = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
                for (int j = 0; j < 3; ++j) n[j] /= l0;
                const float p = n[3] * n[0] + n[4] * n[1] + n[5] * n[2];
                for (int j = 0; j < 3; ++j) n[3 + j] -= p * n[j];
                const float l1 = std::sqrt(n[3] * n[3] + n[4] * n[4] + n[5] * n[5]);
                for (int j = 0; j < 3; ++j) n[3 + j] /= l1;
                n[6] = n[1] * n[5] - n[2] * n[4];
                n[7] = n[2] * n[3] - n[0] * n[5];
                n[8] = n[0] * n[4] - n[1] * n[3];
                t[0] = n[0]; t[1] = n[1]; t[2] = n[2];
                t[4] = n[3]; t[5] = n[4]; t[6] = n[5];
                t[8] = n[6]; t[9] = n[7]; t[10] = n[8];
            }
            if (b.radius > 0.f) {
                const float rad = b.radius;
                const float lo[3] = {-lx / 2.0f + rad, -ly / 2.0f + rad, -lz / 2.0f + rad};
                const float hi[3] = {lx / 2.0f - rad, 10.0f - rad, lz / 2.0f - rad};
                const int ci[3] = {3, 7, 11};
                for (int a = 0; a < 3; ++a) {
                    if (t[ci[a]] < lo[a]) { t[ci[a]] = lo[a]; if (v[a] < 0.f) v[a] = 0.f; }
                    else if (t[ci[a]] > hi[a]) { t[ci[a]] = hi[a]; if (v[a] > 0.f) v[a] = 0.f; }
                }
            }
        }
    }
    int set_body_dynamics(int body, int enabled, const float* ii, float radius) override {
        if (body < 0 || body >= (int)bodies.size()) return 1;
        Body& b = bodies[body];
        if (enabled && (!b.can_move || !(b.mass > 0))) return 1;
        b.dynamic = enabled ? 1 : 0;
        for (int a = 0; a < 3; ++a) b.inv_inertia[a] = enabled && ii ? ii[a] : 0.f;
        b.radius = enabled ? radius : 0.f;
        return 0;
    }
    int body_state(int body, float* rot, float* lin, float* ang) override {
        if (body < 0 || body >= (int)bodies.size()) return 1;
        const Body& b = bodies[body];
        if (rot) std::memcpy(rot, b.rot, sizeof b.rot);
        if (lin) std::memcpy(lin, b.lin, sizeof b.lin);
        if (ang) std::memcpy(ang, b.ang, sizeof b.ang);
        return 0;
    }

    int run_stage(int s) override {
        switch (s) {
        case ORC_S_BOUNDARY_SYNC: boundary_sync(false); break;
        case ORC_S_HASHES: compute_hashes(pos, N, hashes, mask); break;
        case ORC_S_SORT: radix_sort_pairs(hashes.data(), mask.data(), N); break;
        case ORC_S_SHUFFLE:
            gather4(pos, mask, pos_s, N);
            gather4(vel, mask, vel_s, N);
            if (cfg.method == 0) gather4(vel_half, mask, vel_half_s, N);
            ids_s.resize(N);
            for (int i = 0; i < N; ++i) ids_s[i] = ids[mask[i]];
            break;
        case ORC_S_CELL_INTERVALS: compute_intervals(pos_s, hashes, N, intervals); break;
        case ORC_S_NEIGH_LIST: neigh_list(pos_s, N, pos_s, intervals, nlist, nlen); break;
        case ORC_S_SB_NEIGH_LIST:
            if (NB > 0) neigh_list(pos_s, N, bpos_s, bintervals, sblist, sblen);
            else { sblist.assign((size_t)cap * std::max(N, 1), 0); sblen.assign(N, 0); }
            break;
        case ORC_S_WC_DENSITY: wc_density(); break;
        case ORC_S_NORMALS: normals(); break;
        case ORC_S_WC_ACCEL: wc_accel(); break;
        case ORC_S_WC_INTEGRATE: wc_integrate(); break;
        case ORC_S_PCI_INIT_DENSITY: pressure.assign(N, 0); pci_init_density(); break;
        case ORC_S_PCI_INIT_FORCES: f_press.assign(4 * (size_t)N, 0); pci_init_forces(); break;
        case ORC_S_PCI_LOOP: pci_loop(cfg.pci_min_iter, cfg.pci_max_iter); break;
        case ORC_S_PCI_INTEGRATE: pci_integrate(); break;
        case ORC_S_BOUNDARY_FORCES: boundary_forces(); integrate_bodies(); break;
        /* one iteration's passes alone (pcisph.cl:302-344, :349-418, :420-504) */
        case ORC_S_PCI_PREDICT: pci_predict(); break;
        case ORC_S_PCI_UPDATE_PRESSURE: pci_update_pressure(); break;
        case ORC_S_PCI_PRESSURE_FORCE: pci_pressure_force(); break;
        default: return 1;
        }
        return 0;
    }
    void pci_step(int min_iter, int max_iter) {
        const int pre[] = {ORC_S_BOUNDARY_SYNC, ORC_S_HASHES, ORC_S_SORT, ORC_S_SHUFFLE,
                           ORC_S_CELL_INTERVALS, ORC_S_NEIGH_LIST, ORC_S_SB_NEIGH_LIST,
                           ORC_S_PCI_INIT_DENSITY, ORC_S_NORMALS, ORC_S_PCI_INIT_FORCES};
        for (int s : pre) run_stage(s);
        pci_loop(min_iter, max_iter);
        run_stage(ORC_S_BOUNDARY_FORCES);
        run_stage(ORC_S_PCI_INTEGRATE);
    }
    int step(int n) override {
        for (int k = 0; k < n; ++k) {
            if (cfg.method == 0) {
                const int seq[] = {ORC_S_BOUNDARY_SYNC, ORC_S_HASHES, ORC_S_SORT, ORC_S_SHUFFLE,
                                   ORC_S_CELL_INTERVALS, ORC_S_NEIGH_LIST, ORC_S_SB_NEIGH_LIST,
                                   ORC_S_WC_DENSITY, ORC_S_NORMALS, ORC_S_WC_ACCEL,
                                   ORC_S_BOUNDARY_FORCES, ORC_S_WC_INTEGRATE};
                for (int s : seq) run_stage(s);
            } else {
                pci_step(cfg.pci_min_iter, cfg.pci_max_iter);
            }
        }
        return 0;
    }

    int set_fluid(const float* p, const float* v, int n) override {
        N = n;
        pos.assign(4 * (size_t)n, 0); vel.assign(4 * (size_t)n, 0); vel_half.assign(4 * (size_t)n, 0);
        ids.resize(n);
        for (int i = 0; i < n; ++i) {
            for (int k = 0; k < 3; ++k) {
                pos[4 * (size_t)i + k] = p[4 * (size_t)i + k];
                if (v) { vel[4 * (size_t)i + k] = v[4 * (size_t)i + k]; vel_half[4 * (size_t)i + k] = v[4 * (size_t)i + k]; }
            }
            pos[4 * (size_t)i + 3] = 1;
            ids[i] = i;
        }
        hashes.assign(n, 0); mask.assign(n, 0);
        density.assign(n, 0); pressure.assign(n, 0); normal.assign(4 * (size_t)n, 0);
        accel.assign(4 * (size_t)n, 0); pos_pred.assign(4 * (size_t)n, 0);
        f_other.assign(4 * (size_t)n, 0); f_press.assign(4 * (size_t)n, 0); dens_var.assign(n, 0);
        pos_s = pos; vel_s = vel; vel_half_s = vel_half; ids_s = ids;
        intervals.assign(2 * gcells, 0);
        nlist.assign((size_t)cap * std::max(n, 1), 0); nlen.assign(n, 0);
        sblist.assign((size_t)cap * std::max(n, 1), 0); sblen.assign(n, 0);
        /* pcisphsimluation.cpp:548-550: one relaxation step, then zero velocities */
        if (cfg.method == 1 && cfg.relax_on_add && n > 0) {
            pci_step(cfg.pci_min_iter, cfg.pci_relax_max_iter > 0 ? cfg.pci_relax_max_iter : 10000);
            std::fill(vel.begin(), vel.end(), R(0));
        }
        return 0;
    }
    /* boundaryhandler.cpp:119-153: append, recompute phi on the raw sampling, sync(true) */
    int add_boundary(const float* p, int n, int mv, const float* rot, const float* lin, const float* ang,
                     float m) override {
        Body b;
        b.raw.assign(p, p + 4 * (size_t)n);
        for (int i = 0; i < n; ++i) b.raw[4 * (size_t)i + 3] = 1;
        b.count = n; b.origin = NB; b.can_move = mv; b.mass = m;
        static const float I[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
        std::memcpy(b.rot, rot ? rot : I, sizeof b.rot);
        for (int k = 0; k < 4; ++k) { b.lin[k] = lin ? lin[k] : 0; b.ang[k] = ang ? ang[k] : 0; }
        bodies.push_back(b);
        NB += n;
        bpos.assign(4 * (size_t)NB, 0); bvel.assign(4 * (size_t)NB, 0);
        for (auto& bb : bodies)
            for (int i = 0; i < bb.count; ++i)
                for (int k = 0; k < 4; ++k) bpos[4 * (size_t)(bb.origin + i) + k] = bb.raw[4 * (size_t)i + k];
        boundary_phi();
        boundary_sync(true);
        return 0;
    }

    void* fptr(int f, long long& n, int& kd) {
        kd = 0;
        switch (f) {
        case ORC_F_POS: n = pos.size(); return pos.data();
        case ORC_F_VEL: n = vel.size(); return vel.data();
        case ORC_F_VEL_HALF: n = vel_half.size(); return vel_half.data();
        case ORC_F_POS_SORTED: n = pos_s.size(); return pos_s.data();
        case ORC_F_VEL_SORTED: n = vel_s.size(); return vel_s.data();
        case ORC_F_VEL_HALF_SORTED: n = vel_half_s.size(); return vel_half_s.data();
        case ORC_F_HASHES: kd = 2; n = hashes.size(); return hashes.data();
        case ORC_F_MASK: kd = 1; n = mask.size(); return mask.data();
        case ORC_F_CELL_INTERVALS: kd = 1; n = intervals.size(); return intervals.data();
        case ORC_F_NEIGH_LIST: kd = 1; n = nlist.size(); return nlist.data();
        case ORC_F_NEIGH_LEN: kd = 1; n = nlen.size(); return nlen.data();
        case ORC_F_SB_NEIGH_LIST: kd = 1; n = sblist.size(); return sblist.data();
        case ORC_F_SB_NEIGH_LEN: kd = 1; n = sblen.size(); return sblen.data();
        case ORC_F_DENSITY: n = density.size(); return density.data();
        case ORC_F_PRESSURE: n = pressure.size(); return pressure.data();
        case ORC_F_NORMAL: n = normal.size(); return normal.data();
        case ORC_F_ACCEL: n = accel.size(); return accel.data();
        case ORC_F_POS_PRED: n = pos_pred.size(); return pos_pred.data();
        case ORC_F_FORCE_OTHER: n = f_other.size(); return f_other.data();
        case ORC_F_FORCE_PRESSURE: n = f_press.size(); return f_press.data();
        case ORC_F_DENS_VAR: n = dens_var.size(); return dens_var.data();
        case ORC_F_BPOS_SORTED: n = bpos_s.size(); return bpos_s.data();
        case ORC_F_BPHI_SORTED: n = bphi_s.size(); return bphi_s.data();
        case ORC_F_BCELL_INTERVALS: kd = 1; n = bintervals.size(); return bintervals.data();
        case ORC_F_BHASHES: kd = 2; n = bhashes.size(); return bhashes.data();
        case ORC_F_BMASK: kd = 1; n = bmask.size(); return bmask.data();
        case ORC_F_BPHI: n = bphi.size(); return bphi.data();
        case ORC_F_BPOS: n = bpos.size(); return bpos.data();
        case ORC_F_BODY_FORCE: n = body_force.size(); return body_force.data();
        case ORC_F_BODY_TORQUE: n = body_torque.size(); return body_torque.data();
        case ORC_F_PCI_ITERS: kd = 1; n = 1; return &pci_iters;
        case ORC_F_PCI_MAXERR: n = pci_maxerr.size(); return pci_maxerr.data();
        case ORC_F_ID: kd = 1; n = ids.size(); return ids.data();
        }
        n = -1;
        return nullptr;
    }
    long long elems(int f) override { long long n; int k; fptr(f, n, k); return n; }
    int kind(int f) override { long long n; int k; fptr(f, n, k); return k; }
    int get(int f, void* out) override {
        long long n; int k; void* p = fptr(f, n, k);
        if (n < 0) return 1;
        std::memcpy(out, p, (size_t)n * (k == 0 ? sizeof(R) : 4));
        return 0;
    }
    int set(int f, const void* in) override {
        long long n; int k; void* p = fptr(f, n, k);
        if (n < 0) return 1;
        std::memcpy(p, in, (size_t)n * (k == 0 ? sizeof(R) : 4));
        return 0;
    }
    void derived(OrcDerived* d) override {
        d->mass = float(mass); d->mass_def = float(mass_def); d->h = float(h); d->h_def = float(h_def);
        d->rest_density_def = float(rho0_def);
        d->poly6_eval = float(poly6_eval); d->poly6_grad = float(poly6_grad); d->spiky_grad = float(spiky_grad);
        d->visc_lapl = float(visc_lapl); d->st_main = float(st_main); d->st_term = float(st_term);
        d->default_eval = float(default_eval); d->boundary_eval = float(boundary_eval); d->pci_delta = float(delta);
        for (int a = 0; a < 3; ++a) { d->grid_origin[a] = gorigin_f[a]; d->grid_dims[a] = gn[a]; }
        d->grid_wrap = gwrap; d->key_bits = key_bits;
    }
    void stats(double* out) override {
        double comp = 0, abse = 0, mxe = -1e300, ke = 0, pe = 0, cx = 0, cy = 0, cz = 0;
        for (int i = 0; i < N; ++i) {
            double e = (double(density[i]) - double(rho0)) / double(rho0);
            comp += std::max(e, 0.0); abse += std::fabs(e); mxe = std::max(mxe, e);
        }
        for (int i = 0; i < N; ++i) {
            V3<R> p = ld(pos, i), v = ld(vel, i);
            ke += 0.5 * double(mass) * double(dot(v, v));
            pe += double(mass) * double(cfg.gravity) * double(p.y);
            cx += p.x; cy += p.y; cz += p.z;
        }
        double inv = N > 0 ? 1.0 / N : 0.0;
        out[0] = comp * inv; out[1] = abse * inv; out[2] = N > 0 ? mxe : 0.0;
        out[3] = ke; out[4] = pe; out[5] = cx * inv; out[6] = cy * inv; out[7] = cz * inv;
    }
};

}  // namespace

extern "C" {

void* orc_create(const OrcConfig* cfg) {
    if (!cfg) return nullptr;
#ifdef _OPENMP
    if (cfg->threads > 0) omp_set_num_threads(cfg->threads);
#endif
    if (cfg->precision == 1) return static_cast<OracleBase*>(new Oracle<double>(*cfg));
    return static_cast<OracleBase*>(new Oracle<float>(*cfg));
}
void orc_destroy(void* o) { delete static_cast<OracleBase*>(o); }
int orc_set_fluid(void* o, const float* p, const float* v, int n) {
    return static_cast<OracleBase*>(o)->set_fluid(p, v, n);
}
int orc_add_boundary(void* o, const float* p, int n, int mv, const float* rot, const float* lin,
                     const float* ang, float mass) {
    return static_cast<OracleBase*>(o)->add_boundary(p, n, mv, rot, lin, ang, mass);
}
int orc_run_stage(void* o, int s) { return static_cast<OracleBase*>(o)->run_stage(s); }
int orc_step(void* o, int n) { return static_cast<OracleBase*>(o)->step(n); }
long long orc_field_elems(void* o, int f) { return static_cast<OracleBase*>(o)->elems(f); }
int orc_field_kind(void* o, int f) { return static_cast<OracleBase*>(o)->kind(f); }
int orc_get(void* o, int f, void* out) { return static_cast<OracleBase*>(o)->get(f, out); }
int orc_set(void* o, int f, const void* in) { return static_cast<OracleBase*>(o)->set(f, in); }
int orc_derived(void* o, OrcDerived* d) { static_cast<OracleBase*>(o)->derived(d); return 0; }
uint32_t orc_morton3(uint32_t x, uint32_t y, uint32_t z) { return morton3(x, y, z); }
void orc_stable_sort_pairs(uint32_t* k, int32_t* v, int n) { radix_sort_pairs(k, v, n); }
int orc_stats(void* o, double* out) { static_cast<OracleBase*>(o)->stats(out); return 0; }
int orc_set_body_dynamics(void* o, int body, int enabled, const float* inv_inertia3, float radius) {
    return static_cast<OracleBase*>(o)->set_body_dynamics(body, enabled, inv_inertia3, radius);
}
int orc_body_state(void* o, int body, float* rot12, float* lin4, float* ang4) {
    return static_cast<OracleBase*>(o)->body_state(body, rot12, lin4, ang4);
}

}  // extern "C"
