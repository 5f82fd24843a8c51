/*
 * sph_adjoint_oracle.cpp -- TEST INFRASTRUCTURE: FP64 CPU restatement of the differentiable
 * WCSPH step (PHYSICS mode, no boundary, no surface tension) and of its adjoint.
 *
 * Used only by the tests and never by the library.  The forward step follows the
 * reference's WCSPH step (fluid/simulation/wcsphsimluation.cpp:40-106; kernels/wcsph.cl:32-79
 * density and Tait pressure, :81-173 pressure and viscosity acceleration with the mass
 * factors of kernels/pcisph.cl:216-219, :176-224 leapfrog integration with the velocity
 * clamps and the container reflection), in double precision and in particle-id order,
 * with complete neighbour sets (every j with r^2 < h^2, no cap).  The backward pass is the
 * reverse-mode derivative of that step, written independently of the CUDA kernels: it
 * scatters each pair's contribution to both particles instead of relying on symmetric
 * lists, and it recomputes each step's neighbour sets from the stored trajectory.  Clamps
 * and the Tait max(0, .) take the subgradients the CUDA adjoint documents (1 strictly
 * inside a clamp, 0 outside; reflection not differentiated).
 */
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif
#include <cmath>
#include <cstdint>
#include <unordered_map>
#include <vector>

extern "C" {
struct OrcAdjParams {
    double h, hh, h2_list, mass, rho0, kgas, mu, g, dt, vmax;
    double lim[3];
    double poly6, spiky, visc_lapl, rmin2;
    int steps;
    int threads;
};
}

namespace {

struct V3 {
    double x, y, z;
};

/* neighbour sets by a hashed cell grid of cell size h (order irrelevant in FP64) */
void neighbours(const OrcAdjParams& P, int n, const std::vector<V3>& x, std::vector<std::vector<int>>& nb) {
    const double cs = P.h;
    std::unordered_map<int64_t, std::vector<int>> cells;
    auto key = [](int64_t a, int64_t b, int64_t c) {
        return ((a + (1 << 20)) << 42) ^ ((b + (1 << 20)) << 21) ^ (c + (1 << 20));
    };
    std::vector<int64_t> cx(n), cy(n), cz(n);
    for (int i = 0; i < n; ++i) {
        cx[i] = (int64_t)std::floor(x[i].x / cs);
        cy[i] = (int64_t)std::floor(x[i].y / cs);
        cz[i] = (int64_t)std::floor(x[i].z / cs);
        cells[key(cx[i], cy[i], cz[i])].push_back(i);
    }
    nb.assign(n, {});
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        for (int dx = -1; dx <= 1; ++dx)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dz = -1; dz <= 1; ++dz) {
                    auto it = cells.find(key(cx[i] + dx, cy[i] + dy, cz[i] + dz));
                    if (it == cells.end()) continue;
                    for (int j : it->second) {
                        const double ddx = x[i].x - x[j].x, ddy = x[i].y - x[j].y, ddz = x[i].z - x[j].z;
                        if (ddx * ddx + ddy * ddy + ddz * ddz < P.h2_list) nb[i].push_back(j);
                    }
                }
    }
}

double clampd(double v, double lo, double hi) { return std::min(std::max(v, lo), hi); }

struct StepOut {
    std::vector<double> rho, p;
    std::vector<V3> a;
};

/* density, pressure, acceleration of one state */
void forces(const OrcAdjParams& P, int n, const std::vector<V3>& x, const std::vector<V3>& v,
            const std::vector<std::vector<int>>& nb, StepOut& o) {
    o.rho.assign(n, 0.0);
    o.p.assign(n, 0.0);
    o.a.assign(n, V3{0, 0, 0});
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        double s = 0.0;
        for (int j : nb[i]) {
            const double dx = x[i].x - x[j].x, dy = x[i].y - x[j].y, dz = x[i].z - x[j].z;
            const double t = P.hh - (dx * dx + dy * dy + dz * dz);
            s += t * t * t;
        }
        const double rho = P.poly6 * P.mass * s;
        const double q = rho / P.rho0;
        const double pv = P.kgas * (std::pow(q, 7) - 1.0);
        o.rho[i] = rho;
        o.p[i] = pv > 0.0 ? pv : 0.0;
    }
    const double K = P.visc_lapl * P.mu * P.mass;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        V3 a{0.0, P.g, 0.0};
        const double ri = o.rho[i];
        if (ri > 0.0) {
            const double Ci = o.p[i] / (ri * ri);
            for (int j : nb[i]) {
                const double rj = o.rho[j];
                const double dx = x[i].x - x[j].x, dy = x[i].y - x[j].y, dz = x[i].z - x[j].z;
                const double r2 = dx * dx + dy * dy + dz * dz;
                if (!(rj > 0.0 && r2 > P.rmin2)) continue;
                const double r = std::sqrt(r2), w = P.h - r;
                const double Cj = o.p[j] / (rj * rj);
                const double fp = -P.mass * P.spiky * (w * w / r) * (Ci + Cj);
                const double fv = K * w / (ri * rj);
                a.x += fp * dx + fv * (v[j].x - v[i].x);
                a.y += fp * dy + fv * (v[j].y - v[i].y);
                a.z += fp * dz + fv * (v[j].z - v[i].z);
            }
        }
        o.a[i] = a;
    }
}

void integrate(const OrcAdjParams& P, int n, std::vector<V3>& x, std::vector<V3>& v, std::vector<V3>& u,
               const std::vector<V3>& a) {
    const double dt = P.dt, vm = P.vmax;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        double vh[3] = {u[i].x + dt * a[i].x, u[i].y + dt * a[i].y, u[i].z + dt * a[i].z};
        const double av[3] = {a[i].x, a[i].y, a[i].z};
        double p[3] = {x[i].x, x[i].y, x[i].z};
        for (int k = 0; k < 3; ++k) p[k] += dt * clampd(vh[k] + dt * av[k], -vm, vm);
        const double vn = std::sqrt(vh[0] * vh[0] + vh[1] * vh[1] + vh[2] * vh[2]);
        const double c[3] = {clampd(p[0], -P.lim[0] / 2, P.lim[0] / 2), clampd(p[1], -P.lim[1] / 2, 10.0),
                             clampd(p[2], -P.lim[2] / 2, P.lim[2] / 2)};
        const double e[3] = {c[0] - p[0], c[1] - p[1], c[2] - p[2]};
        const double d = std::sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
        if (d > 0.0 && vn > 0.0) {
            double s[3];
            for (int k = 0; k < 3; ++k) s[k] = e[k] > 0 ? 1.0 : (e[k] < 0 ? -1.0 : 0.0);
            const double sl = std::sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
            for (double& t : s) t /= sl;
            const double rest = d / (dt * vn);
            const double kk = (1.0 + rest) * (vh[0] * s[0] + vh[1] * s[1] + vh[2] * s[2]);
            for (int k = 0; k < 3; ++k) {
                vh[k] -= kk * s[k];
                p[k] = c[k];
            }
        }
        x[i] = V3{p[0], p[1], p[2]};
        v[i] = V3{clampd(vh[0] + 0.5 * dt * av[0], -vm, vm), clampd(vh[1] + 0.5 * dt * av[1], -vm, vm),
                  clampd(vh[2] + 0.5 * dt * av[2], -vm, vm)};
        u[i] = V3{clampd(vh[0], -vm, vm), clampd(vh[1], -vm, vm), clampd(vh[2], -vm, vm)};
    }
}

std::vector<V3> load(const double* a, int n) {
    std::vector<V3> r(n);
    for (int i = 0; i < n; ++i) r[i] = V3{a[3 * i], a[3 * i + 1], a[3 * i + 2]};
    return r;
}
void store(const std::vector<V3>& r, double* a) {
    for (size_t i = 0; i < r.size(); ++i) {
        a[3 * i] = r[i].x;
        a[3 * i + 1] = r[i].y;
        a[3 * i + 2] = r[i].z;
    }
}
bool in_open(double x, double vm) { return x > -vm && x < vm; }

}  // namespace

extern "C" {

int orc_adj_forward(const OrcAdjParams* P, int n, const double* x0, const double* v0, double* xT, double* vT,
                    int* max_neigh) {
#ifdef _OPENMP
    if (P->threads > 0) omp_set_num_threads(P->threads);
#endif
    std::vector<V3> x = load(x0, n), v = load(v0, n), u = v;
    std::vector<std::vector<int>> nb;
    StepOut o;
    int mx = 0;
    for (int t = 0; t < P->steps; ++t) {
        neighbours(*P, n, x, nb);
        for (auto& l : nb) mx = std::max(mx, (int)l.size());
        forces(*P, n, x, v, nb, o);
        integrate(*P, n, x, v, u, o.a);
    }
    if (xT) store(x, xT);
    if (vT) store(v, vT);
    if (max_neigh) *max_neigh = mx;
    return 0;
}

int orc_adj_backward(const OrcAdjParams* P, int n, const double* x0, const double* v0, const double* gxT,
                     const double* gvT, double* gx0, double* gv0, double* gmu, double* gk) {
    const int T = P->steps;
    std::vector<std::vector<V3>> X(T + 1), Vv(T + 1), U(T + 1);
    std::vector<StepOut> O(T);
    X[0] = load(x0, n);
    Vv[0] = load(v0, n);
    U[0] = Vv[0];
    std::vector<std::vector<int>> nb;
    for (int t = 0; t < T; ++t) {
        neighbours(*P, n, X[t], nb);
        forces(*P, n, X[t], Vv[t], nb, O[t]);
        X[t + 1] = X[t];
        Vv[t + 1] = Vv[t];
        U[t + 1] = U[t];
        integrate(*P, n, X[t + 1], Vv[t + 1], U[t + 1], O[t].a);
    }
    std::vector<V3> lx = load(gxT, n), lv(n, V3{0, 0, 0}), lu(n, V3{0, 0, 0});
    if (gvT) lv = load(gvT, n);
    double sum_mu = 0.0, sum_k = 0.0;
    const double dt = P->dt, vm = P->vmax, K = P->visc_lapl * P->mu * P->mass;
    for (int t = T - 1; t >= 0; --t) {
        const std::vector<V3>& x = X[t];
        const std::vector<V3>& v = Vv[t];
        const StepOut& o = O[t];
        neighbours(*P, n, x, nb);
        /* integrate */
        std::vector<V3> la(n), nlu(n);
        for (int i = 0; i < n; ++i) {
            const double av[3] = {o.a[i].x, o.a[i].y, o.a[i].z};
            const double uu[3] = {U[t][i].x, U[t][i].y, U[t][i].z};
            const double gx[3] = {lx[i].x, lx[i].y, lx[i].z}, gv[3] = {lv[i].x, lv[i].y, lv[i].z},
                         gu[3] = {lu[i].x, lu[i].y, lu[i].z};
            double ra[3], ru[3];
            for (int k = 0; k < 3; ++k) {
                const double vh = uu[k] + dt * av[k];
                const double mp = in_open(vh + dt * av[k], vm) ? 1.0 : 0.0;
                const double mv = in_open(vh + 0.5 * dt * av[k], vm) ? 1.0 : 0.0;
                const double mu_ = in_open(vh, vm) ? 1.0 : 0.0;
                const double gvh = dt * mp * gx[k] + mv * gv[k] + mu_ * gu[k];
                ra[k] = dt * gvh + dt * dt * mp * gx[k] + 0.5 * dt * mv * gv[k];
                ru[k] = gvh;
            }
            la[i] = V3{ra[0], ra[1], ra[2]};
            nlu[i] = V3{ru[0], ru[1], ru[2]};
        }
        /* forces: scatter every ordered pair (i, j) of a_i to both particles */
        std::vector<double> lC(n, 0.0), lR(n, 0.0);
        std::vector<V3> nlx = lx, nlv(n, V3{0, 0, 0});
        for (int i = 0; i < n; ++i) {
            const double ri = o.rho[i];
            if (!(ri > 0.0)) continue;
            const double Ci = o.p[i] / (ri * ri), Ri = 1.0 / ri;
            const V3 A = la[i];
            double sm[3] = {0, 0, 0};
            for (int j : nb[i]) {
                const double rj = o.rho[j];
                const double dx = x[i].x - x[j].x, dy = x[i].y - x[j].y, dz = x[i].z - x[j].z;
                const double r2 = dx * dx + dy * dy + dz * dz;
                if (!(rj > 0.0 && r2 > P->rmin2)) continue;
                const double r = std::sqrt(r2), w = P->h - r;
                const double Cj = o.p[j] / (rj * rj), Rj = 1.0 / rj;
                const double d[3] = {dx, dy, dz};
                const double Av[3] = {A.x, A.y, A.z};
                const double dA = dx * A.x + dy * A.y + dz * A.z;
                /* pressure term f = c0 (Ci + Cj) s(r) d, c0 = -m spiky, s = w^2 / r */
                const double c0 = -P->mass * P->spiky, s = w * w / r, sp = -w * (P->h + r) / (r * r);
                lC[i] += c0 * s * dA;
                lC[j] += c0 * s * dA;
                double g[3];
                for (int k = 0; k < 3; ++k) g[k] = c0 * (Ci + Cj) * (s * Av[k] + sp * dA * d[k] / r);
                /* viscosity term f = K Ri Rj w (vj - vi) */
                const double dv[3] = {v[j].x - v[i].x, v[j].y - v[i].y, v[j].z - v[i].z};
                const double dvA = dv[0] * A.x + dv[1] * A.y + dv[2] * A.z;
                lR[i] += K * Rj * w * dvA;
                lR[j] += K * Ri * w * dvA;
                for (int k = 0; k < 3; ++k) g[k] += -K * Ri * Rj * dvA * d[k] / r;
                nlx[i].x += g[0]; nlx[i].y += g[1]; nlx[i].z += g[2];
                nlx[j].x -= g[0]; nlx[j].y -= g[1]; nlx[j].z -= g[2];
                const double cv = K * Ri * Rj * w;
                nlv[j].x += cv * A.x; nlv[j].y += cv * A.y; nlv[j].z += cv * A.z;
                nlv[i].x -= cv * A.x; nlv[i].y -= cv * A.y; nlv[i].z -= cv * A.z;
                for (int k = 0; k < 3; ++k) sm[k] += Rj * w * dv[k];
            }
            sum_mu += P->visc_lapl * P->mass * Ri * (sm[0] * A.x + sm[1] * A.y + sm[2] * A.z);
        }
        /* pressure / density chain */
        std::vector<double> lrho(n, 0.0);
        for (int i = 0; i < n; ++i) {
            const double rho = o.rho[i];
            if (!(rho > 0.0)) continue;
            const double q = rho / P->rho0, pv = P->kgas * (std::pow(q, 7) - 1.0);
            const bool act = pv > 0.0;
            const double dp = act ? 7.0 * P->kgas * std::pow(q, 6) / P->rho0 : 0.0;
            const double dpk = act ? std::pow(q, 7) - 1.0 : 0.0;
            lrho[i] = lC[i] * (dp / (rho * rho) - 2.0 * o.p[i] / (rho * rho * rho)) - lR[i] / (rho * rho);
            sum_k += lC[i] * dpk / (rho * rho);
        }
        /* density: rho_i = poly6 m sum_j (hh - r^2)^3 */
        for (int i = 0; i < n; ++i)
            for (int j : nb[i]) {
                if (j == i) continue;
                const double dx = x[i].x - x[j].x, dy = x[i].y - x[j].y, dz = x[i].z - x[j].z;
                const double t = P->hh - (dx * dx + dy * dy + dz * dz);
                const double q = -6.0 * P->poly6 * P->mass * t * t * lrho[i];
                nlx[i].x += q * dx; nlx[i].y += q * dy; nlx[i].z += q * dz;
                nlx[j].x -= q * dx; nlx[j].y -= q * dy; nlx[j].z -= q * dz;
            }
        lx = nlx;
        lv = nlv;
        lu = nlu;
    }
    if (gx0) store(lx, gx0);
    if (gv0) {
        std::vector<V3> g(n);
        for (int i = 0; i < n; ++i) g[i] = V3{lv[i].x + lu[i].x, lv[i].y + lu[i].y, lv[i].z + lu[i].z};
        store(g, gv0);
    }
    if (gmu) *gmu = sum_mu;
    if (gk) *gk = sum_k;
    return 0;
}

}  // extern "C"
