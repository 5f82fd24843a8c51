/*
 * sph_context.cu -- the solver context behind include/sph_capi.h.
 *
 * Host responsibilities of the reference's solver classes, GB300-first:
 *   - constants: fluid/simulation/wcsphsimluation.cpp:165-202, pcisphsimluation.cpp:230-278,
 *     429-469 (PCISPH delta), mullerconstants.cpp:4-38, boundaryhandler.cpp:144,306-309,
 *     grid.cpp:61-68, and the 6-decimal -D rounding of opencl/clcompiler.cpp:50-54;
 *   - memory: one device arena per context holding every SoA array (replaces CLAllocator,
 *     opencl/clallocator.h), carved by carve() below;
 *   - the step: WCSPHSimulation::simulate (wcsphsimluation.cpp:40-106) and
 *     PCISPHSimulation::_simulate_pcisph_step (pcisphsimluation.cpp:72-165) as one sequence
 *     of launches on the context stream, captured once into a CUDA graph and replayed;
 *   - boundary handling: BoundaryHandler (boundaryhandler.cpp:95-349); static bodies are
 *     transformed, sorted and given their Psi once, not re-sorted every step.
 */
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "sph_ctx.cuh"

namespace {
std::mutex g_err_mu;
std::string g_last_create_error;

int fail(sph_ctx* x, int code, const std::string& msg) {
    if (x) x->err = msg;
    else {
        std::lock_guard<std::mutex> lk(g_err_mu);
        g_last_create_error = msg;
    }
    return code;
}
int cuda_fail(sph_ctx* x, cudaError_t e, const char* where) {
    return fail(x, SPH_E_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}
#define SPH_CUDA(x, call)                                 \
    do {                                                  \
        cudaError_t _e = (call);                          \
        if (_e != cudaSuccess) return cuda_fail(x, _e, #call); \
    } while (0)

float round6(float v) {
    char buf[64];
    snprintf(buf, sizeof buf, "%.6f", (double)v);
    return strtof(buf, nullptr);
}

/* pcisphsimluation.cpp:429-469, float arithmetic as written there */
float pci_delta(float h, float r, float mass, float rho0, float dt, float spiky, float poly) {
    const float sqr_h = h * h;
    float beta = 2.0f * std::pow((dt * mass) / rho0, 2.0f);
    float vs[3] = {0.f, 0.f, 0.f}, ss[3] = {0.f, 0.f, 0.f}, vdv = 0.f;
    for (float x = -h - r; x <= h + r; x += 2.0f * r)
        for (float y = -h - r; y <= h + r; y += 2.0f * r)
            for (float z = -h - r; z <= h + r; z += 2.0f * r) {
                float r2 = (x * x + y * y + z * z);
                float rn = std::sqrt(r2);
                if (r2 < sqr_h) {
                    float sf = spiky * (h - rn) * (h - rn) * (1.0 / rn);
                    float f = poly * (sqr_h - r2) * (sqr_h - r2);
                    float sv[3] = {sf * x, sf * y, sf * z};
                    float v[3] = {f * x, f * y, f * z};
                    for (int i = 0; i < 3; i++) {
                        vs[i] += v[i];
                        ss[i] += sv[i];
                        vdv += v[i] * sv[i];
                    }
                }
            }
    float sds = 0.f;
    for (int i = 0; i < 3; i++) sds += ss[i] * vs[i];
    return -1.0f / (beta * (-sds - vdv));
}

int derive(sph_ctx* x) {
    const sph_params& p = x->p;
    Const& c = x->c;
    c = Const{};
    const bool compat = p.mode == SPH_MODE_COMPAT;
    const float h = p.support_radius, r = p.particle_radius, rho0 = p.rest_density;
    if (!(h > 0.f) || !(r > 0.f) || !(rho0 > 0.f) || !(p.time_step > 0.f))
        return fail(x, SPH_E_INVALID, "support_radius, particle_radius, rest_density and time_step must be > 0");
    c.compat = compat ? 1 : 0;
    c.monaghan = (compat && p.kernels == SPH_KERNELS_MONAGHAN) ? 1 : 0;
    c.cap = p.neigh_cap > 0 ? p.neigh_cap : 50;
    c.h = h;
    c.h_def = round6(h);
    c.h2_list = c.h_def * c.h_def;
    c.rho0 = rho0;
    c.mu = p.k_viscosity;
    c.sigma = p.surface_tension;
    c.kgas = p.gas_stiffness;
    c.g = -p.gravity;
    c.dt = p.time_step;
    c.vmax = p.max_vel;
    c.lim_x = x->lim[0];
    c.lim_y = x->lim[1];
    c.lim_z = x->lim[2];
    c.pci_eta = p.pcisph_error_ratio;
    c.pci_min_iter = p.pcisph_min_iterations;
    c.pci_max_iter = p.pcisph_max_iterations;
    float t = 1e-5f;
    if ((double)t > 1e-5) t = std::nextafter(t, 0.0f);
    c.rmin_wc = t;
    c.rmin2_wc = t * t;
    /* cell skipping bound with a 1e-3 relative margin, far above the rounding of the cell
     * coordinates (<= 2^-13 cell units for grids up to 1024 cells per axis) */
    c.cull2 = (c.h2_list / (h * h)) * 1.001f;
    if (p.method == SPH_WCSPH) {
        const float mf = rho0 * std::pow(2.0f * r, 3.0f) / 1.0f;
        c.mass = mf;
        c.mass_def = round6(mf);
        c.rho0_def = rho0;
        c.poly6_eval = (float)(315.0 / (64.0 * M_PI * std::pow((double)h, 9.0)));
        c.poly6_grad = (float)(-945.0 / (32.0 * M_PI * std::pow((double)h, 9.0)));
        c.spiky_grad = (float)(-45.0 / (M_PI * std::pow((double)h, 6.0)));
        c.visc_lapl = (float)(45.0 / (M_PI * std::pow((double)h, 6.0)));
        c.default_eval = c.poly6_eval;
    } else {
        const float mf = rho0 * std::pow(2.0f * r, 3.0f) / (compat ? 1.15f : 1.0f);
        c.mass = mf;
        c.mass_def = round6(mf);
        c.rho0_def = round6(rho0);
        const float e = compat ? 365.0f : 315.0f;
        c.default_eval = (float)(e / (64.0f * M_PI * std::pow(h, 9.0f)));
        c.poly6_grad = (float)(-945.0f / (32.0f * M_PI * std::pow(h, 9.0f)));
        c.visc_lapl = (float)(45.0f / (M_PI * std::pow(h, 6.0f)));
        c.spiky_grad = (float)(-45.0f / (M_PI * std::pow(h, 6.0f)));
        c.poly6_eval = c.default_eval;
        c.delta = pci_delta(h, r, mf, rho0, p.time_step, c.spiky_grad, c.poly6_grad);
    }
    c.st_main = (float)(32.0f / (M_PI * std::pow(h, 9.0f)));
    c.st_term = std::pow(h, 6.0f) / 64.0f;
    {
        const float e = compat ? 365.0f : 315.0f;
        c.boundary_eval = (float)(e / (64.0f * M_PI * std::pow(h, 9.0f)));
    }
    c.bforce_spiky = (float)(-45.0f / (M_PI * std::pow((double)h, 6.0)));
    c.cell = h;
    if (compat) {
        const float size = p.grid_size > 0.f ? p.grid_size : 5.0f;
        const int cps = (int)std::ceil(size / h);
        c.ox = c.oy = c.oz = -(size / 2.0f);
        c.nx = c.ny = c.nz = cps;
        c.wrap = 1;
        c.key_bits = 32;
    } else {
        const float m = p.grid_margin > 0.f ? p.grid_margin : 2.0f;
        float o[3];
        int n[3], mx = 1;
        for (int a = 0; a < 3; ++a) {
            const float L = x->lim[a];
            o[a] = -(L / 2.0f) - m * h;
            n[a] = (int)std::ceil((L + 2.0f * m * h) / h);
            if (n[a] < 1) n[a] = 1;
            mx = n[a] > mx ? n[a] : mx;
        }
        int bits = 0;
        while ((1 << bits) < mx) ++bits;
        if (bits > 10) return fail(x, SPH_E_INVALID, "grid exceeds 1024 cells per axis (Morton keys are 3x10 bits)");
        c.ox = o[0]; c.oy = o[1]; c.oz = o[2];
        c.nx = n[0]; c.ny = n[1]; c.nz = n[2];
        c.wrap = 0;
        c.key_bits = 3 * bits;
    }
    c.ncells = (long long)c.nx * c.ny * c.nz;
    if (!x->scene_in.empty()) {
        /* batched: one container-fitted grid per scene, cells concatenated in one table;
         * sort key = scene id above the Morton bits of the largest grid */
        if (compat || p.method != SPH_WCSPH)
            return fail(x, SPH_E_INVALID, "batched contexts run WCSPH in PHYSICS mode");
        const float m = p.grid_margin > 0.f ? p.grid_margin : 2.0f;
        x->h_scenes.assign(x->scene_in.size(), sph::SceneDev{});
        long long base = 0;
        int mx = 1;
        for (size_t s = 0; s < x->scene_in.size(); ++s) {
            const sph_ctx::SceneIn& in = x->scene_in[s];
            sph::SceneDev& sd = x->h_scenes[s];
            float o[3];
            int n[3];
            for (int a = 0; a < 3; ++a) {
                const float L = in.lim[a];
                o[a] = -(L / 2.0f) - m * h;
                n[a] = std::max(1, (int)std::ceil((L + 2.0f * m * h) / h));
                mx = std::max(mx, n[a]);
            }
            sd.ox = o[0]; sd.oy = o[1]; sd.oz = o[2];
            sd.nx = n[0]; sd.ny = n[1]; sd.nz = n[2];
            sd.ncells = (long long)n[0] * n[1] * n[2];
            sd.cell_base = base;
            base += sd.ncells;
            sd.lim_x = in.lim[0]; sd.lim_y = in.lim[1]; sd.lim_z = in.lim[2];
            sd.mu = in.mu; sd.kgas = in.kgas;
            sd.first = in.first; sd.count = in.count; sd.first_b = in.first_b; sd.count_b = in.count_b;
        }
        int bits = 0;
        while ((1 << bits) < mx) ++bits;
        int sbits = 0;
        while ((1u << sbits) < x->scene_in.size()) ++sbits;
        if (bits > 10 || 3 * bits + sbits > 32)
            return fail(x, SPH_E_INVALID, "scene grids too large for 32-bit (scene, Morton) keys");
        c.batched = 1;
        c.scene_shift = 3 * bits;
        c.key_bits = 3 * bits + sbits;
        c.ncells = base;
    }
    if (c.ncells > (1LL << 31) - 1) return fail(x, SPH_E_INVALID, "grid has more than 2^31 cells");
    c.n = x->N;
    c.nb = x->NB;
    return SPH_OK;
}

/* Arena carving with 256-byte alignment. */
struct Carver {
    size_t off = 0;
    char* base = nullptr;
    template <class T>
    T* take(size_t count) {
        off = (off + 255) & ~size_t(255);
        T* ptr = base ? reinterpret_cast<T*>(base + off) : nullptr;
        off += count * sizeof(T) + 16;
        return ptr;
    }
};

void carve(sph_ctx* x, Carver& cv) {
    Bufs& b = x->b;
    const size_t n = (size_t)(x->N > 0 ? x->N : 1), nb = (size_t)(x->NB > 0 ? x->NB : 1);
    const size_t cap = (size_t)x->c.cap;
    const size_t nbod = x->bodies.empty() ? 1 : x->bodies.size();
    b.pos = cv.take<float4>(n); b.vel = cv.take<float4>(n); b.vhalf = cv.take<float4>(n);
    b.pos_s = cv.take<float4>(n); b.vel_s = cv.take<float4>(n); b.vhalf_s = cv.take<float4>(n);
    b.normal = cv.take<float4>(n); b.accel = cv.take<float4>(n); b.pos_pred = cv.take<float4>(n);
    b.f_other = cv.take<float4>(n); b.f_press = cv.take<float4>(n);
    b.density = cv.take<float>(n); b.pressure = cv.take<float>(n); b.dens_var = cv.take<float>(n);
    b.pci_c = cv.take<float>(n);
    b.pci_pc = cv.take<float4>(n);
    b.aux = cv.take<float4>(n);
    b.nrec = cv.take<float4>(2 * n);
    b.prho = cv.take<float4>(n);
    b.keys = cv.take<uint32_t>(n); b.keys_alt = cv.take<uint32_t>(n);
    b.mask = cv.take<int32_t>(n); b.mask_alt = cv.take<int32_t>(n);
    b.ids = cv.take<int32_t>(n); b.ids_s = cv.take<int32_t>(n);
    b.tab = cv.take<int2>((size_t)x->c.ncells);
    b.cell_prev = cv.take<int32_t>(n);
    b.noff = cv.take<int32_t>(32);
    b.nlist = cv.take<int32_t>(cap * n); b.nlen = cv.take<int32_t>(n);
    b.sblist = cv.take<int32_t>(cap * n); b.sblen = cv.take<int32_t>(n);
    b.sort_ws = cv.take<char>(sph::sort_workspace_bytes((int)n, x->c.key_bits));
    b.inc_ws = cv.take<char>(sph::sort_inc_workspace_bytes((int)n));
    b.braw = cv.take<float4>(nb); b.bpos = cv.take<float4>(nb); b.bvel = cv.take<float4>(nb);
    b.bpos_s = cv.take<float4>(nb);
    b.bphi = cv.take<float>(nb); b.bphi_s = cv.take<float>(nb);
    b.bbody = cv.take<int32_t>(nb); b.bbody_s = cv.take<int32_t>(nb);
    b.bkeys = cv.take<uint32_t>(nb); b.bkeys_alt = cv.take<uint32_t>(nb);
    b.bmask = cv.take<int32_t>(nb); b.bmask_alt = cv.take<int32_t>(nb);
    b.btab = cv.take<int2>((size_t)x->c.ncells);
    b.bcell_prev = cv.take<int32_t>(nb);
    b.bnear = cv.take<uint8_t>((size_t)x->c.ncells);
    b.bsort_ws = cv.take<char>(sph::sort_workspace_bytes((int)nb, x->c.key_bits));
    b.body_xf = cv.take<float>(20 * nbod);
    b.body_range = cv.take<int32_t>(4 * nbod);
    b.body_force = cv.take<float4>(nbod); b.body_torque = cv.take<float4>(nbod);
    b.bft = cv.take<float4>(2 * nb);
    b.body_dyn = cv.take<float>(8 * nbod);
    b.flags = cv.take<unsigned>(4);
    b.pci_iters = cv.take<int32_t>(4);
    b.pci_maxerr = cv.take<float>((size_t)x->max_iter_slots);
    b.barrier = cv.take<unsigned>(4);
    b.stats = cv.take<double>(8);
    /* every context has a scene table; a single-scene context has one entry */
    x->d_scenes = cv.take<sph::SceneDev>(x->scene_in.empty() ? 1 : x->scene_in.size());
    x->d_scene_of = nullptr;
    x->d_scene_stats = nullptr;
    if (!x->scene_in.empty()) {
        x->d_scene_of = cv.take<int32_t>(n);
        x->d_scene_stats = cv.take<double>(8 * x->scene_in.size());
    }
    /* persistent scene tiles: at most one per 32 particles of a scene plus one per scene */
    b.tiles = cv.take<sph::SceneTile>(x->scene_in.empty() ? 1 : n / sph::kTileParticles + x->scene_in.size() + 1);
    b.tile_next = cv.take<unsigned>(4);
}

/* The scene tile table of a batched context: each scene's particle range cut into tiles of
 * at most 32 particles (one warp), in scene order; and the grid of the persistent launches
 * whose CTAs take chunks of tiles from a counter.  Uploaded synchronously (a host vector). */
int upload_tiles(sph_ctx* x) {
    x->c.ntiles = 0;
    x->c.tile_blocks = 0;
    if (x->scene_in.empty() || x->N <= 0 || !x->b.tiles) return SPH_OK;
    x->h_tiles.clear();
    for (size_t sc = 0; sc < x->scene_in.size(); ++sc) {
        const int first = x->scene_in[sc].first, count = x->scene_in[sc].count;
        const int T = sph::kTileParticles;
        for (int a = 0; a < count; a += T)
            x->h_tiles.push_back(sph::SceneTile{(int)sc, first + a, count - a < T ? count - a : T, 0});
    }
    if (x->h_tiles.empty()) return SPH_OK;
    const int per_sm = x->tile_ctas > 0 ? x->tile_ctas : (2048 / x->bs > 0 ? 2048 / x->bs : 1);
    const long long blocks = (long long)x->num_sms * per_sm;
    x->c.ntiles = (int)x->h_tiles.size();
    const long long warps_needed = (x->c.ntiles + x->bs / 32 - 1) / (x->bs / 32);
    x->c.tile_blocks = (int)(blocks < warps_needed ? blocks : warps_needed);
    SPH_CUDA(x, cudaStreamSynchronize(x->stream));
    SPH_CUDA(x, cudaMemcpy(const_cast<sph::SceneTile*>(x->b.tiles), x->h_tiles.data(),
                           sizeof(sph::SceneTile) * x->h_tiles.size(), cudaMemcpyHostToDevice));
    return SPH_OK;
}

void drop_graph(sph_ctx* x) {
    if (x->gexec) {
        cudaGraphExecDestroy(x->gexec);
        x->gexec = nullptr;
    }
    if (x->host_gexec) {
        cudaGraphExecDestroy(x->host_gexec);
        x->host_gexec = nullptr;
    }
    x->host_key[0] = x->host_key[1] = x->host_key[2] = nullptr;
    x->graph_ok = true;
    x->host_graph_ok = true;
}

/* Sorts the boundary particles (boundaryhandler.cpp:216-236) and builds their cell table. */
void boundary_sort(sph_ctx* x) {
    Bufs& b = x->b;
    const cudaStream_t s = x->stream;
    Const cb = x->c;
    /* batched: the boundary body of scene s is body s, so body ids are scene ids */
    sph::launch_hashes(s, cb, b.bpos, x->NB, b.bkeys, b.bmask, b.btab, b.bcell_prev, b.flags, x->bs, b.scenes,
                       b.scene_of ? b.bbody : nullptr);
    sph::sort_pairs(s, b.bkeys, b.bmask, b.bkeys_alt, b.bmask_alt, x->NB, x->c.key_bits, b.bsort_ws, b.flags,
                    x->num_sms, &b.bkeys_sorted, &b.bmask_sorted);
    sph::launch_gather_boundary(s, x->NB, b.bmask_sorted, b.bpos, b.bpos_s, b.bbody, b.bbody_s, b.bphi, b.bphi_s,
                                x->bs);
    sph::launch_cell_ranges(s, cb, b.bpos_s, b.bkeys_sorted, x->NB, b.btab, b.bcell_prev, b.flags, x->bs, b.scenes,
                            b.scene_of ? b.bbody_s : nullptr);
    sph::launch_bnd_near(s, cb, b, x->NB, x->bs);
}

bool uses_lists(const sph_ctx* x) { return x->p.method == SPH_PCISPH || x->p.neighbor_mode == SPH_NEIGH_LIST; }

int run_stage_impl(sph_ctx* x, int stage) {
    Bufs& b = x->b;
    const Const& c = x->c;
    const cudaStream_t s = x->stream;
    const int bs = x->bs;
    switch (stage) {
    case SPH_S_BOUNDARY_SYNC:
        if (x->NB > 0 && x->any_movable) {
            sph::launch_bnd_transform(s, b, (int)x->bodies.size(), x->NB, c.compat != 0, true, bs);
            boundary_sort(x);
        }
        break;
    case SPH_S_HASHES:
        sph::launch_hashes(s, c, b.pos, x->N, b.keys, b.mask, b.tab, b.cell_prev, b.flags, bs, b.scenes, b.scene_of);
        x->cur_keys = b.keys;
        x->cur_mask = b.mask;
        break;
    case SPH_S_SORT:
        /* the stable sort of the keys as an update of the last step's order */
        sph::sort_pairs_incremental(s, b.keys, x->N, c.key_bits, b.keys_alt, b.mask_alt, b.inc_ws, b.sort_ws,
                                    b.flags, x->num_sms, x->side, x->ev_fork, x->ev_join);
        b.keys_sorted = b.keys_alt;
        b.mask_sorted = b.mask_alt;
        x->cur_keys = b.keys_sorted;
        x->cur_mask = b.mask_sorted;
        break;
    case SPH_S_SHUFFLE:
        sph::launch_gather(s, x->N, b.mask_sorted, b.pos, b.pos_s, b.vel, b.vel_s,
                           x->p.method == SPH_WCSPH ? b.vhalf : nullptr, b.vhalf_s, b.ids, b.ids_s, bs);
        break;
    case SPH_S_CELL_INTERVALS:
        sph::launch_cell_ranges(s, c, b.pos_s, b.keys_sorted, x->N, b.tab, b.cell_prev, b.flags, bs, b.scenes,
                                b.scene_of);
        break;
    case SPH_S_NEIGH_LIST:
    case SPH_S_SB_NEIGH_LIST:
        sph::launch_neigh_lists(s, c, b.pos_s, b.tab, b.bpos_s, b.btab, b.nlist, b.nlen, b.sblist, b.sblen, bs,
                                b.scenes, b.scene_of, b.bnear, b.noff);
        break;
    case SPH_S_WC_DENSITY:
        sph::launch_wc_density(s, c, b, x->p.neighbor_mode == SPH_NEIGH_LIST, bs);
        break;
    case SPH_S_NORMALS:
        sph::launch_aux(s, c, b, bs);   /* the density field may have been set from outside */
        sph::launch_normals(s, c, b, uses_lists(x), bs);
        break;
    case SPH_S_WC_ACCEL:
        sph::launch_aux(s, c, b, bs);
        sph::launch_wc_forces(s, c, b, x->p.neighbor_mode == SPH_NEIGH_LIST, false, true, bs);
        break;
    case SPH_S_WC_INTEGRATE:
        sph::launch_wc_integrate(s, c, b, bs);
        break;
    case SPH_S_PCI_INIT_DENSITY:
        sph::launch_pci_init_density(s, c, b, bs);
        break;
    case SPH_S_PCI_INIT_FORCES:
        sph::launch_pci_init_forces(s, c, b, bs);
        break;
    case SPH_S_PCI_LOOP: {
        cudaMemsetAsync(b.pci_maxerr, 0, sizeof(float) * x->max_iter_slots, s);
        cudaMemsetAsync(b.barrier, 0, 4 * sizeof(unsigned), s);
        cudaError_t e = sph::launch_pci_loop(s, c, b, c.pci_min_iter, c.pci_max_iter, x->coop_blocks, bs, false);
        if (e != cudaSuccess) return cuda_fail(x, e, "cooperative launch of the PCISPH loop");
        break;
    }
    case SPH_S_PCI_INTEGRATE:
        sph::launch_pci_integrate(s, c, b, bs);
        break;
    case SPH_S_BOUNDARY_FORCES:
        if (x->any_massive) sph::launch_bnd_forces(s, c, b, (int)x->bodies.size(), bs);
        if (x->any_dynamic) sph::launch_body_integrate(s, c, b, (int)x->bodies.size());
        break;
    case SPH_S_PCI_PREDICT:
    case SPH_S_PCI_UPDATE_PRESSURE:
    case SPH_S_PCI_PRESSURE_FORCE:
        if (x->p.method != SPH_PCISPH) return fail(x, SPH_E_INVALID, "PCISPH stage on a non-PCISPH context");
        if (stage == SPH_S_PCI_PREDICT) sph::launch_pci_predict(s, c, b, bs);
        else if (stage == SPH_S_PCI_UPDATE_PRESSURE) sph::launch_pci_update_pressure(s, c, b, bs);
        else sph::launch_pci_pressure_force(s, c, b, bs);
        break;
    default:
        return fail(x, SPH_E_INVALID, "unknown stage id");
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(x, e, "kernel launch");
    return SPH_OK;
}

/* One full step: the fused sequence of WCSPHSimulation::simulate / _simulate_pcisph_step. */
/* Profiling marks: when x->prof is set, an event is recorded after each kernel group of the
 * step so sph_profile_step can report per-kernel device time (never inside a graph). */
void mark(sph_ctx* x, const char* name) {
    nvtxMarkA(name);   /* a stage boundary on the timeline of an attached profiler */
    if (!x->prof) return;
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, x->stream);
    x->prof->push_back(e);
    x->prof_names.push_back(name);
}

/* The host buffers of sph_simulate_host; chunked: the force pass's parts download their
 * particles' new state as they finish (single-scene WCSPH with the copy stream). */
struct HostState {
    float *pos4, *vel4, *vhalf4;
    bool chunked;
};
static void download_range(sph_ctx* x, const HostState& h, size_t i0, size_t i1, cudaStream_t st) {
    const size_t off = 4 * i0, bytes = 16 * (i1 - i0);
    cudaMemcpyAsync(h.pos4 + off, x->b.pos + i0, bytes, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(h.vel4 + off, x->b.vel + i0, bytes, cudaMemcpyDeviceToHost, st);
    if (h.vhalf4) cudaMemcpyAsync(h.vhalf4 + off, x->b.vhalf + i0, bytes, cudaMemcpyDeviceToHost, st);
}

/* vel_ready: null, or an event after which the unsorted velocities are in place (the host
 * step's uploads); the step then gathers them after the list pass, which does not read them.
 * out: null, or the host buffers the step's new state goes to. */
int enqueue_step(sph_ctx* x, int pci_max_iter, cudaEvent_t vel_ready, const HostState* out) {
    if (x->N <= 0) return SPH_OK;
    Bufs& b = x->b;
    const Const& c = x->c;
    const cudaStream_t s = x->stream;
    const int bs = x->bs;
    int rc;
    mark(x, "start");
    const int pre[] = {SPH_S_BOUNDARY_SYNC, SPH_S_HASHES, SPH_S_SORT};
    const char* pre_names[] = {"boundary_sync", "k_hashes", "sort"};
    for (int k = 0; k < 3; ++k) {
        if (pre[k] == SPH_S_BOUNDARY_SYNC && !(x->NB > 0 && x->any_movable)) continue;
        if (pre[k] == SPH_S_HASHES) {
            /* the hashes with the incremental sort's first pass */
            sph::sort_inc_begin(s, b.inc_ws, x->N);
            sph::launch_hashes_flags(s, c, b.pos, x->N, b.keys, b.tab, b.cell_prev, b.flags, b.scenes, b.scene_of,
                                     sph::sort_inc_flags_args(b.inc_ws, x->N));
            x->cur_keys = b.keys;
        } else if (pre[k] == SPH_S_SORT) {
            sph::sort_pairs_incremental(s, b.keys, x->N, c.key_bits, b.keys_alt, b.mask_alt, b.inc_ws, b.sort_ws,
                                        b.flags, x->num_sms, x->side, x->ev_fork, x->ev_join, true);
            b.keys_sorted = b.keys_alt;
            b.mask_sorted = b.mask_alt;
            x->cur_keys = b.keys_sorted;
            x->cur_mask = b.mask_sorted;
        } else if ((rc = run_stage_impl(x, pre[k])) != SPH_OK) {
            return rc;
        }
        mark(x, pre_names[k]);
    }
    /* the SHUFFLE and CELL_INTERVALS stages in one pass */
    const bool late_vel = vel_ready != nullptr;
    float4* const vh = x->p.method == SPH_WCSPH ? b.vhalf : nullptr;
    sph::launch_gather_ranges(s, c, x->N, b.mask_sorted, b.pos, b.pos_s, late_vel ? nullptr : b.vel, b.vel_s,
                              late_vel ? nullptr : vh, b.vhalf_s, b.ids, b.ids_s, b.keys_sorted, b.tab, b.cell_prev,
                              b.flags, bs, b.scenes, b.scene_of);
    mark(x, "k_gather_ranges");
    /* the velocities' part of the gather, once they have arrived (after the list pass) */
    auto gather_vel = [&]() {
        if (!late_vel) return;
        cudaStreamWaitEvent(s, vel_ready, 0);
        sph::launch_gather(s, x->N, b.mask_sorted, b.vel, b.vel_s, vh, b.vhalf_s, nullptr, nullptr, nullptr, nullptr,
                           bs);
        mark(x, "k_gather_vel");
    };
    if (x->p.method == SPH_WCSPH) {
        const bool lists = x->p.neighbor_mode == SPH_NEIGH_LIST;
        if (lists) {
            sph::launch_lists_density(s, c, b, bs);
            mark(x, "k_lists_density");
        } else {
            sph::launch_wc_density(s, c, b, false, bs);
            mark(x, "k_wc_density");
        }
        gather_vel();
        const bool pack = lists && c.sigma != 0.f;
        if (c.sigma != 0.f) {
            sph::launch_normals(s, c, b, lists, bs, pack, lists);   /* k_lists_density wrote prho */
            mark(x, "k_normals");
        }
        if (x->any_massive) {
            sph::launch_bnd_forces(s, c, b, (int)x->bodies.size(), bs);
            if (x->any_dynamic) sph::launch_body_integrate(s, c, b, (int)x->bodies.size());
            mark(x, "k_bnd_forces");
        }
        if (out && out->chunked) {
            /* the force pass (with the integration) in parts, each part's new state downloaded
             * on the copy stream while the next part computes */
            const int nb = (x->N + bs - 1) / bs;
            const int K = sph_ctx::kOutChunks;
            for (int k = 0; k < K; ++k) {
                const int b0 = (int)((long long)nb * k / K), b1 = (int)((long long)nb * (k + 1) / K);
                if (b1 <= b0) continue;
                sph::Const ck = c;
                ck.block0 = b0;
                ck.blocks = b1 - b0;
                sph::launch_wc_forces(s, ck, b, lists, true, false, bs, pack);
                const size_t i0 = (size_t)b0 * bs, i1 = std::min((size_t)b1 * bs, (size_t)x->N);
                cudaEventRecord(x->ev_chunk[k], s);
                cudaStreamWaitEvent(x->copy_stream, x->ev_chunk[k], 0);
                download_range(x, *out, i0, i1, x->copy_stream);
            }
            cudaEventRecord(x->ev_copy, x->copy_stream);
            cudaStreamWaitEvent(s, x->ev_copy, 0);
        } else {
            sph::launch_wc_forces(s, c, b, lists, true, false, bs, pack);
        }
        mark(x, "k_wc_forces");
    } else {
        if (!c.compat && !c.batched) {
            /* the lists and the initial density in one pass */
            sph::launch_lists_density_pci(s, c, b, bs);
            mark(x, "k_lists_density");
        } else {
            sph::launch_neigh_lists(s, c, b.pos_s, b.tab, b.bpos_s, b.btab, b.nlist, b.nlen, b.sblist, b.sblen, bs,
                                    b.scenes, b.scene_of, b.bnear, b.noff);
            mark(x, "k_neigh_lists");
            sph::launch_pci_init_density(s, c, b, bs);
            mark(x, "k_pci_init_density");
        }
        gather_vel();
        /* with surface tension the normal pass also writes the packed per-neighbour records
         * (velocity, normal, 1/rho) that the force pass reads */
        const bool pack = c.sigma != 0.f;
        if (pack) {
            sph::launch_normals(s, c, b, true, bs, true, !c.compat && !c.batched);   /* after k_lists_density_pci */
            mark(x, "k_normals");
        }
        sph::launch_pci_init_forces(s, c, b, bs, pack);
        mark(x, "k_pci_init_forces");
        cudaMemsetAsync(b.pci_maxerr, 0, sizeof(float) * x->max_iter_slots, s);
        cudaMemsetAsync(b.barrier, 0, 4 * sizeof(unsigned), s);
        if (x->any_massive) {
            cudaError_t e = sph::launch_pci_loop(s, c, b, c.pci_min_iter, pci_max_iter, x->coop_blocks, bs, false);
            if (e != cudaSuccess) return cuda_fail(x, e, "cooperative launch of the PCISPH loop");
            mark(x, "k_pci_loop");
            sph::launch_bnd_forces(s, c, b, (int)x->bodies.size(), bs);
            if (x->any_dynamic) sph::launch_body_integrate(s, c, b, (int)x->bodies.size());
            mark(x, "k_bnd_forces");
            sph::launch_pci_integrate(s, c, b, bs);
            mark(x, "k_pci_integrate");
        } else {
            cudaError_t e = sph::launch_pci_loop(s, c, b, c.pci_min_iter, pci_max_iter, x->coop_blocks, bs, true);
            if (e != cudaSuccess) return cuda_fail(x, e, "cooperative launch of the PCISPH loop");
            mark(x, "k_pci_loop");
        }
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(x, e, "step launch");
    return SPH_OK;
}

int build_graph(sph_ctx* x) {
    drop_graph(x);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(x->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) { x->graph_ok = false; cudaGetLastError(); return SPH_OK; }
    int rc = enqueue_step(x, x->c.pci_max_iter, nullptr, nullptr);
    e = cudaStreamEndCapture(x->stream, &g);
    if (rc != SPH_OK || e != cudaSuccess || !g) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        x->graph_ok = false;
        x->err.clear();
        return SPH_OK;
    }
    {
        size_t nn = 0;
        x->graph_kernels = 0;
        if (cudaGraphGetNodes(g, nullptr, &nn) == cudaSuccess && nn > 0) {
            std::vector<cudaGraphNode_t> nodes(nn);
            if (cudaGraphGetNodes(g, nodes.data(), &nn) == cudaSuccess)
                for (size_t k = 0; k < nn; ++k) {
                    cudaGraphNodeType t;
                    if (cudaGraphNodeGetType(nodes[k], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel)
                        ++x->graph_kernels;
                }
        }
        cudaGetLastError();
    }
    e = cudaGraphInstantiate(&x->gexec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        cudaGetLastError();
        x->gexec = nullptr;
        x->graph_ok = false;
    }
    return SPH_OK;
}

void free_arena(sph_ctx* x) {
    drop_graph(x);
    if (x->arena) {
        cudaFree(x->arena);
        x->arena = nullptr;
    }
    x->arena_bytes = 0;
    x->b = Bufs{};
    x->has_state = false;
}

/* (Re)allocates everything and uploads the scene.  With keep = true the current fluid
 * state on the device is carried over (add_boundary / set_rect_limits keep the fluid). */
int rebuild(sph_ctx* x, bool keep) {
    std::vector<float> kp, kv, kvh;
    std::vector<int32_t> kid;
    if (keep && x->has_state && x->N > 0) {
        kp.resize(4 * (size_t)x->N); kv.resize(kp.size()); kvh.resize(kp.size()); kid.resize(x->N);
        SPH_CUDA(x, cudaStreamSynchronize(x->stream));
        SPH_CUDA(x, cudaMemcpy(kp.data(), x->b.pos, kp.size() * 4, cudaMemcpyDeviceToHost));
        SPH_CUDA(x, cudaMemcpy(kv.data(), x->b.vel, kp.size() * 4, cudaMemcpyDeviceToHost));
        SPH_CUDA(x, cudaMemcpy(kvh.data(), x->b.vhalf, kp.size() * 4, cudaMemcpyDeviceToHost));
        SPH_CUDA(x, cudaMemcpy(kid.data(), x->b.ids, kid.size() * 4, cudaMemcpyDeviceToHost));
    } else {
        keep = false;
    }
    if (x->any_dynamic && x->b.body_xf) {
        /* dynamic bodies moved on the device: keep their current pose and velocities */
        SPH_CUDA(x, cudaStreamSynchronize(x->stream));
        for (size_t k = 0; k < x->bodies.size(); ++k)
            SPH_CUDA(x, cudaMemcpy(x->bodies[k].xf, x->b.body_xf + 20 * k, sizeof x->bodies[k].xf,
                                   cudaMemcpyDeviceToHost));
    }
    /* The new arena is allocated before the old one is freed, so a refused allocation (or a
     * refused derivation) leaves the context as it was: sizes, constants, buffers and the
     * device state.  Growth therefore needs the old and the new arena at once. */
    const int old_n = x->N, old_nb = x->NB, old_slots = x->max_iter_slots;
    const Const old_c = x->c;
    const Bufs old_b = x->b;
    sph::SceneDev* const old_scenes = x->d_scenes;
    int32_t* const old_scene_of = x->d_scene_of;
    double* const old_scene_stats = x->d_scene_stats;
    auto restore = [&]() {
        x->N = old_n; x->NB = old_nb; x->max_iter_slots = old_slots;
        x->c = old_c;
        x->b = old_b;
        x->d_scenes = old_scenes; x->d_scene_of = old_scene_of; x->d_scene_stats = old_scene_stats;
    };
    x->N = (int)(x->vol_pos.size() / 4);
    x->NB = (int)(x->braw_host.size() / 4);
    int rc = derive(x);
    if (rc != SPH_OK) {
        restore();
        return rc;
    }
    {
        const int relax_iter = x->p.pcisph_relax_max_iterations > 0 ? x->p.pcisph_relax_max_iterations : 10000;
        x->max_iter_slots = std::max(std::max(x->p.pcisph_max_iterations, relax_iter), 1);
    }
    Carver dry;
    carve(x, dry);
    const size_t bytes = dry.off + 256;
    void* fresh = nullptr;
    cudaError_t e;
    if (x->inject_alloc) {
        /* injected allocator failure: the allocation is refused as cudaMalloc refuses one */
        x->inject_alloc = false;
        e = cudaErrorMemoryAllocation;
    } else {
        e = cudaMalloc(&fresh, bytes);
        if (e != cudaSuccess) cudaGetLastError();
    }
    if (e != cudaSuccess) {
        restore();
        return fail(x, SPH_E_NOMEM, "device arena of " + std::to_string(bytes) + " bytes: " + cudaGetErrorString(e));
    }
    free_arena(x);
    x->arena = static_cast<char*>(fresh);
    x->arena_bytes = bytes;
    Carver real;
    real.base = x->arena;
    carve(x, real);
    Bufs& b = x->b;
    const cudaStream_t s = x->stream;
    SPH_CUDA(x, cudaMemsetAsync(x->arena, 0, x->arena_bytes, s));
    SPH_CUDA(x, cudaMemsetAsync(b.cell_prev, 0xff, sizeof(int32_t) * (x->N > 0 ? x->N : 1), s));
    SPH_CUDA(x, cudaMemsetAsync(b.bcell_prev, 0xff, sizeof(int32_t) * (x->NB > 0 ? x->NB : 1), s));
    {
        int32_t off[32] = {0};
        sph::neigh_linear_offsets(x->c.nx, x->c.ny, off);
        SPH_CUDA(x, cudaMemcpyAsync(b.noff, off, sizeof off, cudaMemcpyHostToDevice, s));
        SPH_CUDA(x, cudaStreamSynchronize(s));   /* off is a stack array */
    }
    if (x->scene_in.empty()) {
        /* the one scene of a single-scene context: its grid and parameters */
        sph::SceneDev sd{};
        const Const& c = x->c;
        sd.ox = c.ox; sd.oy = c.oy; sd.oz = c.oz;
        sd.nx = c.nx; sd.ny = c.ny; sd.nz = c.nz;
        sd.cell_base = 0;
        sd.ncells = c.ncells;
        sd.lim_x = c.lim_x; sd.lim_y = c.lim_y; sd.lim_z = c.lim_z;
        sd.mu = c.mu; sd.kgas = c.kgas;
        sd.first = 0; sd.count = x->N; sd.first_b = 0; sd.count_b = x->NB;
        x->h_scenes.assign(1, sd);
    } else {
        std::vector<int32_t> so(x->N > 0 ? x->N : 1, 0);
        for (size_t sc = 0; sc < x->scene_in.size(); ++sc)
            for (int i = 0; i < x->scene_in[sc].count; ++i) so[x->scene_in[sc].first + i] = (int32_t)sc;
        SPH_CUDA(x, cudaMemcpyAsync(x->d_scene_of, so.data(), 4 * so.size(), cudaMemcpyHostToDevice, s));
        b.scene_of = x->d_scene_of;
    }
    SPH_CUDA(x, cudaMemcpyAsync(x->d_scenes, x->h_scenes.data(), sizeof(sph::SceneDev) * x->h_scenes.size(),
                                cudaMemcpyHostToDevice, s));
    b.scenes = x->d_scenes;
    if (x->N > 0) {
        std::vector<float> p4(x->vol_pos), v4(x->vol_vel);
        std::vector<int32_t> ids(x->N);
        for (int i = 0; i < x->N; ++i) {
            p4[4 * (size_t)i + 3] = 1.f;
            v4[4 * (size_t)i + 3] = 0.f;
            ids[i] = i;
        }
        const float* pp = keep ? kp.data() : p4.data();
        const float* vv = keep ? kv.data() : v4.data();
        const float* vh = keep ? kvh.data() : v4.data();
        const int32_t* ii = keep ? kid.data() : ids.data();
        SPH_CUDA(x, cudaMemcpyAsync(b.pos, pp, 16 * (size_t)x->N, cudaMemcpyHostToDevice, s));
        SPH_CUDA(x, cudaMemcpyAsync(b.vel, vv, 16 * (size_t)x->N, cudaMemcpyHostToDevice, s));
        SPH_CUDA(x, cudaMemcpyAsync(b.vhalf, vh, 16 * (size_t)x->N, cudaMemcpyHostToDevice, s));
        SPH_CUDA(x, cudaMemcpyAsync(b.ids, ii, 4 * (size_t)x->N, cudaMemcpyHostToDevice, s));
        /* the sorted copies start equal to the state so that fields read before a step are defined */
        SPH_CUDA(x, cudaMemcpyAsync(b.pos_s, b.pos, 16 * (size_t)x->N, cudaMemcpyDeviceToDevice, s));
        SPH_CUDA(x, cudaMemcpyAsync(b.vel_s, b.vel, 16 * (size_t)x->N, cudaMemcpyDeviceToDevice, s));
        SPH_CUDA(x, cudaMemcpyAsync(b.vhalf_s, b.vhalf, 16 * (size_t)x->N, cudaMemcpyDeviceToDevice, s));
        SPH_CUDA(x, cudaMemcpyAsync(b.ids_s, b.ids, 4 * (size_t)x->N, cudaMemcpyDeviceToDevice, s));
    }
    x->cur_keys = b.keys;
    x->cur_mask = b.mask;
    b.keys_sorted = b.keys;
    b.mask_sorted = b.mask;
    b.bkeys_sorted = b.bkeys;
    b.bmask_sorted = b.bmask;
    /* boundary: raw particles, body table, transform all bodies (sync(true)), sort, Psi */
    x->any_movable = false;
    x->any_massive = false;
    x->any_dynamic = false;
    if (x->NB > 0) {
        std::vector<int32_t> body(x->NB), range(4 * x->bodies.size());
        std::vector<float> xf(20 * x->bodies.size()), dyn(8 * x->bodies.size(), 0.f);
        std::vector<float> raw(x->braw_host);
        for (size_t k = 0; k < x->bodies.size(); ++k) {
            const SphBody& bd = x->bodies[k];
            for (int i = 0; i < bd.count; ++i) {
                body[bd.origin + i] = (int)k;
                raw[4 * (size_t)(bd.origin + i) + 3] = 1.f;
            }
            range[4 * k] = bd.origin; range[4 * k + 1] = bd.count;
            range[4 * k + 2] = bd.can_move; range[4 * k + 3] = bd.mass > 0.f ? 1 : 0;
            std::memcpy(&xf[20 * k], bd.xf, sizeof bd.xf);
            x->any_movable |= bd.can_move != 0;
            x->any_massive |= bd.mass > 0.f;
            dyn[8 * k] = bd.dynamic ? 1.f : 0.f;
            dyn[8 * k + 1] = bd.mass;
            for (int a = 0; a < 3; ++a) dyn[8 * k + 2 + a] = bd.inv_inertia[a];
            dyn[8 * k + 5] = bd.radius;
            x->any_dynamic |= bd.dynamic != 0;
        }
        SPH_CUDA(x, cudaMemcpyAsync(b.body_dyn, dyn.data(), 4 * dyn.size(), cudaMemcpyHostToDevice, s));
        SPH_CUDA(x, cudaMemcpyAsync(b.braw, raw.data(), 16 * (size_t)x->NB, cudaMemcpyHostToDevice, s));
        SPH_CUDA(x, cudaMemcpyAsync(b.bbody, body.data(), 4 * (size_t)x->NB, cudaMemcpyHostToDevice, s));
        SPH_CUDA(x, cudaMemcpyAsync(b.body_range, range.data(), 4 * range.size(), cudaMemcpyHostToDevice, s));
        SPH_CUDA(x, cudaMemcpyAsync(b.body_xf, xf.data(), 4 * xf.size(), cudaMemcpyHostToDevice, s));
        sph::launch_bnd_transform(s, b, (int)x->bodies.size(), x->NB, x->c.compat != 0, false, x->bs);
        boundary_sort(x);
        sph::launch_bnd_phi(s, x->c, b, x->p.boundary_phi_coeff > 0.f ? x->p.boundary_phi_coeff : 1.0f, x->bs);
        SPH_CUDA(x, cudaGetLastError());
    }
    x->coop_blocks = sph::pci_loop_blocks(x->num_sms, x->bs);
    int trc = upload_tiles(x);
    if (trc != SPH_OK) return trc;
    x->has_state = true;
    SPH_CUDA(x, cudaGetLastError());
    return SPH_OK;
}

/* PCISPH relaxation after add_volume (pcisphsimluation.cpp:548-550). */
int relax(sph_ctx* x) {
    if (x->p.method != SPH_PCISPH || !x->p.relax_on_add || x->N <= 0) return SPH_OK;
    int relax_iter = x->p.pcisph_relax_max_iterations > 0 ? x->p.pcisph_relax_max_iterations : 10000;
    int rc = enqueue_step(x, relax_iter, nullptr, nullptr);
    if (rc != SPH_OK) return rc;
    SPH_CUDA(x, cudaMemsetAsync(x->b.vel, 0, 16 * (size_t)x->N, x->stream));
    return SPH_OK;
}

const int kFieldKind[SPH_F_COUNT] = {
    0, 0, 0, 0, 0, 0, 2, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 2, 1, 0, 0, 0, 0, 1, 0, 1};

void* field_ptr(sph_ctx* x, int f, long long& elems) {
    Bufs& b = x->b;
    const long long n = x->N, nb = x->NB, cap = x->c.cap, nbod = (long long)x->bodies.size();
    elems = -1;
    switch (f) {
    case SPH_F_POS: elems = 4 * n; return b.pos;
    case SPH_F_VEL: elems = 4 * n; return b.vel;
    case SPH_F_VEL_HALF: elems = 4 * n; return b.vhalf;
    case SPH_F_POS_SORTED: elems = 4 * n; return b.pos_s;
    case SPH_F_VEL_SORTED: elems = 4 * n; return b.vel_s;
    case SPH_F_VEL_HALF_SORTED: elems = 4 * n; return b.vhalf_s;
    case SPH_F_HASHES: elems = n; return x->cur_keys;
    case SPH_F_MASK: elems = n; return x->cur_mask;
    case SPH_F_CELL_INTERVALS: elems = 2 * x->c.ncells; return b.tab;
    case SPH_F_NEIGH_LIST: elems = cap * (n > 0 ? n : 1); return b.nlist;
    case SPH_F_NEIGH_LEN: elems = n; return b.nlen;
    case SPH_F_SB_NEIGH_LIST: elems = cap * (n > 0 ? n : 1); return b.sblist;
    case SPH_F_SB_NEIGH_LEN: elems = n; return b.sblen;
    case SPH_F_DENSITY: elems = n; return b.density;
    case SPH_F_PRESSURE: elems = n; return b.pressure;
    case SPH_F_NORMAL: elems = 4 * n; return b.normal;
    case SPH_F_ACCEL: elems = 4 * n; return b.accel;
    case SPH_F_POS_PRED: elems = 4 * n; return b.pos_pred;
    case SPH_F_FORCE_OTHER: elems = 4 * n; return b.f_other;
    case SPH_F_FORCE_PRESSURE: elems = 4 * n; return b.f_press;
    case SPH_F_DENS_VAR: elems = n; return b.dens_var;
    case SPH_F_BPOS_SORTED: elems = 4 * nb; return b.bpos_s;
    case SPH_F_BPHI_SORTED: elems = nb; return b.bphi_s;
    case SPH_F_BCELL_INTERVALS: elems = 2 * x->c.ncells; return b.btab;
    case SPH_F_BHASHES: elems = nb; return b.bkeys_sorted;
    case SPH_F_BMASK: elems = nb; return b.bmask_sorted;
    case SPH_F_BPHI: elems = nb; return b.bphi;
    case SPH_F_BPOS: elems = 4 * nb; return b.bpos;
    case SPH_F_BODY_FORCE: elems = 4 * nbod; return b.body_force;
    case SPH_F_BODY_TORQUE: elems = 4 * nbod; return b.body_torque;
    case SPH_F_PCI_ITERS: elems = 1; return b.pci_iters;
    case SPH_F_PCI_MAXERR: {
        int it = 0;
        if (b.pci_iters) {
            cudaStreamSynchronize(x->stream);
            cudaMemcpy(&it, b.pci_iters, 4, cudaMemcpyDeviceToHost);
        }
        elems = it;
        return b.pci_maxerr;
    }
    case SPH_F_ID: elems = n; return b.ids;
    }
    return nullptr;
}

int check_ctx(sph_ctx* x) {
    if (!x) return SPH_E_INVALID;
    cudaSetDevice(x->device);
    return SPH_OK;
}

void bump_default_params(sph_params* p) {
    p->grid_size = 5.0f;
    p->grid_margin = 2.0f;
    p->boundary_phi_coeff = 1.0f;
    p->neigh_cap = 50;
    p->pcisph_min_iterations = 3;
    p->pcisph_relax_max_iterations = 10000;
    p->use_graph = 1;
    p->neighbor_mode = SPH_NEIGH_LIST;
}

/* cached scratch for the standalone sort entry point */
struct SortCache {
    std::mutex mu;
    void* ws = nullptr;
    size_t ws_bytes = 0;
    uint32_t* kalt = nullptr;
    int32_t* valt = nullptr;
    unsigned* flags = nullptr;
    size_t n_cap = 0;
    int device = -1;
    cudaEvent_t done = nullptr;   /* the last sort's end: the next one, on any stream, waits for it */
};
SortCache g_sort;

}  // namespace

int sph_ctx_fail(sph_ctx* x, int code, const std::string& msg) { return fail(x, code, msg); }

static bool same_or_built(const sph_ctx* x, const void* const* key) {
    return x->host_key[0] == key[0] && x->host_key[1] == key[1] && x->host_key[2] == key[2];
}

static void release_side(sph_ctx* x) {
    if (x->side) cudaStreamDestroy(x->side);
    if (x->ev_fork) cudaEventDestroy(x->ev_fork);
    if (x->ev_join) cudaEventDestroy(x->ev_join);
    if (x->copy_stream) cudaStreamDestroy(x->copy_stream);
    if (x->ev_copy) cudaEventDestroy(x->ev_copy);
    if (x->ev_vel) cudaEventDestroy(x->ev_vel);
    for (auto& e : x->ev_chunk) {
        if (e) cudaEventDestroy(e);
        e = nullptr;
    }
    x->side = x->copy_stream = nullptr;
    x->ev_fork = x->ev_join = x->ev_copy = x->ev_vel = nullptr;
}

/* One step with the state on the host (sph_simulate_host): position in on the context
 * stream, velocities in on the copy stream (the step waits for them only before its
 * velocity gather, after the list pass), the step, the state back out. */
static int enqueue_host_step(sph_ctx* x, float* pos4, float* vel4, float* vhalf4) {
    const cudaStream_t s = x->stream;
    const size_t bytes = 16 * (size_t)x->N;
    Bufs& b = x->b;
    const bool wc = x->p.method == SPH_WCSPH && vhalf4 != nullptr;
    if (cudaMemcpyAsync(b.pos, pos4, bytes, cudaMemcpyHostToDevice, s) != cudaSuccess)
        return cuda_fail(x, cudaGetLastError(), "position upload");
    cudaEvent_t vel_ready = nullptr;
    if (x->copy_stream && x->ev_copy && x->ev_vel) {
        cudaEventRecord(x->ev_copy, s);
        cudaStreamWaitEvent(x->copy_stream, x->ev_copy, 0);
        cudaMemcpyAsync(b.vel, vel4, bytes, cudaMemcpyHostToDevice, x->copy_stream);
        if (wc) cudaMemcpyAsync(b.vhalf, vhalf4, bytes, cudaMemcpyHostToDevice, x->copy_stream);
        cudaEventRecord(x->ev_vel, x->copy_stream);
        vel_ready = x->ev_vel;
    } else {
        cudaMemcpyAsync(b.vel, vel4, bytes, cudaMemcpyHostToDevice, s);
        if (wc) cudaMemcpyAsync(b.vhalf, vhalf4, bytes, cudaMemcpyHostToDevice, s);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(x, e, "velocity upload");
    HostState out{pos4, vel4, wc ? vhalf4 : nullptr, false};
    /* the WCSPH force pass of a single-scene context ends the step: its parts download as
     * they finish */
    out.chunked = vel_ready != nullptr && x->p.method == SPH_WCSPH && !x->c.batched;
    int rc = enqueue_step(x, x->c.pci_max_iter, vel_ready, &out);
    if (rc != SPH_OK) return rc;
    if (!out.chunked) download_range(x, out, 0, (size_t)x->N, s);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(x, e, "state download");
    return SPH_OK;
}

extern "C" {

void sph_default_params(int method, sph_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof *p);
    bump_default_params(p);
    p->mode = SPH_MODE_COMPAT;
    if (method == SPH_PCISPH) {
        /* config.pci */
        p->method = SPH_PCISPH;
        p->time_step = 0.005f;
        p->max_vel = 20.0f;
        p->particle_radius = 0.008f;
        p->support_radius = 0.032f;
        p->pcisph_max_iterations = 3;
        p->pcisph_error_ratio = 0.01f;
        p->rest_density = 1000.0f;
        p->k_viscosity = 1.7f;
        p->gravity = 9.8f;
        p->gas_stiffness = 500.0f;
        p->surface_tension = 1.0f;
        p->relax_on_add = 1;
    } else {
        /* config.wc */
        p->method = SPH_WCSPH;
        p->time_step = 0.0012f;
        p->max_vel = 10.0f;
        p->particle_radius = 0.008f;
        p->support_radius = 0.032f;
        p->pcisph_max_iterations = 7;
        p->pcisph_error_ratio = 0.01f;
        p->rest_density = 1000.0f;
        p->k_viscosity = 0.00001f;
        p->gravity = 9.8f;
        p->gas_stiffness = 750.0f;
        p->surface_tension = 0.001f;
    }
}

int sph_batch_create(const sph_params* params, int nscenes, const sph_scene_desc* scenes, sph_ctx** out) {
    if (!params || !scenes || !out || nscenes <= 0) return fail(nullptr, SPH_E_INVALID, "null argument or no scenes");
    *out = nullptr;
    if (params->method != SPH_WCSPH || params->mode != SPH_MODE_PHYSICS)
        return fail(nullptr, SPH_E_INVALID, "batched contexts run WCSPH in PHYSICS mode");
    if (nscenes > 65536) return fail(nullptr, SPH_E_OVERFLOW, "more than 65536 scenes");
    sph_ctx* x = nullptr;
    int rc = sph_create(params, &x);
    if (rc != SPH_OK) return rc;
    long long nf = 0, nb = 0;
    for (int s = 0; s < nscenes; ++s) {
        const sph_scene_desc& d = scenes[s];
        if (d.n_fluid < 0 || d.n_boundary < 0 || (d.n_fluid > 0 && !d.fluid_pos4) ||
            (d.n_boundary > 0 && !d.boundary_pos4) || !(d.container[0] > 0.f && d.container[1] > 0.f &&
                                                         d.container[2] > 0.f)) {
            sph_destroy(x);
            return fail(nullptr, SPH_E_INVALID, "scene " + std::to_string(s) + ": bad description");
        }
        sph_ctx::SceneIn in;
        for (int a = 0; a < 3; ++a) in.lim[a] = d.container[a];
        in.mu = d.k_viscosity;
        in.kgas = d.gas_stiffness;
        in.first = (int)nf;
        in.count = d.n_fluid;
        in.first_b = (int)nb;
        in.count_b = d.n_boundary;
        x->scene_in.push_back(in);
        x->vol_pos.insert(x->vol_pos.end(), d.fluid_pos4, d.fluid_pos4 + 4 * (size_t)d.n_fluid);
        const size_t old = x->vol_vel.size();
        x->vol_vel.resize(old + 4 * (size_t)d.n_fluid, 0.f);
        if (d.fluid_vel4 && d.n_fluid > 0) std::memcpy(&x->vol_vel[old], d.fluid_vel4, 16 * (size_t)d.n_fluid);
        /* one static boundary body per scene (identity transform), so body id = scene id */
        SphBody bd;
        bd.origin = (int)nb;
        bd.count = d.n_boundary;
        static const float I[20] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0};
        std::memcpy(bd.xf, I, sizeof bd.xf);
        x->bodies.push_back(bd);
        if (d.n_boundary > 0)
            x->braw_host.insert(x->braw_host.end(), d.boundary_pos4, d.boundary_pos4 + 4 * (size_t)d.n_boundary);
        nf += d.n_fluid;
        nb += d.n_boundary;
        if (nf > 0x3fffffff || nb > 0x3fffffff) {
            sph_destroy(x);
            return fail(nullptr, SPH_E_OVERFLOW, "more than 2^30 particles");
        }
    }
    rc = rebuild(x, false);
    if (rc != SPH_OK) {
        std::string m = x->err;
        sph_destroy(x);
        return fail(nullptr, rc, m);
    }
    *out = x;
    return SPH_OK;
}

int sph_batch_scene_count(const sph_ctx* x) { return x ? (int)x->scene_in.size() : 0; }

int sph_batch_scene_range(const sph_ctx* x, int scene, int* first, int* count) {
    if (!x || scene < 0 || scene >= (int)x->scene_in.size() || !first || !count) return SPH_E_INVALID;
    *first = x->scene_in[scene].first;
    *count = x->scene_in[scene].count;
    return SPH_OK;
}

int sph_batch_scene_grid(const sph_ctx* x, int scene, float* origin3, int* dims3, long long* cell_base) {
    if (!x || scene < 0 || scene >= (int)x->h_scenes.size() || !origin3 || !dims3) return SPH_E_INVALID;
    const sph::SceneDev& sd = x->h_scenes[scene];
    origin3[0] = sd.ox; origin3[1] = sd.oy; origin3[2] = sd.oz;
    dims3[0] = sd.nx; dims3[1] = sd.ny; dims3[2] = sd.nz;
    if (cell_base) *cell_base = sd.cell_base;
    return SPH_OK;
}

int sph_batch_stats(sph_ctx* x, double* out8, int nscenes) {
    if (check_ctx(x) || !out8) return SPH_E_INVALID;
    if (x->scene_in.empty()) return fail(x, SPH_E_STATE, "not a batched context");
    if (nscenes != (int)x->scene_in.size()) return fail(x, SPH_E_INVALID, "nscenes must equal the scene count");
    sph::launch_scene_stats(x->stream, x->c, x->b, x->d_scene_stats, nscenes);
    SPH_CUDA(x, cudaGetLastError());
    std::vector<double> raw(8 * (size_t)nscenes);
    SPH_CUDA(x, cudaStreamSynchronize(x->stream));
    SPH_CUDA(x, cudaMemcpy(raw.data(), x->d_scene_stats, 8 * sizeof(double) * nscenes, cudaMemcpyDeviceToHost));
    for (int s = 0; s < nscenes; ++s) {
        const double* r = &raw[8 * (size_t)s];
        double* o = out8 + 8 * (size_t)s;
        const double n = x->scene_in[s].count > 0 ? (double)x->scene_in[s].count : 1.0;
        unsigned long long bits;
        std::memcpy(&bits, &r[2], 8);
        unsigned u = (unsigned)bits;
        u = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
        float mx;
        std::memcpy(&mx, &u, 4);
        o[0] = r[0] / n; o[1] = r[1] / n; o[2] = x->scene_in[s].count > 0 ? (double)mx : 0.0;
        o[3] = r[3]; o[4] = r[4];
        o[5] = r[5] / n; o[6] = r[6] / n; o[7] = r[7] / n;
    }
    return SPH_OK;
}

int sph_describe(const sph_params* params, const float container3[3], sph_derived* out) {
    if (!params || !out) return SPH_E_INVALID;
    sph_ctx tmp;
    tmp.p = *params;
    if (container3)
        for (int a = 0; a < 3; ++a) tmp.lim[a] = container3[a];
    int rc = derive(&tmp);
    if (rc != SPH_OK) return fail(nullptr, rc, tmp.err);
    const Const& c = tmp.c;
    out->mass = c.mass; out->mass_def = c.mass_def; out->h = c.h; out->h_def = c.h_def;
    out->rest_density_def = c.rho0_def;
    out->poly6_eval = c.poly6_eval; out->poly6_grad = c.poly6_grad; out->spiky_grad = c.spiky_grad;
    out->visc_lapl = c.visc_lapl; out->st_main = c.st_main; out->st_term = c.st_term;
    out->default_eval = c.default_eval; out->boundary_eval = c.boundary_eval; out->pci_delta = c.delta;
    out->grid_origin[0] = c.ox; out->grid_origin[1] = c.oy; out->grid_origin[2] = c.oz;
    out->grid_dims[0] = c.nx; out->grid_dims[1] = c.ny; out->grid_dims[2] = c.nz;
    out->grid_wrap = c.wrap;
    out->key_bits = c.key_bits;
    return SPH_OK;
}

int sph_cuda_available(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n > 0 ? 1 : 0;
}

int sph_create(const sph_params* params, sph_ctx** out) {
    if (!params || !out) return fail(nullptr, SPH_E_INVALID, "null argument");
    *out = nullptr;
    if (params->method != SPH_WCSPH && params->method != SPH_PCISPH)
        return fail(nullptr, SPH_E_INVALID, "method must be SPH_WCSPH or SPH_PCISPH");
    if (params->mode != SPH_MODE_COMPAT && params->mode != SPH_MODE_PHYSICS)
        return fail(nullptr, SPH_E_INVALID, "mode must be SPH_MODE_COMPAT or SPH_MODE_PHYSICS");
    if (params->kernels != SPH_KERNELS_MULLER &&
        !(params->kernels == SPH_KERNELS_MONAGHAN && params->mode == SPH_MODE_COMPAT))
        return fail(nullptr, SPH_E_INVALID, "kernels must be SPH_KERNELS_MULLER, or SPH_KERNELS_MONAGHAN in COMPAT mode");
    if (!sph_cuda_available()) return fail(nullptr, SPH_E_CUDA, "no CUDA device visible");
    sph_ctx* x = new sph_ctx();
    x->p = *params;
    if (x->p.block_size > 0) x->bs = x->p.block_size;
    if (x->bs % 32 != 0 || x->bs > 256) {
        delete x;
        return fail(nullptr, SPH_E_INVALID, "block_size must be a multiple of 32 up to 256");
    }
    cudaGetDevice(&x->device);
    cudaDeviceGetAttribute(&x->num_sms, cudaDevAttrMultiProcessorCount, x->device);
    cudaError_t e = cudaStreamCreateWithFlags(&x->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete x;
        return fail(nullptr, SPH_E_CUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
    }
    x->own_stream = true;
    if (cudaStreamCreateWithFlags(&x->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&x->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&x->ev_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaStreamCreateWithFlags(&x->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&x->ev_copy, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&x->ev_vel, cudaEventDisableTiming) != cudaSuccess ||
        [&]() {
            for (auto& e : x->ev_chunk)
                if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return true;
            return false;
        }()) {
        cudaGetLastError();   /* then everything runs on the main stream */
        release_side(x);
    }
    int rc = derive(x);
    if (rc != SPH_OK) {
        std::string m = x->err;
        cudaStreamDestroy(x->stream);
        release_side(x);
        delete x;
        return fail(nullptr, rc, m);
    }
    *out = x;
    return SPH_OK;
}

int sph_destroy(sph_ctx* x) {
    if (!x) return SPH_OK;
    cudaSetDevice(x->device);
    if (x->stream) cudaStreamSynchronize(x->stream);
    free_arena(x);
    cudaFree(x->render_buf);
    cudaFree(x->render_sort);
    cudaFree(x->frame_buf);
    if (x->own_stream && x->stream) cudaStreamDestroy(x->stream);
    if (x->side) cudaStreamSynchronize(x->side);
    if (x->copy_stream) cudaStreamSynchronize(x->copy_stream);
    release_side(x);
    delete x;
    return SPH_OK;
}

const char* sph_last_error(const sph_ctx* x) {
    if (x) return x->err.c_str();
    return g_last_create_error.c_str();
}

int sph_set_stream(sph_ctx* x, void* stream) {
    if (check_ctx(x)) return SPH_E_INVALID;
    cudaStreamSynchronize(x->stream);
    if (x->own_stream) cudaStreamDestroy(x->stream);
    x->stream = (cudaStream_t)stream;
    x->own_stream = false;
    drop_graph(x);
    return SPH_OK;
}

int sph_set_block_size(sph_ctx* x, int block_size) {
    if (check_ctx(x)) return SPH_E_INVALID;
    if (block_size % 32 != 0 || block_size < 32 || block_size > 256)
        return fail(x, SPH_E_INVALID, "block_size must be a multiple of 32 from 32 to 256");
    cudaStreamSynchronize(x->stream);
    x->p.block_size = block_size;
    x->bs = block_size;
    x->coop_blocks = sph::pci_loop_blocks(x->num_sms, x->bs);
    drop_graph(x);
    return upload_tiles(x);
}

int sph_set_tile_shape(sph_ctx* x, int ctas_per_sm) {
    if (check_ctx(x)) return SPH_E_INVALID;
    if (x->scene_in.empty()) return fail(x, SPH_E_INVALID, "sph_set_tile_shape: not a batched context");
    if (ctas_per_sm < 0 || ctas_per_sm > 64) return fail(x, SPH_E_INVALID, "ctas_per_sm must be 0..64");
    cudaStreamSynchronize(x->stream);
    x->tile_ctas = ctas_per_sm;
    drop_graph(x);
    return upload_tiles(x);
}

int sph_get_tile_shape(const sph_ctx* x, int* tile_particles, int* ctas_per_sm, int* ntiles, int* blocks) {
    if (!x || !tile_particles || !ctas_per_sm || !ntiles || !blocks) return SPH_E_INVALID;
    *tile_particles = sph::kTileParticles;
    *ctas_per_sm = x->tile_ctas;
    *ntiles = x->c.ntiles;
    *blocks = x->c.tile_blocks;
    return SPH_OK;
}

int sph_reset(sph_ctx* x, const sph_params* params) {
    if (check_ctx(x) || !params) return SPH_E_INVALID;
    if (params->block_size % 32 != 0 || params->block_size > 256 || params->block_size < 0)
        return fail(x, SPH_E_INVALID, "block_size must be a multiple of 32 up to 256");
    const sph_params old_p = x->p;
    const int old_bs = x->bs;
    x->p = *params;
    x->bs = x->p.block_size > 0 ? x->p.block_size : 256;
    int rc = rebuild(x, false);
    if (rc != SPH_OK) {
        if (rc == SPH_E_NOMEM) { x->p = old_p; x->bs = old_bs; }   /* the context is unchanged */
        return rc;
    }
    return relax(x);
}

int sph_set_rect_limits(sph_ctx* x, float w, float h, float d) {
    if (check_ctx(x)) return SPH_E_INVALID;
    if (!x->scene_in.empty()) return fail(x, SPH_E_STATE, "a batched context sets containers per scene");
    if (!(w > 0.f && h > 0.f && d > 0.f)) return fail(x, SPH_E_INVALID, "container extents must be > 0");
    const float old_lim[3] = {x->lim[0], x->lim[1], x->lim[2]};
    x->lim[0] = w; x->lim[1] = h; x->lim[2] = d;
    if (!x->has_state) return derive(x);
    const int rc = rebuild(x, true);
    if (rc == SPH_E_NOMEM) std::memcpy(x->lim, old_lim, sizeof old_lim);   /* the context is unchanged */
    return rc;
}

int sph_add_volume(sph_ctx* x, const float* pos4, const float* vel4, int n) {
    if (check_ctx(x)) return SPH_E_INVALID;
    if (!x->scene_in.empty()) return fail(x, SPH_E_STATE, "a batched context takes its particles at creation");
    if (n < 0 || (n > 0 && !pos4)) return fail(x, SPH_E_INVALID, "bad particle array");
    const size_t old = x->vol_pos.size();
    if (old / 4 + (size_t)n > (size_t)0x3fffffff) return fail(x, SPH_E_OVERFLOW, "more than 2^30 particles");
    x->vol_pos.insert(x->vol_pos.end(), pos4, pos4 + 4 * (size_t)n);
    x->vol_vel.resize(old + 4 * (size_t)n, 0.f);
    if (vel4) std::memcpy(&x->vol_vel[old], vel4, 16 * (size_t)n);
    int rc = rebuild(x, false);
    if (rc != SPH_OK) {
        if (rc == SPH_E_NOMEM) {   /* the context is unchanged: the volume is not added */
            x->vol_pos.resize(old);
            x->vol_vel.resize(old);
        }
        return rc;
    }
    return relax(x);
}

int sph_add_boundary(sph_ctx* x, const float* pos4, int n, int can_move, const float* rot3x4, const float* lin4,
                     const float* ang4, float mass) {
    if (check_ctx(x)) return SPH_E_INVALID;
    if (!x->scene_in.empty()) return fail(x, SPH_E_STATE, "a batched context takes its boundaries at creation");
    if (n <= 0 || !pos4) return fail(x, SPH_E_INVALID, "bad boundary array");
    SphBody bd;
    bd.origin = (int)(x->braw_host.size() / 4);
    bd.count = n;
    bd.can_move = can_move ? 1 : 0;
    bd.mass = mass;
    static const float I[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
    std::memcpy(bd.xf, rot3x4 ? rot3x4 : I, 12 * sizeof(float));
    for (int k = 0; k < 4; ++k) {
        bd.xf[12 + k] = lin4 ? lin4[k] : 0.f;
        bd.xf[16 + k] = ang4 ? ang4[k] : 0.f;
    }
    const size_t old = x->braw_host.size();
    if (old / 4 + (size_t)n > (size_t)0x3fffffff) return fail(x, SPH_E_OVERFLOW, "more than 2^30 particles");
    x->bodies.push_back(bd);
    x->braw_host.insert(x->braw_host.end(), pos4, pos4 + 4 * (size_t)n);
    const int rc = rebuild(x, true);
    if (rc == SPH_E_NOMEM) {   /* the context is unchanged: the body is not added */
        x->bodies.pop_back();
        x->braw_host.resize(old);
    }
    return rc;
}

int sph_set_body_transform(sph_ctx* x, int body, const float* rot3x4, const float* lin4, const float* ang4) {
    if (check_ctx(x)) return SPH_E_INVALID;
    if (body < 0 || body >= (int)x->bodies.size()) return fail(x, SPH_E_INVALID, "bad body index");
    SphBody& bd = x->bodies[body];
    if (rot3x4) std::memcpy(bd.xf, rot3x4, 12 * sizeof(float));
    for (int k = 0; k < 4; ++k) {
        if (lin4) bd.xf[12 + k] = lin4[k];
        if (ang4) bd.xf[16 + k] = ang4[k];
    }
    if (x->b.body_xf)
        SPH_CUDA(x, cudaMemcpyAsync(x->b.body_xf + 20 * body, bd.xf, sizeof bd.xf, cudaMemcpyHostToDevice, x->stream));
    return SPH_OK;
}

int sph_set_body_dynamics(sph_ctx* x, int body, int enabled, const float* inv_inertia3, float radius) {
    if (check_ctx(x)) return SPH_E_INVALID;
    if (!x->scene_in.empty()) return fail(x, SPH_E_STATE, "a batched context has static boundaries only");
    if (body < 0 || body >= (int)x->bodies.size()) return fail(x, SPH_E_INVALID, "bad body index");
    SphBody& bd = x->bodies[body];
    if (enabled && (!bd.can_move || !(bd.mass > 0.f)))
        return fail(x, SPH_E_INVALID, "a dynamic body must be movable and have a mass > 0");
    if (enabled && (!inv_inertia3 || !(inv_inertia3[0] >= 0.f) || !(inv_inertia3[1] >= 0.f) ||
                    !(inv_inertia3[2] >= 0.f) || !(radius >= 0.f)))
        return fail(x, SPH_E_INVALID, "inverse inertia and radius must be >= 0");
    if (x->any_dynamic && x->b.body_xf) {
        SPH_CUDA(x, cudaStreamSynchronize(x->stream));
        SPH_CUDA(x, cudaMemcpy(bd.xf, x->b.body_xf + 20 * body, sizeof bd.xf, cudaMemcpyDeviceToHost));
    }
    bd.dynamic = enabled ? 1 : 0;
    for (int a = 0; a < 3; ++a) bd.inv_inertia[a] = enabled ? inv_inertia3[a] : 0.f;
    bd.radius = enabled ? radius : 0.f;
    x->any_dynamic = false;
    for (const SphBody& o : x->bodies) x->any_dynamic |= o.dynamic != 0;
    if (x->b.body_dyn) {
        const float d[8] = {bd.dynamic ? 1.f : 0.f, bd.mass, bd.inv_inertia[0], bd.inv_inertia[1], bd.inv_inertia[2],
                            bd.radius, 0.f, 0.f};
        SPH_CUDA(x, cudaMemcpyAsync(x->b.body_dyn + 8 * body, d, sizeof d, cudaMemcpyHostToDevice, x->stream));
        SPH_CUDA(x, cudaStreamSynchronize(x->stream));
    }
    drop_graph(x);
    return SPH_OK;
}

int sph_get_body_state(sph_ctx* x, int body, float* rot3x4, float* lin4, float* ang4) {
    if (check_ctx(x)) return SPH_E_INVALID;
    if (body < 0 || body >= (int)x->bodies.size()) return fail(x, SPH_E_INVALID, "bad body index");
    float xf[20];
    std::memcpy(xf, x->bodies[body].xf, sizeof xf);
    if (x->b.body_xf) {
        SPH_CUDA(x, cudaStreamSynchronize(x->stream));
        SPH_CUDA(x, cudaMemcpy(xf, x->b.body_xf + 20 * body, sizeof xf, cudaMemcpyDeviceToHost));
    }
    if (rot3x4) std::memcpy(rot3x4, xf, 12 * sizeof(float));
    if (lin4) std::memcpy(lin4, xf + 12, 4 * sizeof(float));
    if (ang4) std::memcpy(ang4, xf + 16, 4 * sizeof(float));
    return SPH_OK;
}

int sph_particle_count(const sph_ctx* x) { return x ? x->N : 0; }
int sph_boundary_particle_count(const sph_ctx* x) { return x ? x->NB : 0; }

namespace {
/* NVTX range for the duration of one API call (a no-op without an attached tool) */
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
};
}  // namespace

int sph_simulate(sph_ctx* x, int nsteps) {
    NvtxRange range("sph_simulate");
    if (check_ctx(x)) return SPH_E_INVALID;
    if (nsteps < 0) return fail(x, SPH_E_INVALID, "nsteps < 0");
    if (!x->has_state || x->N <= 0) return SPH_OK;
    if (x->inject == SPH_FAULT_BARRIER_STALL && nsteps > 0) {
        /* one step outside the graph with the stall in its launch parameters */
        drop_graph(x);
        x->inject = 0;
        x->c.barrier_extra = 1;
        const int rc = enqueue_step(x, x->c.pci_max_iter, nullptr, nullptr);
        x->c.barrier_extra = 0;
        if (rc != SPH_OK) return rc;
        return sph_simulate(x, nsteps - 1);
    }
    if (x->p.use_graph && x->graph_ok && !x->gexec) {
        int rc = build_graph(x);
        if (rc != SPH_OK) return rc;
    }
    for (int k = 0; k < nsteps; ++k) {
        if (x->gexec) {
            SPH_CUDA(x, cudaGraphLaunch(x->gexec, x->stream));
        } else {
            int rc = enqueue_step(x, x->c.pci_max_iter, nullptr, nullptr);
            if (rc != SPH_OK) return rc;
        }
    }
    if (nsteps > 0) {
        /* the HASHES and MASK fields show the last step's sort (a graph launch does not run
         * enqueue_step's host code, and a stage call may have pointed them elsewhere) */
        x->cur_keys = x->b.keys_sorted;
        x->cur_mask = x->b.mask_sorted;
    }
    return SPH_OK;
}

int sph_profile_step(sph_ctx* x, int nsteps, float* ms_out, int max_groups, int* ngroups, char* names,
                     size_t names_len) {
    NvtxRange range("sph_profile_step");
    if (check_ctx(x) || nsteps <= 0 || !ms_out || !ngroups) return SPH_E_INVALID;
    if (!x->has_state || x->N <= 0) return fail(x, SPH_E_STATE, "no particles added");
    std::vector<cudaEvent_t> ev;
    std::vector<double> acc;
    std::vector<const char*> nm;
    int rc = SPH_OK;
    for (int k = 0; k < nsteps && rc == SPH_OK; ++k) {
        ev.clear();
        x->prof_names.clear();
        x->prof = &ev;
        rc = enqueue_step(x, x->c.pci_max_iter, nullptr, nullptr);
        x->prof = nullptr;
        if (rc != SPH_OK) break;
        cudaError_t e = cudaStreamSynchronize(x->stream);
        if (e != cudaSuccess) { rc = cuda_fail(x, e, "profiled step"); break; }
        if (acc.empty()) {
            acc.assign(ev.size() > 0 ? ev.size() - 1 : 0, 0.0);
            nm.assign(x->prof_names.begin() + (x->prof_names.empty() ? 0 : 1), x->prof_names.end());
        }
        for (size_t g = 1; g < ev.size() && g - 1 < acc.size(); ++g) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ev[g - 1], ev[g]);
            acc[g - 1] += ms;
        }
        for (auto e2 : ev) cudaEventDestroy(e2);
    }
    x->prof_names.clear();
    if (rc != SPH_OK) return rc;
    const int ng = (int)acc.size();
    *ngroups = ng;
    for (int g = 0; g < ng && g < max_groups; ++g) ms_out[g] = (float)(acc[g] / nsteps);
    if (names && names_len) {
        std::string all;
        for (int g = 0; g < ng; ++g) {
            if (g) all += ",";
            all += nm[g];
        }
        std::strncpy(names, all.c_str(), names_len - 1);
        names[names_len - 1] = 0;
    }
    return SPH_OK;
}

int sph_inject_fault(sph_ctx* x, int kind) {
    if (check_ctx(x)) return SPH_E_INVALID;
    if (kind == SPH_FAULT_NONE) {
        x->inject = 0;
        x->inject_alloc = false;
        return SPH_OK;
    }
    if (kind == SPH_FAULT_ALLOC_FAIL) {
        x->inject_alloc = true;
        return SPH_OK;
    }
    if (kind != SPH_FAULT_BARRIER_STALL) return fail(x, SPH_E_INVALID, "unknown fault kind");
    if (x->p.method != SPH_PCISPH) return fail(x, SPH_E_STATE, "the barrier stall needs a PCISPH context");
    x->inject = kind;
    return SPH_OK;
}

int sph_run_stage(sph_ctx* x, int stage) {
    NvtxRange range("sph_run_stage");
    if (check_ctx(x)) return SPH_E_INVALID;
    if (!x->has_state) return fail(x, SPH_E_STATE, "no particles added");
    return run_stage_impl(x, stage);
}

int sph_simulate_host(sph_ctx* x, float* pos4, float* vel4, float* vhalf4, int nsteps) {
    NvtxRange range("sph_simulate_host");
    if (check_ctx(x)) return SPH_E_INVALID;
    if (nsteps < 0) return fail(x, SPH_E_INVALID, "nsteps < 0");
    if (!x->has_state || x->N <= 0 || nsteps == 0) return SPH_OK;
    if (!pos4 || !vel4 || (x->p.method == SPH_WCSPH && !vhalf4))
        return fail(x, SPH_E_INVALID, "sph_simulate_host: pos4, vel4 (and vhalf4 for WCSPH) are required");
    if (x->inject == SPH_FAULT_BARRIER_STALL) return fail(x, SPH_E_STATE, "sph_simulate_host: a fault is armed");
    const void* key[3] = {pos4, vel4, vhalf4};
    const bool same = x->host_key[0] == key[0] && x->host_key[1] == key[1] && x->host_key[2] == key[2];
    if (x->p.use_graph && x->host_graph_ok && (!x->host_gexec || !same)) {
        /* one graph per set of host buffers: the copies' pointers are part of it (a capture
         * that fails, e.g. on pageable buffers, leaves the stream-ordered path) */
        if (x->host_gexec) {
            cudaGraphExecDestroy(x->host_gexec);
            x->host_gexec = nullptr;
        }
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(x->stream, cudaStreamCaptureModeThreadLocal);
        int rc = e == cudaSuccess ? enqueue_host_step(x, pos4, vel4, vhalf4) : SPH_E_CUDA;
        if (e == cudaSuccess) e = cudaStreamEndCapture(x->stream, &g);
        if (rc == SPH_OK && e == cudaSuccess && g) e = cudaGraphInstantiate(&x->host_gexec, g, 0);
        if (g) cudaGraphDestroy(g);
        if (rc != SPH_OK || e != cudaSuccess || !x->host_gexec) {
            cudaGetLastError();
            x->err.clear();
            x->host_gexec = nullptr;
            x->host_graph_ok = false;
        } else {
            x->host_key[0] = key[0];
            x->host_key[1] = key[1];
            x->host_key[2] = key[2];
        }
    }
    for (int k = 0; k < nsteps; ++k) {
        if (x->host_gexec && same_or_built(x, key)) {
            SPH_CUDA(x, cudaGraphLaunch(x->host_gexec, x->stream));
        } else {
            const int rc = enqueue_host_step(x, pos4, vel4, vhalf4);
            if (rc != SPH_OK) return rc;
        }
    }
    x->cur_keys = x->b.keys_sorted;
    x->cur_mask = x->b.mask_sorted;
    return SPH_OK;
}

int sph_step_kernel_launches(sph_ctx* x, int* launches) {
    if (check_ctx(x) || !launches) return SPH_E_INVALID;
    *launches = 0;
    if (x->p.use_graph && x->graph_ok && !x->gexec && x->has_state && x->N > 0) {
        int rc = build_graph(x);
        if (rc != SPH_OK) return rc;
    }
    if (x->gexec) *launches = x->graph_kernels;
    return SPH_OK;
}

int sph_synchronize(sph_ctx* x) {
    if (check_ctx(x)) return SPH_E_INVALID;
    SPH_CUDA(x, cudaStreamSynchronize(x->stream));
    return SPH_OK;
}

int sph_device_flags(sph_ctx* x, unsigned* flags, int clear) {
    if (check_ctx(x) || !flags) return SPH_E_INVALID;
    *flags = 0;
    if (!x->b.flags) return SPH_OK;
    SPH_CUDA(x, cudaStreamSynchronize(x->stream));
    SPH_CUDA(x, cudaMemcpy(flags, x->b.flags, sizeof(unsigned), cudaMemcpyDeviceToHost));
    if (clear) SPH_CUDA(x, cudaMemset(x->b.flags, 0, sizeof(unsigned)));
    return SPH_OK;
}

long long sph_field_elems(const sph_ctx* cx, int field) {
    sph_ctx* x = const_cast<sph_ctx*>(cx);
    if (!x || field < 0 || field >= SPH_F_COUNT) return -1;
    long long n;
    field_ptr(x, field, n);
    return n;
}

int sph_field_kind(int field) {
    if (field < 0 || field >= SPH_F_COUNT) return -1;
    return kFieldKind[field];
}

int sph_get_field(sph_ctx* x, int field, void* host, size_t bytes) {
    if (check_ctx(x) || !host) return SPH_E_INVALID;
    if (field < 0 || field >= SPH_F_COUNT) return fail(x, SPH_E_INVALID, "unknown field id");
    long long n;
    void* p = field_ptr(x, field, n);
    if (!p || n < 0) return fail(x, SPH_E_STATE, "field not allocated");
    if (bytes != (size_t)n * 4) return fail(x, SPH_E_INVALID, "byte count does not match the field size");
    SPH_CUDA(x, cudaStreamSynchronize(x->stream));
    if (n > 0) SPH_CUDA(x, cudaMemcpy(host, p, bytes, cudaMemcpyDeviceToHost));
    return SPH_OK;
}

int sph_get_field_async(sph_ctx* x, int field, void* host, size_t bytes) {
    if (check_ctx(x) || !host) return SPH_E_INVALID;
    if (field < 0 || field >= SPH_F_COUNT) return fail(x, SPH_E_INVALID, "unknown field id");
    long long n;
    void* p = field_ptr(x, field, n);
    if (!p || n < 0) return fail(x, SPH_E_STATE, "field not allocated");
    if (bytes != (size_t)n * 4) return fail(x, SPH_E_INVALID, "byte count does not match the field size");
    if (n > 0) SPH_CUDA(x, cudaMemcpyAsync(host, p, bytes, cudaMemcpyDeviceToHost, x->stream));
    return SPH_OK;
}

int sph_set_field_async(sph_ctx* x, int field, const void* host, size_t bytes) {
    if (check_ctx(x) || !host) return SPH_E_INVALID;
    if (field < 0 || field >= SPH_F_COUNT) return fail(x, SPH_E_INVALID, "unknown field id");
    long long n;
    void* p = field_ptr(x, field, n);
    if (!p || n < 0) return fail(x, SPH_E_STATE, "field not allocated");
    if (bytes != (size_t)n * 4) return fail(x, SPH_E_INVALID, "byte count does not match the field size");
    if (n > 0) SPH_CUDA(x, cudaMemcpyAsync(p, host, bytes, cudaMemcpyHostToDevice, x->stream));
    return SPH_OK;
}

int sph_set_field(sph_ctx* x, int field, const void* host, size_t bytes) {
    if (check_ctx(x) || !host) return SPH_E_INVALID;
    if (field < 0 || field >= SPH_F_COUNT) return fail(x, SPH_E_INVALID, "unknown field id");
    long long n;
    void* p = field_ptr(x, field, n);
    if (!p || n < 0) return fail(x, SPH_E_STATE, "field not allocated");
    if (bytes != (size_t)n * 4) return fail(x, SPH_E_INVALID, "byte count does not match the field size");
    SPH_CUDA(x, cudaStreamSynchronize(x->stream));
    if (n > 0) SPH_CUDA(x, cudaMemcpy(p, host, bytes, cudaMemcpyHostToDevice));
    return SPH_OK;
}

int sph_field_device_ptr(sph_ctx* x, int field, void** dptr) {
    if (check_ctx(x) || !dptr) return SPH_E_INVALID;
    long long n;
    *dptr = field_ptr(x, field, n);
    if (!*dptr) return fail(x, SPH_E_STATE, "field not allocated");
    return SPH_OK;
}

int sph_body_forces(sph_ctx* x, float* force4, float* torque4, int bodies) {
    if (check_ctx(x)) return SPH_E_INVALID;
    if (bodies != (int)x->bodies.size()) return fail(x, SPH_E_INVALID, "bodies must equal the number of bodies");
    if (bodies == 0) return SPH_OK;
    SPH_CUDA(x, cudaStreamSynchronize(x->stream));
    if (force4) SPH_CUDA(x, cudaMemcpy(force4, x->b.body_force, 16 * (size_t)bodies, cudaMemcpyDeviceToHost));
    if (torque4) SPH_CUDA(x, cudaMemcpy(torque4, x->b.body_torque, 16 * (size_t)bodies, cudaMemcpyDeviceToHost));
    return SPH_OK;
}

int sph_stats(sph_ctx* x, double* out8) {
    if (check_ctx(x) || !out8) return SPH_E_INVALID;
    if (!x->has_state) return fail(x, SPH_E_STATE, "no particles added");
    sph::launch_stats(x->stream, x->c, x->b);
    SPH_CUDA(x, cudaGetLastError());
    double raw[8];
    SPH_CUDA(x, cudaStreamSynchronize(x->stream));
    SPH_CUDA(x, cudaMemcpy(raw, x->b.stats, sizeof raw, cudaMemcpyDeviceToHost));
    const double n = x->N > 0 ? (double)x->N : 1.0;
    unsigned long long bits;
    std::memcpy(&bits, &raw[2], 8);
    unsigned u = (unsigned)bits;
    u = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
    float mx;
    std::memcpy(&mx, &u, 4);
    out8[0] = raw[0] / n;
    out8[1] = raw[1] / n;
    out8[2] = x->N > 0 ? (double)mx : 0.0;
    out8[3] = raw[3];
    out8[4] = raw[4];
    out8[5] = raw[5] / n;
    out8[6] = raw[6] / n;
    out8[7] = raw[7] / n;
    return SPH_OK;
}

int sph_sort_pairs(uint32_t* d_keys, int32_t* d_vals, int n, int key_bits, void* stream) {
    if (n < 0 || key_bits < 1 || key_bits > 32 || (n > 0 && (!d_keys || !d_vals)))
        return fail(nullptr, SPH_E_INVALID, "sph_sort_pairs: bad arguments");
    if (n <= 1) return SPH_OK;
    std::lock_guard<std::mutex> lk(g_sort.mu);
    int dev = 0;
    cudaGetDevice(&dev);
    const size_t need = sph::sort_workspace_bytes(n, key_bits);
    if (g_sort.device != dev || g_sort.n_cap < (size_t)n || g_sort.ws_bytes < need) {
        if (g_sort.ws && g_sort.device == dev) {
            cudaFree(g_sort.ws); cudaFree(g_sort.kalt); cudaFree(g_sort.valt); cudaFree(g_sort.flags);
        }
        if (g_sort.done && g_sort.device == dev) cudaEventDestroy(g_sort.done);
        g_sort.done = nullptr;
        g_sort.ws = nullptr; g_sort.kalt = nullptr; g_sort.valt = nullptr; g_sort.flags = nullptr;
        g_sort.ws_bytes = 0; g_sort.n_cap = 0;
        g_sort.device = dev;
        size_t ncap = (size_t)n;
        size_t wsb = sph::sort_workspace_bytes(n, 32);
        if (cudaMalloc(&g_sort.ws, wsb) != cudaSuccess || cudaMalloc(&g_sort.kalt, 4 * ncap) != cudaSuccess ||
            cudaMalloc(&g_sort.valt, 4 * ncap) != cudaSuccess || cudaMalloc(&g_sort.flags, 16) != cudaSuccess) {
            cudaGetLastError();
            return fail(nullptr, SPH_E_NOMEM, "sph_sort_pairs: scratch allocation failed");
        }
        cudaMemset(g_sort.flags, 0, 16);
        if (cudaEventCreateWithFlags(&g_sort.done, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            g_sort.done = nullptr;
        }
        g_sort.ws_bytes = wsb;
        g_sort.n_cap = ncap;
    }
    int sms = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaStream_t s = (cudaStream_t)stream;
    /* calls on different streams share the scratch: each waits on the GPU for the previous
       one (outside stream capture, where an outside event cannot be waited on) */
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(s, &cap);
    const bool order = g_sort.done && cap == cudaStreamCaptureStatusNone;
    if (order) cudaStreamWaitEvent(s, g_sort.done, 0);
    uint32_t* kr;
    int32_t* vr;
    sph::sort_pairs(s, d_keys, d_vals, g_sort.kalt, g_sort.valt, n, key_bits, g_sort.ws, g_sort.flags, sms, &kr, &vr);
    if (kr != d_keys) {
        cudaMemcpyAsync(d_keys, kr, 4 * (size_t)n, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(d_vals, vr, 4 * (size_t)n, cudaMemcpyDeviceToDevice, s);
    }
    if (order) cudaEventRecord(g_sort.done, s);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "sph_sort_pairs");
    return SPH_OK;
}

}  // extern "C"
