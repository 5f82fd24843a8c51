/*
 * sph_device.cuh -- device-side building blocks shared by the SPH kernels (sm_103a).
 *
 * Data layout in HBM (one context): structure-of-arrays, particle i of every array is the
 * same particle, arrays indexed in Morton order of the current step:
 *   float4 pos/vel/vel_half (x, y, z, w; w = 1 for positions, 0 otherwise), float density,
 *   pressure, int cell table int2[cells] = [start, end) into the sorted arrays.
 * The cell coordinate, Morton key and linear cell id follow kernels/grid.h:7-13,74-108 and
 * kernels/morton.h:37-56; the neighbour traversal order follows grid.h:15-49 (own cell
 * first, then the 26 offsets), ascending particle index inside a cell, with the
 * NEIGH_LIST_MAX_LENGTH cap of grid.cl:163-177.
 */
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace sph {

/* Kernel constants derived on the host (sph_context.cu: derive_constants). */
struct Const {
    /* grid: origin, cell size, dimensions; wrap = 1 reproduces grid.h:82-88 */
    float ox, oy, oz, cell;
    int nx, ny, nz, wrap;
    long long ncells;
    float h2_list;       /* CELL_SIZE^2 of grid.cl:3 (6-decimal -D rounding in COMPAT) */
    int n, nb, cap, compat;
    float h, h_def;      /* kernel argument h; SUPPORT_RADIUS -D constant */
    float mass, mass_def, rho0, rho0_def, kgas, mu, sigma, g;
    float poly6_eval, poly6_grad, spiky_grad, visc_lapl, st_main, st_term;
    float default_eval, boundary_eval, delta, bforce_spiky;
    float dt, vmax, lim_x, lim_y, lim_z;
    float pci_eta;
    int pci_min_iter, pci_max_iter;
    int barrier_extra;   /* 0; 1 only for an injected barrier stall (sph_inject_fault) */
    int key_bits;
    float rmin_wc;       /* largest float <= 1e-5: wcsph.cl:152 compares r > 0.00001 (a double) */
    float rmin2_wc;      /* rmin_wc^2: the same guard on r^2 */
    float cull2;         /* (h_list / cell)^2 * (1 + 1e-4): face-distance bound for skipping cells */
    int batched;         /* 1: per-scene grid and parameters from a SceneDev table */
    int scene_shift;     /* Morton bits below the scene id in the sort key */
    int monaghan;        /* COMPAT with the Monaghan kernels (sph_params::kernels) */
    int ntiles;          /* batched: entries of the scene tile table (SceneTile) */
    int tile_blocks;     /* batched: CTAs of a persistent launch over the tiles */
    int block0, blocks;  /* single-scene passes launched in parts: blocks [block0, block0 + blocks)
                            of the whole pass (0, 0: the whole pass in one launch) */
};

/* One scene of a batched context: its grid (origin, dimensions, offset of its cells in the
 * concatenated cell table), its parameters and its particle range. */
struct SceneDev {
    float ox, oy, oz, lim_x;
    int nx, ny, nz, first;
    long long cell_base, ncells;
    float lim_y, lim_z, mu, kgas;
    int count, first_b, count_b, pad;
};

/* The constants of the scene a particle belongs to: grid, viscosity, stiffness, container. */
__device__ __forceinline__ void apply_scene(Const& c, const SceneDev& s) {
    c.ox = s.ox; c.oy = s.oy; c.oz = s.oz;
    c.nx = s.nx; c.ny = s.ny; c.nz = s.nz;
    c.ncells = s.ncells;
    c.mu = s.mu; c.kgas = s.kgas;
    c.lim_x = s.lim_x; c.lim_y = s.lim_y; c.lim_z = s.lim_z;
}
/* Switches c to particle i's scene and returns that scene's offset in the cell tables.
 * Every context has a scene table (one entry for a single scene, scene_of null), and the
 * update is unconditional: with nvcc 13.0 for sm_103a at -O3, updating a copy of the
 * by-value kernel parameter only under a runtime condition (if (table) ...) left the first
 * member (ox) at the parameter's value, while an unconditional update keeps every member. */
__device__ __forceinline__ long long scene_setup(Const& c, const SceneDev* scenes, const int32_t* scene_of, int i) {
    const int sid = scene_of ? scene_of[i] : 0;
    const SceneDev& sd = scenes[sid];
    apply_scene(c, sd);
    return sd.cell_base;
}
/* A per-scene tile of a batched context: particles [first, first + count) of scene
 * `scene`, count at most 32 (one warp).  Tiles never straddle scenes. */
constexpr int kTileParticles = 32;
struct SceneTile {
    int scene, first, count, pad;
};

/* Runs f(c, cell_base, i) for the particles of a launch.  Single scene (BATCH = false): one
 * particle per thread of a flat grid, the parameter's constants.  Batched: a persistent
 * grid of tile_blocks CTAs takes the scene tiles from a counter (*next, zero before the
 * launch), one contiguous chunk of blockDim / 32 tiles per CTA at a time, one tile per
 * warp, so the work balances dynamically however uneven the tiles are and the warps of a
 * CTA work on adjacent particles (whose neighbour cells they share in L1); a tile's scene
 * constants are read once, at a warp-uniform address, for its 32 particles (one per lane),
 * instead of being looked up per particle.  f must not use warp-collective operations (a
 * tile's lanes beyond its count are idle). */
template <bool BATCH, class F>
__device__ __forceinline__ void for_each_particle(const Const& c0, const SceneTile* __restrict__ tiles,
                                                  const SceneDev* __restrict__ scenes, unsigned* next, F&& f) {
    if constexpr (BATCH) {
        __shared__ int s_chunk;
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
#pragma unroll 1
        for (;;) {
            if (threadIdx.x == 0) s_chunk = (int)atomicAdd(next, (unsigned)warps);
            __syncthreads();
            const int t = s_chunk + warp;
            __syncthreads();   /* every thread has read s_chunk before it is written again */
            if (t - warp >= c0.ntiles) break;
            if (t < c0.ntiles) {
                const SceneTile tl = tiles[t];
                if (lane < tl.count) {
                    Const c = c0;
                    const SceneDev& sd = scenes[tl.scene];
                    apply_scene(c, sd);
                    f(c, sd.cell_base, tl.first + lane);
                }
            }
        }
    } else {
        const int i = (c0.block0 + (int)blockIdx.x) * (int)blockDim.x + (int)threadIdx.x;
        if (i < c0.n) f(c0, 0LL, i);
    }
}

/* Compile-time choice: single-scene kernels (BATCH = false) use the parameter's grid and
 * carry no scene code at all; batched kernels always apply the particle's scene. */
template <bool BATCH>
__device__ __forceinline__ long long scene_setup_t(Const& c, const SceneDev* scenes, const int32_t* scene_of, int i) {
    if constexpr (BATCH) return scene_setup(c, scenes, scene_of, i);
    else return 0;
}

constexpr unsigned kFlagNan = 1u, kFlagEscaped = 2u, kFlagTimeout = 4u, kFlagOverflow = 8u,
                   kFlagNonconverged = 16u;

/* ---- IEEE helpers that the compiler may not contract into FMAs ---------------------- */
__device__ __forceinline__ float r2_exact(float dx, float dy, float dz) {
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

/* kernels/morton.h:37-56 with OpenCL C semantics (shift by 32 is a shift by 0; 64-bit
 * masks truncated to 32 bits). */
__host__ __device__ __forceinline__ uint32_t split_by_3(uint32_t a) {
    uint32_t x = a & 0x1fffffu;
    x = x & 0x0000ffffu;
    x = (x | (x << 16)) & 0xff0000ffu;
    x = (x | (x << 8)) & 0x0f00f00fu;
    x = (x | (x << 4)) & 0xc30c30c3u;
    x = (x | (x << 2)) & 0x49249249u;
    return x;
}
__host__ __device__ __forceinline__ uint32_t morton3(uint32_t x, uint32_t y, uint32_t z) {
    return (split_by_3(x) | (split_by_3(y) << 1)) | (split_by_3(z) << 2);
}

/* One axis of get_grid_coordinates (grid.h:74-91): floor((p - origin) / h) with IEEE
 * subtraction and division; COMPAT wraps modulo n, PHYSICS clamps into [0, n). */
__device__ __forceinline__ float axis_floor(float p, float o, float h) { return floorf(__fdiv_rn(__fsub_rn(p, o), h)); }
__device__ __forceinline__ int axis_clamp(float f, int n, int wrap) {
    if (wrap) {
        if (!(f > -1e9f && f < 1e9f)) f = 0.f;
        int c = (int)f + n;
        return c % n;
    }
    if (!(f >= 0.f)) return 0;
    if (f > (float)(n - 1)) return n - 1;
    return (int)f;
}
__device__ __forceinline__ int axis_cell(float p, float o, float h, int n, int wrap) {
    return axis_clamp(axis_floor(p, o, h), n, wrap);
}
__device__ __forceinline__ void cell_of(const Const& c, float x, float y, float z, int& cx, int& cy, int& cz) {
    cx = axis_cell(x, c.ox, c.cell, c.nx, c.wrap);
    cy = axis_cell(y, c.oy, c.cell, c.ny, c.wrap);
    cz = axis_cell(z, c.oz, c.cell, c.nz, c.wrap);
}
/* CELL_ID (grid.h:7): x + nx * (y + ny * z). */
__device__ __forceinline__ long long cell_lin(const Const& c, int x, int y, int z) {
    return (long long)x + (long long)c.nx * ((long long)y + (long long)c.ny * (long long)z);
}
/* Linear id of a neighbour cell, false when it is outside the table.  COMPAT keeps the
 * reference's unchecked linear arithmetic (a -1 / n coordinate reads the adjacent row)
 * and only rejects ids outside [0, cells); PHYSICS rejects coordinates outside the grid. */
__device__ __forceinline__ bool neigh_cell(const Const& c, int x, int y, int z, long long& id) {
    if (c.wrap) {
        id = cell_lin(c, x, y, z);
        return id >= 0 && id < c.ncells;
    }
    if ((unsigned)x >= (unsigned)c.nx || (unsigned)y >= (unsigned)c.ny || (unsigned)z >= (unsigned)c.nz)
        return false;
    id = cell_lin(c, x, y, z);
    return true;
}
/* CELL_NEIGH_OFFSET (grid.h:15-49): o = 0 is the own cell; o = 1..26 enumerate
 * (dx, dy, dz) in {-1,0,1}^3 \ {0} with dx slowest, dz fastest. */
__device__ __forceinline__ void neigh_offset(int o, int& dx, int& dy, int& dz) {
    if (o == 0) { dx = dy = dz = 0; return; }
    int t = o - 1;
    t += (t >= 13) ? 1 : 0;
    dx = t / 9 - 1;
    dy = (t / 3) % 3 - 1;
    dz = t % 3 - 1;
}

/* Squared distance, in cell units, from a particle to the face of the neighbour cell in
 * direction o (-1, 0, +1) along one axis, given its fractional position fr in its cell. */
__device__ __forceinline__ float face_gap2(int o, float fr) {
    const float g = o < 0 ? fr : (o > 0 ? 1.0f - fr : 0.0f);
    return g * g;
}

/* Visits the neighbours j of a point (px, py, pz) among the particles npos[] binned in
 * table tab, in the reference's list order, keeping at most c.cap with r^2 < h2_list.
 * f(j, pj, dx, dy, dz) receives the neighbour and d = p - pj (IEEE subtraction).
 * EXACT: r^2 as uncontracted IEEE sum (bit-exact membership, used for the lists and in
 * COMPAT); otherwise FMA-contracted (membership can differ only for r within an ulp of h,
 * where every smoothing kernel is zero).
 * On the clamped PHYSICS grid, a neighbour cell whose nearest face is farther than h from
 * the particle cannot hold a neighbour and is skipped (same visits, same order), and the
 * cap is checked once per cell when the cell cannot overflow it. */
template <bool EXACT, class F>
__device__ __forceinline__ int scan_neighbors(const Const& c, float px, float py, float pz,
                                              const int2* __restrict__ tab, const float4* __restrict__ npos,
                                              F&& f) {
    const float qx = __fdiv_rn(__fsub_rn(px, c.ox), c.cell);
    const float qy = __fdiv_rn(__fsub_rn(py, c.oy), c.cell);
    const float qz = __fdiv_rn(__fsub_rn(pz, c.oz), c.cell);
    int cx, cy, cz;
    cell_of(c, px, py, pz, cx, cy, cz);
    /* fractional positions; an axis that was clamped (or the wrapped COMPAT grid) culls nothing */
    const bool cull = !c.wrap;
    float fx = qx - floorf(qx), fy = qy - floorf(qy), fz = qz - floorf(qz);
    const bool inx = cull && floorf(qx) == (float)cx, iny = cull && floorf(qy) == (float)cy,
               inz = cull && floorf(qz) == (float)cz;
    int cnt = 0;
#pragma unroll 1
    for (int o = 0; o < 27 && cnt < c.cap; ++o) {
        int ox, oy, oz;
        neigh_offset(o, ox, oy, oz);
        if (cull) {
            const float g = (inx ? face_gap2(ox, fx) : 0.f) + (iny ? face_gap2(oy, fy) : 0.f) +
                            (inz ? face_gap2(oz, fz) : 0.f);
            if (g > c.cull2) continue;
        }
        long long id;
        if (!neigh_cell(c, cx + ox, cy + oy, cz + oz, id)) continue;
        const int2 r = __ldg(&tab[id]);
        if (cnt + (r.y - r.x) <= c.cap) {
#pragma unroll 2
            for (int j = r.x; j < r.y; ++j) {
                const float4 pj = __ldg(&npos[j]);
                const float dx = __fsub_rn(px, pj.x), dy = __fsub_rn(py, pj.y), dz = __fsub_rn(pz, pj.z);
                const float r2 = EXACT ? r2_exact(dx, dy, dz) : dx * dx + dy * dy + dz * dz;
                if (r2 < c.h2_list) {
                    f(j, pj, dx, dy, dz);
                    ++cnt;
                }
            }
        } else {
#pragma unroll 1
            for (int j = r.x; j < r.y && cnt < c.cap; ++j) {
                const float4 pj = __ldg(&npos[j]);
                const float dx = __fsub_rn(px, pj.x), dy = __fsub_rn(py, pj.y), dz = __fsub_rn(pz, pj.z);
                const float r2 = EXACT ? r2_exact(dx, dy, dz) : dx * dx + dy * dy + dz * dz;
                if (r2 < c.h2_list) {
                    f(j, pj, dx, dy, dz);
                    ++cnt;
                }
            }
        }
    }
    return cnt;
}

/* The scan of scan_neighbors<true> (same cells, order, cap and exact r^2), written for the
 * list builder: every candidate runs the same instructions and f(hit, j, r2, k) applies the
 * hit (k = the entries kept so far, the slot of a hit) with predicated stores and selects
 * instead of a branch, so the lanes of a warp that
 * walk the same cell stay converged whichever of them hit.  The particle's cell (cx, cy, cz)
 * comes from the caller.  No cell is skipped by distance: in a warp the lanes that share a
 * cell would skip different cells, so the warp walks their union anyway, and measured on
 * GB300 the skipping test cost more than it saved. */
#ifndef SPH_BUILD_UNROLL
#define SPH_BUILD_UNROLL 2
#endif
#ifndef SPH_BUILD_PAIRS
#define SPH_BUILD_PAIRS 1
#endif
constexpr int kBuildUnroll = SPH_BUILD_UNROLL;
/* CELL_NEIGH_OFFSET order as (dx + 1) | (dy + 1) << 2 | (dz + 1) << 4, one byte per offset. */
#define SPH_NEIGH_CODES                                                                                  \
    0x15, 0x00, 0x10, 0x20, 0x04, 0x14, 0x24, 0x08, 0x18, 0x28, 0x01, 0x11, 0x21, 0x05, 0x25, 0x09, 0x19, \
        0x29, 0x02, 0x12, 0x22, 0x06, 0x16, 0x26, 0x0a, 0x1a, 0x2a
static __constant__ uint8_t kNeighCode[27] = {SPH_NEIGH_CODES};
/* Linear cell-id offsets of the 27 neighbour cells, in the order above, on an nx x ny x nz
 * grid (host side; the list builder reads them for cells away from the grid's faces). */
inline void neigh_linear_offsets(int nx, int ny, int32_t* out27) {
    static const uint8_t codes[27] = {SPH_NEIGH_CODES};
    for (int o = 0; o < 27; ++o) {
        const int ox = (codes[o] & 3) - 1, oy = ((codes[o] >> 2) & 3) - 1, oz = ((codes[o] >> 4) & 3) - 1;
        out27[o] = ox + nx * oy + nx * ny * oz;
    }
}
template <class F>
__device__ __forceinline__ int build_scan(const Const& c, float px, float py, float pz, int cx, int cy, int cz,
                                          const int2* __restrict__ tab, const float4* __restrict__ npos,
                                          const int32_t* __restrict__ noff, F&& f) {
    const float h2 = c.h2_list;
    int cnt = 0;
    /* PHYSICS grid: 32-bit cell ids (the grid has < 2^31 cells) and no bounds test for a cell
     * whose 26 neighbours are all inside the grid */
    const bool interior = !c.wrap && cx > 0 && cy > 0 && cz > 0 && cx < c.nx - 1 && cy < c.ny - 1 &&
                          cz < c.nz - 1;
    const int sy = c.nx, sz = c.nx * c.ny;
    const int base = cx + sy * cy + sz * cz;
#pragma unroll 1
    for (int o = 0; o < 27 && cnt < c.cap; ++o) {
        long long id;
        if (interior && noff != nullptr) {
            id = base + __ldg(&noff[o]);   /* one load, the same address in every lane */
        } else {
            const int code = kNeighCode[o];
            const int ox = (code & 3) - 1, oy = ((code >> 2) & 3) - 1, oz = ((code >> 4) & 3) - 1;
            if (interior) {
                id = base + ox + sy * oy + sz * oz;
            } else if (!neigh_cell(c, cx + ox, cy + oy, cz + oz, id)) {
                continue;
            }
        }
        const int2 r = __ldg(&tab[id]);
        if (cnt + (r.y - r.x) <= c.cap) {
            const float4* __restrict__ q = npos + r.x;
#if SPH_BUILD_PAIRS
            /* two candidates a trip, loaded together, then an odd last one */
            int j = r.x;
#pragma unroll 1
            for (; j + 1 < r.y; j += 2, q += 2) {
                const float4 pa = __ldg(q), pb = __ldg(q + 1);
                const float ra = r2_exact(__fsub_rn(px, pa.x), __fsub_rn(py, pa.y), __fsub_rn(pz, pa.z));
                const float rb = r2_exact(__fsub_rn(px, pb.x), __fsub_rn(py, pb.y), __fsub_rn(pz, pb.z));
                const bool ha = ra < h2, hb = rb < h2;
                f(ha, j, ra, cnt);
                cnt += ha ? 1 : 0;
                f(hb, j + 1, rb, cnt);
                cnt += hb ? 1 : 0;
            }
            if (j < r.y) {
                const float4 pj = __ldg(q);
                const float r2 = r2_exact(__fsub_rn(px, pj.x), __fsub_rn(py, pj.y), __fsub_rn(pz, pj.z));
                const bool hit = r2 < h2;
                f(hit, j, r2, cnt);
                cnt += hit ? 1 : 0;
            }
#else
#pragma unroll kBuildUnroll
            for (int j = r.x; j < r.y; ++j, ++q) {
                const float4 pj = __ldg(q);
                const float r2 = r2_exact(__fsub_rn(px, pj.x), __fsub_rn(py, pj.y), __fsub_rn(pz, pj.z));
                const bool hit = r2 < h2;
                f(hit, j, r2, cnt);
                cnt += hit ? 1 : 0;
            }
#endif
        } else {
#pragma unroll 1
            for (int j = r.x; j < r.y && cnt < c.cap; ++j) {
                const float4 pj = __ldg(&npos[j]);
                const float r2 = r2_exact(__fsub_rn(px, pj.x), __fsub_rn(py, pj.y), __fsub_rn(pz, pj.z));
                const bool hit = r2 < h2;
                f(hit, j, r2, cnt);
                cnt += hit ? 1 : 0;
            }
        }
    }
    return cnt;
}

/* Entry k of a column-major list row (row + k * n): one widening multiply-add on the entry
 * count instead of a 64-bit pointer advanced per candidate; n4 = 4 n bytes (n < 2^30). */
__device__ __forceinline__ int* list_slot(char* row, int k, unsigned n4) {
    return reinterpret_cast<int*>(row + (unsigned long long)(unsigned)k * n4);
}

/* Visits the materialised list of particle i (column-major list[k * n + i], grid.cl:174).
 * The pass is bound by the latency of the dependent loads (list entry, then the
 * neighbour's data), so U entries and their positions are loaded before the U visits
 * run.  PIPE also loads the next U entries (the rows live in HBM: 200 bytes per particle)
 * before the current U visits, so their latency overlaps the visits: measured on GB300 it
 * speeds up both walks that use it two entries deep: the normal pass 0.310 -> 0.291 ms at
 * 4M four deep and 0.272 ms two deep (eight deep 0.471 ms at 66 registers), the force pass
 * 0.699 -> 0.667 ms two deep.  PRED (with PIPE) drops the separate tail: a last, partial
 * batch loads the particle itself in place of the missing entries and skips their visits;
 * the force pass walks that way four deep, 0.628 -> 0.600 ms (the normal pass 0.320 ms four
 * deep, so it stays two deep without PRED).  The visits run in list order either way, so
 * every sum keeps the list's order. */
#ifndef SPH_LIST_UNROLL
#define SPH_LIST_UNROLL 4
#endif

template <int U = SPH_LIST_UNROLL, bool PIPE = false, bool PRED = false, class F>
__device__ __forceinline__ void list_neighbors(int i, int n, const int* __restrict__ list, int len,
                                               const float4* __restrict__ npos, float px, float py, float pz,
                                               F&& f) {
    const size_t sn = (size_t)n;
    const int* __restrict__ p = list + i;
    int k = 0;
    if (!PIPE) {
#pragma unroll 1
        for (; k + U <= len; k += U, p += U * sn) {
            int j[U];
            float4 q[U];
#pragma unroll
            for (int u = 0; u < U; ++u) j[u] = __ldg(p + u * sn);
#pragma unroll
            for (int u = 0; u < U; ++u) q[u] = __ldg(&npos[j[u]]);
#pragma unroll
            for (int u = 0; u < U; ++u)
                f(j[u], q[u], __fsub_rn(px, q[u].x), __fsub_rn(py, q[u].y), __fsub_rn(pz, q[u].z));
        }
    } else if (PRED) {
        /* batches of U; a last, partial batch loads its missing entries as the particle
         * itself (a valid index) and does not visit them */
        int jn[U];
#pragma unroll
        for (int u = 0; u < U; ++u) jn[u] = u < len ? __ldg(p + u * sn) : i;
#pragma unroll 1
        for (; k < len; k += U) {
            int j[U];
            float4 q[U];
#pragma unroll
            for (int u = 0; u < U; ++u) j[u] = jn[u];
#pragma unroll
            for (int u = 0; u < U; ++u) q[u] = __ldg(&npos[j[u]]);
            p += U * sn;
#pragma unroll
            for (int u = 0; u < U; ++u) jn[u] = k + U + u < len ? __ldg(p + u * sn) : i;
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (k + u < len) f(j[u], q[u], __fsub_rn(px, q[u].x), __fsub_rn(py, q[u].y), __fsub_rn(pz, q[u].z));
        }
        return;
    } else if (len >= U) {
        int jn[U];
#pragma unroll
        for (int u = 0; u < U; ++u) jn[u] = __ldg(p + u * sn);
        p += U * sn;
#pragma unroll 1
        for (;;) {
            int j[U];
            float4 q[U];
#pragma unroll
            for (int u = 0; u < U; ++u) j[u] = jn[u];
#pragma unroll
            for (int u = 0; u < U; ++u) q[u] = __ldg(&npos[j[u]]);
            k += U;
            const bool more = k + U <= len;
            if (more) {
#pragma unroll
                for (int u = 0; u < U; ++u) jn[u] = __ldg(p + u * sn);
                p += U * sn;
            }
#pragma unroll
            for (int u = 0; u < U; ++u)
                f(j[u], q[u], __fsub_rn(px, q[u].x), __fsub_rn(py, q[u].y), __fsub_rn(pz, q[u].z));
            if (!more) break;
        }
    }
#pragma unroll 1
    for (; k < len; ++k, p += sn) {
        const int j = __ldg(p);
        const float4 pj = __ldg(&npos[j]);
        f(j, pj, __fsub_rn(px, pj.x), __fsub_rn(py, pj.y), __fsub_rn(pz, pj.z));
    }
}

/* Neighbour source: either the cell scan or the materialised list, same order. */
template <bool LIST, bool EXACT = true>
struct Neigh {
    const int2* tab;
    const int* list;
    const int* len;
    const float4* npos;
    template <bool PIPE = false, int U = SPH_LIST_UNROLL, bool PRED = false, class F>
    __device__ __forceinline__ void visit(const Const& c, int i, float px, float py, float pz, F&& f) const {
        if (LIST) list_neighbors<U, PIPE, PRED>(i, c.n, list, __ldg(&len[i]), npos, px, py, pz, f);
        else scan_neighbors<EXACT>(c, px, py, pz, tab, npos, f);
    }
};

/* kernels/monaghan_kernels.h:7-47, the Monaghan cubic spline that kernels/kernels.h
 * selects when a program is built without USE_MULLER_KERNELS; hd = SUPPORT_RADIUS (the -D
 * constant), the normalisers and the arithmetic in the kernel text's order.  Used only by
 * COMPAT contexts with sph_params::kernels = SPH_KERNELS_MONAGHAN. */
__device__ __forceinline__ float mon_eval(float hd) { return 1.0f / (3.14159265358979323846f * ((hd * hd) * hd)); }
__device__ __forceinline__ float mon_grad(float hd) {
    return -3.0f / (3.14159265358979323846f * (((hd * hd) * hd) * hd));
}
__device__ __forceinline__ float w_monaghan(float r, float h, float hd) {
    const float q = r / h;
    if (r <= h) return mon_eval(hd) * ((1.0f - 1.5f * (q * q)) + 0.75f * ((q * q) * q));
    if (r <= 2.0f * h) {
        const float t = 2.0f - q;
        return (mon_eval(hd) * 0.25f) * ((t * t) * t);
    }
    return 0.f;
}
/* grad_w_monaghan(r, rn, h): the inner branch subtracts 0.75 rn / h^2 from every component */
__device__ __forceinline__ void grad_w_monaghan(float rx, float ry, float rz, float rn, float h, float hd, float& gx,
                                                float& gy, float& gz) {
    const float g = mon_grad(hd);
    if (rn <= h) {
        const float c = 0.75f * (rn / (h * h)), ih = 1.0f / h;
        gx = (g * rx) * ih - c;
        gy = (g * ry) * ih - c;
        gz = (g * rz) * ih - c;
    } else if (rn <= 2.0f * h) {
        const float ir = 1.0f / rn, t = 2.0f - rn / h, q = t * t;
        gx = (((g * rx) * 0.25f) * ir) * q;
        gy = (((g * ry) * 0.25f) * ir) * q;
        gz = (((g * rz) * 0.25f) * ir) * q;
    } else {
        gx = rx * 0.f;
        gy = ry * 0.f;
        gz = rz * 0.f;
    }
}
__device__ __forceinline__ float lapl_w_monaghan(float rn, float h, float hd) {
    const float l = 3.0f * mon_grad(hd);
    if (rn <= h) return l * (1.0f / h - 1.5f * (rn / (h * h)));
    if (rn <= 2.0f * h) {
        const float t = 2.0f - rn / h;
        return l * (((1.0f / (0.25f * rn)) * (t * t) - 1.0f / rn) + rn / (4.0f * (h * h)));
    }
    return 0.f;
}

/* pown(x, n) restated as left-to-right repeated multiplication. */
__device__ __forceinline__ float pown2(float x) { return x * x; }
__device__ __forceinline__ float pown3(float x) { return (x * x) * x; }
/* Rounded products (__fmul_rn): the equation of state subtracts 1 from the power, and a
 * contracted last multiply (one FMA with the -1) would round once where the kernel text
 * rounds twice, so the pressure would not be the EOS of the density bit for bit. */
__device__ __forceinline__ float pown7(float x) {
    float r = __fmul_rn(x, x);
    r = __fmul_rn(r, x); r = __fmul_rn(r, x); r = __fmul_rn(r, x); r = __fmul_rn(r, x); r = __fmul_rn(r, x);
    return r;
}
/* kernels/surface_tension.h:23-50 */
__device__ __forceinline__ float st_corr(float rho0, float di, float dj) { return 2.0f * rho0 / (di + dj); }
__device__ __forceinline__ float st_kernel(float r, float h, float c) {
    if (r <= 0.5f * h) {
        float t1 = h - r;
        float t2 = (t1 * t1 * t1) * (r * r * r);
        return 2.0f * t2 - c;
    } else if (r <= h) {
        float t1 = h - r;
        return (t1 * t1 * t1) * (r * r * r);
    }
    return 0.0f;
}
/* st_kernel with selects instead of branches (same arithmetic, same values). */
__device__ __forceinline__ float st_kernel_sel(float r, float h, float c) {
    const float t1 = h - r;
    const float t2 = (t1 * t1 * t1) * (r * r * r);
    const float inner = 2.0f * t2 - c;
    return r <= 0.5f * h ? inner : (r <= h ? t2 : 0.0f);
}
/* OpenCL clamp = fmin(fmax(x, lo), hi) and sign(). */
__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
__device__ __forceinline__ float signf(float x) {
    if (x > 0.f) return 1.f;
    if (x < 0.f) return -1.f;
    if (x != x) return 0.f;
    return x;
}
__device__ __forceinline__ float len3(float x, float y, float z) { return sqrtf(x * x + y * y + z * z); }


}  // namespace sph
