/*
 * sph_grid.cu -- uniform-grid binning kernels.
 *
 *   k_hashes      compute_hashes (kernels/grid.cl:20-39): Morton key + identity mask; also
 *                 clears the cell-table entries the previous step wrote, so the table never
 *                 needs the O(cells) fill of fluid/simulation/grid.cpp:41.
 *   k_gather      clshuffle (opencl/algorithms/clshuffle.h:12-58) for every fluid array in
 *                 one pass: dst[i] = src[mask[i]].
 *   k_cell_ranges compute_cell_intervals (kernels/grid.cl:60-123): [start, end) per occupied
 *                 cell from adjacent sorted keys (neighbours read from L1, no local-memory
 *                 staging or barrier needed on this hardware).
 *   k_neigh_lists compute_neigh_list (kernels/grid.cl:145-182) for the fluid and the boundary
 *                 tables in one launch, column-major list[k * n + i].
 * All are HBM-streaming kernels.
 */
#include "sph_kernels.cuh"

namespace sph {

__global__ void k_hashes(Const c0, const float4* __restrict__ pos, int n, uint32_t* __restrict__ keys,
                         int32_t* __restrict__ mask, int2* __restrict__ tab, const int32_t* __restrict__ cell_prev,
                         unsigned* __restrict__ flags, const SceneDev* __restrict__ scenes,
                         const int32_t* __restrict__ scene_of) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (cell_prev) {
        const int pc = cell_prev[i];
        if (pc >= 0) tab[pc] = make_int2(0, 0);
    }
    Const c = c0;
    const uint32_t sid = scene_of ? (uint32_t)scene_of[i] : 0u;
    scene_setup(c, scenes, scene_of, i);
    const float4 p = pos[i];
    int cx, cy, cz;
    cell_of(c, p.x, p.y, p.z, cx, cy, cz);
    /* batched: the scene id above the Morton bits keeps every scene's range contiguous */
    keys[i] = (sid << c.scene_shift) | morton3((uint32_t)cx, (uint32_t)cy, (uint32_t)cz);
    if (mask) mask[i] = i;   /* the identity values of the stage API (the step's sort needs none) */
    if (!c.wrap) {
        /* PHYSICS grid clamps: report particles outside it (informational) */
        const float fx = floorf(__fdiv_rn(__fsub_rn(p.x, c.ox), c.cell));
        const float fy = floorf(__fdiv_rn(__fsub_rn(p.y, c.oy), c.cell));
        const float fz = floorf(__fdiv_rn(__fsub_rn(p.z, c.oz), c.cell));
        const bool out = !(fx >= 0.f && fx < (float)c.nx && fy >= 0.f && fy < (float)c.ny && fz >= 0.f &&
                           fz < (float)c.nz);
        if (out) atomicOr(flags, kFlagEscaped);
    }
}

__global__ void k_gather(int n, const int32_t* __restrict__ perm, const float4* __restrict__ a,
                         float4* __restrict__ as, const float4* __restrict__ b, float4* __restrict__ bs,
                         const float4* __restrict__ c3, float4* __restrict__ cs, const int32_t* __restrict__ ids,
                         int32_t* __restrict__ ids_s) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int src = perm[i];
    as[i] = __ldg(&a[src]);
    bs[i] = __ldg(&b[src]);
    if (c3) cs[i] = __ldg(&c3[src]);
    if (ids) ids_s[i] = __ldg(&ids[src]);
}

__global__ void k_gather_boundary(int n, const int32_t* __restrict__ perm, const float4* __restrict__ pos,
                                  float4* __restrict__ pos_s, const int32_t* __restrict__ body,
                                  int32_t* __restrict__ body_s, const float* __restrict__ phi,
                                  float* __restrict__ phi_s) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int src = perm[i];
    pos_s[i] = pos[src];
    body_s[i] = body[src];
    if (phi) phi_s[i] = phi[src];
}

/* Global cell id of a sorted particle: linear id in its scene's grid + the scene's offset;
 * -1 when outside the table. */
__device__ __forceinline__ long long global_cell(const Const& c0, const float4& p, const SceneDev* scenes,
                                                 const int32_t* scene_of, int i) {
    Const c = c0;
    const long long base = scene_setup(c, scenes, scene_of, i);
    int x, y, z;
    cell_of(c, p.x, p.y, p.z, x, y, z);
    const long long id = cell_lin(c, x, y, z);
    return (id >= 0 && id < c.ncells) ? base + id : -1;
}

__global__ void k_cell_ranges(Const c, const float4* __restrict__ spos, const uint32_t* __restrict__ keys, int n,
                              int2* __restrict__ tab, int32_t* __restrict__ cell_out, unsigned* __restrict__ flags,
                              const SceneDev* __restrict__ scenes, const int32_t* __restrict__ scene_of) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int* t = reinterpret_cast<int*>(tab);
    const long long id0 = global_cell(c, spos[i], scenes, scene_of, i);
    const bool ok0 = id0 >= 0;
    if (!ok0) atomicOr(flags, kFlagEscaped);
    cell_out[i] = ok0 ? (int)id0 : -1;
    if (i == n - 1) {
        if (ok0) t[2 * id0 + 1] = i + 1;
    } else {
        const uint32_t h0 = keys[i], h1 = keys[i + 1];
        if (h0 < h1) {
            const long long id1 = global_cell(c, spos[i + 1], scenes, scene_of, i + 1);
            if (ok0) t[2 * id0 + 1] = i + 1;
            if (id1 >= 0) t[2 * id1] = i + 1;
        }
    }
}

/* k_gather and k_cell_ranges in one pass for the fused step: the thread of sorted particle i
 * already holds its position, and the position of particle i + 1 is fetched only where a
 * cell ends (h0 < h1).  Same results as the two kernels. */
__global__ void k_gather_ranges(Const c, int n, const int32_t* __restrict__ perm, const float4* __restrict__ a,
                                float4* __restrict__ as, const float4* __restrict__ b, float4* __restrict__ bs,
                                const float4* __restrict__ c3, float4* __restrict__ cs,
                                const int32_t* __restrict__ ids, int32_t* __restrict__ ids_s,
                                const uint32_t* __restrict__ keys, int2* __restrict__ tab,
                                int32_t* __restrict__ cell_out, unsigned* __restrict__ flags,
                                const SceneDev* __restrict__ scenes, const int32_t* __restrict__ scene_of) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int src = __ldg(&perm[i]);
    const float4 p = __ldg(&a[src]);
    as[i] = p;
    bs[i] = __ldg(&b[src]);
    if (c3) cs[i] = __ldg(&c3[src]);
    if (ids) ids_s[i] = __ldg(&ids[src]);
    int* t = reinterpret_cast<int*>(tab);
    const long long id0 = global_cell(c, p, scenes, scene_of, i);
    const bool ok0 = id0 >= 0;
    if (!ok0) atomicOr(flags, kFlagEscaped);
    cell_out[i] = ok0 ? (int)id0 : -1;
    if (i == n - 1) {
        if (ok0) t[2 * id0 + 1] = i + 1;
    } else {
        const uint32_t h0 = __ldg(&keys[i]), h1 = __ldg(&keys[i + 1]);
        if (h0 < h1) {
            const float4 p1 = __ldg(&a[__ldg(&perm[i + 1])]);
            const long long id1 = global_cell(c, p1, scenes, scene_of, i + 1);
            if (ok0) t[2 * id0 + 1] = i + 1;
            if (id1 >= 0) t[2 * id1] = i + 1;
        }
    }
}

__global__ void k_neigh_lists(Const c0, const float4* __restrict__ spos, const int2* __restrict__ tab0,
                              const float4* __restrict__ bpos_s, const int2* __restrict__ btab0,
                              int* __restrict__ nlist, int* __restrict__ nlen, int* __restrict__ sblist,
                              int* __restrict__ sblen, const SceneDev* __restrict__ scenes,
                              const int32_t* __restrict__ scene_of, const uint8_t* __restrict__ bnear,
                              const int32_t* __restrict__ noff) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c0.n) return;
    Const c = c0;
    const long long base = scene_setup(c, scenes, scene_of, i);
    const int2* tab = tab0 + base;
    const int2* btab = btab0 + base;
    const float4 pi = spos[i];
    int cx, cy, cz;
    cell_of(c, pi.x, pi.y, pi.z, cx, cy, cz);
    const int* nof = c.batched ? nullptr : noff;
    char* const lrow = reinterpret_cast<char*>(nlist + i);
    const unsigned n4 = 4u * (unsigned)c.n;
    const int k = build_scan(c, pi.x, pi.y, pi.z, cx, cy, cz, tab, spos, nof, [&](bool hit, int j, float, int slot) {
        if (hit) *list_slot(lrow, slot, n4) = j;
    });
    nlen[i] = k;
    int kb = 0;
    /* boundary cells only where bnear marks one within a cell (PHYSICS grid) */
    if (c.nb > 0 && (c.wrap || bnear == nullptr || bnear[base + cell_lin(c, cx, cy, cz)] != 0)) {
        char* const brow = reinterpret_cast<char*>(sblist + i);
        kb = build_scan(c, pi.x, pi.y, pi.z, cx, cy, cz, btab, bpos_s, nof, [&](bool hit, int j, float, int slot) {
            if (hit) *list_slot(brow, slot, n4) = j;
        });
    }
    sblen[i] = kb;
}

static inline int blocks_for(long long n, int bs) { return (int)((n + bs - 1) / bs); }

void launch_hashes(cudaStream_t s, const Const& c, const float4* pos, int n, uint32_t* keys, int32_t* mask,
                   int2* tab, const int32_t* cell_prev, unsigned* flags, int bs, const SceneDev* scenes,
                   const int32_t* scene_of) {
    if (n <= 0) return;
    k_hashes<<<blocks_for(n, bs), bs, 0, s>>>(c, pos, n, keys, mask, tab, cell_prev, flags, scenes, scene_of);
}
void launch_gather(cudaStream_t s, int n, const int32_t* perm, const float4* a, float4* as, const float4* b,
                   float4* bs_, const float4* c3, float4* cs, const int32_t* ids, int32_t* ids_s, int bs) {
    if (n <= 0) return;
    k_gather<<<blocks_for(n, bs), bs, 0, s>>>(n, perm, a, as, b, bs_, c3, cs, ids, ids_s);
}
void launch_gather_boundary(cudaStream_t s, int n, const int32_t* perm, const float4* pos, float4* pos_s,
                            const int32_t* body, int32_t* body_s, const float* phi, float* phi_s, int bs) {
    if (n <= 0) return;
    k_gather_boundary<<<blocks_for(n, bs), bs, 0, s>>>(n, perm, pos, pos_s, body, body_s, phi, phi_s);
}
void launch_gather_ranges(cudaStream_t s, const Const& c, int n, const int32_t* perm, const float4* a, float4* as,
                          const float4* b, float4* bs_, const float4* c3, float4* cs, const int32_t* ids,
                          int32_t* ids_s, const uint32_t* keys, int2* tab, int32_t* cell_out, unsigned* flags, int bs,
                          const SceneDev* scenes, const int32_t* scene_of) {
    if (n <= 0) return;
    k_gather_ranges<<<blocks_for(n, bs), bs, 0, s>>>(c, n, perm, a, as, b, bs_, c3, cs, ids, ids_s, keys, tab,
                                                     cell_out, flags, scenes, scene_of);
}
void launch_cell_ranges(cudaStream_t s, const Const& c, const float4* spos, const uint32_t* keys, int n,
                        int2* tab, int32_t* cell_out, unsigned* flags, int bs, const SceneDev* scenes,
                        const int32_t* scene_of) {
    if (n <= 0) return;
    k_cell_ranges<<<blocks_for(n, bs), bs, 0, s>>>(c, spos, keys, n, tab, cell_out, flags, scenes, scene_of);
}
void launch_neigh_lists(cudaStream_t s, const Const& c, const float4* spos, const int2* tab, const float4* bpos_s,
                        const int2* btab, int* nlist, int* nlen, int* sblist, int* sblen, int bs,
                        const SceneDev* scenes, const int32_t* scene_of, const uint8_t* bnear,
                        const int32_t* noff) {
    if (c.n <= 0) return;
    k_neigh_lists<<<blocks_for(c.n, bs), bs, 0, s>>>(c, spos, tab, bpos_s, btab, nlist, nlen, sblist, sblen, scenes,
                                                     scene_of, bnear, noff);
}

}  // namespace sph
