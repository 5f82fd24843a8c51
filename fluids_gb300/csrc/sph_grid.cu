/*
 * sph_grid.cu -- uniform-grid binning kernels.
 *
 *   k_hashes      compute_hashes (kernels/grid.cl:20-39): Morton key + identity mask; also
 *                 clears the cell-table entries the previous step wrote, so the table never
 *                 needs the O(cells) fill of fluid/simulation/grid.cpp:41.  k_hashes_flags
 *                 is the fused step's form, which also runs the incremental sort's first
 *                 pass on the keys.
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

/* compute_hashes for particle i: clears the cell-table entry its previous cell left, returns
 * its key (and reports a particle outside a PHYSICS grid). */
__device__ __forceinline__ uint32_t hash_particle(const Const& c0, const float4 p, int i, int2* __restrict__ tab,
                                                  int pc, unsigned* __restrict__ flags,
                                                  const SceneDev* __restrict__ scenes,
                                                  const int32_t* __restrict__ scene_of) {
    if (pc >= 0) tab[pc] = make_int2(0, 0);
    Const c = c0;
    const uint32_t sid = scene_of ? (uint32_t)scene_of[i] : 0u;
    scene_setup(c, scenes, scene_of, i);
    /* cell_of, with each axis's division done once for the cell and the escape test */
    const float fx = axis_floor(p.x, c.ox, c.cell), fy = axis_floor(p.y, c.oy, c.cell),
                fz = axis_floor(p.z, c.oz, c.cell);
    if (!c.wrap) {
        /* PHYSICS grid clamps: report particles outside it (informational) */
        const bool out = !(fx >= 0.f && fx < (float)c.nx && fy >= 0.f && fy < (float)c.ny && fz >= 0.f &&
                           fz < (float)c.nz);
        if (out) atomicOr(flags, kFlagEscaped);
    }
    const int cx = axis_clamp(fx, c.nx, c.wrap), cy = axis_clamp(fy, c.ny, c.wrap), cz = axis_clamp(fz, c.nz, c.wrap);
    /* batched: the scene id above the Morton bits keeps every scene's range contiguous */
    return (sid << c.scene_shift) | morton3((uint32_t)cx, (uint32_t)cy, (uint32_t)cz);
}

__global__ void k_hashes(Const c0, const float4* __restrict__ pos, int n, uint32_t* __restrict__ keys,
                         int32_t* __restrict__ mask, int2* __restrict__ tab, const int32_t* __restrict__ cell_prev,
                         unsigned* __restrict__ flags, const SceneDev* __restrict__ scenes,
                         const int32_t* __restrict__ scene_of) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    keys[i] = hash_particle(c0, pos[i], i, tab, cell_prev ? cell_prev[i] : -1, flags, scenes, scene_of);
    if (mask) mask[i] = i;   /* the identity values of the stage API */
}

/* k_hashes of the fused step with the incremental sort's first pass (k_inc_flags of
 * sph_sort.cu) on the keys it computes: tiles of kIncTile particles, kIncItems a thread. */
__global__ void __launch_bounds__(256) k_hashes_flags(Const c0, const float4* __restrict__ pos, int n,
                                                      uint32_t* __restrict__ keys, int2* __restrict__ tab,
                                                      const int32_t* __restrict__ cell_prev,
                                                      unsigned* __restrict__ flags,
                                                      const SceneDev* __restrict__ scenes,
                                                      const int32_t* __restrict__ scene_of, IncFlags inc) {
    constexpr int kItems = kIncItems;
    __shared__ uint32_t s_wcnt[8];
    __shared__ uint32_t s_base;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wbase = ((int)blockIdx.x * kIncTile) + warp * (32 * kItems);   /* n < 2^31 */
    const bool have_prev = *inc.valid != 0u;
    if (!have_prev && blockIdx.x == 0 && tid == 0) *inc.over = 1u;   /* no previous result: a full sort */
    float4 p[kItems];
    int pc[kItems];
    uint32_t old[kItems];
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const int idx = wbase + k * 32 + lane;
        const bool in = idx < n;
        p[k] = in ? __ldg(&pos[idx]) : make_float4(0.f, 0.f, 0.f, 0.f);
        pc[k] = in && cell_prev ? __ldg(&cell_prev[idx]) : -1;
        old[k] = in ? __ldg(&inc.prev[idx]) : 0u;
    }
    uint32_t cnt = 0, word[kItems], key[kItems];
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const int w0 = wbase + k * 32, idx = w0 + lane;
        key[k] = 0u;
        if (idx < n) {
            key[k] = hash_particle(c0, p[k], idx, tab, pc[k], flags, scenes, scene_of);
            keys[idx] = key[k];
        }
        word[k] = __ballot_sync(0xffffffffu, idx < n && (!have_prev || key[k] != old[k]));
        if (lane == 0 && w0 < n) inc.bits[w0 >> 5] = word[k];
        cnt += (uint32_t)__popc(word[k]);
    }
    if (lane == 0) s_wcnt[warp] = cnt;
    __syncthreads();
    if (tid == 0) {
        uint32_t total = 0;
#pragma unroll
        for (int w = 0; w < 8; ++w) total += s_wcnt[w];
        inc.tcnt[blockIdx.x] = total;
        s_base = have_prev && total ? atomicAdd(inc.lcount, total) : 0u;
    }
    __syncthreads();
    if (!have_prev || cnt == 0) return;
    uint32_t run = s_base;
    for (int w = 0; w < warp; ++w) run += s_wcnt[w];
    const unsigned lt = (1u << lane) - 1u;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        if ((word[k] >> lane) & 1u)
            inc.list[run + (uint32_t)__popc(word[k] & lt)] = make_int2(wbase + k * 32 + lane, (int)key[k]);
        run += (uint32_t)__popc(word[k]);
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
    if (b) bs[i] = __ldg(&b[src]);
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
    if (b) bs[i] = __ldg(&b[src]);   /* null: the velocities are gathered later */
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
void launch_hashes_flags(cudaStream_t s, const Const& c, const float4* pos, int n, uint32_t* keys, int2* tab,
                         const int32_t* cell_prev, unsigned* flags, const SceneDev* scenes, const int32_t* scene_of,
                         const IncFlags& inc) {
    if (n <= 0) return;
    k_hashes_flags<<<blocks_for(n, kIncTile), 256, 0, s>>>(c, pos, n, keys, tab, cell_prev, flags, scenes, scene_of,
                                                           inc);
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
