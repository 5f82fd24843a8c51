/*
 * sph_sort.cu -- stable LSD onesweep radix sort of (uint32 key, int32 value) pairs.
 *
 * Replaces clsort<cl_uint, cl_int> (opencl/algorithms/clsort.h:13-35), which calls the
 * external clogs 1.5.1 Radixsort (a stable LSD radix sort).  The permutation of a stable
 * ascending sort is unique, so any correct stable sort reproduces it bit for bit.
 *
 * Algorithm (Adinets & Merrill, "Onesweep", 2022):
 *   1. k_sort_hist: one read of the keys builds the 256-bin histogram of every 8-bit digit
 *      pass at once (warp match_any aggregation into shared counters).
 *   2. per pass, k_onesweep: each CTA takes the next tile id from an atomic counter (so
 *      tiles are scheduled in order), ranks its kTile keys stably (warp match_any per
 *      32-key round, per-warp digit counters), publishes its per-digit counts, and looks
 *      back over earlier tiles' published counts (decoupled look-back) for its global
 *      digit offsets.  Keys are then reordered in shared memory by digit and written out
 *      so that consecutive threads write consecutive addresses of a digit bucket.
 * Traffic per pass: 8 B read + 8 B written per pair.
 * Every look-back wait is bounded: after kSpinLimit polls the CTA sets SPH_FLAG_TIMEOUT in
 * the flag word, treats the missing count as 0 and finishes (the result is then wrong);
 * with in-order tile ids the wait always ends.  A context's step sorts into the context's
 * flag word, which sph_device_flags reads (SPH_FLAG_TIMEOUT); the standalone entry points
 * sph_sort_pairs and sph_sort_pairs_noalloc do not read their flag word back.
 */
#include "sph_kernels.cuh"

namespace sph {

namespace {
constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kItems = 16;
constexpr int kTile = kThreads * kItems;   /* 4096 keys per tile */
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagInc = 2u << 30;
constexpr uint32_t kValMask = (1u << 30) - 1u;
constexpr long long kSpinLimit = 1LL << 22;

__device__ __forceinline__ uint32_t ld_volatile(const uint32_t* p) {
    return *reinterpret_cast<const volatile uint32_t*>(p);
}
__device__ __forceinline__ void st_volatile(uint32_t* p, uint32_t v) {
    *reinterpret_cast<volatile uint32_t*>(p) = v;
}

/* Exclusive prefix sum over the 256 values held one per thread (blockDim = 256). */
__device__ __forceinline__ uint32_t block_exclusive_scan_256(uint32_t v, uint32_t* s_warp) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < kWarps ? s_warp[lane] : 0u;
#pragma unroll
        for (int d = 1; d < kWarps; d <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, d);
            if (lane >= d) w += y;
        }
        if (lane < kWarps) s_warp[lane] = w;
    }
    __syncthreads();
    uint32_t before = warp > 0 ? s_warp[warp - 1] : 0u;
    __syncthreads();
    return before + x - v;
}
}  // namespace

/* Histogram of all digit passes: hist[pass][256].  Each thread loads kHistItems keys
 * (coalesced across the warp) before it ranks any, so that their loads are in flight
 * together; per key and pass, the lanes holding the same digit add their count once. */
constexpr int kHistItems = 8;
__global__ void __launch_bounds__(kThreads) k_sort_hist(const uint32_t* __restrict__ keys, int n, int passes,
                                                        uint32_t* __restrict__ hist) {
    __shared__ uint32_t s_hist[4][256];
    for (int t = threadIdx.x; t < 4 * 256; t += kThreads) (&s_hist[0][0])[t] = 0u;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const long long step = (long long)gridDim.x * kThreads * kHistItems;
    for (long long base = (long long)blockIdx.x * kThreads * kHistItems; base < n; base += step) {
        uint32_t k[kHistItems];
#pragma unroll
        for (int u = 0; u < kHistItems; ++u) {
            const long long i = base + (long long)u * kThreads + threadIdx.x;
            k[u] = i < n ? __ldg(&keys[i]) : 0u;
        }
#pragma unroll
        for (int u = 0; u < kHistItems; ++u) {
            const long long i = base + (long long)u * kThreads + threadIdx.x;
            const bool valid = i < n;
            const unsigned active = __ballot_sync(0xffffffffu, valid);
            if (valid) {
                for (int p = 0; p < passes; ++p) {
                    const uint32_t d = (k[u] >> (8 * p)) & 255u;
                    const unsigned peers = __match_any_sync(active, d);
                    if (lane == __ffs(peers) - 1) atomicAdd(&s_hist[p][d], (uint32_t)__popc(peers));
                }
            }
        }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < passes * 256; t += kThreads) {
        const uint32_t v = (&s_hist[0][0])[t];
        if (v) atomicAdd(&hist[t], v);
    }
}

__global__ void __launch_bounds__(kThreads) k_onesweep(const uint32_t* __restrict__ kin, const int32_t* __restrict__ vin,
                                                       uint32_t* __restrict__ kout, int32_t* __restrict__ vout, int n,
                                                       int shift, int pass, int tiles,
                                                       const uint32_t* __restrict__ hist,
                                                       uint32_t* __restrict__ counters, uint32_t* __restrict__ status,
                                                       unsigned* __restrict__ flags) {
    __shared__ uint32_t s_keys[kTile];
    __shared__ int32_t s_vals[kTile];
    __shared__ uint32_t s_whist[kWarps][256];
    __shared__ uint32_t s_tprefix[256];
    __shared__ uint32_t s_dbase[256];
    __shared__ uint32_t s_scan[kWarps];
    __shared__ uint32_t s_tile;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(&counters[pass], 1u);
    for (int t = tid; t < kWarps * 256; t += kThreads) (&s_whist[0][0])[t] = 0u;
    __syncthreads();
    const int tile = (int)s_tile;
    const long long base = (long long)tile * kTile;
    const long long wbase = base + (long long)warp * (32 * kItems);
    const unsigned lt_mask = (1u << lane) - 1u;

    uint32_t key[kItems];
    int32_t val[kItems];
    uint32_t rank[kItems];
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const long long idx = wbase + k * 32 + lane;
        const bool valid = idx < n;
        key[k] = valid ? __ldg(&kin[idx]) : 0xffffffffu;   /* tail keys sort last and are not written */
        val[k] = valid ? __ldg(&vin[idx]) : 0;
    }
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const uint32_t d = (key[k] >> shift) & 255u;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const uint32_t before = s_whist[warp][d];
        __syncwarp();
        if ((peers & lt_mask) == 0u) s_whist[warp][d] = before + (uint32_t)__popc(peers);
        __syncwarp();
        rank[k] = before + (uint32_t)__popc(peers & lt_mask);
    }
    __syncthreads();

    /* thread tid owns digit d = tid: per-warp exclusive offsets and the tile's count */
    const int d = tid;
    uint32_t cnt = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
        const uint32_t c = s_whist[w][d];
        s_whist[w][d] = cnt;
        cnt += c;
    }
    /* publish this tile's aggregate (tile 0 publishes its inclusive prefix directly) */
    uint32_t* st = status + ((size_t)pass * tiles + tile) * 256;
    uint32_t prior = 0;
    if (tile == 0) {
        st_volatile(&st[d], kFlagInc | cnt);
    } else {
        st_volatile(&st[d], kFlagAgg | cnt);
        for (int t = tile - 1; t >= 0; --t) {
            const uint32_t* sp = status + ((size_t)pass * tiles + t) * 256 + d;
            uint32_t s = ld_volatile(sp);
            long long spins = 0;
            while ((s & (kFlagAgg | kFlagInc)) == 0u) {
                if (++spins > kSpinLimit) {
                    atomicOr(flags, kFlagTimeout);
                    s = kFlagInc;
                    break;
                }
                __nanosleep(32);
                s = ld_volatile(sp);
            }
            prior += s & kValMask;
            if (s & kFlagInc) break;
        }
        st_volatile(&st[d], kFlagInc | ((prior + cnt) & kValMask));
    }
    /* global base of digit d for this tile: bucket start + counts of earlier tiles */
    const uint32_t bucket = block_exclusive_scan_256(hist[(size_t)pass * 256 + d], s_scan);
    const uint32_t tpre = block_exclusive_scan_256(cnt, s_scan);
    s_tprefix[d] = tpre;
    s_dbase[d] = bucket + prior;
    __syncthreads();

    /* reorder the tile in shared memory by digit (stable) */
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const uint32_t dk = (key[k] >> shift) & 255u;
        const uint32_t slot = s_tprefix[dk] + s_whist[warp][dk] + rank[k];
        s_keys[slot] = key[k];
        s_vals[slot] = val[k];
    }
    __syncthreads();
    const int nvalid = (int)min((long long)kTile, (long long)n - base);
    for (int s = tid; s < nvalid; s += kThreads) {
        const uint32_t kk = s_keys[s];
        const uint32_t dk = (kk >> shift) & 255u;
        const uint32_t dest = s_dbase[dk] + (uint32_t)s - s_tprefix[dk];
        kout[dest] = kk;
        vout[dest] = s_vals[s];
    }
}

int sort_passes(int key_bits) { return key_bits <= 0 ? 0 : (key_bits + 7) / 8; }
int sort_tiles(int n) { return (n + kTile - 1) / kTile; }

size_t sort_workspace_bytes(int n, int key_bits) {
    const int passes = sort_passes(key_bits);
    return (size_t)(4 * 256 + 64) * 4 + (size_t)passes * sort_tiles(n) * 256 * 4;
}

void sort_pairs(cudaStream_t s, uint32_t* k0, int32_t* v0, uint32_t* k1, int32_t* v1, int n, int key_bits,
                void* ws, unsigned* flags, int num_sms, uint32_t** kres, int32_t** vres) {
    *kres = k0;
    *vres = v0;
    const int passes = sort_passes(key_bits);
    if (n <= 1 || passes == 0) return;
    const int tiles = sort_tiles(n);
    uint32_t* hist = reinterpret_cast<uint32_t*>(ws);
    uint32_t* counters = hist + 4 * 256;
    uint32_t* status = counters + 64;
    cudaMemsetAsync(ws, 0, sort_workspace_bytes(n, key_bits), s);
    int hblocks = min((n + kThreads * kHistItems - 1) / (kThreads * kHistItems), 4 * num_sms);
    if (hblocks < 1) hblocks = 1;
    k_sort_hist<<<hblocks, kThreads, 0, s>>>(k0, n, passes, hist);
    uint32_t *ki = k0, *ko = k1;
    int32_t *vi = v0, *vo = v1;
    for (int p = 0; p < passes; ++p) {
        k_onesweep<<<tiles, kThreads, 0, s>>>(ki, vi, ko, vo, n, 8 * p, p, tiles, hist, counters, status, flags);
        uint32_t* tk = ki; ki = ko; ko = tk;
        int32_t* tv = vi; vi = vo; vo = tv;
    }
    *kres = ki;
    *vres = vi;
}

}  // namespace sph
