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
 * sph_sort_pairs and sph_sort_pairs_noalloc do not read their flag word back.  A grid
 * smaller than the tile count loops over tiles (the gated use below).
 *
 * The step's sort (sort_pairs_incremental, second half of this file) computes the same
 * permutation as an update of the previous step's sorted keys: only the particles whose key
 * changed are searched for and merged; the onesweep runs, gated, when there is no previous
 * result or too many particles moved.
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
                                                        uint32_t* __restrict__ hist, const unsigned* __restrict__ gate) {
    __shared__ uint32_t s_hist[4][256];
    if (gate && *gate == 0u) return;   /* a sort that an earlier kernel found unnecessary */
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
                                                       unsigned* __restrict__ flags, const unsigned* __restrict__ gate) {
    __shared__ uint32_t s_keys[kTile];
    __shared__ int32_t s_vals[kTile];
    __shared__ uint32_t s_whist[kWarps][256];
    __shared__ uint32_t s_tprefix[256];
    __shared__ uint32_t s_dbase[256];
    __shared__ uint32_t s_scan[kWarps];
    __shared__ uint32_t s_tile;

    if (gate && *gate == 0u) return;   /* the whole grid leaves together */
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    /* a grid smaller than the tile count loops: each CTA takes tiles until none is left
     * (a tile's look-back waits only on tiles taken before it, by CTAs that are running) */
    for (;;) {
    if (tid == 0) s_tile = atomicAdd(&counters[pass], 1u);
    for (int t = tid; t < kWarps * 256; t += kThreads) (&s_whist[0][0])[t] = 0u;
    __syncthreads();
    const int tile = (int)s_tile;
    if (tile >= tiles) return;
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
        val[k] = valid ? (vin ? __ldg(&vin[idx]) : (int32_t)idx) : 0;   /* no vin: the identity */
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
    if ((int)gridDim.x >= tiles) return;   /* one tile per CTA */
    __syncthreads();                        /* the next tile reuses the shared arrays */
    }
}

int sort_passes(int key_bits) { return key_bits <= 0 ? 0 : (key_bits + 7) / 8; }
int sort_tiles(int n) { return (n + kTile - 1) / kTile; }

size_t sort_workspace_bytes(int n, int key_bits) {
    const int passes = sort_passes(key_bits);
    return (size_t)(4 * 256 + 64) * 4 + (size_t)passes * sort_tiles(n) * 256 * 4;
}

/* gate: null, or a flag word an earlier kernel of the stream wrote; every kernel of the sort
 * leaves at once while it is 0.  v0 may be null for identity values. */
static void sort_pairs_impl(cudaStream_t s, const uint32_t* k0, const int32_t* v0, uint32_t* k1, int32_t* v1,
                            uint32_t* k2, int32_t* v2, int n, const unsigned* gate, int key_bits, void* ws,
                            unsigned* flags, int num_sms, uint32_t** kres, int32_t** vres) {
    const int passes = sort_passes(key_bits);
    const int tiles = sort_tiles(n);
    uint32_t* hist = reinterpret_cast<uint32_t*>(ws);
    uint32_t* counters = hist + 4 * 256;
    uint32_t* status = counters + 64;
    cudaMemsetAsync(ws, 0, sort_workspace_bytes(n, key_bits), s);
    /* a gated sort usually leaves at once: its grids are one wave of looping CTAs */
    int hblocks = min((n + kThreads * kHistItems - 1) / (kThreads * kHistItems), (gate ? 1 : 4) * num_sms);
    if (hblocks < 1) hblocks = 1;
    const int sblocks = gate ? min(tiles, 2 * num_sms) : tiles;
    k_sort_hist<<<hblocks, kThreads, 0, s>>>(k0, n, passes, hist, gate);
    /* pass p reads the previous pass's output and writes (k1, v1) or (k2, v2) in turn */
    const uint32_t* ki = k0;
    const int32_t* vi = v0;
    for (int p = 0; p < passes; ++p) {
        uint32_t* ko = (p & 1) ? k2 : k1;
        int32_t* vo = (p & 1) ? v2 : v1;
        k_onesweep<<<sblocks, kThreads, 0, s>>>(ki, vi, ko, vo, n, 8 * p, p, tiles, hist, counters, status, flags,
                                                gate);
        ki = ko;
        vi = vo;
    }
    *kres = const_cast<uint32_t*>(ki);
    *vres = const_cast<int32_t*>(vi);
}

void sort_pairs(cudaStream_t s, uint32_t* k0, int32_t* v0, uint32_t* k1, int32_t* v1, int n, int key_bits,
                void* ws, unsigned* flags, int num_sms, uint32_t** kres, int32_t** vres) {
    *kres = k0;
    *vres = v0;
    if (n <= 1 || sort_passes(key_bits) == 0) return;
    sort_pairs_impl(s, k0, v0, k1, v1, k0, v0, n, nullptr, key_bits, ws, flags, num_sms, kres, vres);
}

/* ---------------------------------------------------------------------------------------
 * Incremental stable sort of a step's cell keys against the previous step's sorted keys.
 *
 * The fluid arrays stay in the previous step's sorted order between steps, so particle i
 * of this step was sorted particle i of the last one and prev[i] is its key then.  Call a
 * particle "stayed" when its key did not change (keys[i] == prev[i]) and "moved" otherwise.
 * prev is non-decreasing, so the stayed particles are already in (key, index) order, and
 * the stable sort of all keys is their merge, by (key, index), with the moved ones.  That
 * holds for any non-decreasing prev.  prev is the workspace's own copy of the last result
 * (written beside the output, so that writes to the output from outside cannot unsort it).
 *
 *   k_inc_flags  per tile of kIncTile positions: the moved flags as ballot words (bits), the
 *                tile's count of moved particles, and the moved (index, key) pairs appended
 *                to a list (one atomic per tile; the list's order does not matter).  The
 *                step's hash kernel does the same pass on the keys it computes
 *                (k_hashes_flags, sph_grid.cu).
 *   k_inc_place  per moved particle (k, i): p = the first position whose (prev[p], p) is
 *                not below (k, i), by binary searches over each tile's first prev key (a
 *                table staged in shared memory), then each word's first prev key within
 *                the tile, then prev within the word.  (k, i, p) goes to bucket p / kIncTile.
 *                The stayed particles at positions [t kIncTile, (t + 1) kIncTile) are all
 *                above the moved particles of the buckets below t and below those of the
 *                buckets above t, so only bucket t's need comparing with them.  The last
 *                CTA turns the tile and bucket counts into prefix sums.
 *   k_inc_merge  per tile t: a bucket particle e is below the stayed particle at position j
 *                exactly when p_e <= j, so a prefix sum of the bucket's insertion points
 *                over the tile gives every stayed particle its count of bucket particles
 *                below it; the bucket's particles are ranked by p and, for equal p, by
 *                (key, index).  A moved particle goes to (stayed before p) + (moved
 *                particles of the buckets below t) + its rank, a stayed particle of stayed
 *                rank a to a + (moved particles of the buckets below t) + (bucket particles
 *                below it).
 *   k_inc_keep   after an overflow, keeps the full sort's keys as prev; marks prev valid.
 * A bucket holds kIncBucket particles.  When one overflows, when more than a sixth of the
 * particles moved (their searches would cost more than a full sort), or when there is no
 * previous result (the first call), the overflow word opens the gated full onesweep sort of
 * all keys (its kernels read the word and leave at once while it is 0; they run on a side
 * stream beside k_inc_merge, which then leaves at once).  Moved particles are 1-2 % of a
 * flowing scene per step: the passes over all particles then read 8 bytes and write 12
 * bytes per particle.
 * ------------------------------------------------------------------------------------- */
namespace {
static_assert(kIncTile == kThreads * kIncItems, "2048 positions = 64 ballot words");
constexpr int kIncShift = 11;
constexpr int kIncWords = kIncTile / 32;
constexpr int kIncBucket = 1024;                 /* moved particles per merge tile before overflow */

struct IncLayout {
    size_t valid, prev, first, sub, bits, list, store, zero, over, lcount, done, bcnt, tcnt, tpre, boff, vscr, total,
        zero_bytes;
    int tiles, words;
    IncLayout(int n) {
        const size_t nn = (size_t)(n > 0 ? n : 1);
        tiles = (int)((nn + kIncTile - 1) / kIncTile);
        words = (int)((nn + 31) / 32);
        size_t off = 0;
        auto take = [&](size_t bytes) {
            const size_t at = off;
            off = (off + bytes + 255) & ~size_t(255);
            return at;
        };
        valid = take(4);
        prev = take(4 * nn);
        first = take(4 * (size_t)tiles);   /* prev at each tile's first position */
        sub = take(4 * (size_t)words);     /* prev at each word's first position */
        bits = take(4 * (size_t)words);
        list = take(8 * nn);
        store = take(16 * (size_t)tiles * kIncBucket);
        /* zeroed by every call: the overflow word, the list length, the count of finished
         * placing CTAs and the bucket counts (the other arrays are written whole) */
        zero_bytes = 4 * (3 + (size_t)tiles);
        zero = take(zero_bytes);
        over = zero;
        lcount = over + 4;
        done = lcount + 4;
        bcnt = done + 4;
        tcnt = take(4 * (size_t)tiles);
        tpre = take(4 * (size_t)tiles);
        boff = take(4 * (size_t)tiles);
        vscr = take(4 * nn);   /* the gated full sort's second value array */
        total = off;
    }
};

/* a key and its index, ordered by key then index */
__device__ __forceinline__ bool pair_less(uint32_t ka, int32_t ia, uint32_t kb, int32_t ib) {
    return ka < kb || (ka == kb && ia < ib);
}
}  // namespace

__global__ void __launch_bounds__(kThreads) k_inc_flags(const uint32_t* __restrict__ keys,
                                                        const uint32_t* __restrict__ prev, int n,
                                                        const unsigned* __restrict__ valid,
                                                        uint32_t* __restrict__ bits, uint32_t* __restrict__ tcnt,
                                                        unsigned* __restrict__ over, int2* __restrict__ list,
                                                        uint32_t* __restrict__ lcount) {
    __shared__ uint32_t s_wcnt[kWarps];
    __shared__ uint32_t s_base;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wbase = ((int)blockIdx.x << kIncShift) + warp * (32 * kIncItems);   /* n < 2^31 */
    const bool have_prev = *valid != 0u;
    if (!have_prev && blockIdx.x == 0 && tid == 0) *over = 1u;   /* no previous result: a full sort */
    uint32_t key[kIncItems], old[kIncItems];
#pragma unroll
    for (int k = 0; k < kIncItems; ++k) {
        const int idx = wbase + k * 32 + lane;
        key[k] = idx < n ? __ldg(&keys[idx]) : 0u;
        old[k] = idx < n ? __ldg(&prev[idx]) : 0u;
    }
    uint32_t cnt = 0, word[kIncItems];
#pragma unroll
    for (int k = 0; k < kIncItems; ++k) {
        const int w0 = wbase + k * 32;
        word[k] = __ballot_sync(0xffffffffu, w0 + lane < n && (!have_prev || key[k] != old[k]));
        if (lane == 0 && w0 < n) bits[w0 >> 5] = word[k];
        cnt += (uint32_t)__popc(word[k]);
    }
    if (lane == 0) s_wcnt[warp] = cnt;
    __syncthreads();
    if (tid == 0) {
        uint32_t total = 0;
#pragma unroll
        for (int w = 0; w < kWarps; ++w) total += s_wcnt[w];
        tcnt[blockIdx.x] = total;
        /* the moved particles go to a list in any order (one atomic per tile): their places
         * are computed from (key, index) alone */
        s_base = have_prev && total ? atomicAdd(lcount, total) : 0u;
    }
    __syncthreads();
    if (!have_prev || cnt == 0) return;
    uint32_t run = s_base;
    for (int w = 0; w < warp; ++w) run += s_wcnt[w];
    const unsigned lt = (1u << lane) - 1u;
#pragma unroll
    for (int k = 0; k < kIncItems; ++k) {
        if ((word[k] >> lane) & 1u)
            list[run + (uint32_t)__popc(word[k] & lt)] = make_int2(wbase + k * 32 + lane, (int)key[k]);
        run += (uint32_t)__popc(word[k]);
    }
}

constexpr int kIncSmemTiles = 8192;   /* tile-first table staged in shared memory up to 16.7M positions */

__global__ void __launch_bounds__(kThreads) k_inc_place(const int2* __restrict__ list,
                                                        const uint32_t* __restrict__ lcount,
                                                        const uint32_t* __restrict__ prev,
                                                        const uint32_t* __restrict__ first,
                                                        const uint32_t* __restrict__ sub, int n, int tiles,
                                                        const unsigned* __restrict__ valid,
                                                        uint32_t* __restrict__ bcnt, int4* __restrict__ store,
                                                        unsigned* __restrict__ over, unsigned* __restrict__ done,
                                                        const uint32_t* __restrict__ tcnt,
                                                        uint32_t* __restrict__ tpre, uint32_t* __restrict__ boff) {
    extern __shared__ uint32_t s_first[];   /* min(tiles, kIncSmemTiles) entries */
    __shared__ uint32_t s_scan[kWarps];
    __shared__ bool s_last;
    if (*valid == 0u) return;   /* no previous result: the full sort runs */
    const int m = (int)*lcount;
    if (m > n / 6) {
        /* past a sixth of the particles moved, the searches cost more than the full sort */
        if (blockIdx.x == 0 && threadIdx.x == 0) *over = 1u;
        return;
    }
    const bool staged = tiles <= kIncSmemTiles;
    if (staged)
        for (int t = threadIdx.x; t < tiles; t += blockDim.x) s_first[t] = __ldg(&first[t]);
    __syncthreads();
    const int words = (n + 31) >> 5;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < m; r += gridDim.x * blockDim.x) {
        const int2 e = __ldg(&list[r]);
        const int i = e.x;
        const uint32_t k = (uint32_t)e.y;
        /* tiles whose first (prev, position) is below (k, i) */
        int lo = 0, hi = tiles;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            const uint32_t fk = staged ? s_first[mid] : __ldg(&first[mid]);
            if (pair_less(fk, mid << kIncShift, k, i)) lo = mid + 1;
            else hi = mid;
        }
        int p = 0;
        if (lo > 0) {
            /* p lies after tile lo - 1's first position: words of that tile whose first
             * (prev, position) is below (k, i) (its first word is) ... */
            int wlo = ((lo - 1) << (kIncShift - 5)) + 1, whi = min(lo << (kIncShift - 5), words);
            while (wlo < whi) {
                const int mid = (wlo + whi) >> 1;
                if (pair_less(__ldg(&sub[mid]), mid << 5, k, i)) wlo = mid + 1;
                else whi = mid;
            }
            /* ... then p after the first position of word wlo - 1, at most at word wlo's */
            int plo = ((wlo - 1) << 5) + 1, phi = min(wlo << 5, n);
            while (plo < phi) {
                const int mid = (plo + phi) >> 1;
                if (pair_less(__ldg(&prev[mid]), mid, k, i)) plo = mid + 1;
                else phi = mid;
            }
            p = plo;
        }
        const int b = min(p >> kIncShift, tiles - 1);
        const uint32_t slot = atomicAdd(&bcnt[b], 1u);
        if (slot < (uint32_t)kIncBucket) store[(size_t)b * kIncBucket + slot] = make_int4((int)k, i, p, 0);
        else *over = 1u;
    }
    /* the last CTA to finish turns the tile counts and bucket counts into exclusive
     * prefixes (tpre, boff) for the merge */
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    const int per = (tiles + kThreads - 1) / kThreads;
    const int t0 = threadIdx.x * per, t1 = min(t0 + per, tiles);
    uint32_t a = 0, c = 0;
    if (per <= 8) {
        uint32_t va[8], vc[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            va[u] = t0 + u < t1 ? __ldcg(&tcnt[t0 + u]) : 0u;
            vc[u] = t0 + u < t1 ? __ldcg(&bcnt[t0 + u]) : 0u;
        }
        uint32_t ra = 0, rc = 0;
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            a += va[u];
            c += vc[u];
        }
        ra = block_exclusive_scan_256(a, s_scan);
        rc = block_exclusive_scan_256(c, s_scan);
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            if (t0 + u < t1) {
                tpre[t0 + u] = ra;
                boff[t0 + u] = rc;
            }
            ra += va[u];
            rc += vc[u];
        }
        return;
    }
    for (int t = t0; t < t1; ++t) {
        a += __ldcg(&tcnt[t]);
        c += __ldcg(&bcnt[t]);
    }
    uint32_t ra = block_exclusive_scan_256(a, s_scan);
    uint32_t rc = block_exclusive_scan_256(c, s_scan);
    for (int t = t0; t < t1; ++t) {
        tpre[t] = ra;
        boff[t] = rc;
        ra += __ldcg(&tcnt[t]);
        rc += __ldcg(&bcnt[t]);
    }
}

/* The merge of tile t.  A bucket particle e with insertion point p_e is below the stayed
 * particle at position j exactly when p_e <= j (the positions before p_e hold pairs below e,
 * the stayed ones from p_e on pairs above it), so each stayed particle's count of bucket
 * particles below it is a prefix sum of the bucket's insertion points over the tile. */
__global__ void __launch_bounds__(kThreads) k_inc_merge(const uint32_t* __restrict__ keys, int n,
                                                        const uint32_t* __restrict__ bits,
                                                        const uint32_t* __restrict__ tcnt,
                                                        const uint32_t* __restrict__ tpre,
                                                        const uint32_t* __restrict__ boff,
                                                        const uint32_t* __restrict__ bcnt,
                                                        const int4* __restrict__ store,
                                                        const unsigned* __restrict__ over,
                                                        uint32_t* __restrict__ kout, int32_t* __restrict__ vout,
                                                        uint32_t* __restrict__ prev, uint32_t* __restrict__ first,
                                                        uint32_t* __restrict__ sub) {
    __shared__ uint32_t s_k[kIncBucket], s_gk[kIncBucket];
    __shared__ int32_t s_i[kIncBucket], s_p[kIncBucket], s_g[kIncBucket], s_gi[kIncBucket];
    __shared__ uint32_t s_at[kIncTile + 1];   /* bucket particles inserted at each position */
    __shared__ uint32_t s_word[kIncWords], s_wpre[kIncWords];
    __shared__ uint32_t s_scan[kWarps];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int t = blockIdx.x;
    const int tbase = t << kIncShift;
    const int tlen = min(kIncTile, n - tbase);
    if (*over != 0u) return;   /* the gated full sort writes the result */
    /* this tile's keys and moved words first (their loads in flight together) */
    const int wbase = warp * (32 * kIncItems);   /* tile-local */
    uint32_t key[kIncItems], word[kIncItems];
#pragma unroll
    for (int k = 0; k < kIncItems; ++k) {
        const int j = wbase + k * 32 + lane;
        key[k] = j < tlen ? __ldg(&keys[tbase + j]) : 0u;
        word[k] = wbase + k * 32 < tlen ? __ldg(&bits[(tbase + wbase + k * 32) >> 5]) : 0u;
    }
    const uint32_t tile_pre = __ldg(&tpre[t]), off = __ldg(&boff[t]), tile_moved = __ldg(&tcnt[t]);
    const int c = min((int)__ldg(&bcnt[t]), kIncBucket);   /* no overflow: at most kIncBucket */
#pragma unroll
    for (int k = 0; k < kIncItems; ++k) s_at[tid * kIncItems + k] = 0u;
    if (tid == 0) s_at[kIncTile] = 0u;
    uint32_t wc = 0;
#pragma unroll
    for (int k = 0; k < kIncItems; ++k) wc += (uint32_t)__popc(word[k]);
    if (lane == 0) s_wpre[warp] = wc;   /* per-warp totals, scanned below */
    __syncthreads();
    for (int e = tid; e < c; e += kThreads) {
        const int4 v = __ldg(&store[(size_t)t * kIncBucket + e]);
        s_k[e] = (uint32_t)v.x;
        s_i[e] = v.y;
        s_p[e] = v.z;
        s_g[e] = (int)atomicAdd(&s_at[v.z - tbase], 1u);   /* p in [tbase, tbase + tlen]; its place in p's group */
    }
    uint32_t wrun = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) wrun += w < warp ? s_wpre[w] : 0u;
    __syncthreads();   /* every warp has read the per-warp totals; s_at is complete */
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < kIncItems; ++k) {
            s_word[warp * kIncItems + k] = word[k];
            s_wpre[warp * kIncItems + k] = wrun;
            wrun += (uint32_t)__popc(word[k]);
        }
    }
    /* inclusive prefix of s_at over the tile's positions (thread tid owns 8 in a row) */
    uint32_t loc[kIncItems], run = 0;
#pragma unroll
    for (int k = 0; k < kIncItems; ++k) {
        run += s_at[tid * kIncItems + k];
        loc[k] = run;
    }
    const uint32_t before = block_exclusive_scan_256(run, s_scan);   /* syncs the block */
#pragma unroll
    for (int k = 0; k < kIncItems; ++k) s_at[tid * kIncItems + k] = before + loc[k];
    __syncthreads();
    /* the bucket's particles: those with a smaller insertion point are below; those with the
     * same point (grouped by it, in any order) compare by (key, index) */
    for (int e = tid; e < c; e += kThreads) {
        const int lp = s_p[e] - tbase;
        const int excl = lp > 0 ? (int)s_at[lp - 1] : 0;
        s_gk[excl + s_g[e]] = s_k[e];
        s_gi[excl + s_g[e]] = s_i[e];
    }
    __syncthreads();
    for (int e = tid; e < c; e += kThreads) {
        const uint32_t k = s_k[e];
        const int32_t i = s_i[e];
        const int p = s_p[e];
        const int lp = p - tbase;
        const int excl = lp > 0 ? (int)s_at[lp - 1] : 0;
        const int gend = lp < kIncTile ? (int)s_at[lp] : c;
        int r = excl;
        for (int f = excl; f < gend; ++f) r += pair_less(s_gk[f], s_gi[f], k, i) ? 1 : 0;
        uint32_t mb = tile_pre + tile_moved;   /* p at the tile's end */
        if (lp < tlen) {
            const int lw = lp >> 5;
            mb = tile_pre + s_wpre[lw] + (uint32_t)__popc(s_word[lw] & ((1u << (lp & 31)) - 1u));
        }
        const int at = p - (int)mb + (int)off + r;
        if (at < 0 || at >= n) continue;   /* never with consistent inputs */
        kout[at] = k;
        vout[at] = i;
        prev[at] = k;
        if ((at & 31) == 0) sub[at >> 5] = k;
        if ((at & (kIncTile - 1)) == 0) first[at >> kIncShift] = k;
    }
    /* the stayed particles of this tile */
    const unsigned lt = (1u << lane) - 1u;
#pragma unroll
    for (int k = 0; k < kIncItems; ++k) {
        const int j = wbase + k * 32 + lane;
        if (j < tlen && !((word[k] >> lane) & 1u)) {
            const int lw = warp * kIncItems + k;
            const int at = tbase + j - (int)(tile_pre + s_wpre[lw] + (uint32_t)__popc(word[k] & lt)) + (int)off +
                           (int)s_at[j];
            if (at < 0 || at >= n) continue;
            kout[at] = key[k];
            vout[at] = tbase + j;
            prev[at] = key[k];
            if ((at & 31) == 0) sub[at >> 5] = key[k];
            if ((at & (kIncTile - 1)) == 0) first[at >> kIncShift] = key[k];
        }
    }
}

/* After the gated full sort: its keys become prev (with the word and tile tables); a
 * single pair needs no sort.  Marks prev valid for the next call either way. */
__global__ void __launch_bounds__(kThreads) k_inc_keep(const uint32_t* __restrict__ keys, int n,
                                                       const unsigned* __restrict__ over, uint32_t* __restrict__ kout,
                                                       int32_t* __restrict__ vout, uint32_t* __restrict__ prev,
                                                       uint32_t* __restrict__ first, uint32_t* __restrict__ sub,
                                                       unsigned* __restrict__ valid) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *valid = 1u;
    if (*over == 0u) return;
    if (n == 1 && blockIdx.x == 0 && threadIdx.x == 0) {
        kout[0] = __ldg(&keys[0]);
        vout[0] = 0;
    }
    for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (long long)gridDim.x * blockDim.x) {
        const uint32_t k = n == 1 ? __ldg(&keys[0]) : kout[j];
        prev[j] = k;
        if ((j & 31) == 0) sub[j >> 5] = k;
        if ((j & (kIncTile - 1)) == 0) first[j >> kIncShift] = k;
    }
}

size_t sort_inc_workspace_bytes(int n) { return IncLayout(n).total; }

IncFlags sort_inc_flags_args(void* inc_ws, int n) {
    const IncLayout L(n);
    char* w = static_cast<char*>(inc_ws);
    return IncFlags{reinterpret_cast<const unsigned*>(w + L.valid), reinterpret_cast<const uint32_t*>(w + L.prev),
                    reinterpret_cast<uint32_t*>(w + L.bits),        reinterpret_cast<uint32_t*>(w + L.tcnt),
                    reinterpret_cast<unsigned*>(w + L.over),        reinterpret_cast<int2*>(w + L.list),
                    reinterpret_cast<uint32_t*>(w + L.lcount)};
}

void sort_inc_begin(cudaStream_t s, void* inc_ws, int n) {
    const IncLayout L(n);
    cudaMemsetAsync(static_cast<char*>(inc_ws) + L.zero, 0, L.zero_bytes, s);
}

void sort_pairs_incremental(cudaStream_t s, const uint32_t* keys, int n, int key_bits, uint32_t* kout,
                            int32_t* vout, void* inc_ws, void* sort_ws, unsigned* flags, int num_sms,
                            cudaStream_t side, cudaEvent_t fork, cudaEvent_t join, bool flags_done) {
    if (n <= 0) return;
    const IncLayout L(n);
    char* w = static_cast<char*>(inc_ws);
    unsigned* valid = reinterpret_cast<unsigned*>(w + L.valid);
    uint32_t* prev = reinterpret_cast<uint32_t*>(w + L.prev);
    uint32_t* first = reinterpret_cast<uint32_t*>(w + L.first);
    uint32_t* sub = reinterpret_cast<uint32_t*>(w + L.sub);
    uint32_t* bits = reinterpret_cast<uint32_t*>(w + L.bits);
    int4* store = reinterpret_cast<int4*>(w + L.store);
    unsigned* over = reinterpret_cast<unsigned*>(w + L.over);
    uint32_t* bcnt = reinterpret_cast<uint32_t*>(w + L.bcnt);
    uint32_t* tcnt = reinterpret_cast<uint32_t*>(w + L.tcnt);
    uint32_t* tpre = reinterpret_cast<uint32_t*>(w + L.tpre);
    uint32_t* boff = reinterpret_cast<uint32_t*>(w + L.boff);
    int2* list = reinterpret_cast<int2*>(w + L.list);
    uint32_t* lcount = reinterpret_cast<uint32_t*>(w + L.lcount);
    unsigned* done = reinterpret_cast<unsigned*>(w + L.done);
    if (!flags_done) {
        cudaMemsetAsync(w + L.zero, 0, L.zero_bytes, s);
        k_inc_flags<<<L.tiles, kThreads, 0, s>>>(keys, prev, n, valid, bits, tcnt, over, list, lcount);
    }
    const size_t fsm = L.tiles <= kIncSmemTiles ? 4 * (size_t)L.tiles : 0;
    k_inc_place<<<4 * num_sms, kThreads, fsm, s>>>(list, lcount, prev, first, sub, n, L.tiles, valid, bcnt, store,
                                                   over, done, tcnt, tpre, boff);
    /* the gated full sort of (keys, identity) on the side stream, beside the merge (one of
     * the two writes the result); prev is its scratch and its last pass writes kout / vout */
    const bool fork_side = side != nullptr && fork != nullptr && join != nullptr;
    cudaStream_t gs = fork_side ? side : s;
    if (fork_side) {
        cudaEventRecord(fork, s);
        cudaStreamWaitEvent(side, fork, 0);
    }
    if (n > 1 && sort_passes(key_bits) > 0) {
        uint32_t* kr;
        int32_t* vr;
        int32_t* vscr = reinterpret_cast<int32_t*>(w + L.vscr);
        const bool odd = (sort_passes(key_bits) & 1) != 0;
        sort_pairs_impl(gs, keys, nullptr, odd ? kout : prev, odd ? vout : vscr, odd ? prev : kout,
                        odd ? vscr : vout, n, over, key_bits, sort_ws, flags, num_sms, &kr, &vr);
    }
    if (fork_side) cudaEventRecord(join, side);
    k_inc_merge<<<L.tiles, kThreads, 0, s>>>(keys, n, bits, tcnt, tpre, boff, bcnt, store, over, kout, vout, prev,
                                             first, sub);
    if (fork_side) cudaStreamWaitEvent(s, join, 0);
    k_inc_keep<<<2 * num_sms, kThreads, 0, s>>>(keys, n, over, kout, vout, prev, first, sub, valid);
}

}  // namespace sph
