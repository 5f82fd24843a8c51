/*
 * sph_sort_noalloc.cu -- the stable (uint32 key, int32 value) sort for callers that cannot
 * allocate device memory.
 *
 * Some host programs cannot call cudaMalloc at the point where they need a sort: an
 * application whose own allocator owns the whole device heap and forbids allocations
 * behind its back, a plug-in called from a frame or simulation callback where an
 * allocation (which can synchronise the device) is not allowed, or code that must not fail
 * for lack of memory once it has started.  sph_sort_pairs caches scratch it allocates on
 * first use, which such callers cannot accept.  This entry point takes the caller's input
 * and output buffers and uses, for every other byte it needs (digit histograms, tile
 * counters, the decoupled look-back status words and the ping-pong key/value copy), the
 * fixed array below, which exists once per GPU that loads the library and stays allocated
 * until the process exits.
 *
 * Limits and behaviour:
 *   - at most SPH_NOALLOC_SORT_MAX_PAIRS (1,048,576) pairs per call; larger n is rejected
 *     with SPH_E_OVERFLOW before anything is launched;
 *   - the array holds 9,441,792 bytes (9.0 MiB) per device;
 *   - the first call on a device looks up the array's device address with
 *     cudaGetSymbolAddress (host code cannot use the array's name as an address); make
 *     that first call before any stream capture;
 *   - every call on a device shares the one array and it keeps the last call's contents;
 *     the parts that must start at zero are cleared at the start of each call, but two
 *     calls whose work overlaps on the GPU (different streams, or different host threads)
 *     race on it: serialise them;
 *   - asynchronous on the given stream; no cudaMalloc, cudaFree or allocating library call;
 *   - the array's address is looked up once per device and kept; it does not survive
 *     cudaDeviceReset (which unloads the module), so a host that resets a device must not
 *     call this entry point on it again; a failed launch forgets the address, and the next
 *     call looks it up again;
 *   - the error check after the launches (cudaGetLastError) also returns, and clears, an
 *     error that earlier asynchronous work on the calling thread left behind;
 *   - a look-back wait that gives up (it cannot on a correct launch: tiles are taken in
 *     order) leaves a wrong result and is not reported by the return code.
 * The kernels are the ones of sph_sort.cu (block size 256); the passes ping-pong between
 * the caller's output and the array's copy so that the input is only read.
 */
#include <cstdint>
#include <mutex>

#include "sph_capi.h"
#include "sph_kernels.cuh"

namespace sph {
__global__ void k_sort_hist(const uint32_t* keys, int n, int passes, uint32_t* hist, const unsigned* gate);
__global__ void k_onesweep(const uint32_t* kin, const int32_t* vin, uint32_t* kout, int32_t* vout, int n,
                           int shift, int pass, int tiles, const uint32_t* hist, uint32_t* counters,
                           uint32_t* status, unsigned* flags, const unsigned* gate);
int sort_tiles(int n);
}  // namespace sph

namespace {
constexpr int kMaxPairs = SPH_NOALLOC_SORT_MAX_PAIRS;
constexpr int kCtaThreads = 256;                        /* block size of the sort kernels */
constexpr size_t kStatusBytes = (size_t)4 * (kMaxPairs / 4096) * 256 * 4;
constexpr size_t kWorkspaceBytes = (size_t)(4 * 256 + 64) * 4 + kStatusBytes;   /* hist, counters, status */
constexpr size_t kFlagsOffset = kWorkspaceBytes;
constexpr size_t kKeysOffset = kFlagsOffset + 256;
constexpr size_t kValsOffset = kKeysOffset + (size_t)4 * kMaxPairs;
constexpr size_t kScratchBytes = kValsOffset + (size_t)4 * kMaxPairs;
static_assert(kScratchBytes == 9441792, "scratch size stated in the header comment");

static __device__ __align__(256) unsigned char g_sort_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_base[kMaxDevices] = {nullptr};
int g_sms[kMaxDevices] = {0};

/* Once per device, with that device current: the device address of g_sort_scratch. */
int scratch_for_current_device(unsigned char** base, int* sms) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return SPH_E_CUDA;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_base[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_sort_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return SPH_E_CUDA;
        }
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) n = 1;
        g_sms[dev] = n;
        g_base[dev] = static_cast<unsigned char*>(p);
    }
    *base = g_base[dev];
    *sms = g_sms[dev];
    return SPH_OK;
}

/* After a failed launch the context may have been lost and the module reloaded: look the
 * address up again on the next call. */
void forget_scratch_for_current_device() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return;
    std::lock_guard<std::mutex> lk(g_mu);
    g_base[dev] = nullptr;
}

bool overlaps(const void* a, size_t na, const void* b, size_t nb) {
    const char* x = static_cast<const char*>(a);
    const char* y = static_cast<const char*>(b);
    return x < y + nb && y < x + na;
}
}  // namespace

extern "C" int sph_sort_pairs_noalloc(const uint32_t* d_keys_in, const int32_t* d_vals_in, uint32_t* d_keys_out,
                                      int32_t* d_vals_out, int n, int key_bits, void* cuda_stream) {
    if (n < 0 || key_bits < 1 || key_bits > 32) return SPH_E_INVALID;
    if (n > kMaxPairs) return SPH_E_OVERFLOW;
    if (n == 0) return SPH_OK;
    if (!d_keys_in || !d_vals_in || !d_keys_out || !d_vals_out) return SPH_E_INVALID;
    const size_t bytes = (size_t)4 * n;
    /* an output may overlap neither input (with an odd pass count the first pass writes the
     * outputs while it still reads the inputs) nor the other output */
    if (overlaps(d_keys_in, bytes, d_keys_out, bytes) || overlaps(d_vals_in, bytes, d_vals_out, bytes) ||
        overlaps(d_keys_in, bytes, d_vals_out, bytes) || overlaps(d_vals_in, bytes, d_keys_out, bytes) ||
        overlaps(d_keys_out, bytes, d_vals_out, bytes))
        return SPH_E_INVALID;
    unsigned char* base = nullptr;
    int sms = 1;
    int rc = scratch_for_current_device(&base, &sms);
    if (rc != SPH_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    if (n == 1) {
        if (cudaMemcpyAsync(d_keys_out, d_keys_in, 4, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
            cudaMemcpyAsync(d_vals_out, d_vals_in, 4, cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
            cudaGetLastError();
            return SPH_E_CUDA;
        }
        return SPH_OK;
    }
    const int passes = sph::sort_passes(key_bits);
    const int tiles = sph::sort_tiles(n);
    const size_t ws = sph::sort_workspace_bytes(n, key_bits);
    if (ws > kWorkspaceBytes) return SPH_E_OVERFLOW;
    uint32_t* hist = reinterpret_cast<uint32_t*>(base);
    uint32_t* counters = hist + 4 * 256;
    uint32_t* status = counters + 64;
    unsigned* flags = reinterpret_cast<unsigned*>(base + kFlagsOffset);
    uint32_t* kalt = reinterpret_cast<uint32_t*>(base + kKeysOffset);
    int32_t* valt = reinterpret_cast<int32_t*>(base + kValsOffset);
    /* what must start at zero: histograms, tile counters, look-back status, the flag word */
    if (cudaMemsetAsync(base, 0, ws, s) != cudaSuccess || cudaMemsetAsync(flags, 0, 4, s) != cudaSuccess) {
        cudaGetLastError();
        return SPH_E_CUDA;
    }
    sph::k_sort_hist<<<2 * sms, kCtaThreads, 0, s>>>(d_keys_in, n, passes, hist, nullptr);
    /* pass p writes the caller's output when (passes - 1 - p) is even, the copy otherwise,
     * so the last pass lands in the output and the input is never written */
    const uint32_t* ki = d_keys_in;
    const int32_t* vi = d_vals_in;
    for (int p = 0; p < passes; ++p) {
        const bool to_out = ((passes - 1 - p) % 2) == 0;
        uint32_t* ko = to_out ? d_keys_out : kalt;
        int32_t* vo = to_out ? d_vals_out : valt;
        sph::k_onesweep<<<tiles, kCtaThreads, 0, s>>>(ki, vi, ko, vo, n, 8 * p, p, tiles, hist, counters, status,
                                                      flags, nullptr);
        ki = ko;
        vi = vo;
    }
    if (cudaGetLastError() != cudaSuccess) {
        forget_scratch_for_current_device();
        return SPH_E_CUDA;
    }
    return SPH_OK;
}
