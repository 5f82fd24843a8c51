/*
 * sph_mesh.cu -- mesh boundary sampling on the GPU: the voxel sampler behind
 * Model::surface_sampling (scene/model.cpp:170-214), which voxelizes the mesh with voxel
 * size = particle spacing and precision = spacing / 10 and takes the 8 corners of every
 * voxel as boundary particles.  The voxelizer is the reference's vendored single-header
 * library (external/voxelizer/voxelizer.h, vx_voxelize, MIT); its algorithm is restated here
 * so that the output is the same list, in the same order, bit for bit:
 *
 *   per triangle (skipped when its area is below 1e-7): the bounding box snapped outwards
 *   to the voxel lattice (vx__map_to_voxel), then voxel centres stepped through the box by
 *   repeated float addition of the voxel size; each voxel [c - s/2, c + s/2] grown by
 *   `precision` is kept when the triangle overlaps it (separating-axis test of
 *   Akenine-Moller: 9 edge-cross-axis tests, the 3 box axes, the triangle's plane);
 *
 *   kept centres go into a 4096-bucket hash table keyed by
 *   (size_t)(x * 73856093) ^ (size_t)(y * 19349663) ^ (size_t)(z * 83492791) mod 4096
 *   (float products; the float -> size_t conversion as x86-64 performs it, which is where
 *   the reference runs: truncation to int64 then reinterpretation), a centre being dropped
 *   when an earlier one in its bucket is within 1e-7 on every axis;
 *
 *   the output walks the buckets in order and each bucket in insertion order.
 *
 * GPU plan: one thread per triangle counts its overlapping voxels; a scan gives each
 * triangle its slots; the same thread writes its centres and bucket keys in its own loop
 * order; a stable sort by bucket keeps insertion order inside each bucket; one thread per
 * bucket replays the duplicate test in that order; a scan of the survivors places the
 * 8 corners of each.  Built with -fmad=false: every multiply and add rounds on its own, as
 * in the reference's x86 build.  Every loop is bounded: a triangle box of more than 2^24
 * voxels is refused on the host before any launch, and on the device a box whose step no
 * longer advances the float, with more than 2^20 steps on an axis or 2^24 voxels, stops the
 * call with SPH_E_OVERFLOW.
 */
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "sph_capi.h"

namespace {

constexpr int kBuckets = 4096;
constexpr int kMaxSteps = 1 << 20;            /* per axis of one triangle's box */
constexpr long long kMaxVoxels = 1ll << 24;    /* per triangle's box */
constexpr double kEps = 1e-7;

struct F3 {
    float x, y, z;
};

__device__ __forceinline__ F3 sub(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }

__device__ __forceinline__ float snap(float p, float s, bool lo) {
    const float v = (p + (p < 0.f ? -1.f : 1.f) * s * 0.5f) / s;
    return (lo ? floorf(v) : ceilf(v)) * s;
}

/* one of the 9 edge tests: projections q0, q1 of two vertices, radius r */
__device__ __forceinline__ bool separated(float q0, float q1, float r) {
    const float mn = q0 < q1 ? q0 : q1, mx = q0 < q1 ? q1 : q0;
    return mn > r || mx < -r;
}

__device__ __forceinline__ bool outside_axis(float a, float b, float c, float h) {
    float mn = a, mx = a;
    if (b < mn) mn = b;
    if (b > mx) mx = b;
    if (c < mn) mn = c;
    if (c > mx) mx = c;
    return mn > h || mx < -h;
}

/* triangle (p1, p2, p3) against the box of centre bc and half size hs */
__device__ bool tri_box(F3 bc, F3 hs, F3 p1, F3 p2, F3 p3) {
    const F3 v1 = sub(p1, bc), v2 = sub(p2, bc), v3 = sub(p3, bc);
    const F3 e1 = sub(v2, v1), e2 = sub(v3, v2), e3 = sub(v1, v3);
    float fx = fabsf(e1.x), fy = fabsf(e1.y), fz = fabsf(e1.z);
    /* edge 1: x axis on vertices 1, 3; y axis on 1, 3; z axis on 2, 3 */
    if (separated(e1.z * v1.y - e1.y * v1.z, e1.z * v3.y - e1.y * v3.z, fz * hs.y + fy * hs.z)) return false;
    if (separated(-e1.z * v1.x + e1.x * v1.z, -e1.z * v3.x + e1.x * v3.z, fz * hs.x + fx * hs.z)) return false;
    if (separated(e1.y * v2.x - e1.x * v2.y, e1.y * v3.x - e1.x * v3.y, fy * hs.x + fx * hs.y)) return false;
    /* edge 2: x on 1, 3; y on 1, 3; z on 1, 2 */
    fx = fabsf(e2.x), fy = fabsf(e2.y), fz = fabsf(e2.z);
    if (separated(e2.z * v1.y - e2.y * v1.z, e2.z * v3.y - e2.y * v3.z, fz * hs.y + fy * hs.z)) return false;
    if (separated(-e2.z * v1.x + e2.x * v1.z, -e2.z * v3.x + e2.x * v3.z, fz * hs.x + fx * hs.z)) return false;
    if (separated(e2.y * v1.x - e2.x * v1.y, e2.y * v2.x - e2.x * v2.y, fy * hs.x + fx * hs.y)) return false;
    /* edge 3: x on 1, 2; y on 1, 2; z on 2, 3 */
    fx = fabsf(e3.x), fy = fabsf(e3.y), fz = fabsf(e3.z);
    if (separated(e3.z * v1.y - e3.y * v1.z, e3.z * v2.y - e3.y * v2.z, fz * hs.y + fy * hs.z)) return false;
    if (separated(-e3.z * v1.x + e3.x * v1.z, -e3.z * v2.x + e3.x * v2.z, fz * hs.x + fx * hs.z)) return false;
    if (separated(e3.y * v2.x - e3.x * v2.y, e3.y * v3.x - e3.x * v3.y, fy * hs.x + fx * hs.y)) return false;
    /* the box's own axes */
    if (outside_axis(v1.x, v2.x, v3.x, hs.x) || outside_axis(v1.y, v2.y, v3.y, hs.y) ||
        outside_axis(v1.z, v2.z, v3.z, hs.z))
        return false;
    /* the triangle's plane */
    const F3 n = {e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x};
    const float d = -(n.x * v1.x + n.y * v1.y + n.z * v1.z);
    const F3 vmin = {n.x > 0.f ? -hs.x : hs.x, n.y > 0.f ? -hs.y : hs.y, n.z > 0.f ? -hs.z : hs.z};
    const F3 vmax = {-vmin.x, -vmin.y, -vmin.z};
    if (n.x * vmin.x + n.y * vmin.y + n.z * vmin.z + d > 0.f) return false;
    return n.x * vmax.x + n.y * vmax.y + n.z * vmax.z + d >= 0.f;
}

/* float -> size_t as x86-64 converts it (the host the reference runs on) */
__device__ __forceinline__ unsigned long long x86_to_size(float f) {
    if (f != f || f < -9.2233720368547758e18f) return 0x8000000000000000ull;
    if (f >= 9.2233720368547758e18f) {
        const float g = f - 9.2233720368547758e18f;
        if (g >= 9.2233720368547758e18f) return 0ull;   /* indefinite value with bit 63 flipped */
        return (unsigned long long)(long long)g ^ 0x8000000000000000ull;
    }
    return (unsigned long long)(long long)f;
}

__device__ __forceinline__ uint32_t bucket_of(F3 c) {
    const unsigned long long a = x86_to_size(c.x * (float)73856093);
    const unsigned long long b = x86_to_size(c.y * (float)19349663);
    const unsigned long long d = x86_to_size(c.z * (float)83492791);
    return (uint32_t)((a ^ b ^ d) % (unsigned long long)kBuckets);
}

struct Grid {
    float sx, sy, sz, prec;
};

/* Visits the overlapping voxels of triangle t in the library's loop order; returns false
 * (and stops) when a loop would not terminate within the step limit. */
template <class F>
__device__ bool triangle_voxels(const Grid& g, const float* __restrict__ v, const uint32_t* __restrict__ ix, int t,
                                F&& f) {
    const uint32_t i0 = ix[3 * t], i1 = ix[3 * t + 1], i2 = ix[3 * t + 2];
    const F3 p1 = {v[3 * i0], v[3 * i0 + 1], v[3 * i0 + 2]};
    const F3 p2 = {v[3 * i1], v[3 * i1 + 1], v[3 * i1 + 2]};
    const F3 p3 = {v[3 * i2], v[3 * i2 + 1], v[3 * i2 + 2]};
    const F3 ab = sub(p2, p1), ac = sub(p3, p1);
    const float a0 = ab.y * ac.z - ab.z * ac.y, a1 = ab.z * ac.x - ab.x * ac.z, a2 = ab.x * ac.y - ab.y * ac.x;
    if ((double)(sqrtf(a0 * a0 + a1 * a1 + a2 * a2) * 0.5f) < kEps) return true;   /* zero-area triangle */
    float mnx = INFINITY, mny = INFINITY, mnz = INFINITY, mxx = -INFINITY, mxy = -INFINITY, mxz = -INFINITY;
    const F3 ps[3] = {p1, p2, p3};
    for (int k = 0; k < 3; ++k) {
        const F3 p = ps[k];
        mxx = mxx > p.x ? mxx : p.x; mxy = mxy > p.y ? mxy : p.y; mxz = mxz > p.z ? mxz : p.z;
        mnx = mnx > p.x ? p.x : mnx; mny = mny > p.y ? p.y : mny; mnz = mnz > p.z ? p.z : mnz;
    }
    const float lx = snap(mnx, g.sx, true), ly = snap(mny, g.sy, true), lz = snap(mnz, g.sz, true);
    const float ux = snap(mxx, g.sx, false), uy = snap(mxy, g.sy, false), uz = snap(mxz, g.sz, false);
    const float hx = g.sx * 0.5f, hy = g.sy * 0.5f, hz = g.sz * 0.5f;
    int nx = 0;
    long long visited = 0;
    for (float x = lx; x < ux; x += g.sx) {
        if (++nx > kMaxSteps || x + g.sx == x) return false;
        int ny = 0;
        for (float y = ly; y < uy; y += g.sy) {
            if (++ny > kMaxSteps || y + g.sy == y) return false;
            int nz = 0;
            for (float z = lz; z < uz; z += g.sz) {
                if (++nz > kMaxSteps || z + g.sz == z || ++visited > kMaxVoxels) return false;
                const F3 lo = {x - hx, y - hy, z - hz}, hi = {x + hx, y + hy, z + hz};
                const F3 c = {(lo.x + hi.x) * 0.5f, (lo.y + hi.y) * 0.5f, (lo.z + hi.z) * 0.5f};
                const F3 hs = {fabsf(hi.x - lo.x) * 0.5f + g.prec, fabsf(hi.y - lo.y) * 0.5f + g.prec,
                               fabsf(hi.z - lo.z) * 0.5f + g.prec};
                if (tri_box(c, hs, p1, p2, p3)) f(c);
            }
        }
    }
    return true;
}

__global__ void k_vox_count(Grid g, const float* v, const uint32_t* ix, int ntri, int* count, unsigned* err) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntri) return;
    int n = 0;   /* at most kMaxVoxels */
    if (!triangle_voxels(g, v, ix, t, [&](F3) { ++n; })) {
        atomicOr(err, 1u);
        n = 0;
    }
    count[t] = n;
}

__global__ void k_vox_emit(Grid g, const float* v, const uint32_t* ix, int ntri, const int* off, float* cand,
                           uint32_t* key, int32_t* val) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntri) return;
    int k = off[t];
    triangle_voxels(g, v, ix, t, [&](F3 c) {
        cand[3 * (size_t)k] = c.x;
        cand[3 * (size_t)k + 1] = c.y;
        cand[3 * (size_t)k + 2] = c.z;
        key[k] = bucket_of(c);
        val[k] = k;
        ++k;
    });
}

__global__ void k_bucket_ranges(const uint32_t* key, int n, int* start, int* end) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t b = key[i];
    if (i == 0 || key[i - 1] != b) start[b] = i;
    if (i == n - 1 || key[i + 1] != b) end[b] = i + 1;
}

/* one thread per bucket: the insertion test replayed in insertion order */
__global__ void k_bucket_dedup(const int* start, const int* end, const int32_t* val, const float* cand, int* keep) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= kBuckets) return;
    const int s = start[b], e = end[b];
    for (int i = s; i < e; ++i) {
        const float* c = cand + 3 * (size_t)val[i];
        bool dup = false;
        for (int j = s; j < i && !dup; ++j) {
            if (!keep[j]) continue;
            const float* q = cand + 3 * (size_t)val[j];
            dup = fabsf(q[0] - c[0]) < kEps && fabsf(q[1] - c[1]) < kEps && fabsf(q[2] - c[2]) < kEps;
        }
        keep[i] = dup ? 0 : 1;
    }
}

__global__ void k_vox_corners(const int* keep, const int* pos, const int32_t* val, const float* cand, int n, float hx,
                              float hy, float hz, float4* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !keep[i]) return;
    const float* c = cand + 3 * (size_t)val[i];
    const float cx = c[0], cy = c[1], cz = c[2];
    /* corner order of the library's unit voxel */
    const float sx[8] = {-hx, -hx, hx, hx, -hx, -hx, hx, hx};
    const float sy[8] = {hy, -hy, -hy, hy, hy, -hy, -hy, hy};
    const float sz[8] = {hz, hz, hz, hz, -hz, -hz, -hz, -hz};
    float4* o = out + 8 * (size_t)pos[i];
#pragma unroll
    for (int k = 0; k < 8; ++k) o[k] = make_float4(sx[k] + cx, sy[k] + cy, sz[k] + cz, 1.0f);
}

/* exclusive scan of n non-negative ints by one block (chunks of 1024), the 64-bit total to
 * *total; the int outputs are meaningful when the total fits in an int */
__global__ void k_scan_one_block(const int* in, int* out, int n, long long* total) {
    __shared__ int warp_sum[32];
    __shared__ long long carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int base = 0; base < n; base += 1024) {
        const int i = base + threadIdx.x;
        const int x = i < n ? in[i] : 0;
        int s = x;
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, s, d);
            if (lane >= d) s += y;
        }
        if (lane == 31) warp_sum[wid] = s;
        __syncthreads();
        if (wid == 0) {
            int w = warp_sum[lane];
            for (int d = 1; d < 32; d <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, w, d);
                if (lane >= d) w += y;
            }
            warp_sum[lane] = w;
        }
        __syncthreads();
        const long long excl = carry + (wid > 0 ? warp_sum[wid - 1] : 0) + s - x;
        if (i < n) out[i] = (int)excl;
        __syncthreads();
        if (threadIdx.x == 1023) carry = excl + x;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

struct DevBufs {
    std::vector<void*> ptrs;
    ~DevBufs() {
        for (void* p : ptrs) cudaFree(p);
    }
    template <class T>
    T* get(size_t n) {
        void* p = nullptr;
        if (cudaMalloc(&p, n ? n * sizeof(T) : sizeof(T)) != cudaSuccess) return nullptr;
        ptrs.push_back(p);
        return static_cast<T*>(p);
    }
};

inline unsigned blocks(long long n, int b) { return (unsigned)((n + b - 1) / b); }

}  // namespace

extern "C" int sph_scene_voxelize(const float* vertices3, int nvertices, const uint32_t* indices, int nindices,
                                  float voxel_size, float precision, float* out4, int cap) {
    if (!vertices3 || !indices || nvertices <= 0 || nindices <= 0 || nindices % 3 != 0 || !(voxel_size > 0.f) ||
        !(precision >= 0.f) || cap < 0)
        return -SPH_E_INVALID;
    for (int i = 0; i < nindices; ++i)
        if (indices[i] >= (uint32_t)nvertices) return -SPH_E_INVALID;
    const int ntri = nindices / 3;
    /* refuse boxes the device loops would take too long over, before any launch */
    for (int t = 0; t < ntri; ++t) {
        double steps = 1.0;
        for (int a = 0; a < 3; ++a) {
            float lo = INFINITY, hi = -INFINITY;
            for (int k = 0; k < 3; ++k) {
                const float c = vertices3[3 * indices[3 * t + k] + a];
                lo = c < lo ? c : lo;
                hi = c > hi ? c : hi;
            }
            if (!(hi - lo < INFINITY)) return -SPH_E_INVALID;   /* non-finite vertex */
            steps *= (double)(hi - lo) / voxel_size + 3.0;
        }
        if (steps > (double)kMaxVoxels) return -SPH_E_OVERFLOW;
    }
    cudaStream_t s = nullptr;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        return -SPH_E_CUDA;
    }
    int result = -SPH_E_CUDA;
    {
        DevBufs d;
        float* v = d.get<float>(3 * (size_t)nvertices);
        uint32_t* ix = d.get<uint32_t>((size_t)nindices);
        int* count = d.get<int>((size_t)ntri);
        int* off = d.get<int>((size_t)ntri);
        long long* total = d.get<long long>(2);
        unsigned* err = d.get<unsigned>(1);
        int* start = d.get<int>(kBuckets);
        int* end = d.get<int>(kBuckets);
        const Grid g{voxel_size, voxel_size, voxel_size, precision};
        long long h_total = 0;
        unsigned h_err = 0;
        bool ok = v && ix && count && off && total && err && start && end;
        ok = ok && cudaMemcpyAsync(v, vertices3, 12 * (size_t)nvertices, cudaMemcpyHostToDevice, s) == cudaSuccess &&
             cudaMemcpyAsync(ix, indices, 4 * (size_t)nindices, cudaMemcpyHostToDevice, s) == cudaSuccess &&
             cudaMemsetAsync(err, 0, 4, s) == cudaSuccess;
        if (ok) {
            k_vox_count<<<blocks(ntri, 128), 128, 0, s>>>(g, v, ix, ntri, count, err);
            k_scan_one_block<<<1, 1024, 0, s>>>(count, off, ntri, total);
            ok = cudaMemcpyAsync(&h_total, total, 8, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
                 cudaMemcpyAsync(&h_err, err, 4, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
                 cudaStreamSynchronize(s) == cudaSuccess;
        }
        if (ok && h_err) result = -SPH_E_OVERFLOW;
        else if (ok && h_total > (1ll << 30)) result = -SPH_E_OVERFLOW;
        else if (ok && h_total == 0) result = 0;
        else if (ok) {
            const int n = (int)h_total;
            float* cand = d.get<float>(3 * (size_t)n);
            uint32_t* key = d.get<uint32_t>((size_t)n);
            int32_t* val = d.get<int32_t>((size_t)n);
            int* keep = d.get<int>((size_t)n);
            int* pos = d.get<int>((size_t)n);
            ok = cand && key && val && keep && pos;
            if (!ok) result = -SPH_E_NOMEM;
            if (ok) {
                k_vox_emit<<<blocks(ntri, 128), 128, 0, s>>>(g, v, ix, ntri, off, cand, key, val);
                ok = sph_sort_pairs(key, val, n, 12, s) == SPH_OK &&
                     cudaMemsetAsync(start, 0, 4 * kBuckets, s) == cudaSuccess &&
                     cudaMemsetAsync(end, 0, 4 * kBuckets, s) == cudaSuccess;
            }
            long long kept = 0;
            if (ok) {
                k_bucket_ranges<<<blocks(n, 256), 256, 0, s>>>(key, n, start, end);
                k_bucket_dedup<<<blocks(kBuckets, 64), 64, 0, s>>>(start, end, val, cand, keep);
                k_scan_one_block<<<1, 1024, 0, s>>>(keep, pos, n, total + 1);
                ok = cudaMemcpyAsync(&kept, total + 1, 8, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
                     cudaStreamSynchronize(s) == cudaSuccess;
            }
            if (ok && kept > INT32_MAX / 8) {
                result = -SPH_E_OVERFLOW;
            } else if (ok) {
                const int nout = (int)(8 * kept);
                result = nout;
                if (out4 && cap >= nout && nout > 0) {
                    float4* o = d.get<float4>((size_t)nout);
                    ok = o != nullptr;
                    if (ok) {
                        k_vox_corners<<<blocks(n, 256), 256, 0, s>>>(keep, pos, val, cand, n, voxel_size * 0.5f,
                                                                      voxel_size * 0.5f, voxel_size * 0.5f, o);
                        ok = cudaMemcpyAsync(out4, o, 16 * (size_t)nout, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
                             cudaStreamSynchronize(s) == cudaSuccess;
                    }
                    if (!ok) result = -SPH_E_CUDA;
                }
            }
        }
        if (cudaGetLastError() != cudaSuccess && result >= 0) result = -SPH_E_CUDA;
        cudaStreamSynchronize(s);
    }
    cudaStreamDestroy(s);
    return result;
}
