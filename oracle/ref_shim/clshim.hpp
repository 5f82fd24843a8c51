/*
 * clshim.hpp -- lets g++ compile the reference's OpenCL C kernels (kernels/NAME.cl) for the
 * CPU so the oracle can be pinned against the reference's own kernel text.
 * TEST INFRASTRUCTURE: built only by oracle/build_ref.sh into oracle/_ref/.
 *
 * What it provides:
 *   - float2/float4/int2/int4 with the OpenCL operators the kernels use, including the
 *     .zx swizzle (read and write) of kernels/wcsph.cl:207 and kernels/pcisph.cl:268,329;
 *   - the builtins the kernels call, restated with IEEE single operations exactly as the
 *     oracle restates them (dot left to right over x,y,z,w; length = sqrt(dot);
 *     normalize = v / length with the zero vector mapped to itself; pown = repeated
 *     multiplication; clamp = min(max()); sign per the OpenCL spec);
 *   - image1d_buffer_t + read_imagef over a plain array (CL_RGBA or CL_R), and a
 *     single-channel image2d_t with the clamp-to-edge / nearest sampler and write_imagef
 *     (kernels/bilateral.cl, kernels/curvatureflow.cl), run by a 2-D NDRange runner;
 *   - the -D program constants as runtime globals (PARTICLE_COUNT, SUPPORT_RADIUS, ...);
 *   - an NDRange runner: work-items of one work-group run as ucontext fibers, and
 *     barrier() switches back to the group scheduler, so local-memory caches and the
 *     early-return-before-barrier pattern behave as on a device.
 * The only source transformation (done by build_ref.sh on copies under oracle/_ref/src)
 * rewrites the vector literals "(int4)(" and "(float4)(" into make_int4( / make_float4(,
 * which C++ would otherwise parse as a cast of a comma expression.
 */
#ifndef CLSHIM_HPP
#define CLSHIM_HPP

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <ucontext.h>
#include <vector>

namespace clshim {
extern int g_particle_count;
extern int g_boundary_particle_count;
extern float g_support_radius;
extern float g_particle_mass;
extern float g_rest_density;
extern float g_cell_size;
extern float g_grid_size;
extern int g_cells_per_side;

struct WorkItem { size_t gid, lid, lsize, group, gid1 = 0; };
extern thread_local WorkItem* tl_cur;
void barrier_impl();

/* Runs kernel body() for every work-item of a 1-D NDRange (global rounded up to a
 * multiple of local, as the reference's launches are). With fibers=false, a barrier()
 * aborts: use it only for kernels that have none. */
void run_ndrange(size_t global, size_t local, bool fibers, const std::function<void()>& body);
/* __local memory of the work-group running on this thread (slot 0..7, at least bytes). */
void* group_local(int slot, size_t bytes);
/* A 2-D NDRange of independent work-items (no barrier), dimension 0 fastest. */
void run_ndrange_2d(size_t gx, size_t gy, const std::function<void()>& body);
}  // namespace clshim

typedef unsigned int uint;

struct float2 { float x, y; };
struct int2 { int x, y; };
struct float3 { float x, y, z; };
inline int2 operator+(const int2& a, const int2& b) { return int2{a.x + b.x, a.y + b.y}; }
inline int2 operator-(const int2& a, const int2& b) { return int2{a.x - b.x, a.y - b.y}; }
inline float2 convert_float2(const int2& a) { return float2{(float)a.x, (float)a.y}; }
inline float fast_length(const float2& a) { return std::sqrt(a.x * a.x + a.y * a.y); }

template <int A, int B>
struct swz2f {
    float v[4];
    operator float2() const { return float2{v[A], v[B]}; }
    swz2f& operator=(const float2& o) { v[A] = o.x; v[B] = o.y; return *this; }
};

struct float4 {
    union {
        struct { float x, y, z, w; };
        float s[4];
        swz2f<2, 0> zx;
    };
};
struct int4 {
    union {
        struct { int x, y, z, w; };
        int s[4];
    };
};

inline float4 make_float4(float a, float b, float c, float d) { float4 r; r.x = a; r.y = b; r.z = c; r.w = d; return r; }
inline int4 make_int4(int a, int b, int c, int d) { int4 r; r.x = a; r.y = b; r.z = c; r.w = d; return r; }

inline float2 operator-(const float2& a) { return float2{-a.x, -a.y}; }
inline float2 operator/(const float2& a, float s) { return float2{a.x / s, a.y / s}; }

inline float4 operator+(const float4& a, const float4& b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline float4 operator-(const float4& a, const float4& b) { return make_float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
inline float4 operator-(const float4& a) { return make_float4(-a.x, -a.y, -a.z, -a.w); }
inline float4 operator*(const float4& a, const float4& b) { return make_float4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
inline float4 operator*(const float4& a, float s) { return make_float4(a.x * s, a.y * s, a.z * s, a.w * s); }
inline float4 operator*(float s, const float4& a) { return make_float4(s * a.x, s * a.y, s * a.z, s * a.w); }
inline float4 operator/(const float4& a, float s) { return make_float4(a.x / s, a.y / s, a.z / s, a.w / s); }
inline float4 operator-(const float4& a, float s) { return make_float4(a.x - s, a.y - s, a.z - s, a.w - s); }
inline float4& operator+=(float4& a, const float4& b) { a = a + b; return a; }
inline float4& operator-=(float4& a, const float4& b) { a = a - b; return a; }
inline float4& operator*=(float4& a, float s) { a = a * s; return a; }
inline int4 operator+(const int4& a, const int4& b) { return make_int4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }

inline float dot(const float4& a, const float4& b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
inline float length(const float4& a) { return std::sqrt(dot(a, a)); }
inline float fast_length(const float4& a) { return std::sqrt(dot(a, a)); }
inline float distance(const float4& a, const float4& b) { return length(a - b); }
inline float4 normalize(const float4& a) {
    float l = length(a);
    if (l == 0.0f) return a;
    return make_float4(a.x / l, a.y / l, a.z / l, a.w / l);
}
inline float4 fast_normalize(const float4& a) { return normalize(a); }
inline float4 cross(const float4& a, const float4& b) {
    return make_float4(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x, 0.0f);
}
/* OpenCL C spec: max(x,y) = (x < y) ? y : x; min(x,y) = (y < x) ? y : x;
 * clamp(x,lo,hi) = fmin(fmax(x, lo), hi). */
inline float max(float a, float b) { return a < b ? b : a; }
inline float min(float a, float b) { return b < a ? b : a; }
inline float clamp(float x, float lo, float hi) { return std::fmin(std::fmax(x, lo), hi); }
inline float2 clamp(const float2& x, const float2& lo, const float2& hi) {
    return float2{clamp(x.x, lo.x, hi.x), clamp(x.y, lo.y, hi.y)};
}
inline float4 clamp(const float4& x, float lo, float hi) {
    return make_float4(clamp(x.x, lo, hi), clamp(x.y, lo, hi), clamp(x.z, lo, hi), clamp(x.w, lo, hi));
}
inline float sign(float x) {
    if (x > 0.0f) return 1.0f;
    if (x < 0.0f) return -1.0f;
    if (x != x) return 0.0f;
    return x;
}
inline float4 sign(const float4& a) { return make_float4(sign(a.x), sign(a.y), sign(a.z), sign(a.w)); }
inline float pown(float x, int n) { float r = x; for (int k = 1; k < n; ++k) r = r * x; return r; }
inline int mad24(int a, int b, int c) { return a * b + c; }

struct image1d_buffer_t { const float* data; int channels; };
inline float4 read_imagef(const image1d_buffer_t& im, int i) {
    if (im.channels == 4) return make_float4(im.data[4 * i], im.data[4 * i + 1], im.data[4 * i + 2], im.data[4 * i + 3]);
    return make_float4(im.data[i], 0.0f, 0.0f, 1.0f);
}

/* single-channel float image; the sampler is always clamp-to-edge, nearest, unnormalised */
typedef int sampler_t;
#define CLK_NORMALIZED_COORDS_FALSE 0
#define CLK_ADDRESS_CLAMP_TO_EDGE 0
#define CLK_FILTER_NEAREST 0
struct image2d_t { float* data; int w, h; };
inline float4 read_imagef(const image2d_t& im, sampler_t, int2 p) {
    const int x = p.x < 0 ? 0 : (p.x >= im.w ? im.w - 1 : p.x);
    const int y = p.y < 0 ? 0 : (p.y >= im.h ? im.h - 1 : p.y);
    return make_float4(im.data[(size_t)y * im.w + x], 0.0f, 0.0f, 1.0f);
}
inline void write_imagef(const image2d_t& im, int2 p, float4 v) { im.data[(size_t)p.y * im.w + p.x] = v.x; }

inline size_t get_global_id(int d) { return d == 0 ? clshim::tl_cur->gid : clshim::tl_cur->gid1; }
inline size_t get_local_id(int) { return clshim::tl_cur->lid; }
inline size_t get_local_size(int) { return clshim::tl_cur->lsize; }
inline size_t get_group_id(int) { return clshim::tl_cur->group; }
#define CLK_LOCAL_MEM_FENCE 1
inline void barrier(int) { clshim::barrier_impl(); }

#define M_PI_F 3.14159265358979323846f

#endif

/* Names of a glue unit: the Monaghan build of a kernel file (CLSHIM_MONAGHAN, kernels.h
 * without USE_MULLER_KERNELS) puts its kernels in namespace <name>_monaghan and exports its
 * entry points as <name>_monaghan, so both builds link into one library. */
#ifdef CLSHIM_MONAGHAN
#define REF_NS(n) n##_monaghan
#define REF_FN(n) n##_monaghan
#else
#define REF_NS(n) n
#define REF_FN(n) n
#endif
