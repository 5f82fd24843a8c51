/*
 * ref_render.cpp -- C entry points running the reference's screen-space smoothing kernels
 * (kernels/bilateral.cl, kernels/curvatureflow.cl) on the CPU over single-channel float
 * images.  TEST INFRASTRUCTURE (oracle/_ref only): pins the CUDA filters of
 * fluids_gb300/csrc/sph_render.cu and generates their golden vectors.  The OpenCL builtins
 * exp, fabs and pow are the C library's single-precision functions.
 */
#include "clshim.hpp"

#include "clshim_kernel_begin.hpp"
namespace ref_bilateral {
inline float exp(float x) { return std::exp(x); }
inline float fabs(float x) { return std::fabs(x); }
#include "bilateral.cl"
}
namespace ref_curvature {
inline float fabs(float x) { return std::fabs(x); }
inline float pow(float a, float b) { return std::pow(a, b); }
#include "curvatureflow.cl"
}
#include "clshim_kernel_end.hpp"

using namespace clshim;

extern "C" {

void ref_bilateral_filter(const float* in, float* out, int width, int height) {
    image2d_t ii{const_cast<float*>(in), width, height}, oo{out, width, height};
    run_ndrange_2d((size_t)width, (size_t)height, [&] { ref_bilateral::bilateral(ii, oo, width, height); });
}

void ref_curvature_flow(const float* in, float* out, int width, int height, float inv_proj_x, float inv_proj_y) {
    image2d_t ii{const_cast<float*>(in), width, height}, oo{out, width, height};
    run_ndrange_2d((size_t)width, (size_t)height,
                   [&] { ref_curvature::curvature_flow(ii, oo, width, height, inv_proj_x, inv_proj_y); });
}

}  // extern "C"
