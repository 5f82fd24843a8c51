/*
 * ref_normals.cpp -- C entry point running the reference's kernels/normals.cl on the CPU.
 * TEST INFRASTRUCTURE (oracle/_ref only).  Arguments as bound by
 * fluid/simulation/pcisphsimluation.cpp:300-307 (positions and densities read as images,
 * local caches of one float4 / one float per work-item).
 */
#include "clshim.hpp"

#include "clshim_kernel_begin.hpp"
namespace REF_NS(ref_normals) {
#include "normals.cl"
}
#include "clshim_kernel_end.hpp"

using namespace clshim;

extern "C" {

void REF_FN(ref_compute_normals)(const float* pos4, const float* dens, float* nrm4, int n, const int32_t* len,
                         const int32_t* list, float w_grad, float mass_define, float support_define,
                         int local_size) {
    g_particle_count = n;
    g_particle_mass = mass_define;
    g_support_radius = support_define;
    const size_t local = local_size > 0 ? (size_t)local_size : 64;
    image1d_buffer_t ip{pos4, 4}, id{dens, 1};
    run_ndrange((size_t)n, local, true, [&] {
        REF_NS(ref_normals)::compute_normals(ip, id, reinterpret_cast<float4*>(nrm4), len, list, w_grad, static_cast<float4*>(group_local(0, sizeof(float4) * local)),
                                     static_cast<float*>(group_local(1, sizeof(float) * local)));
    });
}

}  // extern "C"
