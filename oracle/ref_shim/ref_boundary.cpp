/*
 * ref_boundary.cpp -- C entry points running the reference's kernels/boundary.cl on the CPU.
 * TEST INFRASTRUCTURE (oracle/_ref only).  The program is built with SUPPORT_RADIUS
 * (fluid/simulation/boundaryhandler.cpp:404-419); arguments follow :238-349.
 */
#include "clshim.hpp"

#include "clshim_kernel_begin.hpp"
namespace REF_NS(ref_boundary) {
#include "boundary.cl"
}
#include "clshim_kernel_end.hpp"

using namespace clshim;

extern "C" {

void REF_FN(ref_boundary_phi)(const float* pos4, float* phi, int count, float rho0, float w_eval, float phi_coeff,
                      float support_define) {
    g_support_radius = support_define;
    g_boundary_particle_count = count;
    run_ndrange((size_t)count, 64, false, [&] {
        REF_NS(ref_boundary)::compute_boundary_phi(reinterpret_cast<const float4*>(pos4), phi, rho0, w_eval, phi_coeff,
                                           count);
    });
}

/* rows: m0, m1, m2 (float4 each, w = 0); lin4, ang4, cm4 (cm.w = 1 as in boundaryhandler.cpp:274). */
void REF_FN(ref_transform_particles)(const float* raw4, float* out4, float* vel4, const float* m0, const float* m1,
                             const float* m2, const float* lin4, const float* ang4, const float* cm4, int count) {
    float4 r0 = make_float4(m0[0], m0[1], m0[2], m0[3]);
    float4 r1 = make_float4(m1[0], m1[1], m1[2], m1[3]);
    float4 r2 = make_float4(m2[0], m2[1], m2[2], m2[3]);
    float4 lin = make_float4(lin4[0], lin4[1], lin4[2], lin4[3]);
    float4 ang = make_float4(ang4[0], ang4[1], ang4[2], ang4[3]);
    float4 cm = make_float4(cm4[0], cm4[1], cm4[2], cm4[3]);
    run_ndrange((size_t)count, 64, false, [&] {
        REF_NS(ref_boundary)::transform_particles(reinterpret_cast<const float4*>(raw4), reinterpret_cast<float4*>(out4),
                                          reinterpret_cast<float4*>(vel4), r0, r1, r2, lin, ang, cm, count);
    });
}

void REF_FN(ref_fluid_force)(float* bpos4, float* bphi, const float* fpos4, const float* fdens, const float* fpres,
                     const int32_t* intervals, float mass, float spiky_grad, float size, float cell_size, int cps,
                     int count, float* force4, float* torque4, const float* center4, const float* fvel4,
                     const float* bvel4, float visc_lapl, float support_define) {
    g_support_radius = support_define;
    REF_NS(ref_boundary)::GridInfo gi;
    gi.size = size; gi.cell_size = cell_size; gi.cells_per_side = cps; gi.cells_count = cps * cps * cps;
    image1d_buffer_t ip{fpos4, 4}, id{fdens, 1}, ipr{fpres, 1}, iv{fvel4, 4};
    float4 center = make_float4(center4[0], center4[1], center4[2], center4[3]);
    run_ndrange((size_t)count, 64, false, [&] {
        REF_NS(ref_boundary)::compute_fluid_force(reinterpret_cast<float4*>(bpos4), bphi, ip, id, ipr,
                                          reinterpret_cast<const int2*>(intervals), mass, spiky_grad, gi, count,
                                          reinterpret_cast<float4*>(force4), reinterpret_cast<float4*>(torque4),
                                          center, iv, reinterpret_cast<const float4*>(bvel4), visc_lapl);
    });
}

}  // extern "C"
