/*
 * ref_pcisph.cpp -- C entry points running the reference's kernels/pcisph.cl on the CPU.
 * TEST INFRASTRUCTURE (oracle/_ref only).  The program is built with PARTICLE_COUNT,
 * SUPPORT_RADIUS, PARTICLE_MASS, REST_DENSITY and COMPUTE_BOUNDARY
 * (fluid/simulation/pcisphsimluation.cpp:501-508); arguments follow :280-392.
 * With no boundary particles the boundary lists have length 0, which gives the same
 * result as building without COMPUTE_BOUNDARY.
 */
#include "clshim.hpp"

#include "clshim_kernel_begin.hpp"
namespace REF_NS(ref_pcisph) {
#include "pcisph.cl"
}
#include "clshim_kernel_end.hpp"

using namespace clshim;

static void set_defines(int n, float support_define, float mass_define, float rho0_define) {
    g_particle_count = n;
    g_support_radius = support_define;
    g_particle_mass = mass_define;
    g_rest_density = rho0_define;
}

extern "C" {

void REF_FN(ref_pci_initial_density)(const float* pos4, float* dens, int n, const int32_t* flen, const int32_t* flist,
                             const int32_t* blist, const int32_t* blen, const float* bpos4, const float* bphi,
                             float w_eval, float support_define, float mass_define, float rho0_define,
                             int local_size) {
    set_defines(n, support_define, mass_define, rho0_define);
    const size_t local = local_size > 0 ? (size_t)local_size : 64;
    image1d_buffer_t ip{pos4, 4}, ib{bpos4, 4}, iphi{bphi, 1};
    run_ndrange((size_t)n, local, true, [&] {
        REF_NS(ref_pcisph)::compute_initial_density(ip, dens, flen, flist, blist, blen, ib, iphi, w_eval, static_cast<float4*>(group_local(0, sizeof(float4) * local)));
    });
}

void REF_FN(ref_pci_initial_forces)(const float* pos4, const float* vel4, const float* dens, const float* nrm4,
                            float* fo4, int n, float mu, float sigma, const int32_t* flen, const int32_t* flist,
                            float visc_lapl, float st_main, float st_term, float support_define,
                            float mass_define, float rho0_define, int local_size) {
    set_defines(n, support_define, mass_define, rho0_define);
    const size_t local = local_size > 0 ? (size_t)local_size : 64;
    image1d_buffer_t ip{pos4, 4}, iv{vel4, 4}, id{dens, 1}, in{nrm4, 4};
    run_ndrange((size_t)n, local, true, [&] {
        REF_NS(ref_pcisph)::compute_initial_forces(ip, iv, id, in, reinterpret_cast<float4*>(fo4), mu, sigma, flen, flist,
                                           visc_lapl, st_main, st_term, static_cast<float4*>(group_local(0, sizeof(float4) * local)), static_cast<float4*>(group_local(1, sizeof(float4) * local)), static_cast<float*>(group_local(3, sizeof(float) * local)),
                                           static_cast<float4*>(group_local(2, sizeof(float4) * local)));
    });
}

void REF_FN(ref_pci_predict_pos)(const float* pos4, const float* vel4, const float* fo4, const float* fp4,
                         float* pred4, int n, float dt, const float* g4, float max_vel, const float* lim4,
                         float support_define, float mass_define, float rho0_define) {
    set_defines(n, support_define, mass_define, rho0_define);
    float4 g = make_float4(g4[0], g4[1], g4[2], g4[3]);
    float4 lim = make_float4(lim4[0], lim4[1], lim4[2], lim4[3]);
    run_ndrange((size_t)n, 64, false, [&] {
        REF_NS(ref_pcisph)::predict_pos(reinterpret_cast<const float4*>(pos4), reinterpret_cast<const float4*>(vel4),
                                reinterpret_cast<const float4*>(fo4), reinterpret_cast<const float4*>(fp4),
                                reinterpret_cast<float4*>(pred4), dt, g, max_vel, lim);
    });
}

void REF_FN(ref_pci_update_pressure)(const float* pred4, float* dens_var, float* pres, int n, float delta,
                             const int32_t* flen, const int32_t* flist, const int32_t* blist,
                             const int32_t* blen, const float* bpos4, const float* bphi, float w_eval,
                             float support_define, float mass_define, float rho0_define, int local_size) {
    set_defines(n, support_define, mass_define, rho0_define);
    const size_t local = local_size > 0 ? (size_t)local_size : 64;
    image1d_buffer_t ip{pred4, 4}, ib{bpos4, 4}, iphi{bphi, 1};
    run_ndrange((size_t)n, local, true, [&] {
        REF_NS(ref_pcisph)::update_pressure(ip, dens_var, pres, delta, flen, flist, blist, blen, ib, iphi, w_eval,
                                    static_cast<float4*>(group_local(0, sizeof(float4) * local)));
    });
}

void REF_FN(ref_pci_pressure_force)(const float* pos4, const float* dens, const float* pres, float* fp4, int n,
                            float size, float cell_size, int cps, const int32_t* flen, const int32_t* flist,
                            const int32_t* blist, const int32_t* blen, const float* bpos4, const float* bphi,
                            float w_grad, float support_define, float mass_define, float rho0_define,
                            int local_size) {
    set_defines(n, support_define, mass_define, rho0_define);
    const size_t local = local_size > 0 ? (size_t)local_size : 64;
    REF_NS(ref_pcisph)::GridInfo gi;
    gi.size = size; gi.cell_size = cell_size; gi.cells_per_side = cps; gi.cells_count = cps * cps * cps;
    image1d_buffer_t ip{pos4, 4}, id{dens, 1}, ipr{pres, 1}, ib{bpos4, 4}, iphi{bphi, 1};
    run_ndrange((size_t)n, local, true, [&] {
        REF_NS(ref_pcisph)::compute_pressure_force(ip, id, ipr, reinterpret_cast<float4*>(fp4), gi, flen, flist, blist,
                                           blen, ib, iphi, w_grad, static_cast<float4*>(group_local(0, sizeof(float4) * local)), static_cast<float*>(group_local(3, sizeof(float) * local)), static_cast<float*>(group_local(4, sizeof(float) * local)));
    });
}

void REF_FN(ref_pci_integrate)(const float* pos4, const float* vel4, const float* fo4, const float* fp4,
                       float* out_pos4, float* out_vel4, int n, float dt, const float* g4, float max_vel,
                       const float* lim4, float support_define, float mass_define, float rho0_define) {
    set_defines(n, support_define, mass_define, rho0_define);
    float4 g = make_float4(g4[0], g4[1], g4[2], g4[3]);
    float4 lim = make_float4(lim4[0], lim4[1], lim4[2], lim4[3]);
    run_ndrange((size_t)n, 64, false, [&] {
        REF_NS(ref_pcisph)::predict_vel_n_pos(reinterpret_cast<const float4*>(pos4), reinterpret_cast<const float4*>(vel4),
                                      reinterpret_cast<const float4*>(fo4), reinterpret_cast<const float4*>(fp4),
                                      reinterpret_cast<float4*>(out_pos4), reinterpret_cast<float4*>(out_vel4), dt, g,
                                      max_vel, lim);
    });
}

}  // extern "C"
