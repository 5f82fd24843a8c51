/*
 * ref_wcsph.cpp -- C entry points running the reference's kernels/wcsph.cl on the CPU.
 * TEST INFRASTRUCTURE (oracle/_ref only).  The WCSPH program is built with PARTICLE_COUNT
 * and SUPPORT_RADIUS (fluid/simulation/wcsphsimluation.cpp:368-370); the kernel argument
 * lists follow wcsphsimluation.cpp:223-279.
 */
#include "clshim.hpp"

#include "clshim_kernel_begin.hpp"
namespace REF_NS(ref_wcsph) {
#include "wcsph.cl"
}
#include "clshim_kernel_end.hpp"

using namespace clshim;

extern "C" {

void REF_FN(ref_wc_density_pressure)(const float* pos4, int n, float* dens, float* pres, float mass,
                             float h, float gas_k, float rho0, float poly6, const int32_t* flen,
                             const int32_t* flist, const int32_t* blist, const int32_t* blen,
                             const float* bpos4, const float* bphi, float support_define) {
    g_particle_count = n;
    g_support_radius = support_define;
    run_ndrange((size_t)n, 128, false, [&] {
        REF_NS(ref_wcsph)::compute_density_pressure(reinterpret_cast<const float4*>(pos4), dens, pres, mass, h,
                                            gas_k, rho0, poly6, flen, flist, blist, blen,
                                            reinterpret_cast<const float4*>(bpos4), bphi);
    });
}

/* sc: poly6_eval, poly6_grad, poly6_lapl, visc_eval, visc_grad, visc_lapl, spiky_eval,
 * spiky_grad, spiky_lapl (kernels/common.h:21-35). g4 = (0, -g, 0, 0). */
void REF_FN(ref_wc_acceleration)(const float* pos4, const float* vel4, const float* nrm4, const float* dens,
                         const float* pres, float* acc4, int n, const float* g4, float mass, float h,
                         float h2, float mu, float sigma, float rho0, const float* sc9,
                         int32_t* flen, int32_t* flist, int32_t* blist, int32_t* blen, float* bpos4,
                         float* bphi, float st_main, float st_term, float support_define) {
    g_particle_count = n;
    g_support_radius = support_define;
    REF_NS(ref_wcsph)::SmoothingConstants sc;
    sc.poly6_eval = sc9[0]; sc.poly6_grad = sc9[1]; sc.poly6_lapl = sc9[2];
    sc.visc_eval = sc9[3]; sc.visc_grad = sc9[4]; sc.visc_lapl = sc9[5];
    sc.spiky_eval = sc9[6]; sc.spiky_grad = sc9[7]; sc.spiky_lapl = sc9[8];
    float4 g = make_float4(g4[0], g4[1], g4[2], g4[3]);
    run_ndrange((size_t)n, 128, false, [&] {
        REF_NS(ref_wcsph)::compute_acceleration(reinterpret_cast<const float4*>(pos4), reinterpret_cast<const float4*>(vel4),
                                        reinterpret_cast<const float4*>(nrm4), dens, pres,
                                        reinterpret_cast<float4*>(acc4), g, mass, h, h2, mu, sigma, rho0, sc,
                                        flen, flist, blist, blen, reinterpret_cast<float4*>(bpos4), bphi,
                                        st_main, st_term);
    });
}

void REF_FN(ref_wc_integrate)(float* pos4, float* vel4, float* vhalf4, float* acc4, int n, float dt,
                      float* out_pos4, float* out_vel4, float* out_vhalf4, float max_vel,
                      const float* limits4, float support_define) {
    g_particle_count = n;
    g_support_radius = support_define;
    float4 lim = make_float4(limits4[0], limits4[1], limits4[2], limits4[3]);
    run_ndrange((size_t)n, 128, false, [&] {
        REF_NS(ref_wcsph)::predict_vel_n_pos(reinterpret_cast<float4*>(pos4), reinterpret_cast<float4*>(vel4),
                                     reinterpret_cast<float4*>(vhalf4), reinterpret_cast<float4*>(acc4), dt,
                                     reinterpret_cast<float4*>(out_pos4), reinterpret_cast<float4*>(out_vel4),
                                     reinterpret_cast<float4*>(out_vhalf4), max_vel, lim);
    });
}

}  // extern "C"
