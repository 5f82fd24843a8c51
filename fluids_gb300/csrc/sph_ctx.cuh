/*
 * sph_ctx.cuh -- the solver context (struct sph_ctx of include/sph_capi.h), shared by the
 * translation units that implement the C ABI (sph_context.cu, sph_adjoint.cu).
 */
#pragma once
#include <string>
#include <vector>

#include "sph_capi.h"
#include "sph_kernels.cuh"

using sph::Bufs;
using sph::Const;

struct SphBody {
    int origin = 0, count = 0, can_move = 0;
    float mass = 0.f;
    float xf[20];   /* rot3x4 (row-major), lin4, ang4 */
    /* rigid-body dynamics (sph_set_body_dynamics): integrated on the device every step */
    int dynamic = 0;
    float inv_inertia[3] = {0.f, 0.f, 0.f};
    float radius = 0.f;
};

struct sph_ctx {
    sph_params p{};
    Const c{};
    Bufs b{};
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    /* a second stream and fork / join events: work that may run beside the main stream's
     * (the gated full sort of the step's incremental sort) */
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    /* sph_simulate_host: the stream and events of the velocity uploads, and the step graph
     * with its copies for one set of host buffers */
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_copy = nullptr, ev_vel = nullptr;
#ifndef SPH_OUT_CHUNKS
#define SPH_OUT_CHUNKS 8   /* e2e at 4M: 2.93 ms per step with 8 parts, 2.97 with 4, 2.94 with 16 */
#endif
    static constexpr int kOutChunks = SPH_OUT_CHUNKS;   /* force pass parts whose results download early */
    cudaEvent_t ev_chunk[kOutChunks] = {};
    cudaGraphExec_t host_gexec = nullptr;
    const void* host_key[3] = {nullptr, nullptr, nullptr};
    bool host_graph_ok = true;
    int device = 0, num_sms = 1;
    std::string err;
    float lim[3] = {0.f, 0.f, 0.f};
    /* host copies of what was added (FluidSimulation::add_volume / add_boundary) */
    std::vector<float> vol_pos, vol_vel;
    std::vector<float> braw_host;
    std::vector<SphBody> bodies;
    int N = 0, NB = 0;
    bool any_movable = false, any_massive = false, any_dynamic = false;
    char* arena = nullptr;
    size_t arena_bytes = 0;
    int max_iter_slots = 1;
    int coop_blocks = 0;
    int bs = 256;
    int tile_ctas = 0;   /* batched: CTAs per SM of the persistent tile launches (0: 2048 / bs) */
    std::vector<sph::SceneTile> h_tiles;
    bool graph_ok = true;
    cudaGraphExec_t gexec = nullptr;
    int graph_kernels = 0;   /* kernel nodes of the step graph */
    uint32_t* cur_keys = nullptr;
    int32_t* cur_mask = nullptr;
    bool has_state = false;
    std::vector<cudaEvent_t>* prof = nullptr;   /* set only by sph_profile_step */
    std::vector<const char*> prof_names;
    std::string prof_list;
    /* batched contexts: one entry per scene (container, viscosity, stiffness, ranges) */
    struct SceneIn {
        float lim[3];
        float mu, kgas;
        int first, count, first_b, count_b;
    };
    std::vector<SceneIn> scene_in;
    std::vector<sph::SceneDev> h_scenes;
    sph::SceneDev* d_scenes = nullptr;
    int32_t* d_scene_of = nullptr;
    double* d_scene_stats = nullptr;
    int inject = 0;   /* one-shot fault for the next step (sph_inject_fault) */
    bool inject_alloc = false;   /* the next arena allocation fails (sph_inject_fault) */
    /* depth-test scratch of sph_render_depth: 8 bytes per pixel */
    void* render_buf = nullptr;
    size_t render_pixels = 0;
    void* render_sort = nullptr;   /* sph_render_depth: 16-bit depth keys and particle order */
    size_t render_sort_bytes = 0;
    void* frame_buf = nullptr;     /* sph_render_frame: depth, blur scratch, normals, colour */
    size_t frame_pixels = 0;
};

/* Records msg as the context's last error (or the last creation error) and returns code. */
int sph_ctx_fail(sph_ctx* x, int code, const std::string& msg);
