/*
 * sph_capi.h -- C ABI of the GB300 SPH particle pipeline (libsph_gb300.so).
 *
 * Drop-in boundary for the per-step particle pipeline of paivett/fluids: the reference's
 * C++ solver classes (fluid/simulation/wcsphsimluation.cpp, pcisphsimluation.cpp,
 * grid.cpp, boundaryhandler.cpp) call these entry points in place of their OpenCL kernel
 * launches (clEnqueueNDRangeKernel / CLKernel::run), clsort, clshuffle, clmax and clsum.
 * Plain C types only: host arrays are float[4*n] (x, y, z, w) as the reference's cl_float4
 * buffers; device pointers are returned as void*.
 *
 * Every function returns SPH_OK (0) or an SPH_E_* status; sph_last_error() describes the
 * last failure.  A context owns one CUDA stream and is not thread-safe; distinct contexts
 * may be driven from different threads.
 */
#ifndef SPH_CAPI_H
#define SPH_CAPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPH_CAPI_VERSION 1

/* Status codes.  Replace CLError::check's exceptions (opencl/clerror.cpp:15-19). */
enum sph_status {
    SPH_OK = 0,
    SPH_E_INVALID = 1,       /* bad argument or parameter */
    SPH_E_CUDA = 2,          /* a CUDA runtime call failed */
    SPH_E_NONCONVERGED = 3,  /* PCISPH stopped at max iterations above the error ratio */
    SPH_E_ESCAPED = 4,       /* a particle left the grid (PHYSICS grid clamps it) */
    SPH_E_NAN = 5,           /* a non-finite position or velocity was produced */
    SPH_E_TIMEOUT = 6,       /* a bounded device wait gave up */
    SPH_E_OVERFLOW = 7,      /* a size limit was exceeded */
    SPH_E_STATE = 8,         /* call not valid in the current state */
    SPH_E_NOMEM = 9          /* device allocation failed */
};

/* Device status word bits (sph_device_flags). */
enum sph_flag {
    SPH_FLAG_NAN = 1u,
    SPH_FLAG_ESCAPED = 2u,
    SPH_FLAG_TIMEOUT = 4u,
    SPH_FLAG_OVERFLOW = 8u,
    SPH_FLAG_NONCONVERGED = 16u,
    SPH_FLAG_NONSMOOTH = 32u   /* adjoint: a velocity clamp or wall reflection was active */
};

enum sph_method { SPH_WCSPH = 0, SPH_PCISPH = 1 };

/* COMPAT follows the reference kernel text (including its defects) for stage parity;
 * PHYSICS applies the documented fixes P1..P7 (container-fitted grid, mass-consistent
 * forces, 315 poly6 normalisation, PCISPH stop test). */
enum sph_mode { SPH_MODE_COMPAT = 0, SPH_MODE_PHYSICS = 1 };

/* Neighbour access: scan the 27 cells in every pass, or materialise per-particle lists
 * once per step (grid.cl:145-182 layout, column-major; the default, measured 2.4x faster
 * for WCSPH on GB300 because the list passes run without divergence).  PCISPH always uses
 * lists. */
enum sph_neighbors { SPH_NEIGH_SCAN = 0, SPH_NEIGH_LIST = 1 };

/* Solver parameters: the union of SimulationSettings (settings/simulationsettings.h) and
 * PhysicsSettings (settings/physicssettings.h) plus the grid constants the reference fixes
 * in code (wcsphsimluation.cpp:26 grid side 5.0, common.h:4 list cap 50). */
typedef struct sph_params {
    int method;                      /* sph_method */
    int mode;                        /* sph_mode */
    float time_step;                 /* s */
    float max_vel;                   /* m/s, per-component clamp */
    float particle_radius;           /* m; lattice spacing = 2 * radius */
    float support_radius;            /* h, m; also the grid cell size */
    int pcisph_min_iterations;       /* pcisphsimluation.h:254 (3) */
    int pcisph_max_iterations;
    float pcisph_error_ratio;        /* eta */
    int pcisph_relax_max_iterations; /* pcisphsimluation.cpp:549 (10000) */
    float rest_density;              /* kg/m^3 */
    float k_viscosity;
    float gravity;                   /* m/s^2, acts along -y */
    float gas_stiffness;             /* Tait k (WCSPH) */
    float surface_tension;
    float grid_size;                 /* COMPAT: cube side centred at the origin (5.0) */
    float grid_margin;               /* PHYSICS: cells of margin around the container (2) */
    float boundary_phi_coeff;        /* BoundaryHandler phi coefficient (1.0) */
    int neigh_cap;                   /* neighbours kept per particle (50) */
    int relax_on_add;                /* PCISPH: relaxation step then v := 0 after add_volume */
    int neighbor_mode;               /* sph_neighbors (WCSPH only) */
    int use_graph;                   /* capture a step in a CUDA graph (1) */
    int block_size;                  /* threads per block of particle kernels (32..256), 0 = 256 */
    int kernels;                     /* sph_kernels: smoothing-kernel family (SPH_KERNELS_MULLER) */
} sph_params;

/* Smoothing-kernel family (kernels/kernels.h:8-37).  The reference builds every program with
 * USE_MULLER_KERNELS (wcsphsimluation.cpp:370, pcisphsimluation.cpp:505,
 * boundaryhandler.cpp:413); without it the kernel text's W_DEFAULT, GRAD_W_DEFAULT,
 * GRAD_W_PRESSURE and LAPL_W_VISCOSITY become the Monaghan cubic spline of
 * kernels/monaghan_kernels.h:7-47 at the same call sites (the host constants are unchanged).
 * SPH_KERNELS_MONAGHAN reproduces that build; it exists in COMPAT mode only. */
enum sph_kernels { SPH_KERNELS_MULLER = 0, SPH_KERNELS_MONAGHAN = 1 };

typedef struct sph_ctx sph_ctx;

/* Field ids for sph_get_field / sph_set_field / sph_field_device_ptr.  "Sorted" arrays are in
 * this step's Morton order; POS/VEL/VEL_HALF hold the state between steps, in the previous
 * step's sorted order, as the reference's unsorted buffers do (wcsphsimluation.cpp:270-279). */
enum sph_field {
    SPH_F_POS = 0, SPH_F_VEL = 1, SPH_F_VEL_HALF = 2,
    SPH_F_POS_SORTED = 3, SPH_F_VEL_SORTED = 4, SPH_F_VEL_HALF_SORTED = 5,
    SPH_F_HASHES = 6, SPH_F_MASK = 7, SPH_F_CELL_INTERVALS = 8,
    SPH_F_NEIGH_LIST = 9, SPH_F_NEIGH_LEN = 10, SPH_F_SB_NEIGH_LIST = 11, SPH_F_SB_NEIGH_LEN = 12,
    SPH_F_DENSITY = 13, SPH_F_PRESSURE = 14, SPH_F_NORMAL = 15, SPH_F_ACCEL = 16,
    SPH_F_POS_PRED = 17, SPH_F_FORCE_OTHER = 18, SPH_F_FORCE_PRESSURE = 19, SPH_F_DENS_VAR = 20,
    SPH_F_BPOS_SORTED = 21, SPH_F_BPHI_SORTED = 22, SPH_F_BCELL_INTERVALS = 23,
    SPH_F_BHASHES = 24, SPH_F_BMASK = 25, SPH_F_BPHI = 26, SPH_F_BPOS = 27,
    SPH_F_BODY_FORCE = 28, SPH_F_BODY_TORQUE = 29, SPH_F_PCI_ITERS = 30, SPH_F_PCI_MAXERR = 31,
    SPH_F_ID = 32, SPH_F_COUNT = 33
};
/* Element kinds returned by sph_field_kind. */
enum sph_kind { SPH_KIND_F32 = 0, SPH_KIND_I32 = 1, SPH_KIND_U32 = 2 };

/* Stage ids for sph_run_stage: one call per reference launch point. */
enum sph_stage {
    SPH_S_BOUNDARY_SYNC = 0,    /* BoundaryHandler::sync (boundaryhandler.cpp:251-294) */
    SPH_S_HASHES = 1,           /* Grid::compute_hashes (grid.cpp:22-34; grid.cl:20-39) */
    SPH_S_SORT = 2,             /* clsort<cl_uint,cl_int> (opencl/algorithms/clsort.h:13-35) */
    SPH_S_SHUFFLE = 3,          /* clshuffle<cl_float4> x3 / x2 (clshuffle.h:12-58) */
    SPH_S_CELL_INTERVALS = 4,   /* Grid::compute_cell_intervals (grid.cpp:36-55; grid.cl:60-123) */
    SPH_S_NEIGH_LIST = 5,       /* Grid::compute_neigh_list (grid.cpp:97-115; grid.cl:145-182) */
    SPH_S_SB_NEIGH_LIST = 6,    /* BoundaryHandler::build_neighbourhood (boundaryhandler.cpp:351-371) */
    SPH_S_WC_DENSITY = 7,       /* compute_density_pressure (wcsph.cl:32-79) */
    SPH_S_NORMALS = 8,          /* compute_normals (normals.cl:23-70) */
    SPH_S_WC_ACCEL = 9,         /* compute_acceleration (wcsph.cl:81-173) */
    SPH_S_WC_INTEGRATE = 10,    /* predict_vel_n_pos (wcsph.cl:176-224) */
    SPH_S_PCI_INIT_DENSITY = 11,/* fill p = 0 + compute_initial_density (pcisph.cl:33-102) */
    SPH_S_PCI_INIT_FORCES = 12, /* fill F_p = 0 + compute_initial_forces (pcisph.cl:134-222) */
    SPH_S_PCI_LOOP = 13,        /* predict/update/force loop + clmax (pcisphsimluation.cpp:129-148) */
    SPH_S_PCI_INTEGRATE = 14,   /* predict_vel_n_pos (pcisph.cl:240-284) */
    SPH_S_BOUNDARY_FORCES = 15, /* BoundaryHandler::apply_fluid_forces (boundaryhandler.cpp:296-349) */
    /* the three passes of one PCISPH loop iteration, each alone on the fields as they are
     * (PCISPH contexts only): */
    SPH_S_PCI_PREDICT = 16,     /* predict_pos (pcisph.cl:302-344): POS_PRED */
    SPH_S_PCI_UPDATE_PRESSURE = 17, /* update_pressure (pcisph.cl:349-418): DENS_VAR, PRESSURE += */
    SPH_S_PCI_PRESSURE_FORCE = 18   /* compute_pressure_force (pcisph.cl:420-504): FORCE_PRESSURE
                                       from POS_SORTED, DENSITY, PRESSURE */
};

/* ---- parameters and lifetime ------------------------------------------------------ */

/* Fills *out with the defaults of the reference's config.wc (method SPH_WCSPH) or
 * config.pci (SPH_PCISPH) in COMPAT mode. */
void sph_default_params(int method, sph_params* out);

/* Creates a solver.  Replaces WCSPHSimulation / PCISPHSimulation construction
 * (wcsphsimluation.cpp:15-34, pcisphsimluation.cpp:19-62, fluidsimulationfactory.h:13-40). */
int sph_create(const sph_params* params, sph_ctx** out);
/* Releases the context and its device memory (wcsphsimluation.cpp:284-308). */
int sph_destroy(sph_ctx* ctx);
/* Text of the last failure on ctx (or of the last failed sph_create when ctx is NULL). */
const char* sph_last_error(const sph_ctx* ctx);
/* FluidSimulation::reset (fluidsimulation.h:47-48): new parameters, particles rebuilt from
 * the volumes and boundaries added so far. */
int sph_reset(sph_ctx* ctx, const sph_params* params);
/* Runs work on a caller stream (cudaStream_t) instead of the context's own stream. */
int sph_set_stream(sph_ctx* ctx, void* cuda_stream);

/* ---- scene -------------------------------------------------------------------------- */

/* FluidSimulation::set_rect_limits (fluidsimulation.h:79; wcsphsimluation.cpp:407-414). */
int sph_set_rect_limits(sph_ctx* ctx, float width, float height, float depth);
/* FluidSimulation::add_volume (fluidsimulation.h:91): appends n particles (host pos4; vel4
 * may be NULL for rest) and re-initialises the solver (wcsphsimluation.cpp:386-405). */
int sph_add_volume(sph_ctx* ctx, const float* pos4, const float* vel4, int n);
/* FluidSimulation::add_boundary (fluidsimulation.h:66-68; boundaryhandler.cpp:95-153):
 * n sampled surface particles in body coordinates, the body's rigid transform rot3x4
 * (row-major 3x4, NULL = identity), linear/angular velocity lin4/ang4 (NULL = 0) and mass
 * (fluid forces are accumulated for mass > 0). */
int sph_add_boundary(sph_ctx* ctx, const float* pos4, int n, int can_move, const float* rot3x4,
                     const float* lin4, const float* ang4, float mass);
/* Updates a body's transform and velocities before the next sync (RigidBody state read by
 * boundaryhandler.cpp:259-274). */
int sph_set_body_transform(sph_ctx* ctx, int body, const float* rot3x4, const float* lin4,
                           const float* ang4);
/* Two-way coupling without a physics engine: the reference hands the fluid's force and
 * torque on each body to Bullet (boundaryhandler.cpp:296-349, scene.cpp:471 makes bodies with
 * mass dynamic).  With enabled != 0 the context itself advances the body every step on the
 * device (semi-implicit Euler under fluid force, fluid torque and gravity; orientation by
 * the angular velocity), so the body moves inside the captured step.  inv_inertia3: inverse
 * principal moments in body coordinates (a solid cube of side s: 6 / (m s^2)); radius > 0
 * keeps the body's centre that far inside the container.  Bodies do not collide with each
 * other.  The body must be movable (can_move) with mass > 0. */
int sph_set_body_dynamics(sph_ctx* ctx, int body, int enabled, const float* inv_inertia3, float radius);
/* Current transform and velocities of a body (the pose RigidBody reports for rendering);
 * synchronises. */
int sph_get_body_state(sph_ctx* ctx, int body, float* rot3x4, float* lin4, float* ang4);
/* FluidSimulation::particle_count / boundary_particle_count (fluidsimulation.h:54,84). */
int sph_particle_count(const sph_ctx* ctx);
int sph_boundary_particle_count(const sph_ctx* ctx);

/* ---- stepping ------------------------------------------------------------------------ */

/* FluidSimulation::simulate (fluidsimulation.h:36) called nsteps times; asynchronous on the
 * context stream (a CUDA graph per step when use_graph = 1). */
int sph_simulate(sph_ctx* ctx, int nsteps);
/* nsteps steps with the particle state on the host: each step uploads pos4, vel4 and (WCSPH)
 * vhalf4 -- 4 floats per particle in the context's current particle order, the layout of the
 * POS, VEL and VEL_HALF fields -- runs the step of sph_simulate and downloads the three back
 * into the same buffers.  The velocity uploads run beside the step's binning, sort and list
 * pass, which do not read them.  Asynchronous on the context stream like sph_simulate; the
 * buffers must stay valid until it completes.  With use_graph = 1 and page-locked buffers
 * the step and its copies are one CUDA graph per set of buffers.  Same results as
 * sph_set_field_async, sph_simulate(ctx, 1) and sph_get_field_async per step.  No
 * counterpart in the reference, whose state stays on the device between steps. */
int sph_simulate_host(sph_ctx* ctx, float* pos4, float* vel4, float* vhalf4, int nsteps);
/* Runs one stage (one reference launch point) on the current state. */
int sph_run_stage(sph_ctx* ctx, int stage);
/* Runs nsteps steps of the same kernel sequence as sph_simulate, without the graph, with a
 * CUDA event after each kernel group (replaces the reference's per-kernel profiling queue,
 * opencl/clenvironment.cpp:45-48 and clmisc.cpp:3-22).  Writes the average device ms per
 * step of each group to ms_out[0..max_groups), the group count to *ngroups and the group
 * names, comma-separated, to names. */
int sph_profile_step(sph_ctx* ctx, int nsteps, float* ms_out, int max_groups, int* ngroups, char* names,
                     size_t names_len);
/* The number of kernel launches in one step's CUDA graph (building the graph if the context
 * steps through one and has none yet); 0 when the context steps without a graph.  No
 * counterpart in the reference, whose launches are the enqueue calls of the step. */
int sph_step_kernel_launches(sph_ctx* ctx, int* launches);
/* Waits for the context stream. */
int sph_synchronize(sph_ctx* ctx);

/* Host-side fault injection for failure-detection tests (no counterpart in the reference,
 * whose only failure path is CLError, opencl/clerror.cpp:15-19).  SPH_FAULT_BARRIER_STALL
 * (PCISPH contexts): the next step's predict-correct kernel waits at its grid barrier for one
 * CTA more than it launched, so every CTA's bounded wait runs out (about a second), sets
 * SPH_FLAG_TIMEOUT and returns; the step's integration is skipped, the context stays usable
 * and the steps after it are normal.  Nothing faults or hangs.  SPH_FAULT_ALLOC_FAIL (any
 * context): the next device-arena allocation (sph_add_volume, sph_add_boundary,
 * sph_set_rect_limits, sph_reset) is refused as cudaMalloc refuses one; the call returns
 * SPH_E_NOMEM and leaves the context as it was (the arena is grown by allocating the new one
 * before freeing the old).  SPH_FAULT_NONE cancels both. */
enum sph_fault { SPH_FAULT_NONE = 0, SPH_FAULT_BARRIER_STALL = 1, SPH_FAULT_ALLOC_FAIL = 2 };
int sph_inject_fault(sph_ctx* ctx, int kind);
/* Reads (and with clear = 1 resets) the device status word; synchronises. */
int sph_device_flags(sph_ctx* ctx, unsigned* flags, int clear);

/* ---- buffers ------------------------------------------------------------------------- */

/* Number of scalar elements of a field (float4 fields count 4 per particle). */
long long sph_field_elems(const sph_ctx* ctx, int field);
/* sph_kind of a field. */
int sph_field_kind(int field);
/* Copies a field to / from host memory (bytes must equal elems * 4); synchronises. */
int sph_get_field(sph_ctx* ctx, int field, void* host, size_t bytes);
int sph_set_field(sph_ctx* ctx, int field, const void* host, size_t bytes);
/* The same copies enqueued on the context's stream, ordered with sph_simulate and returning
 * at once: the host memory must stay valid until sph_synchronize (pinned memory makes the
 * copy asynchronous; pageable memory is copied synchronously by the driver).  For a host
 * program that uploads and reads back state every frame without a host wait per array. */
int sph_get_field_async(sph_ctx* ctx, int field, void* host, size_t bytes);
int sph_set_field_async(sph_ctx* ctx, int field, const void* host, size_t bytes);
/* Device address of a field (replaces the cl_mem / GL VBO buffers of clallocator.h). */
int sph_field_device_ptr(sph_ctx* ctx, int field, void** dptr);
/* Sum of fluid force / torque per body (boundaryhandler.cpp:338-346), float[4*bodies]. */
int sph_body_forces(sph_ctx* ctx, float* force4, float* torque4, int bodies);
/* Rollout statistics of the last step, out[8]: mean max(rho-rho0,0)/rho0, mean
 * |rho-rho0|/rho0, max (rho-rho0)/rho0, kinetic energy, potential energy (m g y), centre
 * of mass x, y, z.  Computed on the device; synchronises. */
int sph_stats(sph_ctx* ctx, double* out8);

/* ---- batched scenes ------------------------------------------------------------------- */

/* One independent scene of a batched context (the reference runs one FluidSimulation per
 * Fluid, scene/fluid.cpp:32; a batch runs many in one launch per stage). */
typedef struct sph_scene_desc {
    float container[3];          /* set_rect_limits of this scene */
    float k_viscosity;           /* per-scene viscosity */
    float gas_stiffness;         /* per-scene Tait stiffness k = rho0 c0^2 / gamma */
    const float* fluid_pos4;     /* n_fluid float4 particles */
    const float* fluid_vel4;     /* initial velocities or NULL */
    int n_fluid;
    const float* boundary_pos4;  /* static boundary particles, world coordinates */
    int n_boundary;
} sph_scene_desc;

/* Creates a context that advances nscenes independent WCSPH scenes (PHYSICS mode) with one
 * launch per stage: every scene keeps its own grid, container, viscosity and stiffness,
 * and its particles stay in one contiguous range of the arrays (the sort key puts the scene
 * id above the Morton bits, which makes the one sort a segmented sort).  The other
 * parameters are shared.  sph_simulate / sph_get_field work as for one scene. */
int sph_batch_create(const sph_params* params, int nscenes, const sph_scene_desc* scenes, sph_ctx** out);
/* Number of scenes (0 for a single-scene context). */
int sph_batch_scene_count(const sph_ctx* ctx);
/* Particle range [first, first + count) of a scene in every fluid field. */
int sph_batch_scene_range(const sph_ctx* ctx, int scene, int* first, int* count);
/* Grid of a scene (Grid::info, grid.h:66-118): origin, cells per axis, offset of its cells
 * in the concatenated cell table. */
int sph_batch_scene_grid(const sph_ctx* ctx, int scene, float* origin3, int* dims3, long long* cell_base);
/* sph_stats for every scene: out8[8 * scene + k]; synchronises. */
int sph_batch_stats(sph_ctx* ctx, double* out8, int nscenes);

/* Threads per block of the step's kernels (a multiple of 32 from 32 to 256), keeping the
 * particle state; the captured step graph is rebuilt on the next sph_simulate.  The launch
 * shape never changes results.  Used by the autotuner (fluids_gb300/autotune.py); the
 * reference fixes its local sizes in the host code (e.g. grid.cpp:53 runs with 32). */
int sph_set_block_size(sph_ctx* ctx, int block_size);

/* Batched contexts (no counterpart in the reference, which steps one scene): the neighbour
 * passes of a batched step (list build + density, normals, forces + integration) run as
 * persistent launches over per-scene tiles -- each scene's particle range cut into tiles of
 * 32 particles, a tile never straddling two scenes -- whose CTAs take the next chunk of
 * tiles (one per warp) from a counter; a warp reads its tile's scene constants once.  The shape of the persistent grid is
 * block_size threads (sph_set_block_size) times SMs x ctas_per_sm CTAs (0 = 2048 /
 * block_size).  The shape never changes results; fluids_gb300/autotune.py picks it.
 * SPH_E_INVALID on a single-scene context. */
int sph_set_tile_shape(sph_ctx* ctx, int ctas_per_sm);
/* The current tile shape: particles per tile, CTAs per SM (0 = automatic), tile count and
 * CTAs of the persistent launches. */
int sph_get_tile_shape(const sph_ctx* ctx, int* tile_particles, int* ctas_per_sm, int* ntiles, int* blocks);

/* ---- differentiable WCSPH (adjoint) ----------------------------------------------------
 * No counterpart in the reference, which has no gradients.  The forward step is the WCSPH
 * step of WCSPHSimulation::simulate (wcsphsimluation.cpp:40-106) in PHYSICS mode; the
 * backward pass runs hand-written adjoint kernels over the same neighbour lists (held fixed
 * per step), recomputing each segment of checkpoint_every steps from its checkpoint.
 * Requirements: a single-scene WCSPH context in PHYSICS mode with fluid particles, no
 * boundary particles and surface_tension = 0 (SPH_E_INVALID otherwise).  The context's
 * grid, container and constants are used; its own particle state is not touched.
 * Particle arrays are float4 (x, y, z, unused) in particle-id order (the order of
 * sph_add_volume), host or device pointers. */
typedef struct sph_adj sph_adj;
int sph_adj_create(sph_ctx* ctx, int steps, int checkpoint_every, sph_adj** out);
/* Frees the handle; valid even after its context was destroyed (no other call is). */
int sph_adj_destroy(sph_adj* adj);
const char* sph_adj_last_error(const sph_adj* adj);
/* Runs `steps` steps from positions x0 and velocities v0 (the half-step velocity starts at
 * v0, as sph_add_volume does) with viscosity mu and Tait stiffness gas_stiffness, keeping a
 * checkpoint every checkpoint_every steps.  Writes the final positions / velocities to
 * xT_4 / vT_4 when they are not NULL.  Synchronises. */
int sph_adj_forward(sph_adj* adj, const float* x0_4, const float* v0_4, float mu, float gas_stiffness,
                    float* xT_4, float* vT_4);
/* Given dL/dx_T (and dL/dv_T, or NULL for zero) of the last forward pass, writes dL/dx0,
 * dL/dv0 (either may be NULL), dL/dmu, dL/dk and dL/dc0 (k = rho0 c0^2 / 7).
 * Deterministic: no atomics in any sum.  Synchronises. */
int sph_adj_backward(sph_adj* adj, const float* gxT_4, const float* gvT_4, float* gx0_4, float* gv0_4,
                     double* g_mu, double* g_stiffness, double* g_c0);
/* SPH_FLAG_* raised since the last forward: OVERFLOW (a list reached the cap, so the lists
 * may not be symmetric), NONSMOOTH (a clamp or reflection was crossed), NAN, ESCAPED. */
int sph_adj_flags(sph_adj* adj, unsigned* flags);
/* Device bytes the adjoint holds (checkpoints, one segment's tape, scratch). */
int sph_adj_tape_bytes(const sph_adj* adj, size_t* bytes);

/* ---- checkpoint / resume -------------------------------------------------------------- */

/* No counterpart in the reference (reset() rebuilds from the scene,
 * pcisphsimluation.cpp:257-266).  Writes what the next step reads: fluid positions,
 * velocities, half-step velocities and particle ids in the context's current order, every
 * body's transform, velocities and dynamics, with the parameters, container and counts, and
 * a checksum.  Synchronises.  Not for batched contexts (SPH_E_STATE). */
int sph_save_state(sph_ctx* ctx, const char* path);
/* Restores a sph_save_state file into a context built from the same scene (same parameters
 * but for block_size / use_graph, container, fluid count, bodies and their particle counts;
 * SPH_E_INVALID otherwise, and for a damaged file).  The steps that follow are bit-identical
 * to the steps that followed the save. */
int sph_load_state(sph_ctx* ctx, const char* path);

/* ---- screen-space surface ------------------------------------------------------------ */

/* The depth, blur, normals and final shading stages of SSpaceFluidRenderer (fluid/render/
 * sspacefluidrenderer.cpp:35-53) as CUDA kernels writing plain device images instead of
 * GL textures: row-major, row 0 at the bottom, width * height floats (depth) or float4
 * (normals, colour).  Reads outside an image clamp to its edge.  All asynchronous. */
typedef struct sph_view {
    float modelview[16];   /* mv_matrix, column-major like a GL uniform */
    float projection[16];  /* pr_matrix (camera.projection()), column-major */
    float point_radius;    /* sprite sphere radius; the renderer uses 0.0625 (:365) */
    float point_scale;     /* viewport width * tan(fov / 2) (:366) */
    int width, height;     /* image size in pixels: each 1..65536, at most 2^28 pixels */
} sph_view;
/* _render_depth_stage (:353-386) with shaders/sspace_fluid_rendering/depth_stage.vert and
 * .frag: every fluid particle of the context is a sphere sprite; d_depth receives at each
 * pixel the NDC depth of the nearest sprite fragment (GL_LESS on the normalised depth, the
 * lower particle index winning a tie) and 0 where no sprite covers it.  No background
 * depth texture: fragments beyond the far plane are dropped.  Runs on the context stream;
 * holds 8 bytes per pixel of scratch in the context. */
int sph_render_depth(sph_ctx* ctx, const sph_view* view, float* d_depth);
/* One pass of kernels/bilateral.cl (BilateralFilter::filter, filters/bilateralfilter.cpp:
 * 28-41): d_in and d_out must differ. */
int sph_filter_bilateral(const float* d_in, float* d_out, int width, int height, void* cuda_stream);
/* _render_blur_stage (:388-407): iterations times bilateral d_depth -> d_tmp -> d_depth. */
int sph_render_smooth(float* d_depth, float* d_tmp, int width, int height, int iterations, void* cuda_stream);
/* One explicit step of kernels/curvatureflow.cl (screen-space mean-curvature flow; the
 * reference ships the kernel without a host caller).  inv_proj_x, inv_proj_y: the inverse
 * projection's x and y scale terms. */
int sph_filter_curvature_flow(const float* d_in, float* d_out, int width, int height, float inv_proj_x,
                              float inv_proj_y, void* cuda_stream);
/* _render_normals_stage (:409-436) with normals_stage.frag: view-space normals (x, y, z, 1)
 * of the depth image, (0, 0, 0, 0) where depth <= 0.  inv_projection: column-major. */
int sph_render_normals(const float* d_depth, float* d_normals4, int width, int height,
                       const float inv_projection[16], void* cuda_stream);
/* _render_final_stage (:438-480) with final_stage.frag: the fluid's colour into d_rgba (float4
 * per pixel, alpha 1).  Inputs: the blurred depth, the normals, a background image (float4
 * per pixel, what the scene rendered behind the fluid; NULL = black) and a cube map for
 * reflections (6 faces of cube_size^2 float4 texels in GL order +x, -x, +y, -y, +z, -z,
 * row 0 at t = 0; NULL = black).  Blinn-Phong specular (exponent 50) for the light direction
 * modelview * (0.7, 1, 0, 0), Schlick Fresnel (r0 = 0.1), reflection from the cube map,
 * refraction of the background offset by 0.01 * normal.xy, attenuation colour
 * (0.2, 0.2, 0.5); background where depth <= 0.  Offset reads are bilinear with clamped
 * coordinates (GL_LINEAR), the cube map read bilinear within the selected face. */
int sph_render_shade(const float* d_depth, const float* d_normals4, const float* d_background4,
                     const float* d_cube4, int cube_size, int width, int height, const float modelview[16],
                     const float inv_projection[16], float* d_rgba, void* cuda_stream);
/* A directional light of the scene file ("lights", scene/scene.cpp:340-364): direction and
 * diffuse colour (r, g, b, a in 0..1, i.e. the file's 0..255 values / 255). */
typedef struct sph_light {
    float direction[3];
    float diffuse[4];
} sph_light;
/* ParticlesRenderer (fluid/render/particlesrenderer.cpp:40-88, shaders/particles.vert/.frag):
 * the context's particles as sphere sprites, each depth-tested at its centre's window depth
 * (the fragment shader writes none; the lower index wins a tie), lit by up to 8 directional
 * lights: (0, 0, 0, 1) + sum of diffuse * (89, 152, 255, 256) / 256 * max(0, n . -dir),
 * n from the point coordinate; clamped to [0, 1] as a fixed-point framebuffer stores it;
 * (0, 0, 0, 1) where no sprite is.  Into d_rgba (float4 per pixel), on the context stream. */
int sph_render_particles(sph_ctx* ctx, const sph_view* view, const sph_light* lights, int nlights, float* d_rgba);
/* GraphicsSettings::render_method (settings/settings.cpp:47-57). */
enum sph_render_method { SPH_RENDER_PARTICLES = 0, SPH_RENDER_SCREEN_SPACE = 1 };
/* A headless frame into rgba_host (width * height float4, row 0 at the bottom):
 * SPH_RENDER_SCREEN_SPACE runs SSpaceFluidRenderer::render (:35-53) — depth,
 * filter_iterations blur iterations, normals and the final stage over a black background
 * without a cube map; SPH_RENDER_PARTICLES runs sph_render_particles with the given lights.
 * The device images are the context's (40 bytes per pixel, kept for the next frame); the
 * inverse projection is computed from view->projection.  Synchronous. */
int sph_render_frame(sph_ctx* ctx, const sph_view* view, int method, int filter_iterations, const sph_light* lights,
                     int nlights, float* rgba_host);

/* ---- primitives ---------------------------------------------------------------------- */

/* clsort<cl_uint, cl_int> (opencl/algorithms/clsort.h:13-35): stable ascending sort of n
 * (key, value) pairs in place in device memory, on the low key_bits bits (1..32) of the
 * key.  Scratch memory is allocated on first use and cached per device; calls on different
 * streams are ordered on the GPU one after the other (not while a stream is being captured:
 * captured calls must not overlap another call on the GPU). */
int sph_sort_pairs(uint32_t* d_keys, int32_t* d_vals, int n, int key_bits, void* cuda_stream);

/* The same stable sort for callers that cannot allocate device memory (no counterpart in
 * the reference).  Host programs whose own allocator owns the device heap, or that sort
 * from a callback where an allocation is not allowed, cannot accept the scratch that
 * sph_sort_pairs allocates; this variant allocates nothing.  The caller passes the input
 * pairs (only read) and separate output buffers; everything else lives in one fixed
 * device array of 9,441,792 bytes per GPU, held until the process exits.  At most
 * SPH_NOALLOC_SORT_MAX_PAIRS pairs (SPH_E_OVERFLOW above that, nothing launched).  The
 * first call on a device looks up the array's address, so make it before any stream
 * capture; the address is kept and does not survive cudaDeviceReset (do not call this
 * again on a device that was reset).  All calls on a device share the array: calls that
 * overlap on the GPU race, so serialise them.  No output may overlap an input or the other
 * output (SPH_E_INVALID).  Asynchronous on cuda_stream; its closing cudaGetLastError also
 * returns and clears an error left by earlier work on the calling thread. */
#define SPH_NOALLOC_SORT_MAX_PAIRS 1048576
int sph_sort_pairs_noalloc(const uint32_t* d_keys_in, const int32_t* d_vals_in, uint32_t* d_keys_out,
                           int32_t* d_vals_out, int n, int key_bits, void* cuda_stream);

/* ---- scene builders (host) ------------------------------------------------------------ */

/* BoxVolume::particles (fluid/simulation/boxvolume.cpp:11-40): fills out4 (capacity cap
 * particles, may be NULL to count) and returns the particle count. */
int sph_scene_box_volume(const float size3[3], const float center3[3], float particle_radius,
                         float* out4, int cap);
/* FishTank::surface_sampling (scene/fishtank.cpp:108-141): container base and four walls,
 * open top. */
int sph_scene_fishtank(float width, float height, float depth, float spacing, float* out4, int cap);
/* Cube::surface_sampling (scene/cube.cpp:136-171): hollow cube shell in body coordinates. */
int sph_scene_cube(float side, float spacing, float* out4, int cap);
/* ModelMesh(path) (mesh/modelmesh.cpp:16-88): reads an OBJ file (v / vn / f records,
 * polygons split into triangle fans as tinyobj does) into one vertex per distinct
 * (position, normal) reference and a triangle index list.  Indices keep only their low 16
 * bits, as the reference's unsigned-short mesh_index does.  Writes *nvertices and
 * *nindices always, the arrays when vcap / icap suffice.  SPH_E_INVALID when the file cannot
 * be read or a face references a missing vertex. */
int sph_scene_load_obj(const char* path, float* vertices3, int vcap, uint32_t* indices, int icap, int* nvertices,
                       int* nindices);
/* Model::surface_sampling (scene/model.cpp:170-214) on the GPU: the vendored voxelizer's
 * vx_voxelize (external/voxelizer/voxelizer.h) of the triangle mesh with cubic voxels of
 * voxel_size (the reference passes the particle spacing and precision = spacing / 10);
 * writes the 8 corners of every voxel, in the voxelizer's output order, as float4 (w = 1).
 * Returns the particle count (8 per voxel); writes nothing when out4 is NULL or cap is
 * below the count.  Negative SPH_E_* on error (SPH_E_OVERFLOW: a triangle spans more than
 * 2^24 voxels or the mesh more than 2^30 voxel hits).  Synchronous. */
int sph_scene_voxelize(const float* vertices3, int nvertices, const uint32_t* indices, int nindices,
                       float voxel_size, float precision, float* out4, int cap);
/* IcoSphereMesh(radius, level) (mesh/icospheremesh.cpp:10-124), level 0..4. */
int sph_scene_icosphere(float radius, int level, float* vertices3, int vcap, uint32_t* indices, int icap,
                        int* nvertices, int* nindices);
/* Sphere::surface_sampling (scene/sphere.cpp:135-171) of IcoSphereMesh(radius, 3): random
 * points on each triangle (a default-seeded std::default_random_engine per triangle), then
 * every mesh vertex; the corner reads and the area formula as written there.  Returns the
 * count, fills out4 up to cap. */
int sph_scene_sphere(float radius, float spacing, float* out4, int cap);
/* Wall::surface_sampling (scene/wall.cpp:142-152): a width x height plane at z = 0 in body
 * coordinates.  Returns the count (-1 for bad arguments), fills out4 up to cap. */
int sph_scene_wall(float width, float height, float spacing, float* out4, int cap);
/* Adds U(-amp, amp) to x, y, z of every particle from a splitmix64 stream seeded by seed. */
void sph_jitter(float* pos4, int n, float amp, uint64_t seed);

/* Whether a CUDA device is visible (does not create a context on failure paths). */
int sph_cuda_available(void);

/* Constants a context derives from params and a container (host only, no GPU needed):
 * the kernel constants of wcsphsimluation.cpp:165-202 / pcisphsimluation.cpp:230-278,429-469
 * and the grid of grid.cpp:61-68 (Grid::info, grid.h:66-118). */
typedef struct sph_derived {
    float mass, mass_def, h, h_def, rest_density_def;
    float poly6_eval, poly6_grad, spiky_grad, visc_lapl, st_main, st_term;
    float default_eval, boundary_eval, pci_delta;
    float grid_origin[3];
    int grid_dims[3];
    int grid_wrap;
    int key_bits;
} sph_derived;
int sph_describe(const sph_params* params, const float container3[3], sph_derived* out);

#ifdef __cplusplus
}
#endif
#endif /* SPH_CAPI_H */
