/*
 * sph_oracle.h -- CPU oracle of the SPH particle pipeline (TEST INFRASTRUCTURE).
 *
 * This is the checker, never the product: only tests/, __graft_entry__.smoke() and
 * bench.py's cpu_baseline leg load it.  It restates, function by function, the
 * reference's OpenCL kernels and the host code that derives their constants:
 *
 *   kernels/grid.h:74-108, kernels/morton.h:37-56, kernels/grid.cl:20-182,
 *   kernels/wcsph.cl:32-224, kernels/normals.cl:23-70, kernels/pcisph.cl:33-504,
 *   kernels/boundary.cl:4-118, kernels/surface_tension.h:23-80,
 *   kernels/muller_kernels.h:9-19,
 *   fluid/simulation/wcsphsimluation.cpp:40-106,165-202,
 *   fluid/simulation/pcisphsimluation.cpp:72-165,230-255,268-393,429-476,532-551,
 *   fluid/simulation/boundaryhandler.cpp:119-153,216-349,
 *   fluid/simulation/mullerconstants.cpp:4-38, opencl/clcompiler.cpp:50-54.
 *
 * Pinning: the float/compat instance is checked stage by stage against the
 * reference's own .cl kernels compiled for the CPU through a shim
 * (oracle/ref_shim, built into oracle/_ref by oracle/build_ref.sh), and against
 * golden vectors generated from that build (tests/golden/).
 *
 * Two modes:
 *   COMPAT  follows the kernel text, including its defects.
 *   PHYSICS fixes only the documented defects P1..P7 (listed in sph_oracle.cpp).
 * Two precisions: float (stage parity, CPU baseline) and double (rollout oracle).
 */
#ifndef SPH_ORACLE_H
#define SPH_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct OrcConfig {
    int method;            /* 0 = WCSPH, 1 = PCISPH */
    int mode;              /* 0 = COMPAT (kernel text), 1 = PHYSICS (documented fixes) */
    int precision;         /* 0 = float, 1 = double */
    int neigh_cap;         /* NEIGH_LIST_MAX_LENGTH, kernels/common.h:4 (50) */
    float time_step, max_vel, particle_radius, support_radius;
    int pci_min_iter, pci_max_iter;   /* pcisphsimluation.h:254 (3), settings */
    float pci_error_ratio;
    int pci_relax_max_iter;           /* pcisphsimluation.cpp:549 (10000) */
    float rest_density, k_viscosity, gravity, gas_stiffness, surface_tension;
    float grid_size;       /* COMPAT cube side (wcsphsimluation.cpp:26: 5.0) */
    float grid_margin;     /* PHYSICS: cells of margin around the container */
    float phi_coeff;       /* BoundaryHandler phi coefficient (1.0) */
    float container[3];    /* set_rect_limits(w, h, d) */
    int relax_on_add;      /* PCISPH: relaxation step + v:=0 after set_fluid */
    int threads;           /* OpenMP threads (0 = runtime default) */
    int kernels;           /* 0 = Mueller (USE_MULLER_KERNELS, the reference's build), 1 = Monaghan (COMPAT) */
} OrcConfig;

enum {
    ORC_S_BOUNDARY_SYNC = 0, ORC_S_HASHES = 1, ORC_S_SORT = 2, ORC_S_SHUFFLE = 3,
    ORC_S_CELL_INTERVALS = 4, ORC_S_NEIGH_LIST = 5, ORC_S_SB_NEIGH_LIST = 6,
    ORC_S_WC_DENSITY = 7, ORC_S_NORMALS = 8, ORC_S_WC_ACCEL = 9, ORC_S_WC_INTEGRATE = 10,
    ORC_S_PCI_INIT_DENSITY = 11, ORC_S_PCI_INIT_FORCES = 12, ORC_S_PCI_LOOP = 13,
    ORC_S_PCI_INTEGRATE = 14, ORC_S_BOUNDARY_FORCES = 15,
    ORC_S_PCI_PREDICT = 16, ORC_S_PCI_UPDATE_PRESSURE = 17, ORC_S_PCI_PRESSURE_FORCE = 18
};

enum {
    ORC_F_POS = 0, ORC_F_VEL = 1, ORC_F_VEL_HALF = 2,
    ORC_F_POS_SORTED = 3, ORC_F_VEL_SORTED = 4, ORC_F_VEL_HALF_SORTED = 5,
    ORC_F_HASHES = 6, ORC_F_MASK = 7, ORC_F_CELL_INTERVALS = 8,
    ORC_F_NEIGH_LIST = 9, ORC_F_NEIGH_LEN = 10, ORC_F_SB_NEIGH_LIST = 11, ORC_F_SB_NEIGH_LEN = 12,
    ORC_F_DENSITY = 13, ORC_F_PRESSURE = 14, ORC_F_NORMAL = 15, ORC_F_ACCEL = 16,
    ORC_F_POS_PRED = 17, ORC_F_FORCE_OTHER = 18, ORC_F_FORCE_PRESSURE = 19, ORC_F_DENS_VAR = 20,
    ORC_F_BPOS_SORTED = 21, ORC_F_BPHI_SORTED = 22, ORC_F_BCELL_INTERVALS = 23,
    ORC_F_BHASHES = 24, ORC_F_BMASK = 25, ORC_F_BPHI = 26, ORC_F_BPOS = 27,
    ORC_F_BODY_FORCE = 28, ORC_F_BODY_TORQUE = 29, ORC_F_PCI_ITERS = 30, ORC_F_PCI_MAXERR = 31,
    ORC_F_ID = 32, ORC_F_COUNT = 33
};

/* Derived constants, exported so tests can compare them with the CUDA host code. */
typedef struct OrcDerived {
    float mass, mass_def, h, h_def, rest_density_def;
    float poly6_eval, poly6_grad, spiky_grad, visc_lapl, st_main, st_term;
    float default_eval, boundary_eval, pci_delta;
    float grid_origin[3]; int grid_dims[3]; int grid_wrap; int key_bits;
} OrcDerived;

void* orc_create(const OrcConfig* cfg);
void  orc_destroy(void* o);
int   orc_set_fluid(void* o, const float* pos4, const float* vel4, int n);
/* rot3x4: row-major 3x4 rigid transform (rotation | translation); lin4/ang4 velocities. */
int   orc_add_boundary(void* o, const float* pos4, int n, int can_move,
                       const float* rot3x4, const float* lin4, const float* ang4, float mass);
int   orc_run_stage(void* o, int stage);
int   orc_step(void* o, int nsteps);
long long orc_field_elems(void* o, int field);   /* scalar elements (float4 -> 4 per particle) */
int   orc_field_kind(void* o, int field);         /* 0 real, 1 int32, 2 uint32 */
int   orc_get(void* o, int field, void* out);     /* copies the field in its native type */
int   orc_set(void* o, int field, const void* in);
int   orc_derived(void* o, OrcDerived* out);
/* Standalone primitives used by known-answer tests. */
uint32_t orc_morton3(uint32_t x, uint32_t y, uint32_t z);
void  orc_stable_sort_pairs(uint32_t* keys, int32_t* vals, int n);
/* Rollout statistics of the last completed step, out[8]:
 * [mean max(rho-rho0,0)/rho0, mean |rho-rho0|/rho0, max (rho-rho0)/rho0,
 *  kinetic energy, potential energy (m g y), centre of mass x, y, z]. */
int   orc_stats(void* o, double* out8);
/* rigid-body dynamics of a movable body with mass (integrated in the BOUNDARY_FORCES stage) */
int   orc_set_body_dynamics(void* o, int body, int enabled, const float* inv_inertia3, float radius);
int   orc_body_state(void* o, int body, float* rot12, float* lin4, float* ang4);

#ifdef __cplusplus
}
#endif
#endif
