/*
 * sph_kernels.cuh -- host-side launchers of the SPH kernels (one per reference launch point).
 */
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "sph_device.cuh"

namespace sph {

/* Device buffers of one context, passed to the launchers. */
struct Bufs {
    /* fluid */
    float4 *pos, *vel, *vhalf;             /* state between steps */
    float4 *pos_s, *vel_s, *vhalf_s;       /* this step's sorted copies */
    float4 *normal, *accel, *pos_pred, *f_other, *f_press;
    float *density, *pressure, *dens_var;
    float* pci_c;                          /* PCISPH loop: p / rho^2 of each particle this iteration */
    float4* pci_pc;                        /* PCISPH loop: (x, y, z, p / rho^2), the force phase's neighbour record */
    float4* aux;                           /* per particle (p/rho^2, 1/rho, rho, p) */
    float4* nrec;                          /* 2 per particle: (v, p/rho^2), (normal, 1/rho) for the force pass */
    float4* prho;                          /* per particle (x, y, z, rho), written by the list + density pass of
                                              the step for the normal pass (one load per neighbour) */
    uint32_t *keys, *keys_alt;
    int32_t *mask, *mask_alt;
    uint32_t* keys_sorted;                 /* where the sort left the keys */
    int32_t* mask_sorted;
    int32_t *ids, *ids_s;
    int2* tab;                             /* fluid cell table */
    int32_t* cell_prev;                    /* cell id of each sorted particle (sparse clear) */
    int32_t* noff;                         /* 27 linear neighbour-cell offsets (single-scene grid) */
    int32_t *nlist, *nlen, *sblist, *sblen;
    void* sort_ws;
    void* inc_ws;                          /* the incremental sort's workspace (holds the last result) */
    /* boundary */
    float4 *braw, *bpos, *bvel, *bpos_s;
    float *bphi, *bphi_s;
    int32_t *bbody, *bbody_s;
    uint32_t *bkeys, *bkeys_alt;
    int32_t *bmask, *bmask_alt;
    uint32_t* bkeys_sorted;
    int32_t* bmask_sorted;
    int2* btab;
    int32_t* bcell_prev;
    uint8_t* bnear;                        /* per cell: 1 when a boundary particle is binned within one cell */
    void* bsort_ws;
    /* per-body data (device) */
    float* body_xf;                        /* 20 floats per body: rot3x4, lin4, ang4 */
    int32_t* body_range;                   /* origin, count, can_move, has_mass per body */
    float4 *body_force, *body_torque;
    float4* bft;                           /* 2 per boundary particle: its fluid force and torque */
    float* body_dyn;                       /* 8 floats per body: dynamic, mass, inv inertia xyz, radius */
    /* batched contexts: scene table and the scene of each fluid particle (ranges never move) */
    const SceneDev* scenes;
    const int32_t* scene_of;
    const SceneTile* tiles;                /* batched: per-scene tiles of 32 particles (Const::ntiles) */
    unsigned* tile_next;                   /* batched: the tile counters of the four tiled passes */
    /* status */
    unsigned* flags;
    int32_t* pci_iters;
    float* pci_maxerr;
    unsigned* barrier;
    double* stats;
};

/* sph_sort.cu */
int sort_passes(int key_bits);
size_t sort_workspace_bytes(int n, int key_bits);
void sort_pairs(cudaStream_t s, uint32_t* k0, int32_t* v0, uint32_t* k1, int32_t* v1, int n, int key_bits,
                void* ws, unsigned* flags, int num_sms, uint32_t** kres, int32_t** vres);
/* The stable sort of keys[0, n) (values: the indices) into kout / vout, computed as an update
 * of the previous call's result kept in inc_ws (bytes: sort_inc_workspace_bytes(n), zeroed
 * once before the first call; sort_ws: sort_workspace_bytes(n, key_bits)).  Same result as
 * sort_pairs over (keys, identity) for every input.  side / fork / join (all or none): a
 * second stream and two events on which the gated full sort runs beside the merge. */
size_t sort_inc_workspace_bytes(int n);
/* The incremental sort's first pass fused into the step's hash kernel: the sort then starts
 * with sort_inc_begin (before the hash kernel) and skips that pass (flags_done). */
constexpr int kIncItems = 8;
constexpr int kIncTile = 256 * kIncItems;
struct IncFlags {
    const unsigned* valid;
    const uint32_t* prev;
    uint32_t* bits;
    uint32_t* tcnt;
    unsigned* over;
    int2* list;
    uint32_t* lcount;
};
IncFlags sort_inc_flags_args(void* inc_ws, int n);
void sort_inc_begin(cudaStream_t s, void* inc_ws, int n);
void sort_pairs_incremental(cudaStream_t s, const uint32_t* keys, int n, int key_bits, uint32_t* kout,
                            int32_t* vout, void* inc_ws, void* sort_ws, unsigned* flags, int num_sms,
                            cudaStream_t side = nullptr, cudaEvent_t fork = nullptr, cudaEvent_t join = nullptr,
                            bool flags_done = false);

/* sph_grid.cu */
/* scenes: the context's scene table (never null); scene_of: scene of each particle, or
 * null for a single-scene context. */
void launch_hashes(cudaStream_t s, const Const& c, const float4* pos, int n, uint32_t* keys, int32_t* mask,
                   int2* tab, const int32_t* cell_prev, unsigned* flags, int bs, const SceneDev* scenes,
                   const int32_t* scene_of);
void launch_hashes_flags(cudaStream_t s, const Const& c, const float4* pos, int n, uint32_t* keys, int2* tab,
                         const int32_t* cell_prev, unsigned* flags, const SceneDev* scenes, const int32_t* scene_of,
                         const IncFlags& inc);
void launch_gather_ranges(cudaStream_t s, const Const& c, int n, const int32_t* perm, const float4* a, float4* as,
                          const float4* b, float4* bs_, const float4* c3, float4* cs, const int32_t* ids,
                          int32_t* ids_s, const uint32_t* keys, int2* tab, int32_t* cell_out, unsigned* flags, int bs,
                          const SceneDev* scenes, const int32_t* scene_of);
void launch_gather(cudaStream_t s, int n, const int32_t* perm, const float4* a, float4* as, const float4* b,
                   float4* bs_, const float4* c3, float4* cs, const int32_t* ids, int32_t* ids_s, int bs);
void launch_gather_boundary(cudaStream_t s, int n, const int32_t* perm, const float4* pos, float4* pos_s,
                            const int32_t* body, int32_t* body_s, const float* phi, float* phi_s, int bs);
void launch_cell_ranges(cudaStream_t s, const Const& c, const float4* spos, const uint32_t* keys, int n,
                        int2* tab, int32_t* cell_out, unsigned* flags, int bs, const SceneDev* scenes,
                        const int32_t* scene_of);
void launch_neigh_lists(cudaStream_t s, const Const& c, const float4* spos, const int2* tab, const float4* bpos_s,
                        const int2* btab, int* nlist, int* nlen, int* sblist, int* sblen, int bs,
                        const SceneDev* scenes, const int32_t* scene_of, const uint8_t* bnear,
                        const int32_t* noff = nullptr);

/* sph_wcsph.cu */
void launch_wc_density(cudaStream_t s, const Const& c, const Bufs& b, bool lists, int bs);
/* pack: also write nrec (the force pass then reads 2 adjacent float4 per neighbour instead of
 * velocity, aux and normal); only the fused step uses it */
/* prho: the step's list + density pass wrote b.prho, which the walk then reads for both the
 * neighbour's position and its density */
void launch_normals(cudaStream_t s, const Const& c, const Bufs& b, bool lists, int bs, bool pack = false,
                    bool prho = false);
void launch_wc_forces(cudaStream_t s, const Const& c, const Bufs& b, bool lists, bool fuse_integrate,
                      bool write_acc, int bs, bool pack = false);
void launch_wc_integrate(cudaStream_t s, const Const& c, const Bufs& b, int bs);
void launch_aux(cudaStream_t s, const Const& c, const Bufs& b, int bs);
/* PHYSICS PCISPH: the neighbour lists and compute_initial_density in one pass */
void launch_lists_density_pci(cudaStream_t s, const Const& c, const Bufs& b, int bs);
void launch_lists_density(cudaStream_t s, const Const& c, const Bufs& b, int bs);
/* the list builder writing rows, entries and densities in id order (remap = sorted -> id) */
void launch_lists_density_remap(cudaStream_t s, const Const& c, const Bufs& b, const int32_t* remap, int bs);

/* sph_pcisph.cu */
void launch_pci_init_density(cudaStream_t s, const Const& c, const Bufs& b, int bs);
void launch_pci_init_forces(cudaStream_t s, const Const& c, const Bufs& b, int bs, bool pack = false);
int pci_loop_blocks(int num_sms, int bs);
cudaError_t launch_pci_loop(cudaStream_t s, const Const& c, const Bufs& b, int min_iter, int max_iter, int blocks,
                            int bs, bool fuse_integrate);
void launch_pci_integrate(cudaStream_t s, const Const& c, const Bufs& b, int bs);
void launch_pci_predict(cudaStream_t s, const Const& c, const Bufs& b, int bs);
void launch_pci_update_pressure(cudaStream_t s, const Const& c, const Bufs& b, int bs);
void launch_pci_pressure_force(cudaStream_t s, const Const& c, const Bufs& b, int bs);

/* sph_boundary.cu */
void launch_bnd_transform(cudaStream_t s, const Bufs& b, int nbodies, int nb, bool compat, bool only_movable,
                          int bs);
void launch_bnd_phi(cudaStream_t s, const Const& c, const Bufs& b, float phi_coeff, int bs);
/* marks bnear for the 27 cells around every sorted boundary particle (after clearing it) */
void launch_bnd_near(cudaStream_t s, const Const& c, const Bufs& b, int nb, int bs);
void launch_bnd_forces(cudaStream_t s, const Const& c, const Bufs& b, int nbodies, int bs);
/* advances every dynamic body by one step under the fluid force and torque and gravity */
void launch_body_integrate(cudaStream_t s, const Const& c, const Bufs& b, int nbodies);
void launch_stats(cudaStream_t s, const Const& c, const Bufs& b);
void launch_scene_stats(cudaStream_t s, const Const& c, const Bufs& b, double* out, int nscenes);

}  // namespace sph
