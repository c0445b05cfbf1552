// Host-side engine state and kernel launch entry points shared by the CUDA translation units.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "tfg.h"
#include "tfg_device.cuh"

namespace tfg {

// Per-particle device state, stored in cell order.  Two copies exist so the counting
// sort can scatter from one into the other.
struct ParticleArrays {
    float4 *pos = nullptr;     // cell-relative x,y,z ; w = type (int bits)
    float4 *vel = nullptr;     // v.x,v.y,v.z ; w = inverse number density
    float4 *aux = nullptr;     // radius, imass, flags (bits), id (bits)
    float4 *fext = nullptr;    // force_i (external) ; w unused
    float4 *pforce = nullptr;  // persistent random force ; w unused
    int32_t *cell = nullptr;   // cell index of each slot
    float *sval = nullptr;     // species values, [s * cap + slot]
    float *sq = nullptr;       // flux increments, [s * cap + slot]
};

// Reduction slots in the device double array.
enum RedSlot : int {
    RED_EPOT_NONBOND = 0,
    RED_EPOT_BOND,
    RED_EPOT_ANGLE,
    RED_KINETIC,
    RED_VIRIAL,
    RED_VOLUME,
    RED_MIGRATIONS,
    RED_SPECIES0,               // kMaxSpecies entries
    RED_COUNT = RED_SPECIES0 + kMaxSpecies,
};

struct PairKernelArgs {
    const SimParams *sims;      // per-simulation parameters (device)
    const int32_t *cell_sim;    // simulation of each global cell (device)
    int nsims;
    int ncells;                 // global cells over all simulations
    int max_type;               // types per simulation (tables are max_type^2 per simulation)
    int nspec;                  // species per particle (all simulations)
    uint32_t flags;             // union of the simulations' TFG_ENGINE_* flags
    int n;
    const float4 *pos;
    const float4 *vel;
    const float4 *aux;
    const float4 *fext;
    const float4 *pforce;
    const int32_t *cell;
    const int32_t *start;       // ncells+1
    const float *sval;
    float *sq;
    int cap;
    float4 *force;              // out: f.xyz, number density
    const PotDev *pots;         // nsims * max_type^2
    const float *blob;
    int blob_floats;
    const PotDev *wpots;        // nsims * 6 * max_type wall potentials
    bool has_wall_pots;         // any simulation has a wall potential
    const FluxSet *fluxes;      // nsims * max_type^2
    const float4 *rforce;       // nsims * max_type: mean, std, duration, enabled
    float4 *pforce_out;         // persistent force updated in place (same as pforce)
    double *red;                // RED_COUNT per simulation
    uint32_t *err;
    int32_t *sig_count;         // signature mode: interacting neighbours per particle
    uint32_t *sig_hash;         // signature mode: order-independent hash of neighbour ids
    int32_t *pair_out;          // signature mode, optional: (lower id, higher id) of each pair found
    unsigned long long *pair_n; // pairs found (the first pair_cap are written)
    long long pair_cap;
    int flux_sub;               // >= 0: flux-only substep pass number (simulations with
                                // nr_fluxsteps - 1 > flux_sub take part); -1: the full pass
    bool has_dpd;               // any type pair uses a DPD potential
    bool has_flux;              // any type pair has fluxes
    // Verlet pair lists (tiled pass, table potentials): per home cell, the staged-index
    // pairs (i | k << 16) within the list radius found at the simulation's last rebuild,
    // one kListEnd marker after each staging chunk, in interleaved groups of 128
    uint32_t *vlist;            // list_k entries per home cell (a multiple of 128)
    int32_t *vlen;              // entries of each home cell's list; -1: none (candidate tests)
    int list_k;
    int *list_need;             // largest list a build asked for (atomicMax)
};

constexpr uint32_t kListEnd = 0xffffffffu;

// Full-stencil kernel: one thread per particle, no atomics.  General path (any number
// of species); force[] must hold the initial force (external + random, density W(0)).
void launch_pair(const PairKernelArgs &a, cudaStream_t s);
// Tiled half-shell kernel (one species at most) plus its overflow pass; force[] must hold
// the initial force, to which both partners' contributions are added atomically.
// `split` = warps per home cell (1, 2, 7 or 14): the cell's 14 tasks are divided into
// that many work items.
// Shared-memory staging of the tiled pass: every potential table and descriptor of the
// arena is staged per CTA when they fit (the usual case for one simulation), else none is
// and they are read through L1.
struct TilePlan {
    int stage_floats = 0;
    int stage_pots = 0;
};
TilePlan plan_pair_tile(int nsims, int max_type, int blob_floats);
// Launch configuration of the nonbonded pass, picked by the autotuner: the work split (warps
// per home cell: 1, 2, 7 or 14, or TFG_PAIR_HOME_OUTER for the home-outer kernel), the
// warps per CTA of the tiled kernel's table variants (8, or 4 with twice the CTAs per SM),
// and the work items a warp takes from the shared counter at a time.
struct TileTune {
    int split = 1;
    int warps = 8;
    int grab = 1;
};
void launch_pair_tile(const PairKernelArgs &a, const TilePlan &plan, int *overflow_list, int *overflow_count, int sms,
                      bool signature, const TileTune &tune, cudaStream_t s);
// Overflow pass of the tiled kernels' table variant: the home cells listed in
// overflow_list[0 .. overflow_count[0]), one warp each, global-memory candidates and atomics.
void launch_pair_overflow(const PairKernelArgs &a, int *overflow_list, int *overflow_count, bool signature, int sms,
                          cudaStream_t s);
// Home-particle-outer pass (split TFG_PAIR_HOME_OUTER): tabulated potentials only, no DPD,
// fluxes or Verlet pair lists.  overflow_count must be zeroed before the launch.
void launch_pair_home(const PairKernelArgs &a, int *overflow_list, int *overflow_count, int sms, bool signature,
                      cudaStream_t s);
inline bool pair_home_eligible(const PairKernelArgs &a) {
    return !a.has_dpd && !(a.nspec > 0 && a.has_flux) && !a.vlist && a.flux_sub < 0;
}
int pair_tile_capacity();
void launch_pair_stencil_fluxonly(const PairKernelArgs &a, cudaStream_t s);
// Flux-only substep pass (a.flux_sub >= 0): species flux increments of the pair set, no
// forces, densities or energies (runner_dopair_fluxonly / runner_doself_fluxonly).
void launch_pair_fluxonly(const PairKernelArgs &a, const TilePlan &plan, int *overflow_list, int *overflow_count,
                          int sms, bool tile, cudaStream_t s);
// Same stencil walk and pair decision as launch_pair, writing only the per-particle
// pair signature (used to prove the pair set bit-exact against the oracle).
void launch_pair_signature(const PairKernelArgs &a, cudaStream_t s);

// Signature mode with an explicit list: append the pair (ida, idb) once.
__device__ __forceinline__ void record_pair(const PairKernelArgs &a, int ida, int idb) {
    if (!a.pair_out) return;
    const unsigned long long p = atomicAdd(a.pair_n, 1ull);
    if ((long long)p < a.pair_cap) {
        a.pair_out[2 * p] = ida < idb ? ida : idb;
        a.pair_out[2 * p + 1] = ida < idb ? idb : ida;
    }
}

// Hash of one neighbour id for the pair signature.
__host__ __device__ inline uint32_t sig_mix(uint32_t id) {
    uint32_t x = id * 2654435761u + 0x9E3779B9u;
    x ^= x >> 15;
    x *= 0x85EBCA6Bu;
    x ^= x >> 13;
    return x;
}

}  // namespace tfg
