// Launch entry points of the non-pair kernels (tfg_kernels.cu).
#pragma once

#include "tfg_internal.h"

namespace tfg {

constexpr int kThreads = 256;

// One re-binning of the whole arena: optional shuffle re-check, counting sort by global
// cell (ranked by particle id inside a cell), scatter from `src` into `dst`, and the
// force initialisation of the coming pair pass.
struct BinArgs {
    int n, cap, ncells, nspec, shuffle;
    const SimParams *sims;
    const int32_t *cell_sim;
    ParticleArrays src, dst;
    int32_t *count, *start, *lidx, *tmp_id, *tmp_src, *dest, *scan_sums, *slot_of_id;
    const float4 *rforce;
    float4 *force;
    float4 *oldx;   // Verlet reference positions by slot (written on rebuild steps), or null
};

void launch_tick(int nsims, SimParams *sims, double *red, cudaStream_t s);
// One thread writes the GPU global timer (ns) into t[k]: phase boundaries of a step, valid
// inside captured graphs (event timing is not).
void launch_stamp(unsigned long long *t, int k, cudaStream_t s);
void launch_setpartp(int n, const float *xg, const SimParams &P, float3 lo, float3 hi, float3 org, float3 ih,
                     int slot0, int32_t *cell, float4 *pos, float4 *aux, const int32_t *type, uint32_t *err,
                     cudaStream_t s);
void launch_relocate(int n, int src0, int dst0, int cap_src, int cap_dst, int nspec, int did, int dcell,
                     const ParticleArrays &src, const ParticleArrays &dst, cudaStream_t s);
void launch_bin(const BinArgs &b, cudaStream_t s);
void launch_bonds(int nb, const SimParams *sims, const int32_t *cell_sim, const int2 *bonds, const int32_t *bslot,
                  const PotDev *bpots, const float *bblob, const int32_t *slot_of_id, const float4 *pos,
                  const float4 *aux, const int32_t *cell, float4 *force, double *red, cudaStream_t s);
void launch_angles(int na, const SimParams *sims, const int32_t *cell_sim, const int4 *angles, const PotDev *bpots,
                   const float *bblob, const int32_t *slot_of_id, const float4 *pos, const int32_t *cell,
                   float4 *force, double *red, cudaStream_t s);
void launch_advance(int n, int cap, int nspec, SimParams *sims, const int32_t *cell_sim,
                    const ParticleArrays &A, const float4 *force, const float *type_mass, const int32_t *type_dyn,
                    const uint32_t *species_flags, const float4 *oldx, double *red, uint32_t *err, cudaStream_t s);
// Fluxes_integrate of flux substep `sub` over every particle of the simulations that have
// that substep (tf_engine_advance.cpp:314-323, tfFlux.cpp:175-202).
void launch_flux_integrate(int n, int cap, int nspec, int sub, const SimParams *sims, const int32_t *cell_sim,
                           const int32_t *cell, float *sval, float *sq, const uint32_t *species_flags,
                           cudaStream_t s);
void launch_gather(int n, int slot0, int cap, int nspec, const SimParams &P, const ParticleArrays &A,
                   const float4 *force, float *x, float *xrel, int32_t *cell, float *v, float *f, float *dens,
                   float *species, float *q, cudaStream_t s);

}  // namespace tfg
