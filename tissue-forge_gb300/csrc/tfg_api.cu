// The C ABI of libtfg.  An engine is a device arena of simulations; the single-simulation
// calls (tfg_set_potential, tfg_load_particles, ...) act on simulation 0 of an engine made
// by tfg_engine_create, and the tfg_batch_* calls name the simulation explicitly.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>

#include "tfg_engine_impl.h"

using namespace tfg;

namespace {

#define CKE(call)                                                                             \
    do {                                                                                      \
        cudaError_t _e = (call);                                                              \
        if (_e != cudaSuccess)                                                                \
            return fail(eng, TFG_E_CUDA, std::string(#call ": ") + cudaGetErrorString(_e));   \
    } while (0)

int make_engine(int device, int max_type, int nspec, tfg_engine **out) {
    if (!out) return TFG_E_INVAL;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return TFG_E_NODEVICE;
    if (device < 0 || device >= ndev || max_type < 1 || max_type > kMaxTypes || nspec < 0 || nspec > kMaxSpecies)
        return TFG_E_INVAL;
    if (cudaSetDevice(device) != cudaSuccess) return TFG_E_CUDA;
    tfg_engine *eng = new (std::nothrow) tfg_engine();
    if (!eng) return TFG_E_OOM;
    eng->device = device;
    eng->max_type = max_type;
    eng->nspec = nspec;
    cudaDeviceGetAttribute(&eng->sms, cudaDevAttrMultiProcessorCount, device);
    if (cudaStreamCreateWithFlags(&eng->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete eng;
        return TFG_E_CUDA;
    }
    eng->own_stream = true;
    for (int k = 0; k < 5; k++) cudaEventCreate(&eng->ev[k]);
    eng->h_bpots.assign(kMaxBondSlots, PotDev{});
    for (auto &p : eng->h_bpots) std::memset(&p, 0, sizeof(p));
    eng->h_btables.assign(kMaxBondSlots, std::vector<float>());
    int rc;
    if ((rc = dalloc(eng, &eng->err, 2)) || (rc = dalloc(eng, &eng->overflow_count, 2)) ||
        (rc = dalloc(eng, &eng->bpots, kMaxBondSlots)) || (rc = dalloc(eng, &eng->stamps, 5))) {
        destroy(eng);
        return rc;
    }
    eng->err_slots = 1;
    cudaMemset(eng->err, 0, 2 * sizeof(uint32_t));
    cudaMemset(eng->overflow_count, 0, 2 * sizeof(int));
    cudaMemset(eng->stamps, 0, sizeof(unsigned long long) * 5);
    if (cudaDeviceSynchronize() != cudaSuccess) {
        destroy(eng);
        return TFG_E_CUDA;
    }
    *out = eng;
    return TFG_OK;
}

int set_type(tfg_engine *eng, int sim, int type, int dynamics, float mass) {
    int rc = sim_check(eng, sim);
    if (rc) return rc;
    if (type < 0 || type >= eng->max_type) return fail(eng, TFG_E_INVAL, "type out of range");
    if (dynamics != TFG_NEWTONIAN && dynamics != TFG_OVERDAMPED) return fail(eng, TFG_E_INVAL, "bad dynamics");
    eng->sims[sim].dyn[type] = dynamics;
    eng->sims[sim].mass[type] = mass;
    eng->tables_dirty = true;
    return TFG_OK;
}

int set_potential(tfg_engine *eng, int sim, int ti, int tj, const tfg_potential *p) {
    int rc = sim_check(eng, sim);
    if (rc) return rc;
    const int T = eng->max_type;
    if (ti < 0 || tj < 0 || ti >= T || tj >= T) return fail(eng, TFG_E_INVAL, "type out of range");
    SimHost &S = eng->sims[sim];
    for (int pass = 0; pass < 2; pass++) {
        const int k = pass == 0 ? ti * T + tj : tj * T + ti;
        if (!p) {
            std::memset(&S.pots[k], 0, sizeof(PotDev));
            S.tables[k].clear();
            continue;
        }
        if (p->kind == TFG_POTENTIAL_KIND_POTENTIAL) {
            if (!p->c || p->n < 1 || p->n > TFG_POTENTIAL_IVALSMAX) return fail(eng, TFG_E_INVAL, "bad table");
            S.tables[k].assign(p->c, p->c + (size_t)(p->n + 1) * kChunk);
        } else if (p->kind != TFG_POTENTIAL_KIND_DPD) {
            return fail(eng, TFG_E_INVAL, "unsupported potential kind");
        }
        S.pots[k] = to_dev(p);
    }
    eng->tables_dirty = true;
    return TFG_OK;
}

int add_flux(tfg_engine *eng, int sim, int ti, int tj, const tfg_flux *f) {
    int rc = sim_check(eng, sim);
    if (rc) return rc;
    if (!f) return TFG_E_INVAL;
    const int T = eng->max_type;
    if (ti < 0 || tj < 0 || ti >= T || tj >= T) return fail(eng, TFG_E_INVAL, "type out of range");
    if (f->index_a < 0 || f->index_a >= eng->nspec || f->index_b < 0 || f->index_b >= eng->nspec)
        return fail(eng, TFG_E_INVAL, "species index out of range");
    SimHost &S = eng->sims[sim];
    FluxSet &fs = S.fluxes[ti * T + tj];
    // Fluxes::addFlux accepts at most fluxes_size*TF_SIMD_SIZE - 1 entries (tfFlux.cpp:216).
    if (fs.count + 1 >= kMaxFluxPerPair) return fail(eng, TFG_E_OVERFLOW, "too many fluxes for this type pair");
    FluxDev &F = fs.f[fs.count++];
    F.kind = f->kind;
    F.type_a = f->type_a;
    F.type_b = f->type_b;
    F.index_a = f->index_a;
    F.index_b = f->index_b;
    F.coef = f->coef;
    F.half_decay = f->decay / 2.f;
    F.target = f->target;
    F.cutoff = f->cutoff > 0 ? f->cutoff : S.P.cutoff;
    if (ti != tj) S.fluxes[tj * T + ti] = fs;
    eng->tables_dirty = true;
    return TFG_OK;
}

int set_species_flags(tfg_engine *eng, int sim, int nr, const uint32_t *flags) {
    int rc = sim_check(eng, sim);
    if (rc) return rc;
    if (nr < 0 || nr > kMaxSpecies || (nr && !flags)) return TFG_E_INVAL;
    for (int s = 0; s < nr; s++) eng->sims[sim].species_flags[s] = flags[s];
    eng->tables_dirty = true;
    return TFG_OK;
}

int set_species_reset(tfg_engine *eng, int sim, int nr, const float *values) {
    int rc = sim_check(eng, sim);
    if (rc) return rc;
    if (nr < 0 || nr > kMaxSpecies || (nr && !values)) return TFG_E_INVAL;
    for (int s = 0; s < nr; s++) eng->sims[sim].P.species_reset[s] = values[s];
    eng->layout_dirty = true;   // parameters are uploaded with the layout
    return TFG_OK;
}

int set_random_force(tfg_engine *eng, int sim, int type, float mean, float std_, int duration_steps) {
    int rc = sim_check(eng, sim);
    if (rc) return rc;
    if (type < 0 || type >= eng->max_type || duration_steps < 1) return TFG_E_INVAL;
    eng->sims[sim].rforce[type] = make_float4(mean, std_, (float)duration_steps, std_ > 0.f ? 1.f : 0.f);
    eng->tables_dirty = true;
    return TFG_OK;
}

int load_bonds(tfg_engine *eng, int sim, int n, const int32_t *i, const int32_t *j, const int32_t *slot) {
    int rc = sim_check(eng, sim);
    if (rc) return rc;
    if (n < 0 || (n > 0 && (!i || !j))) return TFG_E_INVAL;
    SimHost &S = eng->sims[sim];
    std::vector<int2> b(n);
    std::vector<int32_t> sl(n, 0);
    for (int k = 0; k < n; k++) {
        if (i[k] < 0 || j[k] < 0 || i[k] >= S.n || j[k] >= S.n) return fail(eng, TFG_E_INVAL, "bond id out of range");
        b[k] = make_int2(i[k], j[k]);
        if (slot) {
            if (slot[k] < 0 || slot[k] >= kMaxBondSlots) return fail(eng, TFG_E_INVAL, "bond slot out of range");
            sl[k] = slot[k];
        }
    }
    S.bonds = std::move(b);
    S.bond_slot = std::move(sl);
    eng->layout_dirty = true;
    return TFG_OK;
}

int load_angles(tfg_engine *eng, int sim, int n, const int32_t *i, const int32_t *j, const int32_t *k,
                const int32_t *slot) {
    int rc = sim_check(eng, sim);
    if (rc) return rc;
    if (n < 0 || (n > 0 && (!i || !j || !k))) return TFG_E_INVAL;
    SimHost &S = eng->sims[sim];
    std::vector<int4> a(n);
    for (int q = 0; q < n; q++) {
        if (i[q] < 0 || j[q] < 0 || k[q] < 0 || i[q] >= S.n || j[q] >= S.n || k[q] >= S.n)
            return fail(eng, TFG_E_INVAL, "angle id out of range");
        const int sl = slot ? slot[q] : 0;
        if (sl < 0 || sl >= kMaxBondSlots) return fail(eng, TFG_E_INVAL, "angle slot out of range");
        a[q] = make_int4(i[q], j[q], k[q], sl);
    }
    S.angles = std::move(a);
    eng->layout_dirty = true;
    return TFG_OK;
}

bool any_particles(const tfg_engine *eng) {
    for (const auto &S : eng->sims)
        if (S.live && S.loaded) return true;
    return false;
}

}  // namespace

extern "C" {

TFG_API const char *tfg_build_info(void) {
    return "libtfg: GB300 (sm_103a) engine for Tissue Forge's per-step particle path";
}

TFG_API const char *tfg_last_error(const tfg_engine *eng) { return eng ? eng->last_error.c_str() : "null engine"; }

TFG_API int tfg_engine_create(const tfg_engine_desc *d, tfg_engine **out) {
    if (!d || !out) return TFG_E_INVAL;
    tfg_engine *eng = nullptr;
    int rc = make_engine(d->device, d->max_type, d->nr_species, &eng);
    if (rc) return rc;
    eng->capacity_hint = std::max(0, d->capacity);
    int sim = 0;
    rc = add_sim(eng, d, &sim);
    if (rc) {
        destroy(eng);
        return rc;
    }
    *out = eng;
    return TFG_OK;
}

TFG_API int tfg_batch_create(int device, int max_type, int nr_species, tfg_engine **out) {
    return make_engine(device, max_type, nr_species, out);
}

TFG_API int tfg_batch_add_sim(tfg_engine *eng, const tfg_engine_desc *desc, int *sim) {
    if (!eng) return TFG_E_INVAL;
    return add_sim(eng, desc, sim);
}

TFG_API int tfg_batch_remove_sim(tfg_engine *eng, int sim) {
    int rc = sim_check(eng, sim);
    if (rc) return rc;
    SimHost &S = eng->sims[sim];
    S.live = false;
    S.x.clear(); S.xrel.clear(); S.cell.clear(); S.v.clear(); S.radius.clear(); S.imass.clear();
    S.species.clear(); S.force_i.clear(); S.type.clear(); S.flags.clear(); S.bonds.clear(); S.angles.clear();
    S.bond_slot.clear(); S.tables.clear(); S.pots.clear(); S.fluxes.clear();
    S.n = 0;
    eng->layout_dirty = true;
    return TFG_OK;
}

TFG_API int tfg_batch_sim_count(const tfg_engine *eng, int *live) {
    if (!eng || !live) return TFG_E_INVAL;
    int c = 0;
    for (const auto &S : eng->sims) c += S.live ? 1 : 0;
    *live = c;
    return TFG_OK;
}

TFG_API int tfg_engine_destroy(tfg_engine *eng) {
    if (!eng) return TFG_E_INVAL;
    destroy(eng);
    return TFG_OK;
}

TFG_API int tfg_engine_set_stream(tfg_engine *eng, void *stream) {
    if (!eng) return TFG_E_INVAL;
    cudaStreamSynchronize(eng->stream);
    if (stream) {
        if (eng->own_stream) cudaStreamDestroy(eng->stream);
        eng->stream = (cudaStream_t)stream;
        eng->own_stream = false;
    } else if (!eng->own_stream) {
        cudaStreamCreateWithFlags(&eng->stream, cudaStreamNonBlocking);
        eng->own_stream = true;
    }
    eng->gen++;
    return TFG_OK;
}

TFG_API int tfg_set_type(tfg_engine *eng, int type, int dynamics, float mass) {
    return set_type(eng, 0, type, dynamics, mass);
}
TFG_API int tfg_batch_set_type(tfg_engine *eng, int sim, int type, int dynamics, float mass) {
    return set_type(eng, sim, type, dynamics, mass);
}
TFG_API int tfg_set_potential(tfg_engine *eng, int ti, int tj, const tfg_potential *p) {
    return set_potential(eng, 0, ti, tj, p);
}
TFG_API int tfg_batch_set_potential(tfg_engine *eng, int sim, int ti, int tj, const tfg_potential *p) {
    return set_potential(eng, sim, ti, tj, p);
}
TFG_API int tfg_add_flux(tfg_engine *eng, int ti, int tj, const tfg_flux *f) { return add_flux(eng, 0, ti, tj, f); }
TFG_API int tfg_batch_add_flux(tfg_engine *eng, int sim, int ti, int tj, const tfg_flux *f) {
    return add_flux(eng, sim, ti, tj, f);
}
TFG_API int tfg_set_species_flags(tfg_engine *eng, int nr, const uint32_t *flags) {
    return set_species_flags(eng, 0, nr, flags);
}
TFG_API int tfg_batch_set_species_flags(tfg_engine *eng, int sim, int nr, const uint32_t *flags) {
    return set_species_flags(eng, sim, nr, flags);
}
TFG_API int tfg_set_species_reset(tfg_engine *eng, int nr, const float *values) {
    return set_species_reset(eng, 0, nr, values);
}
TFG_API int tfg_batch_set_species_reset(tfg_engine *eng, int sim, int nr, const float *values) {
    return set_species_reset(eng, sim, nr, values);
}
TFG_API int tfg_set_stop(tfg_engine *eng, int64_t step) { return set_stop_sim(eng, 0, step); }
TFG_API int tfg_batch_set_stop(tfg_engine *eng, int sim, int64_t step) { return set_stop_sim(eng, sim, step); }
TFG_API int tfg_set_random_force(tfg_engine *eng, int type, float mean, float std_, int duration_steps) {
    return set_random_force(eng, 0, type, mean, std_, duration_steps);
}
TFG_API int tfg_batch_set_random_force(tfg_engine *eng, int sim, int type, float mean, float std_,
                                       int duration_steps) {
    return set_random_force(eng, sim, type, mean, std_, duration_steps);
}

TFG_API int tfg_load_particles(tfg_engine *eng, int n, const float *x, const float *v, const int32_t *type,
                               const float *radius, const float *imass, const uint32_t *flags, const float *species,
                               const float *force_i) {
    if (!x && n > 0) return TFG_E_INVAL;
    return load_sim(eng, 0, n, x, nullptr, nullptr, v, type, radius, imass, flags, species, force_i);
}
TFG_API int tfg_batch_load_particles(tfg_engine *eng, int sim, int n, const float *x, const float *v,
                                     const int32_t *type, const float *radius, const float *imass,
                                     const uint32_t *flags, const float *species, const float *force_i) {
    if (!x && n > 0) return TFG_E_INVAL;
    return load_sim(eng, sim, n, x, nullptr, nullptr, v, type, radius, imass, flags, species, force_i);
}
TFG_API int tfg_load_particles_binned(tfg_engine *eng, int n, const int32_t *cell, const float *xrel, const float *v,
                                      const int32_t *type, const float *radius, const float *imass,
                                      const uint32_t *flags, const float *species, const float *force_i) {
    if ((!cell || !xrel) && n > 0) return TFG_E_INVAL;
    return load_sim(eng, 0, n, nullptr, cell, xrel, v, type, radius, imass, flags, species, force_i);
}
TFG_API int tfg_batch_load_particles_binned(tfg_engine *eng, int sim, int n, const int32_t *cell, const float *xrel,
                                            const float *v, const int32_t *type, const float *radius,
                                            const float *imass, const uint32_t *flags, const float *species,
                                            const float *force_i) {
    if ((!cell || !xrel) && n > 0) return TFG_E_INVAL;
    return load_sim(eng, sim, n, nullptr, cell, xrel, v, type, radius, imass, flags, species, force_i);
}

TFG_API int tfg_set_bonded_potential(tfg_engine *eng, int slot, const tfg_potential *p) {
    if (!eng || slot < 0 || slot >= kMaxBondSlots || !p) return TFG_E_INVAL;
    if (p->kind != TFG_POTENTIAL_KIND_POTENTIAL || !p->c || p->n < 1)
        return fail(eng, TFG_E_INVAL, "bonded potentials must be tables");
    eng->h_btables[slot].assign(p->c, p->c + (size_t)(p->n + 1) * kChunk);
    eng->h_bpots[slot] = to_dev(p);
    eng->tables_dirty = true;
    return TFG_OK;
}
TFG_API int tfg_load_bonds(tfg_engine *eng, int n, const int32_t *i, const int32_t *j, const int32_t *slot) {
    return load_bonds(eng, 0, n, i, j, slot);
}
TFG_API int tfg_batch_load_bonds(tfg_engine *eng, int sim, int n, const int32_t *i, const int32_t *j,
                                 const int32_t *slot) {
    return load_bonds(eng, sim, n, i, j, slot);
}
TFG_API int tfg_load_angles(tfg_engine *eng, int n, const int32_t *i, const int32_t *j, const int32_t *k,
                            const int32_t *slot) {
    return load_angles(eng, 0, n, i, j, k, slot);
}
TFG_API int tfg_batch_load_angles(tfg_engine *eng, int sim, int n, const int32_t *i, const int32_t *j,
                                  const int32_t *k, const int32_t *slot) {
    return load_angles(eng, sim, n, i, j, k, slot);
}

TFG_API int tfg_autotune(tfg_engine *eng, int *split) {
    if (!eng) return TFG_E_INVAL;
    if (!any_particles(eng)) return fail(eng, TFG_E_STATE, "no particles loaded");
    int rc = commit(eng);
    if (rc) return rc;
    rc = autotune(eng);
    if (split) *split = eng->split;
    return rc;
}

TFG_API int tfg_set_split(tfg_engine *eng, int split) {
    if (!eng || !(split == 1 || split == 2 || split == 7 || split == 14 || split == TFG_PAIR_HOME_OUTER))
        return TFG_E_INVAL;
    eng->split = split;
    eng->tune_auto = false;
    eng->gen++;
    return TFG_OK;
}

TFG_API int tfg_step(tfg_engine *eng, int nsteps) {
    if (!eng || nsteps < 0) return TFG_E_INVAL;
    if (!any_particles(eng)) return fail(eng, TFG_E_STATE, "no particles loaded");
    int rc = commit(eng);
    if (rc) return rc;
    if ((rc = tune_if_needed(eng))) return rc;
    return run_steps(eng, nsteps);
}

TFG_API int tfg_set_graphs(tfg_engine *eng, int enable) {
    if (!eng) return TFG_E_INVAL;
    eng->use_graphs = enable != 0;
    return TFG_OK;
}

TFG_API int tfg_query(tfg_engine *eng, int *idle) {
    if (!eng || !idle) return TFG_E_INVAL;
    cudaError_t e = cudaStreamQuery(eng->stream);
    if (e == cudaErrorNotReady) {
        *idle = 0;
        return TFG_OK;
    }
    if (e != cudaSuccess) return fail(eng, TFG_E_CUDA, cudaGetErrorString(e));
    *idle = 1;
    return TFG_OK;
}

TFG_API int tfg_batch_step(tfg_engine *eng, int nsteps) { return tfg_step(eng, nsteps); }

TFG_API int tfg_force_only(tfg_engine *eng, int with_bonded) {
    if (!eng) return TFG_E_INVAL;
    if (!any_particles(eng)) return fail(eng, TFG_E_STATE, "no particles loaded");
    int rc = commit(eng);
    if (rc) return rc;
    if ((rc = tune_if_needed(eng))) return rc;
    cudaStream_t s = eng->stream;
    advance_clocks(eng);
    launch_tick((int)eng->order.size(), eng->sims_dev, eng->red, s);
    rc = bin(eng, 1);
    if (rc) return rc;
    return force_pass(eng, with_bonded != 0, false);
}

// The pair pass's own walk and pair decision in signature mode (no forces): per-particle
// partner count and id hash, and optionally the explicit pair list.
static int signature_pass(tfg_engine *eng, int32_t *count, uint32_t *hash, int64_t cap, int32_t *pairs,
                          int64_t *npairs) {
    int rc = commit(eng);
    if (rc) return rc;
    const int n = eng->n;
    if (npairs) *npairs = 0;
    if (n == 0) return TFG_OK;
    if (eng->split == 0) eng->split = 1;
    const int64_t pc = pairs ? std::max<int64_t>(cap, 0) : 0;
    // signature words, then the pair counter (8-byte aligned), then the pair list
    const size_t words = (size_t)2 * n + 2 + (size_t)2 * pc;
    int32_t *dbuf = nullptr;
    rc = dalloc(eng, &dbuf, words + 1);
    if (rc) return rc;
    int32_t *base = dbuf + (reinterpret_cast<uintptr_t>(dbuf) % 8 ? 1 : 0);
    PairKernelArgs a = pair_args(eng);
    a.sig_count = base;
    a.sig_hash = reinterpret_cast<uint32_t *>(base + n);
    unsigned long long *cnt_dev = reinterpret_cast<unsigned long long *>(base + 2 * (size_t)n + ((size_t)n % 2 ? 1 : 0));
    if (pairs) {
        a.pair_n = cnt_dev;
        a.pair_out = reinterpret_cast<int32_t *>(cnt_dev + 1);
        a.pair_cap = pc;
    }
    cudaMemsetAsync(dbuf, 0, sizeof(int32_t) * (words + 1), eng->stream);
    if (use_tile(eng))
        launch_pair_tile(a, tile_plan(eng, eng->split), eng->overflow_list, eng->overflow_count, eng->sms, true,
                         tune_of(eng), eng->stream);
    else
        launch_pair_signature(a, eng->stream);
    if (count) cudaMemcpyAsync(count, a.sig_count, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, eng->stream);
    if (hash) cudaMemcpyAsync(hash, a.sig_hash, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, eng->stream);
    unsigned long long found = 0;
    if (pairs) cudaMemcpyAsync(&found, cnt_dev, sizeof(found), cudaMemcpyDeviceToHost, eng->stream);
    cudaError_t e = cudaStreamSynchronize(eng->stream);
    if (e == cudaSuccess && pairs && found) {
        const size_t take = (size_t)std::min<int64_t>((int64_t)found, pc);
        e = cudaMemcpy(pairs, a.pair_out, sizeof(int32_t) * 2 * take, cudaMemcpyDeviceToHost);
    }
    cudaFree(dbuf);
    if (e != cudaSuccess) return fail(eng, TFG_E_CUDA, cudaGetErrorString(e));
    if (npairs) *npairs = (int64_t)found;
    return check_launch(eng);
}

TFG_API int tfg_pair_signature(tfg_engine *eng, int32_t *count, uint32_t *hash) {
    if (!eng || !count || !hash) return TFG_E_INVAL;
    return signature_pass(eng, count, hash, 0, nullptr, nullptr);
}

TFG_API int tfg_pair_list(tfg_engine *eng, int64_t cap, int32_t *pairs, int64_t *count) {
    if (!eng || !count || cap < 0 || (cap > 0 && !pairs)) return TFG_E_INVAL;
    if (cap == 0) {   // count only: a one-pair buffer that is not copied out
        int32_t dummy[2];
        return signature_pass(eng, nullptr, nullptr, 1, dummy, count);
    }
    return signature_pass(eng, nullptr, nullptr, cap, pairs, count);
}

TFG_API int tfg_sync(tfg_engine *eng) {
    if (!eng) return TFG_E_INVAL;
    CKE(cudaStreamSynchronize(eng->stream));
    int rc = check_launch(eng);
    if (rc) return rc;
    return read_err(eng);
}

TFG_API int tfg_get_count(const tfg_engine *eng, int *n) {
    if (!eng || !n || eng->sims.empty()) return TFG_E_INVAL;
    *n = eng->sims[0].n;
    return TFG_OK;
}
TFG_API int tfg_batch_get_count(const tfg_engine *eng, int sim, int *n) {
    if (!eng || !n || sim < 0 || sim >= (int)eng->sims.size() || !eng->sims[sim].live) return TFG_E_INVAL;
    *n = eng->sims[sim].n;
    return TFG_OK;
}

TFG_API int tfg_download(tfg_engine *eng, float *x, float *xrel, int32_t *cell, float *v, float *f, float *density,
                         float *species, float *q) {
    return download_sim(eng, 0, x, xrel, cell, v, f, density, species, q);
}
TFG_API int tfg_batch_download(tfg_engine *eng, int sim, float *x, float *xrel, int32_t *cell, float *v, float *f,
                               float *density, float *species, float *q) {
    return download_sim(eng, sim, x, xrel, cell, v, f, density, species, q);
}

TFG_API int tfg_get_reductions(tfg_engine *eng, tfg_reductions *out) { return reductions_sim(eng, 0, out); }
TFG_API int tfg_set_boundary(tfg_engine *eng, int wall, const tfg_boundary *bc) {
    return set_boundary_sim(eng, 0, wall, bc);
}
TFG_API int tfg_batch_set_boundary(tfg_engine *eng, int sim, int wall, const tfg_boundary *bc) {
    return set_boundary_sim(eng, sim, wall, bc);
}
TFG_API int tfg_set_boundary_potential(tfg_engine *eng, int wall, int type, const tfg_potential *p) {
    return set_boundary_potential_sim(eng, 0, wall, type, p);
}
TFG_API int tfg_batch_set_boundary_potential(tfg_engine *eng, int sim, int wall, int type, const tfg_potential *p) {
    return set_boundary_potential_sim(eng, sim, wall, type, p);
}
TFG_API int tfg_batch_get_reductions(tfg_engine *eng, int sim, tfg_reductions *out) {
    return reductions_sim(eng, sim, out);
}
TFG_API int tfg_set_pair_lists(tfg_engine *eng, int enable) {
    if (!eng) return TFG_E_INVAL;
    eng->lists_wanted = enable != 0;   // applied at the next step; lists fill at the next rebuild
    return TFG_OK;
}
TFG_API int tfg_get_verlet(tfg_engine *eng, int64_t *rebuilds, float *maxdx) {
    if (!eng) return TFG_E_INVAL;
    return verlet_sim(eng, 0, rebuilds, maxdx);
}
TFG_API int tfg_get_tuning(tfg_engine *eng, int *split, int *warps, int *grab) {
    if (!eng) return TFG_E_INVAL;
    if (split) *split = eng->split;
    if (warps) *warps = eng->tune_warps;
    if (grab) *grab = eng->tune_grab;
    return TFG_OK;
}

TFG_API int tfg_set_tuning(tfg_engine *eng, int split, int warps, int grab) {
    if (!eng || !(split == 1 || split == 2 || split == 7 || split == 14 || split == TFG_PAIR_HOME_OUTER) ||
        !(warps == 4 || warps == 8) || grab < 1 || grab > 8)
        return TFG_E_INVAL;
    eng->split = split;
    eng->tune_warps = warps;
    eng->tune_grab = grab;
    eng->tune_auto = false;
    eng->gen++;
    return TFG_OK;
}

TFG_API int tfg_set_deterministic(tfg_engine *eng, int enable) {
    if (!eng) return TFG_E_INVAL;
    if (eng->deterministic != (enable != 0)) {
        eng->deterministic = enable != 0;
        eng->gen++;
    }
    return TFG_OK;
}

TFG_API int tfg_batch_resume(tfg_engine *eng, int sim, int64_t steps, const float *q) {
    int rc = sim_check(eng, sim);
    if (rc) return rc;
    SimHost &S = eng->sims[sim];
    if (steps < 0) return fail(eng, TFG_E_INVAL, "negative step count");
    if (!S.pending) return fail(eng, TFG_E_STATE, "resume applies to particles loaded since the last step");
    S.time = steps;
    if (q) S.q_pending.assign(q, q + (size_t)S.n * eng->nspec);
    else S.q_pending.clear();
    return TFG_OK;
}

TFG_API int tfg_batch_sim_status(tfg_engine *eng, int sim, int *status) {
    if (!eng) return TFG_E_INVAL;
    return sim_status(eng, sim, status);
}

TFG_API int tfg_batch_get_verlet(tfg_engine *eng, int sim, int64_t *rebuilds, float *maxdx) {
    if (!eng) return TFG_E_INVAL;
    return verlet_sim(eng, sim, rebuilds, maxdx);
}

TFG_API int tfg_get_phase_ms(tfg_engine *eng, float ms[4]) {
    if (!eng || !ms) return TFG_E_INVAL;
    unsigned long long t[5];
    CKE(cudaMemcpyAsync(t, eng->stamps, sizeof(t), cudaMemcpyDeviceToHost, eng->stream));
    CKE(cudaStreamSynchronize(eng->stream));
    for (int k = 0; k < 4; k++) ms[k] = t[k + 1] >= t[k] && t[0] ? (float)((t[k + 1] - t[k]) * 1e-6) : -1.f;
    return TFG_OK;
}

TFG_API int tfg_set_phase_timing(tfg_engine *eng, int enable) {
    if (!eng) return TFG_E_INVAL;
    if (eng->phase_timing != (enable != 0)) eng->gen++;
    eng->phase_timing = enable != 0;
    return TFG_OK;
}

}  // extern "C"
