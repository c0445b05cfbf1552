// Stand-in for the batch C ABI (tfg_batch_*), linked with the real server code
// (tissue-forge_gb300/host/tfg_server.cpp) into a CPU-only test library, so that the
// server's admission, chunking and retirement logic is tested without a GPU.
//
// A simulation here is a particle count and a step counter.  A step advances every live
// simulation that has not reached its stop (tfg_batch_set_stop); a simulation loaded with
// a non-finite coordinate fails at its first step with TFG_E_NAN (reported by the next
// tfg_sync, as the device engine reports it).  A chunk
// stays "in flight" for a few tfg_query calls, so that requests arrive while it runs.
// Downloads return the step count in every coordinate, so a test can check that each
// request ran exactly its step count.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>

#include "tfg.h"

namespace {
struct FakeSim {
    int n = 0;
    long long steps = 0, stop_at = -1;
    bool poison = false;
    int status = TFG_OK;
};
int g_max_chunk = 0, g_min_chunk = 1 << 30, g_max_live = 0, g_chunks = 0, g_masked = 0;
}  // namespace

struct tfg_engine {
    std::map<int, FakeSim> sims;
    int next = 0;
    int busy = 0;
    int pending = TFG_OK;
    std::string err;
};

extern "C" {

// Chunk statistics since the last call; `masked` counts the simulation-steps that chunks
// ran past a member's stop.
TFG_API int tfg_fake_log(int *max_chunk, int *min_chunk, int *max_live, int *chunks, int *masked) {
    *max_chunk = g_max_chunk;
    *min_chunk = g_min_chunk;
    *max_live = g_max_live;
    *chunks = g_chunks;
    *masked = g_masked;
    g_masked = 0;
    g_max_chunk = 0;
    g_min_chunk = 1 << 30;
    g_max_live = 0;
    g_chunks = 0;
    return TFG_OK;
}

TFG_API int tfg_batch_create(int, int, int, tfg_engine **out) {
    *out = new tfg_engine();
    return TFG_OK;
}
TFG_API int tfg_engine_destroy(tfg_engine *e) {
    delete e;
    return TFG_OK;
}
TFG_API const char *tfg_last_error(const tfg_engine *e) { return e ? e->err.c_str() : ""; }
TFG_API int tfg_set_bonded_potential(tfg_engine *, int, const tfg_potential *) { return TFG_OK; }
TFG_API int tfg_batch_add_sim(tfg_engine *e, const tfg_engine_desc *, int *sim) {
    *sim = e->next++;
    e->sims[*sim] = FakeSim();
    return TFG_OK;
}
TFG_API int tfg_batch_remove_sim(tfg_engine *e, int sim) {
    return e->sims.erase(sim) ? TFG_OK : TFG_E_INVAL;
}
TFG_API int tfg_batch_set_type(tfg_engine *, int, int, int, float) { return TFG_OK; }
TFG_API int tfg_batch_set_potential(tfg_engine *, int, int, int, const tfg_potential *p) {
    return p ? TFG_OK : TFG_E_INVAL;
}
TFG_API int tfg_batch_add_flux(tfg_engine *, int, int, int, const tfg_flux *) { return TFG_OK; }
TFG_API int tfg_batch_set_species_flags(tfg_engine *, int, int, const uint32_t *) { return TFG_OK; }
TFG_API int tfg_batch_set_random_force(tfg_engine *, int, int, float, float, int) { return TFG_OK; }
TFG_API int tfg_batch_set_species_reset(tfg_engine *, int, int, const float *) { return TFG_OK; }
TFG_API int tfg_batch_set_stop(tfg_engine *e, int sim, int64_t step) {
    auto it = e->sims.find(sim);
    if (it == e->sims.end() || step < -1) return TFG_E_INVAL;
    it->second.stop_at = step;
    return TFG_OK;
}
TFG_API int tfg_batch_set_boundary(tfg_engine *, int, int, const tfg_boundary *) { return TFG_OK; }
TFG_API int tfg_batch_set_boundary_potential(tfg_engine *, int, int, int, const tfg_potential *) { return TFG_OK; }
TFG_API int tfg_batch_load_particles(tfg_engine *e, int sim, int n, const float *x, const float *, const int32_t *,
                                     const float *, const float *, const uint32_t *, const float *,
                                     const float *) {
    FakeSim &s = e->sims[sim];
    s.n = n;
    for (int k = 0; k < 3 * n; k++)
        if (!std::isfinite(x[k])) s.poison = true;
    return TFG_OK;
}
TFG_API int tfg_batch_load_bonds(tfg_engine *, int, int, const int32_t *, const int32_t *, const int32_t *) {
    return TFG_OK;
}
TFG_API int tfg_batch_load_angles(tfg_engine *, int, int, const int32_t *, const int32_t *, const int32_t *,
                                  const int32_t *) {
    return TFG_OK;
}
TFG_API int tfg_batch_step(tfg_engine *e, int nsteps) {
    if (nsteps < 1) return TFG_E_INVAL;
    g_chunks++;
    if (nsteps > g_max_chunk) g_max_chunk = nsteps;
    if (nsteps < g_min_chunk) g_min_chunk = nsteps;
    int live = 0;
    for (auto &kv : e->sims) {
        FakeSim &s = kv.second;
        long long k = nsteps;
        if (s.stop_at >= 0) k = std::max(0LL, std::min(k, s.stop_at - s.steps));
        g_masked += (int)(nsteps - k);
        s.steps += k;
        live++;
        if (k > 0 && s.poison && s.status == TFG_OK) {
            s.status = TFG_E_NAN;
            e->pending = TFG_E_NAN;
        }
    }
    if (live > g_max_live) g_max_live = live;
    e->busy = 3;
    return TFG_OK;
}
TFG_API int tfg_query(tfg_engine *e, int *idle) {
    if (e->busy > 0) e->busy--;
    *idle = e->busy == 0;
    return TFG_OK;
}
TFG_API int tfg_sync(tfg_engine *e) {
    e->busy = 0;
    const int rc = e->pending;
    e->pending = TFG_OK;
    if (rc) e->err = "non-finite particle position";
    return rc;
}
TFG_API int tfg_batch_sim_status(tfg_engine *e, int sim, int *status) {
    auto it = e->sims.find(sim);
    if (it == e->sims.end()) return TFG_E_INVAL;
    *status = it->second.status;
    return TFG_OK;
}
TFG_API int tfg_batch_get_count(const tfg_engine *e, int sim, int *n) {
    auto it = e->sims.find(sim);
    if (it == e->sims.end()) return TFG_E_INVAL;
    *n = it->second.n;
    return TFG_OK;
}
TFG_API int tfg_batch_download(tfg_engine *e, int sim, float *x, float *, int32_t *, float *v, float *, float *,
                               float *, float *) {
    const FakeSim &s = e->sims[sim];
    for (int k = 0; k < 3 * s.n; k++) {
        if (x) x[k] = (float)s.steps;
        if (v) v[k] = (float)s.n;
    }
    return TFG_OK;
}
TFG_API int tfg_batch_get_reductions(tfg_engine *e, int sim, tfg_reductions *out) {
    std::memset(out, 0, sizeof(*out));
    out->steps = e->sims[sim].steps;
    return TFG_OK;
}

}  // extern "C"
