// Continuous batching of simulation requests behind the C ABI (tfg_server_*, tfg_request_*).
//
// The reference runs one simulation per process and has no server; this layer sits on the
// batch C ABI of this library (tfg_batch_*).  A request records a whole simulation model
// host-side; the server keeps one batch per model family (types, species) on its own stream,
// admits requests under an HBM budget and a particles-in-flight cap, advances every batch in
// chunks cut at the nearest finishing simulation, and retires finished or failed simulations
// at chunk boundaries, so new requests join without waiting for a batch to drain.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <new>
#include <set>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "tfg.h"

namespace {

using Clock = std::chrono::steady_clock;

// A potential copied with its table.
struct PotCopy {
    tfg_potential p{};
    std::vector<float> c;
    void set(const tfg_potential *src) {
        p = *src;
        c.clear();
        if (src->c && src->kind == TFG_POTENTIAL_KIND_POTENTIAL && src->n >= 0)
            c.assign(src->c, src->c + (size_t)(src->n + 1) * TFG_POTENTIAL_CHUNK);
        p.c = c.empty() ? nullptr : c.data();
    }
    const tfg_potential *get() {
        p.c = c.empty() ? nullptr : c.data();
        return &p;
    }
};

// Arena bytes of one simulation: two particle buffers (five float4 arrays, cell index,
// value and increment per species), the force buffer and the binning scratch per
// particle; start/count/cell-simulation words per cell; bonds and angles.
int64_t footprint(int n, int nspec, int64_t ncells, int nb, int na) {
    const int64_t per_particle = 2 * (5 * 16 + 4 + 8 * std::max(1, nspec)) + 16 + 5 * 4;
    return (int64_t)n * per_particle + ncells * 16 + nb * 12 + na * 16;
}

}  // namespace

struct tfg_request {
    tfg_engine_desc desc{};
    int max_type = 1, nspec = 0, nsteps = 0;
    struct Type { int type, dynamics; float mass; };
    struct Pair { int ti, tj; PotCopy pot; };
    struct FluxAdd { int ti, tj; tfg_flux f; };
    struct RForce { int type; float mean, std; int dur; };
    struct Wall { int wall; tfg_boundary bc; };
    struct WallPot { int wall, type; bool none; PotCopy pot; };
    struct Slot { int slot; PotCopy pot; };
    std::vector<Type> types;
    std::vector<std::unique_ptr<Pair>> pots;
    std::vector<FluxAdd> fluxes;
    std::vector<uint32_t> species_flags;
    std::vector<float> species_reset;
    std::vector<RForce> rforces;
    std::vector<Wall> walls;
    std::vector<std::unique_ptr<WallPot>> wall_pots;
    std::vector<std::unique_ptr<Slot>> bonded;
    int n = 0;
    std::vector<float> x, v, radius, imass, species, force_i;
    std::vector<int32_t> type;
    std::vector<uint32_t> flags;
    std::vector<int32_t> bi, bj, bslot, ai, aj, ak, aslot;
    bool loaded = false;

    int64_t ncells() const { return (int64_t)desc.cells[0] * desc.cells[1] * desc.cells[2]; }
    int64_t bytes() const { return footprint(n, nspec, ncells(), (int)bi.size(), (int)ai.size()); }
    double work() const { return (double)n * nsteps; }
};

namespace {

struct Record {
    int state = TFG_REQ_QUEUED;
    int status = TFG_OK;
    double t_submit = -1, t_admit = -1, t_done = -1;
    std::unique_ptr<tfg_request> req;   // until admitted
    int n = 0, nspec = 0;
    std::vector<float> x, v, species;
    tfg_reductions red{};
    int64_t particles = 0, bytes = 0;
};

struct Active {
    int64_t id;
    int remaining;
};

struct Lane {
    tfg_engine *batch = nullptr;
    std::map<int, Active> active;     // by simulation id in the batch
    std::set<int> in_chunk;           // simulations stepping in the running chunk
    int running = 0;                  // steps of the running chunk (0: idle)
    Clock::time_point t_launch{};     // start of the running chunk
    Clock::time_point t_done{};       // completion of the last chunk, while simulations remain
    bool waiting = false;             // t_done is set: the batch waits for its next chunk
};

}  // namespace

struct tfg_server {
    tfg_server_desc desc{};
    Clock::time_point t0;
    std::map<std::pair<int, int>, Lane> lanes;
    std::unordered_map<int64_t, Record> records;
    std::vector<int64_t> arrived;     // submitted, not yet admitted, in submission order
    std::vector<int64_t> finished;    // finished or failed since the last take
    int64_t next_id = 1;
    tfg_server_stats st{};
    std::string last_error;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
    int fail(int code, const std::string &m) {
        last_error = m;
        return code;
    }
};

namespace {

// Bonded potentials are slots of a whole batch, so requests whose bonded tables differ go
// to different batches: the lane key carries a hash of them.
uint64_t bonded_key(const tfg_request &q) {
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](const void *p, size_t n) {
        const unsigned char *b = static_cast<const unsigned char *>(p);
        for (size_t k = 0; k < n; k++) h = (h ^ b[k]) * 1099511628211ull;
    };
    for (const auto &s : q.bonded) {
        mix(&s->slot, sizeof(s->slot));
        tfg_potential hdr = s->pot.p;
        hdr.c = nullptr;
        mix(&hdr, sizeof(hdr));
        if (!s->pot.c.empty()) mix(s->pot.c.data(), s->pot.c.size() * sizeof(float));
    }
    return h;
}

int lane_for(tfg_server *S, const tfg_request &q, Lane **out) {
    const uint64_t bk = bonded_key(q);
    const auto key = std::make_pair(q.max_type * 64 + q.nspec, (int)(bk ^ (bk >> 32)));
    Lane &L = S->lanes[key];
    if (!L.batch) {
        int rc = tfg_batch_create(S->desc.device, q.max_type, q.nspec, &L.batch);
        if (rc) {
            S->lanes.erase(key);
            return S->fail(rc, "tfg_batch_create failed");
        }
        for (const auto &s : q.bonded)
            if ((rc = tfg_set_bonded_potential(L.batch, s->slot, s->pot.get()))) return S->fail(rc, "bonded potential");
    }
    *out = &L;
    return TFG_OK;
}

// Replay a recorded request into its lane's batch as a new simulation.
int replay(tfg_engine *b, tfg_request &q, int *sim_out) {
    int sim = -1, rc;
    if ((rc = tfg_batch_add_sim(b, &q.desc, &sim))) return rc;
    *sim_out = sim;
    for (const auto &t : q.types)
        if ((rc = tfg_batch_set_type(b, sim, t.type, t.dynamics, t.mass))) return rc;
    for (auto &p : q.pots)
        if ((rc = tfg_batch_set_potential(b, sim, p->ti, p->tj, p->pot.get()))) return rc;
    for (const auto &f : q.fluxes)
        if ((rc = tfg_batch_add_flux(b, sim, f.ti, f.tj, &f.f))) return rc;
    if (!q.species_flags.empty() &&
        (rc = tfg_batch_set_species_flags(b, sim, (int)q.species_flags.size(), q.species_flags.data())))
        return rc;
    if (!q.species_reset.empty() &&
        (rc = tfg_batch_set_species_reset(b, sim, (int)q.species_reset.size(), q.species_reset.data())))
        return rc;
    for (const auto &r : q.rforces)
        if ((rc = tfg_batch_set_random_force(b, sim, r.type, r.mean, r.std, r.dur))) return rc;
    for (const auto &w : q.walls)
        if ((rc = tfg_batch_set_boundary(b, sim, w.wall, &w.bc))) return rc;
    for (auto &w : q.wall_pots)
        if ((rc = tfg_batch_set_boundary_potential(b, sim, w->wall, w->type, w->none ? nullptr : w->pot.get())))
            return rc;
    auto ptr = [](const auto &v) { return v.empty() ? nullptr : v.data(); };
    if ((rc = tfg_batch_load_particles(b, sim, q.n, ptr(q.x), ptr(q.v), ptr(q.type), ptr(q.radius), ptr(q.imass),
                                       ptr(q.flags), ptr(q.species), ptr(q.force_i))))
        return rc;
    if (!q.bi.empty() &&
        (rc = tfg_batch_load_bonds(b, sim, (int)q.bi.size(), q.bi.data(), q.bj.data(), ptr(q.bslot))))
        return rc;
    if (!q.ai.empty() &&
        (rc = tfg_batch_load_angles(b, sim, (int)q.ai.size(), q.ai.data(), q.aj.data(), q.ak.data(), ptr(q.aslot))))
        return rc;
    return TFG_OK;
}

void finish(tfg_server *S, int64_t id, int state, int status) {
    Record &R = S->records[id];
    R.state = state;
    R.status = status;
    R.t_done = S->now();
    R.req.reset();
    S->finished.push_back(id);
    if (state == TFG_REQ_DONE) S->st.completed++;
    else S->st.failed++;
}

bool fits(const tfg_server *S, const Record &R) {
    if (S->st.bytes_in_flight + R.bytes > S->desc.budget_bytes) return false;
    return S->desc.max_particles <= 0 || S->st.particles_in_flight == 0 ||
           S->st.particles_in_flight + R.particles <= S->desc.max_particles;
}

// Admit arrived requests in policy order while they fit (the first that does not fit waits
// at the head, as a queue).
int admit_inner(tfg_server *S);

int admit(tfg_server *S) {
    if (S->arrived.empty()) return TFG_OK;
    const auto t0 = Clock::now();
    const int rc = admit_inner(S);
    S->st.admit_s += std::chrono::duration<double>(Clock::now() - t0).count();
    return rc;
}

int admit_inner(tfg_server *S) {
    if (S->desc.policy == TFG_SERVER_LEAST_WORK)
        std::stable_sort(S->arrived.begin(), S->arrived.end(), [&](int64_t a, int64_t b) {
            return S->records[a].particles * (double)S->records[a].req->nsteps <
                   S->records[b].particles * (double)S->records[b].req->nsteps;
        });
    size_t k = 0;
    for (; k < S->arrived.size(); k++) {
        const int64_t id = S->arrived[k];
        Record &R = S->records[id];
        if (!fits(S, R)) break;
        Lane *L = nullptr;
        int rc = lane_for(S, *R.req, &L);
        if (rc) return rc;
        int sim = -1;
        rc = replay(L->batch, *R.req, &sim);
        // the simulation stops itself at its step count, so chunks need not end there
        if (rc == TFG_OK) rc = tfg_batch_set_stop(L->batch, sim, R.req->nsteps);
        if (rc) {
            if (sim >= 0) tfg_batch_remove_sim(L->batch, sim);
            S->last_error = std::string("request ") + std::to_string(id) + ": " + tfg_last_error(L->batch);
            finish(S, id, TFG_REQ_FAILED, rc);
            continue;
        }
        L->active[sim] = Active{id, R.req->nsteps};
        R.state = TFG_REQ_RUNNING;
        R.t_admit = S->now();
        R.nspec = R.req->nspec;
        S->st.bytes_in_flight += R.bytes;
        S->st.particles_in_flight += R.particles;
        R.req.reset();
    }
    S->arrived.erase(S->arrived.begin(), S->arrived.begin() + k);
    int64_t live = 0;
    for (auto &kv : S->lanes) live += (int64_t)kv.second.active.size();
    S->st.max_concurrent = std::max(S->st.max_concurrent, live);
    return TFG_OK;
}

void retire(tfg_server *S, Lane &L, int sim, int state, int status) {
    const Active a = L.active[sim];
    Record &R = S->records[a.id];
    if (state == TFG_REQ_DONE && !S->desc.discard_results) {
        int n = 0;
        if (tfg_batch_get_count(L.batch, sim, &n) == TFG_OK) {
            R.n = n;
            R.x.resize((size_t)3 * n);
            R.v.resize((size_t)3 * n);
            R.species.resize((size_t)n * R.nspec);
            int rc = tfg_batch_download(L.batch, sim, R.x.data(), nullptr, nullptr, R.v.data(), nullptr, nullptr,
                                        R.nspec ? R.species.data() : nullptr, nullptr);
            if (rc == TFG_OK) rc = tfg_batch_get_reductions(L.batch, sim, &R.red);
            if (rc != TFG_OK) {
                state = TFG_REQ_FAILED;
                status = rc;
            }
        }
    }
    tfg_batch_remove_sim(L.batch, sim);
    L.active.erase(sim);
    S->st.bytes_in_flight -= R.bytes;
    S->st.particles_in_flight -= R.particles;
    finish(S, a.id, state, status);
}

// An error reported by a batch call.  Particle errors (TFG_E_NAN, TFG_E_TOOFAST,
// TFG_E_RANGE) retire exactly the simulations whose status carries them; any other error
// means the batch itself failed (device or allocation), and every member fails with it.
int handle_error(tfg_server *S, Lane &L, int rc) {
    if (rc == TFG_OK) return 0;
    if (rc == TFG_E_NAN || rc == TFG_E_TOOFAST || rc == TFG_E_RANGE) {
        std::vector<std::pair<int, int>> bad;
        for (auto &kv : L.active) {
            int st = TFG_OK;
            if (tfg_batch_sim_status(L.batch, kv.first, &st) == TFG_OK && st != TFG_OK) bad.push_back({kv.first, st});
        }
        for (auto &b : bad) retire(S, L, b.first, TFG_REQ_FAILED, b.second);
        return (int)bad.size();
    }
    S->last_error = tfg_last_error(L.batch);
    std::vector<int> all;
    for (auto &kv : L.active) all.push_back(kv.first);
    for (int sid : all) retire(S, L, sid, TFG_REQ_FAILED, rc);
    return (int)all.size();
}

// The running chunk of lane L has completed on the device: account its steps, retire the
// failed and the finished simulations.
int complete_chunk(tfg_server *S, Lane &L) {
    struct Timed {
        tfg_server *S;
        Clock::time_point t0;
        ~Timed() { S->st.retire_s += std::chrono::duration<double>(Clock::now() - t0).count(); }
    } timed{S, Clock::now()};
    const int rc = tfg_sync(L.batch);
    const auto t_end = Clock::now();
    if (L.running) S->st.busy_s += std::chrono::duration<double>(t_end - L.t_launch).count();
    for (int sid : L.in_chunk) {
        auto it = L.active.find(sid);
        if (it != L.active.end()) it->second.remaining -= L.running;
    }
    L.running = 0;
    L.in_chunk.clear();
    int done = handle_error(S, L, rc);
    std::vector<int> fin;
    for (auto &kv : L.active)
        if (kv.second.remaining <= 0) fin.push_back(kv.first);
    for (int sid : fin) retire(S, L, sid, TFG_REQ_DONE, TFG_OK);
    L.waiting = !L.active.empty();
    L.t_done = t_end;
    return done + (int)fin.size();
}

// Start the next chunk on every idle batch with simulations: the quantum, or the longest
// remaining step count when that is shorter.  Members that reach their step count inside
// the chunk stop on the device (tfg_batch_set_stop) and wait there until the chunk ends,
// so a chunk is not cut short and the batch is re-laid out once per chunk at most.
// Returns the requests retired on the way (zero-step requests, or a chunk that failed to
// start).
int launch_idle(tfg_server *S) {
    int done = 0;
    for (auto &kv : S->lanes) {
        Lane &L = kv.second;
        if (L.running || L.active.empty()) continue;
        int longest = 0;
        for (auto &a : L.active) longest = std::max(longest, a.second.remaining);
        const int chunk = std::min(S->desc.quantum, longest);
        if (chunk <= 0) {   // zero-step requests finish at once
            L.running = 0;
            L.in_chunk.clear();
            done += complete_chunk(S, L);
            continue;
        }
        L.in_chunk.clear();
        for (auto &a : L.active) L.in_chunk.insert(a.first);
        L.running = chunk;
        const auto t0 = Clock::now();
        if (L.waiting) S->st.gap_s += std::chrono::duration<double>(t0 - L.t_done).count();
        L.waiting = false;
        L.t_launch = t0;
        const int rs = tfg_batch_step(L.batch, chunk);
        S->st.launch_s += std::chrono::duration<double>(Clock::now() - t0).count();
        S->st.chunks++;
        if (rs != TFG_OK) {
            // the chunk did not run as a whole: no steps are accounted, the failed leave
            L.running = 0;
            L.in_chunk.clear();
            done += handle_error(S, L, rs);
        }
    }
    return done;
}

}  // namespace

extern "C" {

TFG_API int tfg_server_create(const tfg_server_desc *desc, tfg_server **out) {
    if (!desc || !out) return TFG_E_INVAL;
    if (desc->policy != TFG_SERVER_LEAST_WORK && desc->policy != TFG_SERVER_FIFO) return TFG_E_INVAL;
    if (desc->quantum < 0 || desc->budget_bytes < 0 || desc->max_particles < 0) return TFG_E_INVAL;
    tfg_server *S = new (std::nothrow) tfg_server();
    if (!S) return TFG_E_OOM;
    S->desc = *desc;
    if (S->desc.quantum == 0) S->desc.quantum = 50;
    if (S->desc.budget_bytes == 0) S->desc.budget_bytes = (int64_t)150 << 30;
    S->t0 = Clock::now();
    *out = S;
    return TFG_OK;
}

TFG_API int tfg_server_destroy(tfg_server *S) {
    if (!S) return TFG_E_INVAL;
    for (auto &kv : S->lanes)
        if (kv.second.batch) tfg_engine_destroy(kv.second.batch);
    delete S;
    return TFG_OK;
}

TFG_API const char *tfg_server_last_error(const tfg_server *S) { return S ? S->last_error.c_str() : ""; }

TFG_API int tfg_request_create(const tfg_engine_desc *desc, int max_type, int nr_species, int nsteps,
                               tfg_request **out) {
    if (!desc || !out || max_type < 1 || nr_species < 0 || nsteps < 0) return TFG_E_INVAL;
    tfg_request *q = new (std::nothrow) tfg_request();
    if (!q) return TFG_E_OOM;
    q->desc = *desc;
    q->max_type = max_type;
    q->nspec = nr_species;
    q->nsteps = nsteps;
    *out = q;
    return TFG_OK;
}

TFG_API int tfg_request_free(tfg_request *q) {
    delete q;
    return TFG_OK;
}

TFG_API int tfg_request_set_type(tfg_request *q, int type, int dynamics, float mass) {
    if (!q || type < 0 || type >= q->max_type) return TFG_E_INVAL;
    q->types.push_back({type, dynamics, mass});
    return TFG_OK;
}

TFG_API int tfg_request_set_potential(tfg_request *q, int ti, int tj, const tfg_potential *p) {
    if (!q || !p || ti < 0 || tj < 0 || ti >= q->max_type || tj >= q->max_type) return TFG_E_INVAL;
    std::unique_ptr<tfg_request::Pair> e(new tfg_request::Pair{ti, tj, PotCopy()});
    e->pot.set(p);
    q->pots.push_back(std::move(e));
    return TFG_OK;
}

TFG_API int tfg_request_add_flux(tfg_request *q, int ti, int tj, const tfg_flux *f) {
    if (!q || !f) return TFG_E_INVAL;
    q->fluxes.push_back({ti, tj, *f});
    return TFG_OK;
}

TFG_API int tfg_request_set_species_flags(tfg_request *q, int nr, const uint32_t *flags) {
    if (!q || nr < 0 || (nr > 0 && !flags)) return TFG_E_INVAL;
    q->species_flags.assign(flags, flags + nr);
    return TFG_OK;
}

TFG_API int tfg_request_set_species_reset(tfg_request *q, int nr, const float *values) {
    if (!q || nr < 0 || (nr > 0 && !values)) return TFG_E_INVAL;
    q->species_reset.assign(values, values + nr);
    return TFG_OK;
}

TFG_API int tfg_request_set_random_force(tfg_request *q, int type, float mean, float std, int duration_steps) {
    if (!q) return TFG_E_INVAL;
    q->rforces.push_back({type, mean, std, duration_steps});
    return TFG_OK;
}

TFG_API int tfg_request_set_boundary(tfg_request *q, int wall, const tfg_boundary *bc) {
    if (!q || !bc) return TFG_E_INVAL;
    q->walls.push_back({wall, *bc});
    return TFG_OK;
}

TFG_API int tfg_request_set_boundary_potential(tfg_request *q, int wall, int type, const tfg_potential *p) {
    if (!q) return TFG_E_INVAL;
    std::unique_ptr<tfg_request::WallPot> e(new tfg_request::WallPot{wall, type, p == nullptr, PotCopy()});
    if (p) e->pot.set(p);
    q->wall_pots.push_back(std::move(e));
    return TFG_OK;
}

TFG_API int tfg_request_set_bonded_potential(tfg_request *q, int slot, const tfg_potential *p) {
    if (!q || !p) return TFG_E_INVAL;
    std::unique_ptr<tfg_request::Slot> e(new tfg_request::Slot{slot, PotCopy()});
    e->pot.set(p);
    q->bonded.push_back(std::move(e));
    return TFG_OK;
}

TFG_API int tfg_request_load_particles(tfg_request *q, int n, const float *x, const float *v, const int32_t *type,
                                       const float *radius, const float *imass, const uint32_t *flags,
                                       const float *species, const float *force_i) {
    if (!q || n < 0 || (n > 0 && !x)) return TFG_E_INVAL;
    auto copy = [](auto &dst, const auto *src, size_t cnt) {
        dst.clear();
        if (src) dst.assign(src, src + cnt);
    };
    q->n = n;
    copy(q->x, x, (size_t)3 * n);
    copy(q->v, v, (size_t)3 * n);
    copy(q->type, type, (size_t)n);
    copy(q->radius, radius, (size_t)n);
    copy(q->imass, imass, (size_t)n);
    copy(q->flags, flags, (size_t)n);
    copy(q->species, species, (size_t)n * q->nspec);
    copy(q->force_i, force_i, (size_t)3 * n);
    q->loaded = true;
    return TFG_OK;
}

TFG_API int tfg_request_load_bonds(tfg_request *q, int n, const int32_t *i, const int32_t *j, const int32_t *slot) {
    if (!q || n < 0 || (n > 0 && (!i || !j))) return TFG_E_INVAL;
    q->bi.assign(i, i + n);
    q->bj.assign(j, j + n);
    q->bslot.clear();
    if (slot) q->bslot.assign(slot, slot + n);
    return TFG_OK;
}

TFG_API int tfg_request_load_angles(tfg_request *q, int n, const int32_t *i, const int32_t *j, const int32_t *k,
                                    const int32_t *slot) {
    if (!q || n < 0 || (n > 0 && (!i || !j || !k))) return TFG_E_INVAL;
    q->ai.assign(i, i + n);
    q->aj.assign(j, j + n);
    q->ak.assign(k, k + n);
    q->aslot.clear();
    if (slot) q->aslot.assign(slot, slot + n);
    return TFG_OK;
}

TFG_API int tfg_server_submit(tfg_server *S, tfg_request *q, int64_t *id) {
    if (!S || !q || !id) return TFG_E_INVAL;
    if (!q->loaded) return S->fail(TFG_E_STATE, "request has no particles");
    if (q->bytes() > S->desc.budget_bytes) return S->fail(TFG_E_OOM, "request larger than the HBM budget");
    const int64_t rid = S->next_id++;
    Record &R = S->records[rid];
    R.t_submit = S->now();
    R.particles = q->n;
    R.bytes = q->bytes();
    R.req.reset(q);
    S->arrived.push_back(rid);
    S->st.submitted++;
    *id = rid;
    return TFG_OK;
}

TFG_API int tfg_server_poll(tfg_server *S, int wait_us, int *completed) {
    if (!S) return TFG_E_INVAL;
    int done = 0;
    int rc = admit(S);
    if (rc == TFG_OK) done += launch_idle(S);
    const auto deadline = Clock::now() + std::chrono::microseconds(std::max(0, wait_us));
    for (;;) {
        bool any_running = false;
        int now_done = 0;
        for (auto &kv : S->lanes) {
            Lane &L = kv.second;
            if (!L.running) continue;
            int idle = 0;
            if (tfg_query(L.batch, &idle) != TFG_OK || idle) now_done += complete_chunk(S, L);
            else any_running = true;
        }
        if (now_done > 0) {
            // slots and memory freed: admit the waiting requests and start the next chunks
            done += now_done;
            if (rc == TFG_OK) rc = admit(S);
            if (rc == TFG_OK) done += launch_idle(S);
            break;
        }
        if (!any_running || Clock::now() >= deadline) break;
        std::this_thread::sleep_for(std::chrono::microseconds(100));
    }
    S->st.queued = (int64_t)S->arrived.size();
    int64_t running = 0;
    for (auto &kv : S->lanes) running += (int64_t)kv.second.active.size();
    S->st.running = running;
    if (completed) *completed = done;
    return rc;
}

TFG_API int tfg_server_take_finished(tfg_server *S, int64_t *ids, int cap, int *n) {
    if (!S || !n || cap < 0 || (cap > 0 && !ids)) return TFG_E_INVAL;
    const int k = std::min(cap, (int)S->finished.size());
    for (int i = 0; i < k; i++) ids[i] = S->finished[i];
    S->finished.erase(S->finished.begin(), S->finished.begin() + k);
    *n = k;
    return TFG_OK;
}

TFG_API int tfg_server_request_info(tfg_server *S, int64_t id, int *state, int *status, double times[3]) {
    if (!S) return TFG_E_INVAL;
    auto it = S->records.find(id);
    if (it == S->records.end()) return S->fail(TFG_E_INVAL, "no such request");
    const Record &R = it->second;
    if (state) *state = R.state;
    if (status) *status = R.status;
    if (times) {
        times[0] = R.t_submit;
        times[1] = R.t_admit;
        times[2] = R.t_done;
    }
    return TFG_OK;
}

TFG_API int tfg_server_result(tfg_server *S, int64_t id, int *n, float *x, float *v, float *species,
                              tfg_reductions *red) {
    if (!S) return TFG_E_INVAL;
    auto it = S->records.find(id);
    if (it == S->records.end()) return S->fail(TFG_E_INVAL, "no such request");
    const Record &R = it->second;
    if (R.state == TFG_REQ_FAILED) return R.status;
    if (R.state != TFG_REQ_DONE) return S->fail(TFG_E_STATE, "request not finished");
    if (n) *n = R.n;
    if (x && !R.x.empty()) std::memcpy(x, R.x.data(), sizeof(float) * R.x.size());
    if (v && !R.v.empty()) std::memcpy(v, R.v.data(), sizeof(float) * R.v.size());
    if (species && !R.species.empty()) std::memcpy(species, R.species.data(), sizeof(float) * R.species.size());
    if (red) *red = R.red;
    return TFG_OK;
}

TFG_API int tfg_server_release(tfg_server *S, int64_t id) {
    if (!S) return TFG_E_INVAL;
    auto it = S->records.find(id);
    if (it == S->records.end()) return S->fail(TFG_E_INVAL, "no such request");
    if (it->second.state != TFG_REQ_DONE && it->second.state != TFG_REQ_FAILED)
        return S->fail(TFG_E_STATE, "request still queued or running");
    S->records.erase(it);
    return TFG_OK;
}

TFG_API int tfg_server_get_stats(tfg_server *S, tfg_server_stats *out) {
    if (!S || !out) return TFG_E_INVAL;
    *out = S->st;
    return TFG_OK;
}

}  // extern "C"
