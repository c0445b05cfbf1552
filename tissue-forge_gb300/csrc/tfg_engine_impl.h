// Host-side engine: one device arena holding one or more simulations.
//
// A simulation is the reference's engine (source/mdcore/include/tfEngine.h:164-418):
// space, potentials, fluxes, types, particles, bonds and angles.  The arena concatenates
// the cells and particles of every live simulation in simulation order, so simulation k
// owns global cells [cell_off, cell_off+ncells) and, once binned, the particle slots
// [id_off, id_off+n) (particles are sorted by global cell).  Loads, additions and
// removals only mark the layout dirty; the next step (or download) re-lays the arena out.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "tfg_kernels.h"

struct SimHost {
    bool live = true;
    tfg_engine_desc desc{};
    tfg::SimParams P{};              // host copy; offsets and pointers filled at layout
    int maxc = 0;
    std::vector<float> orig;         // cell origins, 3 * maxc (axis-major)
    int n = 0;                       // particles of this simulation
    bool loaded = false;             // a particle load happened
    bool in_arena = false;           // its particles live in the current arena
    int arena_slot0 = 0, arena_cell_off = 0;
    // particle data waiting for the next layout
    bool pending = false, pending_binned = false;
    std::vector<float> x, xrel, v, radius, imass, species, force_i;
    std::vector<int32_t> cell, type;
    std::vector<uint32_t> flags;
    // interaction model (max_type^2 potentials and fluxes, per-type arrays)
    std::vector<tfg::PotDev> pots;
    std::vector<std::vector<float>> tables;
    std::vector<tfg::FluxSet> fluxes;
    std::vector<float4> rforce;
    std::vector<float> mass;
    std::vector<int32_t> dyn;
    std::vector<uint32_t> species_flags;
    std::vector<int2> bonds;         // local ids
    std::vector<int32_t> bond_slot;
    std::vector<int4> angles;        // local ids, w = slot
    int64_t time = 0;
    tfg_boundary walls[6];           // as set (NO_SLIP already turned into VELOCITY)
    std::vector<tfg::PotDev> wpots;  // 6 x max_type wall potentials
    std::vector<std::vector<float>> wtables;
    int status = 0;                  // first error of this simulation (TFG_E_*), sticky
    std::vector<float> q_pending;    // flux increments to restore at the next layout (id order)
};

struct tfg_engine {
    int device = 0, max_type = 1, nspec = 0, sms = 1;
    std::vector<SimHost> sims;       // by simulation id; removed ones have live == false
    std::vector<int> order;          // live simulation ids in arena order (current layout)
    int n = 0, cap = 0, ncells = 0, cells_cap = 0, cur = 0;
    tfg::ParticleArrays A[2];
    float4 *force = nullptr;
    float4 *oldx = nullptr;          // Verlet reference positions by slot
    int oldx_cap = 0;
    // Verlet pair lists of the tiled pass (table variants): list_k entries per home cell
    bool lists_wanted = true;        // tfg_set_pair_lists
    bool lists_on = false;
    uint32_t *vlist = nullptr;
    int32_t *vlen = nullptr;
    size_t vlist_cap = 0, vlen_cap = 0;
    int list_k = 0;
    int *list_need = nullptr;        // device: largest list a build asked for
    int *list_need_host = nullptr;   // pinned copy, read once its event has completed
    cudaEvent_t ev_need = nullptr;
    bool need_pending = false;
    int32_t *count = nullptr, *start = nullptr, *lidx = nullptr, *tmp_id = nullptr, *tmp_src = nullptr,
            *dest = nullptr, *slot_of_id = nullptr, *scan_sums = nullptr, *cell_sim = nullptr;
    int *overflow_list = nullptr, *overflow_count = nullptr;
    tfg::SimParams *sims_dev = nullptr;
    int sims_cap = 0;
    float *corig = nullptr;
    size_t corig_cap = 0;
    tfg::PotDev *pots = nullptr;
    size_t pots_cap = 0;
    float *blob = nullptr;
    size_t blob_cap = 0;
    int blob_floats = 0;
    tfg::FluxSet *fluxes = nullptr;
    size_t fluxes_cap = 0;
    float4 *rforce = nullptr;
    float *type_mass = nullptr;
    int32_t *type_dyn = nullptr;
    size_t types_cap = 0;
    uint32_t *species_flags = nullptr;
    size_t spec_cap = 0;
    int2 *bonds = nullptr;
    int32_t *bond_slot = nullptr;
    int4 *angles = nullptr;
    int nb = 0, na = 0, bcap = 0, acap = 0;
    tfg::PotDev *wpots = nullptr;     // nsims x 6 x max_type wall potentials
    size_t wpots_cap = 0;
    bool has_wall_pots = false;
    tfg::PotDev *bpots = nullptr;
    float *bblob = nullptr;
    size_t bblob_cap = 0;
    std::vector<tfg::PotDev> h_bpots;
    std::vector<std::vector<float>> h_btables;
    double *red = nullptr;
    size_t red_cap = 0;
    // device error words: err[0] for the engine, err[1 + q] for the simulation at arena
    // slot q (order[q]); collected into SimHost::status and pending_err at every read
    uint32_t *err = nullptr;
    int err_slots = 0;               // simulation words allocated after err[0]
    uint32_t pending_err = 0;        // engine bits collected but not yet reported
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    cudaEvent_t ev[5] = {};          // autotuner timing
    unsigned long long *stamps = nullptr;  // device: global-timer stamps of the phases of a step
    bool phase_timing = true;
    std::string last_error;
    bool layout_dirty = true, tables_dirty = true;
    bool has_dpd = false, has_flux = false;
    int max_fluxsteps = 1;           // largest nr_fluxsteps of a simulation with fluxes
    uint32_t flags_all = 0;          // TFG_ENGINE_NO_DENSITY only when every simulation sets it
    int split = 0;                   // tiled pair pass: warps per home cell (0 = not tuned)
    bool tune_auto = false;          // the tuple is the autotuner's (not fixed by the caller)
    int64_t tuned_n = 0;             // particles when the autotuner last ran
    int tune_warps = 8;              // tiled pair pass: warps per CTA (table variants: 8 or 4)
    int tune_grab = 1;               // tiled pair pass: work items per grab
    bool deterministic = false;      // pair pass without atomics (stencil kernel): reproducible bits
    int capacity_hint = 0;
    // tiled-pass staging plan, cached for (generation, split)
    tfg::TilePlan plan;
    uint64_t plan_gen = 0;
    int plan_split = 0;
    // CUDA graphs of one step, one per starting buffer parity (a step swaps the particle
    // buffers).  `gen` changes whenever a captured launch argument may have changed
    // (layout, tables, split, stream); a graph captured under another generation is
    // captured again, after one eager step of the new generation (`eager_gen`).
    bool use_graphs = true;
    uint64_t gen = 1;
    uint64_t graph_gen[2] = {0, 0};
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    int graph_next[2] = {1, 0};      // buffer index after a replay from each parity
    uint64_t eager_gen = 0;
};

namespace tfg {

int fail(tfg_engine *e, int code, const std::string &msg);

// (Re)allocate a device buffer of `count` elements (freeing the old one).
template <typename T> int dalloc(tfg_engine *eng, T **p, size_t count) {
    if (*p) { cudaFree(*p); *p = nullptr; }
    if (count == 0) return TFG_OK;
    cudaError_t e = cudaMalloc((void **)p, sizeof(T) * count);
    if (e != cudaSuccess) {
        *p = nullptr;
        return fail(eng, TFG_E_OOM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    return TFG_OK;
}
int check_launch(tfg_engine *eng);
int read_err(tfg_engine *eng);
int collect_errors(tfg_engine *eng);            // device error words -> SimHost::status, pending_err
int sim_status(tfg_engine *eng, int sim, int *status);
int sim_check(tfg_engine *eng, int sim);        // TFG_OK when `sim` names a live simulation
int add_sim(tfg_engine *eng, const tfg_engine_desc *d, int *out);
int commit(tfg_engine *eng);                    // re-lay the arena out and upload tables when dirty
int bin(tfg_engine *eng, int shuffle);
int force_pass(tfg_engine *eng, bool bonded, bool timed);
int one_step(tfg_engine *eng, bool advance, bool timed);
void advance_clocks(tfg_engine *eng);           // host clocks, by k_tick's rule (stops included)
int set_stop_sim(tfg_engine *eng, int sim, int64_t step);
int enqueue_step(tfg_engine *eng, bool advance, bool timed);
int flux_substeps(tfg_engine *eng);  // one_step without the host clock
int graph_step(tfg_engine *eng);                // one step replayed from a captured graph
int run_steps(tfg_engine *eng, int nsteps);     // nsteps steps, graphs where they apply
int autotune(tfg_engine *eng, bool splits_only = false);
int tune_if_needed(tfg_engine *eng);   // first tuning, or a re-tune after the batch grew or shrank 4x
inline TileTune tune_of(const tfg_engine *eng) {
    TileTune t;
    t.split = eng->split;
    t.warps = eng->tune_warps;
    t.grab = eng->tune_grab;
    return t;
}
int prepare_lists(tfg_engine *eng, bool relaid);  // allocate / invalidate the Verlet pair lists
int check_lists(tfg_engine *eng);                 // grow them when a build asked for more
PairKernelArgs pair_args(tfg_engine *eng);
const TilePlan &tile_plan(tfg_engine *eng, int split);
bool use_tile(const tfg_engine *eng);
PotDev to_dev(const tfg_potential *p);
int load_sim(tfg_engine *eng, int sim, int n, const float *xg, const int32_t *cellv, const float *xrel,
             const float *v, const int32_t *type, const float *radius, const float *imass, const uint32_t *flags,
             const float *species, const float *force_i);
int download_sim(tfg_engine *eng, int sim, float *x, float *xrel, int32_t *cell, float *v, float *f, float *dens,
                 float *species, float *q);
int reductions_sim(tfg_engine *eng, int sim, tfg_reductions *out);
int verlet_sim(tfg_engine *eng, int sim, int64_t *rebuilds, float *maxdx);
int set_boundary_sim(tfg_engine *eng, int sim, int wall, const tfg_boundary *bc);
int set_boundary_potential_sim(tfg_engine *eng, int sim, int wall, int type, const tfg_potential *p);
void resolve_boundaries(SimHost &S);   // periodicity and wall flags into S.P
void destroy(tfg_engine *eng);

}  // namespace tfg
