// tfg_oracle -- CPU restatement of Tissue Forge's per-step particle path.
//
// TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU engine: the
// tests, the smoke check and the CPU-baseline leg of the benchmark load it; the
// product never does.  It restates the reference's mdcore CPU engine (version 0.2.1)
// in the same operation order, in FP32 without FMA contraction (compiled with
// -ffp-contract=off), with an optional FP64 evaluation mode that keeps the FP32
// pair decisions and table indices but evaluates forces in double.
//
// Parity status: the reference cannot be built here (its Magnum/Corrade/libsbml
// submodules are empty and it needs GL/GLFW/assimp), and its own tests hold no golden
// vectors for this path (every Python test ends in `def test_pass(): pass`, the C/C++
// tests only check HRESULTs).  Parity is therefore UNPINNED by the reference; the
// restatement is pinned by analytic known-answer tests and committed golden fixtures.
//
// Restated functions (file:line in source/mdcore of the reference):
//   space geometry / cell origins        src/tfSpace.cpp:737-770
//   task list (27-stencil, id1<id2)      src/tfSpace.cpp:893-1019
//   space_getsid / cell_flip / sortIDs   src/tfSpace.cpp:79-114, src/tfSpace_cell.cpp:54-99
//   space_setpartp (load binning)        src/tfSpace.cpp:432-475
//   space_prepare (f = force_i, W(0))    src/tfSpace.cpp:168-208
//   space_shuffle_local + welcome        src/tfSpace.cpp:274-391, tfSpace_cell.cpp:187-237
//   runner_dosort (16-bit keys)          src/tf_runner_dosort.cpp:64-126
//   runner_dopair (sorted window)        src/tf_runner_dopair.cpp:72-332
//   runner_doself                        src/tf_runner_dopair.cpp:514-758
//   fptype_r2 (scalar branch)            include/tf_fptype.h:204-210 (VECTORIZE undefined :54)
//   potential_eval / _ex / _r            src/tf_potential_eval.h:74-194
//   potential_eval_super_ex              src/tf_potential_eval.h:207-272
//   dpd_eval                             src/tf_dpd_eval.h:32-76
//   flux_eval_ex                         src/tf_flux_eval.h:32-103
//   W (cubic spline number density)      src/tf_smoothing_kernel.h:49-67
//   bond_eval                            src/tfBond.cpp:97-345
//   angle_eval                           src/tfAngle.cpp:90-382
//   cell_advance_forward_euler           src/tf_engine_advance.cpp:140-247
//   engine_advance_forward_euler         src/tf_engine_advance.cpp:309-480
//   Fluxes_integrate                     src/tfFlux.cpp:175-202
//   gaussian_force                       src/tfForce.cpp:211-223
//   engine_kinetic_energy                src/tfEngine.cpp:1893-1925
// Where the reference draws from std::mt19937 (angle random plane, Gaussian force) or
// uses a deterministic stand-in (DPD random term), this oracle uses the same
// Philox4x32-10 counter streams as the GPU engine (see philox() below).
#include "../include/tfg.h"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

namespace {

// ---------------- Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) ----------------
struct U4 { uint32_t x, y, z, w; };

static inline void mulhilo(uint32_t a, uint32_t b, uint32_t &hi, uint32_t &lo) {
    uint64_t p = (uint64_t)a * (uint64_t)b;
    hi = (uint32_t)(p >> 32);
    lo = (uint32_t)p;
}

static U4 philox(U4 c, uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; r++) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo(0xD2511F53u, c.x, hi0, lo0);
        mulhilo(0xCD9E8D57u, c.z, hi1, lo1);
        U4 n = {hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
        c = n;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}
// (0,1) uniform from 24 high bits.
static inline float u01(uint32_t u) { return (float)(u >> 8) * 5.9604644775390625e-8f + 2.98023223876953125e-8f; }

enum : uint32_t { STREAM_DPD = 0xD0D0u, STREAM_FORCE = 0xF0F0u, STREAM_ANGLE = 0xA0A0u, STREAM_WALL = 0xB0B0u };

// ---------------- reference constants ----------------
const char kSortID[27] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 0,
                          12, 11, 10, 9, 8, 7, 6, 5, 4, 3, 2, 1, 0};
const char kFlip[27] = {1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 0,
                        0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
const float kShiftN[13 * 3] = {
    5.773502691896258e-01f, 5.773502691896258e-01f, 5.773502691896258e-01f,
    7.071067811865475e-01f, 7.071067811865475e-01f, 0.0f,
    5.773502691896258e-01f, 5.773502691896258e-01f, -5.773502691896258e-01f,
    7.071067811865475e-01f, 0.0f, 7.071067811865475e-01f,
    1.0f, 0.0f, 0.0f,
    7.071067811865475e-01f, 0.0f, -7.071067811865475e-01f,
    5.773502691896258e-01f, -5.773502691896258e-01f, 5.773502691896258e-01f,
    7.071067811865475e-01f, -7.071067811865475e-01f, 0.0f,
    5.773502691896258e-01f, -5.773502691896258e-01f, -5.773502691896258e-01f,
    0.0f, 7.071067811865475e-01f, 7.071067811865475e-01f,
    0.0f, 1.0f, 0.0f,
    0.0f, 7.071067811865475e-01f, -7.071067811865475e-01f,
    0.0f, 0.0f, 1.0f,
};

// ---------------- data ----------------
template <typename R> struct Part {
    R f[4];             // force; f[3] = number density
    double fmag;        // sum of |contribution| (force-error normalisation)
    float fi[3];        // force_i (external)
    float v[4];         // velocity; v[3] = inverse number density
    float x[4];         // cell-relative position
    float ox[3];        // Verlet reference position (space_cell::oldx)
    float pf[3];        // persistent (random) force
    float imass, radius;
    int id, type;
    uint32_t flags;
};

template <typename R> struct Pot {
    bool set = false;
    uint32_t kind = 0, flags = 0;
    float alpha[4] = {0, 0, 0, 0};
    float r0_plusone = 0, a = 0, b = 0;
    int n = 0;
    std::vector<float> c;
    std::vector<R> cr;  // table in evaluation precision
    float dalpha = 0, dgamma = 0, dsigma = 0;
};

struct FluxEntry { tfg_flux f; };

template <typename R> struct Cell {
    int loc[3];
    float origin[3];
    std::vector<Part<R>> parts, incoming;
    std::vector<unsigned> sortlist;   // 13 * count keys
    R epot = 0;
    R computed_volume = 0;
    double virial = 0;
    std::mutex mtx;
    bool migrated_in = false;
};

struct Task { int type; int sid; int i, j; };   // type 0 = self, 1 = pair

struct BondRec { int i, j, slot; };
struct AngleRec { int i, j, k, slot; };

template <typename R> struct Engine {
    tfg_engine_desc d{};
    float origin[3], dim[3], h[3], ih[3];
    int cdim[3];
    float cutoff, cutoff2;
    int ncells = 0;
    std::vector<Cell<R>> cells;
    std::vector<Task> tasks;
    std::vector<int> sortflags;
    std::vector<std::vector<int>> owned;           // task indices per owner cell
    std::vector<std::vector<int>> colour_classes;  // owner cells that may run concurrently
    int max_type = 1, nspec = 0;
    std::vector<Pot<R>> pots;                    // max_type^2
    std::vector<std::vector<tfg_flux>> fluxes;   // max_type^2
    std::vector<int> dyn;
    std::vector<float> mass;
    std::vector<float> rf_mean, rf_std;
    std::vector<int> rf_dur;
    std::vector<uint32_t> species_flags;
    std::vector<float> species_reset;   // StateVector::reset values (state/tfStateVector.cpp:36-44)
    std::vector<float> svec;    // n * nspec (by id)
    std::vector<R> sq;          // n * nspec (by id)
    std::vector<Pot<R>> bpots;  // bonded slots
    std::vector<BondRec> bonds;
    std::vector<AngleRec> angles;
    int nparts = 0;
    int64_t time = 0;
    float dt = 0.01f, dt_flux = 0.01f;
    int nthreads = 1;
    bool brute = false;          // brute-force pair enumeration instead of sorted windows
    bool ref_dpd_random = false; // reproduce the reference's deterministic DPD "random" term
    bool density = true;
    bool flux_only = false;      // flux substep pass: fluxes only (runner_*_fluxonly)
    // boundary conditions, walls 0..5 = left, right, front, back, bottom, top
    tfg_boundary walls_set[6];   // as set
    tfg_boundary walls[6];       // in effect (check_periodicy applied)
    unsigned periodic = 7;       // bit k: axis k periodic
    std::vector<Pot<R>> wpots;   // 6 x max_type
    bool tasks_dirty = false;
    int nr_fluxsteps = 1;
    // Verlet mode (engine_flag_verlet): skin, rebuild flag, space::maxdx, rebuild count
    bool verlet = false;
    float skin = 0.f;
    bool verlet_rebuild = true;
    float verlet_maxdx = 0.f;
    int64_t verlet_rebuilds = 0;
    R epot_nonbond = 0, epot_bond = 0, epot_angle = 0;
    double kinetic = 0, virial = 0, computed_volume = 0;
    int64_t migrations = 0, straight_angles = 0;
    std::atomic<int64_t> window_skips{0};
    std::string err;
    // per-id lookup (rebuilt on demand)
    std::vector<int> where_cell, where_slot;
    std::vector<uint8_t> migrated;  // particle migrated during the last advance (flux deferral)
    bool want_sig = false;
    std::vector<int32_t> sig_cnt;
    std::vector<uint32_t> sig_hash;
    bool record_pairs = false;
    std::vector<std::pair<int, int>> pairs;
    std::mutex pair_mtx;
};

template <typename R> static inline float Wdens(float r2, float hcut) {
    // Cubic-spline number density.  The reference's x86 qsqrt() is 1/_mm_rsqrt_ss
    // (~12-bit); this restatement uses the correctly rounded sqrt.
    float r = std::sqrt(r2);
    float x = r / hcut;
    float y;
    if (x < 1.f) {
        float x2 = x * x;
        y = 1.f - (3.f / 2.f) * x2 + (3.f / 4.f) * x2 * x;
    } else if (x >= 1.f && x < 2.f) {
        float arg = 2.f - x;
        y = (1.f / 4.f) * arg * arg * arg;
    } else {
        y = 0.f;
    }
    return y / (M_PI * hcut * hcut * hcut);
}

template <typename R> static inline int cellid(const Engine<R> &e, int i, int j, int k) {
    return (i * e.cdim[1] + j) * e.cdim[2] + k;
}

// space_getsid: shift from ci to cj, wrapped; flips so that the sort id is canonical.
template <typename R> static int getsid(const Engine<R> &e, int &ci, int &cj, float *shift) {
    for (int k = 0; k < 3; k++) {
        shift[k] = e.cells[cj].origin[k] - e.cells[ci].origin[k];
        if (shift[k] * 2 > e.dim[k]) shift[k] -= e.dim[k];
        else if (shift[k] * 2 < -e.dim[k]) shift[k] += e.dim[k];
    }
    int sid = 0;
    for (int k = 0; k < 3; k++) sid = 3 * sid + ((shift[k] < 0) ? 0 : ((shift[k] > 0) ? 2 : 1));
    if (kFlip[sid]) {
        std::swap(ci, cj);
        shift[0] = -shift[0]; shift[1] = -shift[1]; shift[2] = -shift[2];
    }
    return kSortID[sid];
}

// Task list (space_init, tfSpace.cpp:893-1019): every cell against its neighbours, kept once
// (id1 < id2) plus self; across the edge of a non-periodic axis there is no neighbour.
template <typename R> static void build_tasks(Engine<R> &e) {
    e.tasks.clear();
    e.sortflags.assign(e.ncells, 0);
    e.owned.clear();
    e.colour_classes.clear();
    for (int i = 0; i < e.cdim[0]; i++)
        for (int j = 0; j < e.cdim[1]; j++)
            for (int k = 0; k < e.cdim[2]; k++) {
                int id1 = cellid(e, i, j, k);
                for (int a = -1; a <= 1; a++) {
                    if (!(e.periodic & 1u) && (i + a < 0 || i + a >= e.cdim[0])) continue;
                    int ii = (i + a + e.cdim[0]) % e.cdim[0];
                    for (int b = -1; b <= 1; b++) {
                        if (!(e.periodic & 2u) && (j + b < 0 || j + b >= e.cdim[1])) continue;
                        int jj = (j + b + e.cdim[1]) % e.cdim[1];
                        for (int c = -1; c <= 1; c++) {
                            if (!(e.periodic & 4u) && (k + c < 0 || k + c >= e.cdim[2])) continue;
                            int kk = (k + c + e.cdim[2]) % e.cdim[2];
                            int id2 = cellid(e, ii, jj, kk);
                            int ci = id1, cj = id2;
                            float sh[3];
                            int sid = getsid(e, ci, cj, sh);
                            if (id1 < id2 || (id1 == id2 && a == 0 && b == 0 && c == 0)) {
                                Task t{id1 == id2 ? 0 : 1, sid, ci, cj};
                                e.tasks.push_back(t);
                                if (t.type == 1) {
                                    e.sortflags[ci] |= 1 << sid;
                                    e.sortflags[cj] |= 1 << sid;
                                }
                            }
                        }
                    }
                }
            }
}

template <typename R> static int init_space(Engine<R> &e, const tfg_engine_desc *d) {
    e.d = *d;
    for (int i = 0; i < 3; i++) {
        e.origin[i] = d->origin[i];
        e.dim[i] = d->dim[i];
        e.cdim[i] = d->cells[i];
        if (e.cdim[i] < 3) return TFG_E_INVAL;
    }
    e.cutoff = d->cutoff;
    e.cutoff2 = e.cutoff * e.cutoff;
    e.ncells = e.cdim[0] * e.cdim[1] * e.cdim[2];
    for (int i = 0; i < 3; i++) {
        e.h[i] = e.dim[i] / e.cdim[i];
        e.ih[i] = 1.0 / e.h[i];
        if ((int)std::ceil(e.cutoff * e.ih[i]) != 1) return TFG_E_INVAL;   // span must be 1
    }
    e.cells = std::vector<Cell<R>>(e.ncells);
    float o[3];
    int l[3];
    for (l[0] = 0; l[0] < e.cdim[0]; l[0]++) {
        o[0] = e.origin[0] + l[0] * e.h[0];
        for (l[1] = 0; l[1] < e.cdim[1]; l[1]++) {
            o[1] = e.origin[1] + l[1] * e.h[1];
            for (l[2] = 0; l[2] < e.cdim[2]; l[2]++) {
                o[2] = e.origin[2] + l[2] * e.h[2];
                Cell<R> &c = e.cells[cellid(e, l[0], l[1], l[2])];
                for (int k = 0; k < 3; k++) { c.loc[k] = l[k]; c.origin[k] = o[k]; }
            }
        }
    }
    for (int w = 0; w < 6; w++) {
        std::memset(&e.walls[w], 0, sizeof(tfg_boundary));
        e.walls[w].kind = TFG_BOUNDARY_PERIODIC;
        e.walls[w].restore = 1.f;
        e.walls_set[w] = e.walls[w];
    }
    e.periodic = 7;
    build_tasks(e);
    e.max_type = std::max(1, d->max_type);
    e.nspec = std::max(0, d->nr_species);
    e.pots.assign(e.max_type * e.max_type, Pot<R>());
    e.fluxes.assign(e.max_type * e.max_type, std::vector<tfg_flux>());
    e.dyn.assign(e.max_type, TFG_NEWTONIAN);
    e.mass.assign(e.max_type, 1.0f);
    e.rf_mean.assign(e.max_type, 0.f);
    e.rf_std.assign(e.max_type, 0.f);
    e.rf_dur.assign(e.max_type, 1);
    e.species_flags.assign(std::max(1, e.nspec), 0u);
    e.species_reset.assign(std::max(1, e.nspec), 0.f);
    e.wpots.assign(6 * e.max_type, Pot<R>());
    e.dt = d->dt;
    // dt_flux = dt / nr_fluxsteps (tfSimulator.cpp:653), an FP32 division
    e.nr_fluxsteps = d->nr_fluxsteps > 0 ? d->nr_fluxsteps : 1;
    e.dt_flux = d->dt / (float)e.nr_fluxsteps;
    e.verlet = (d->flags & TFG_ENGINE_VERLET) != 0;
    e.skin = std::fmin(e.h[0], std::fmin(e.h[1], e.h[2])) - e.cutoff;   // tfEngine.cpp:231
    return TFG_OK;
}

template <typename R> static void copy_pot(Pot<R> &dst, const tfg_potential *p) {
    dst.set = true;
    dst.kind = p->kind;
    dst.flags = p->flags;
    for (int k = 0; k < 4; k++) dst.alpha[k] = p->alpha[k];
    dst.r0_plusone = p->r0_plusone;
    dst.a = p->a; dst.b = p->b; dst.n = p->n;
    dst.dalpha = p->dpd_alpha; dst.dgamma = p->dpd_gamma; dst.dsigma = p->dpd_sigma;
    if (p->kind == TFG_POTENTIAL_KIND_POTENTIAL && p->c) {
        dst.c.assign(p->c, p->c + (size_t)(p->n + 1) * TFG_POTENTIAL_CHUNK);
        dst.cr.assign(dst.c.begin(), dst.c.end());
    }
}

// ---- potential evaluation (FP32 index, R-precision polynomial) ----
// potential_eval_ex: radius shift/scale, clamp to a, interval index, Horner in x.
template <typename R> static bool pot_eval_ex(const Pot<R> &p, float ri, float rj, float r2f, R r2,
                                              R &e, R &f) {
    const float eps = FLT_EPSILON;
    float r = std::sqrt(r2f);
    if (p.flags & TFG_POTENTIAL_SCALED) r = r / (ri + rj);
    else if (p.flags & TFG_POTENTIAL_SHIFTED) r = r - (ri + rj) + p.r0_plusone;
    r = r < p.a ? p.a : r;
    unsigned ind = std::max(0.0f, p.alpha[0] + r * (p.alpha[1] + r * p.alpha[2]));
    if (r > p.b || ind > (unsigned)p.n) return false;
    R rr, ro;
    if (sizeof(R) == sizeof(float)) {
        rr = r;
        float rf = std::sqrt(r2f);
        ro = rf < eps ? eps : rf;
    } else {
        R rd = std::sqrt(r2);
        ro = rd < (R)eps ? (R)eps : rd;
        if (p.flags & TFG_POTENTIAL_SCALED) rd = rd / ((R)ri + (R)rj);
        else if (p.flags & TFG_POTENTIAL_SHIFTED) rd = rd - ((R)ri + (R)rj) + (R)p.r0_plusone;
        rr = rd < (R)p.a ? (R)p.a : rd;
    }
    const R *c = &p.cr[ind * TFG_POTENTIAL_CHUNK];
    R x = (rr - c[0]) * c[1];
    R ee = c[2] * x + c[3], eff = c[2];
    for (int k = 4; k < TFG_POTENTIAL_CHUNK; k++) {
        eff = eff * x + ee;
        ee = ee * x + c[k];
    }
    e = ee;
    f = eff * c[1] / ro;
    return true;
}

// potential_eval (no epsilon guard, int index, no range check): used by bonds.
template <typename R> static void pot_eval(const Pot<R> &p, float r2f, R &e, R &f) {
    float r = std::sqrt(r2f);
    int ind = std::max(0.0f, p.alpha[0] + r * (p.alpha[1] + r * p.alpha[2]));
    const R *c = &p.cr[ind * TFG_POTENTIAL_CHUNK];
    R rr = r;
    R x = (rr - c[0]) * c[1];
    R ee = c[2] * x + c[3], eff = c[2];
    for (int k = 4; k < TFG_POTENTIAL_CHUNK; k++) {
        eff = eff * x + ee;
        ee = ee * x + c[k];
    }
    e = ee;
    f = eff * c[1] / rr;
}

// potential_eval_r (r given directly): used by angles.
template <typename R> static bool pot_eval_r(const Pot<R> &p, float r, R &e, R &f) {
    int ind = std::max(0.0f, p.alpha[0] + r * (p.alpha[1] + r * p.alpha[2]));
    if (ind > p.n) return false;
    const R *c = &p.cr[ind * TFG_POTENTIAL_CHUNK];
    R rr = r;
    R x = (rr - c[0]) * c[1];
    R ee = c[2] * x + c[3], eff = c[2];
    for (int k = 4; k < TFG_POTENTIAL_CHUNK; k++) {
        eff = eff * x + ee;
        ee = ee * x + c[k];
    }
    e = ee;
    f = eff * c[1];
    return true;
}

static inline float dpd_gauss(uint64_t seed, int64_t step, int ida, int idb) {
    int lo = std::min(ida, idb), hi = std::max(ida, idb);
    U4 r = philox({(uint32_t)step, (uint32_t)lo, (uint32_t)hi, STREAM_DPD},
                  (uint32_t)seed, (uint32_t)(seed >> 32));
    float u1 = u01(r.x), u2 = u01(r.y);
    return std::sqrt(-2.0f * std::log(u1)) * std::cos(6.283185307179586f * u2);
}

// One interacting pair (r2 <= cutoff^2): density, flux, potential (tf_runner_dopair.cpp:172-258).
static inline uint32_t sig_mix(uint32_t id) {
    uint32_t x = id * 2654435761u + 0x9E3779B9u;
    x ^= x >> 15;
    x *= 0x85EBCA6Bu;
    x ^= x >> 13;
    return x;
}

template <typename R> static void interact(Engine<R> &e, Part<R> &pi, Part<R> &pj, const float *dx,
                                           float r2f, R &epot, double &vir) {
    // per-particle pair signature (each particle's cell is owned by the running task)
    if (e.want_sig && !e.flux_only) {
        e.sig_cnt[pi.id]++;
        e.sig_cnt[pj.id]++;
        e.sig_hash[pi.id] += sig_mix((uint32_t)pj.id);
        e.sig_hash[pj.id] += sig_mix((uint32_t)pi.id);
    }
    if (e.record_pairs && !e.flux_only) {
        std::lock_guard<std::mutex> g(e.pair_mtx);
        e.pairs.push_back({std::min(pi.id, pj.id), std::max(pi.id, pj.id)});
    }
    if (e.density && !e.flux_only) {
        float nd = Wdens<R>(r2f, e.cutoff);
        pi.f[3] += nd;
        pj.f[3] += nd;
    }
    const int idx = e.max_type * pi.type + pj.type;
    const Pot<R> &pot = e.pots[idx];
    const std::vector<tfg_flux> &fl = e.fluxes[idx];
    if (!pot.set && fl.empty()) return;
    R dxr[3] = {(R)dx[0], (R)dx[1], (R)dx[2]};
    R r2 = dxr[0] * dxr[0] + dxr[1] * dxr[1] + dxr[2] * dxr[2];
    if (sizeof(R) == sizeof(float)) r2 = r2f;

    if (!fl.empty() && e.nspec > 0) {
        // flux_eval_ex
        R r = std::sqrt(r2);
        for (const tfg_flux &F : fl) {
            R fc = F.cutoff > 0 ? (R)F.cutoff : (R)e.cutoff;
            if (r > fc) continue;
            R term = 1 - r / fc;
            term = term * term;
            Part<R> *a = pi.type == F.type_a ? &pi : &pj;
            Part<R> *b = pj.type == F.type_b ? &pj : &pi;
            R ssi = e.svec[(size_t)a->id * e.nspec + F.index_a];
            R ssj = e.svec[(size_t)b->id * e.nspec + F.index_b];
            R q = term;
            if (F.kind == TFG_FLUX_FICK) {
                q *= (R)F.coef * (ssi - ssj);
            } else if (F.kind == TFG_FLUX_SECRETE) {
                R qq = (R)F.coef * (ssi - (R)F.target);
                R scale = qq > 0.f;
                q *= scale * qq;
            } else {
                R qq = (R)F.coef * ((R)F.target - ssj) * ssi;
                R scale = qq > 0.f;
                q *= scale * qq;
            }
            R half_decay = (R)F.decay / 2.f;
            R &qi = e.sq[(size_t)a->id * e.nspec + F.index_a];
            R &qj = e.sq[(size_t)b->id * e.nspec + F.index_b];
            qi = qi - q - half_decay * ssi;
            qj = qj + q - half_decay * ssj;
        }
    }
    if (!pot.set || e.flux_only) return;
    if (pot.kind == TFG_POTENTIAL_KIND_DPD) {
        // dpd_eval
        const float eps = FLT_EPSILON;
        const R delta = (R)(1.f / std::sqrt(e.dt));
        R r = std::sqrt(r2);
        R ro = r < (R)eps ? (R)eps : r;
        if (pot.flags & TFG_POTENTIAL_SHIFTED) r = r - ((R)pi.radius + (R)pj.radius);
        if (r > (R)pot.b) return;
        r = r >= (R)pot.a ? r : (R)pot.a;
        R ev[3] = {dxr[0] / ro, dxr[1] / ro, dxr[2] / ro};
        R vv[3] = {(R)pi.v[0] - (R)pj.v[0], (R)pi.v[1] - (R)pj.v[1], (R)pi.v[2] - (R)pj.v[2]};
        R omega_c = r < 0.f ? (R)1 : (1 - r / (R)pot.b);
        R fc = (R)pot.dalpha * omega_c;
        R omega_d = omega_c * omega_c;
        R edv = ev[0] * vv[0] + ev[1] * vv[1] + ev[2] * vv[2];
        R fd = -(R)pot.dgamma * omega_d * edv;
        R xi = e.ref_dpd_random ? (R)1 : (R)dpd_gauss(e.d.seed, e.time, pi.id, pj.id);
        R fr = (R)pot.dsigma * omega_c * xi * delta;
        R f = fc + fd + fr;
        for (int k = 0; k < 3; k++) {
            pj.f[k] = pj.f[k] - f * ev[k];
            pi.f[k] = pi.f[k] + f * ev[k];
        }
        pi.fmag += std::fabs((double)f);
        pj.fmag += std::fabs((double)f);
        // virial: f_ij . r_ij with r_ij = ev * ro
        vir += (double)f * (double)ro;
        return;
    }
    R ee, f;
    if (pot_eval_ex(pot, pi.radius, pj.radius, r2f, r2, ee, f)) {
        for (int k = 0; k < 3; k++) {
            R w = f * dxr[k];
            pi.f[k] -= w;
            pj.f[k] += w;
        }
        double mag = std::fabs((double)f) * std::sqrt((double)r2);
        pi.fmag += mag;
        pj.fmag += mag;
        epot += ee;
        vir += -(double)f * (double)r2;
    }
}

template <typename R> static void do_sort(Engine<R> &e, int cid) {
    Cell<R> &c = e.cells[cid];
    int count = (int)c.parts.size();
    c.sortlist.assign((size_t)13 * count, 0u);
    if (count == 0) return;
    float bias = std::sqrt(e.h[0] * e.h[0] + e.h[1] * e.h[1] + e.h[2] * e.h[2]);
    float dscale = (float)SHRT_MAX / (2 * bias);
    int flags = e.sortflags[cid];
    for (int sid = 0; sid < 13; sid++) {
        if (!(flags & (1 << sid))) continue;
        const float *sn = &kShiftN[3 * sid];
        unsigned *ip = &c.sortlist[(size_t)count * sid];
        for (int i = 0; i < count; i++) {
            const Part<R> &p = c.parts[i];
            ip[i] = ((unsigned)i << 16) |
                    (unsigned)(dscale * (bias + p.x[0] * sn[0] + p.x[1] * sn[1] + p.x[2] * sn[2]));
        }
        std::sort(ip, ip + count, [](unsigned a, unsigned b) { return (a & 0xffff) > (b & 0xffff); });
    }
}

template <typename R> static void do_pair(Engine<R> &e, int ci0, int cj0, R &epot_out) {
    int ci = ci0, cj = cj0;
    Cell<R> &A0 = e.cells[ci], &B0 = e.cells[cj];
    if (A0.parts.empty() || B0.parts.empty()) return;
    float shift[3];
    int sid = getsid(e, ci, cj, shift);
    Cell<R> &A = e.cells[ci], &B = e.cells[cj];
    int ni = (int)A.parts.size(), nj = (int)B.parts.size();
    R epot = 0;
    double vir = 0;
    if (e.brute) {
        for (int i = 0; i < ni; i++) {
            Part<R> &pi = A.parts[i];
            float pix[3] = {pi.x[0] - shift[0], pi.x[1] - shift[1], pi.x[2] - shift[2]};
            for (int j = 0; j < nj; j++) {
                Part<R> &pj = B.parts[j];
                float dx[3] = {pix[0] - pj.x[0], pix[1] - pj.x[1], pix[2] - pj.x[2]};
                float r2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
                if (r2 > e.cutoff2) continue;
                interact(e, pi, pj, dx, r2, epot, vir);
            }
        }
    } else {
        float bias = std::sqrt(e.h[0] * e.h[0] + e.h[1] * e.h[1] + e.h[2] * e.h[2]);
        float dscale = (float)SHRT_MAX / (2 * bias);
        int dmaxdist = 2 + dscale * (e.cutoff + 2 * e.verlet_maxdx);   // tf_runner_dopair.cpp:115-117
        float nshift = std::sqrt(shift[0] * shift[0] + shift[1] * shift[1] + shift[2] * shift[2]);
        int dnshift = dscale * nshift;
        const unsigned *ip = &A.sortlist[(size_t)ni * sid];
        const unsigned *jp = &B.sortlist[(size_t)nj * sid];
        for (int i = 0; i < ni; i++) {
            // unsigned arithmetic as in the reference: a negative gap wraps and ends the loop
            if ((jp[nj - 1] & 0xffff) + dnshift - (ip[i] & 0xffff) > (unsigned)dmaxdist) {
                if (i == 0 && (int)((jp[nj - 1] & 0xffff) + dnshift - (ip[i] & 0xffff)) < 0) e.window_skips++;
                break;
            }
            Part<R> &pi = A.parts[ip[i] >> 16];
            float pix[3] = {pi.x[0] - shift[0], pi.x[1] - shift[1], pi.x[2] - shift[2]};
            for (int j = nj - 1; j >= 0 && (jp[j] & 0xffff) + dnshift - (ip[i] & 0xffff) < (unsigned)dmaxdist; j--) {
                Part<R> &pj = B.parts[jp[j] >> 16];
                float dx[3] = {pix[0] - pj.x[0], pix[1] - pj.x[1], pix[2] - pj.x[2]};
                float r2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
                if (r2 > e.cutoff2) continue;
                interact(e, pi, pj, dx, r2, epot, vir);
            }
        }
    }
    A.epot += epot;
    A.virial += vir;
    epot_out += epot;
}

template <typename R> static void add_random_force(Engine<R> &e, Part<R> &p) {
    int t = p.type;
    if (e.rf_std[t] <= 0.f) return;
    if ((e.time + p.id) % e.rf_dur[t] == 0) {
        U4 r = philox({(uint32_t)e.time, (uint32_t)p.id, 0u, STREAM_FORCE},
                      (uint32_t)e.d.seed, (uint32_t)(e.d.seed >> 32));
        float theta = 6.283185307179586f * u01(r.x);
        float phi = std::acos(1.f - 2.f * u01(r.y));
        float g = std::sqrt(-2.0f * std::log(u01(r.z))) * std::cos(6.283185307179586f * u01(r.w));
        float rr = e.rf_mean[t] + e.rf_std[t] * g;
        p.pf[0] = rr * std::sin(phi) * std::cos(theta);
        p.pf[1] = rr * std::sin(phi) * std::sin(theta);
        p.pf[2] = rr * std::cos(phi);
    }
    for (int k = 0; k < 3; k++) p.f[k] += p.pf[k];
    p.fmag += std::sqrt((double)p.pf[0] * p.pf[0] + (double)p.pf[1] * p.pf[1] + (double)p.pf[2] * p.pf[2]);
}

static inline float wall_gauss(uint64_t seed, int64_t step, int id, int wall) {
    U4 r = philox({(uint32_t)step, (uint32_t)id, (uint32_t)wall, STREAM_WALL}, (uint32_t)seed, (uint32_t)(seed >> 32));
    float u1 = u01(r.x), u2 = u01(r.y);
    return std::sqrt(-2.0f * std::log(u1)) * std::cos(6.283185307179586f * u2);
}

template <typename R> static bool on_wall(const Engine<R> &e, int w, const int *loc) {
    const unsigned active = TFG_BOUNDARY_FREESLIP | TFG_BOUNDARY_VELOCITY | TFG_BOUNDARY_POTENTIAL;
    if (!(e.walls[w].kind & active)) return false;
    const int ax = w >> 1;
    return (w & 1) ? loc[ax] + 1 == e.cdim[ax] : loc[ax] == 0;
}

// Periodic wall flag of a cell along axis k (space_init, tfSpace.cpp:812-830): the low
// wall's at index 0 when that wall is PERIODIC, else the high wall's at index cdim-1; -1 none.
template <typename R> static int periodic_side(const Engine<R> &e, int k, int l) {
    if (l == 0 && (e.walls[2 * k].kind & TFG_BOUNDARY_PERIODIC)) return 0;
    if (l + 1 == e.cdim[k] && (e.walls[2 * k + 1].kind & TFG_BOUNDARY_PERIODIC)) return 1;
    return -1;
}

// apply_boundary_particle_crossing (tfBoundaryConditions.cpp:676-735): for the axes whose
// cell index changes, in order x, y, z, on a periodic axis, with both cells flagged periodic
// on that axis, the destination's wall decides; the state vector is reset once.
template <typename R> static bool crossing_resets(const Engine<R> &e, const int *src, const int *dst) {
    for (int k = 0; k < 3; k++) {
        if (src[k] == dst[k] || !((e.periodic >> k) & 1u)) continue;
        const int ss = periodic_side(e, k, src[k]), ds = periodic_side(e, k, dst[k]);
        if (ss < 0 || ds < 0) continue;
        if (e.walls[2 * k + ds].kind & TFG_BOUNDARY_RESETTING) return true;
    }
    return false;
}

// boundary_eval (tf_boundary_eval.h:192-254) with boundary_potential_eval_ex (:146-188) and
// dpd_boundary_eval (tf_dpd_eval.h:78-120): wall potentials of particle p in cell c.
template <typename R> static void boundary_eval(Engine<R> &e, const Cell<R> &c, Part<R> &p, R &epot) {
    for (int w = 0; w < 6; w++) {
        if (!on_wall(e, w, c.loc)) continue;
        const Pot<R> &pot = e.wpots[w * e.max_type + p.type];
        if (!pot.set) continue;
        const int ax = w >> 1;
        float r = (w & 1) ? e.h[ax] - p.x[ax] : p.x[ax];
        if (!(r <= pot.b)) continue;
        const float dxa = (w & 1) ? -r : r;
        const float r2 = r * r;
        if (pot.kind == TFG_POTENTIAL_KIND_DPD) {
            const float eps = FLT_EPSILON;
            const R delta = (R)(1.f / std::sqrt(e.dt));
            R rr = std::sqrt((R)r2);
            R ro = rr < (R)eps ? (R)eps : rr;
            if (pot.flags & TFG_POTENTIAL_SHIFTED) rr = rr - ((R)p.radius + (R)e.walls[w].radius);
            if (rr > (R)pot.b) continue;
            rr = rr >= (R)pot.a ? rr : (R)pot.a;
            R ea = (R)dxa / ro;
            R va = (R)p.v[ax] - (R)e.walls[w].velocity[ax];
            R omega_c = rr < 0 ? (R)1 : (1 - rr / (R)pot.b);
            R xi = e.ref_dpd_random ? (R)1 : (R)wall_gauss(e.d.seed, e.time, p.id, w);
            R f = (R)pot.dalpha * omega_c - (R)pot.dgamma * omega_c * omega_c * (ea * va) +
                  (R)pot.dsigma * omega_c * xi * delta;
            p.f[ax] += f * ea;
            p.fmag += std::fabs((double)f);
        } else {
            R ee, f;
            if (pot_eval_ex(pot, p.radius, e.walls[w].radius, r2, (R)r2, ee, f)) {
                p.f[ax] -= f * (R)dxa;
                p.fmag += std::fabs((double)f * dxa);
                epot += ee;
            }
        }
    }
}

template <typename R> static void do_self(Engine<R> &e, int cid, R &epot_out) {
    Cell<R> &c = e.cells[cid];
    int count = (int)c.parts.size();
    R epot = 0;
    double vir = 0;
    for (int i = 0; i < count; i++) {
        Part<R> &pi = c.parts[i];
        if (!e.flux_only) {
            add_random_force(e, pi);
            boundary_eval(e, c, pi, epot);
        }
        for (int j = i + 1; j < count; j++) {
            Part<R> &pj = c.parts[j];
            float dx[3] = {pi.x[0] - pj.x[0], pi.x[1] - pj.x[1], pi.x[2] - pj.x[2]};
            float r2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
            if (r2 > e.cutoff2) continue;
            interact(e, pi, pj, dx, r2, epot, vir);
        }
    }
    c.epot += epot;
    c.virial += vir;
    epot_out += epot;
}

template <typename R> static void rebuild_index(Engine<R> &e) {
    e.where_cell.assign(e.nparts, -1);
    e.where_slot.assign(e.nparts, -1);
    for (int c = 0; c < e.ncells; c++)
        for (int s = 0; s < (int)e.cells[c].parts.size(); s++) {
            int id = e.cells[c].parts[s].id;
            e.where_cell[id] = c;
            e.where_slot[id] = s;
        }
}

template <typename R> static Part<R> &part_of(Engine<R> &e, int id) {
    return e.cells[e.where_cell[id]].parts[e.where_slot[id]];
}

// bond_eval (tfBond.cpp:97-345), harmonic-style table potentials only.
template <typename R> static void eval_bonds(Engine<R> &e) {
    R epot = 0;
    for (const BondRec &b : e.bonds) {
        const Pot<R> &pot = e.bpots[b.slot];
        if (!pot.set) continue;
        Part<R> &pi = part_of(e, b.i), &pj = part_of(e, b.j);
        const int *li = e.cells[e.where_cell[b.i]].loc, *lj = e.cells[e.where_cell[b.j]].loc;
        float pix[3];
        for (int k = 0; k < 3; k++) {
            int s = li[k] - lj[k];
            if (s > 1) s = -1;
            else if (s < -1) s = 1;
            pix[k] = pi.x[k] + e.h[k] * s;
        }
        float dx[3] = {pix[0] - pj.x[0], pix[1] - pj.x[1], pix[2] - pj.x[2]};
        float r2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
        // potential_eval_adjust_distance2
        float r = std::sqrt(r2);
        if (pot.flags & TFG_POTENTIAL_SCALED) r = r / (pi.radius + pj.radius);
        else if (pot.flags & TFG_POTENTIAL_SHIFTED) r = r - (pi.radius + pj.radius) + pot.r0_plusone;
        float _r2 = r * r;
        if (_r2 > pot.b * pot.b) continue;
        _r2 = std::fmax(_r2, pot.a * pot.a);
        R ee, eff;
        pot_eval(pot, _r2, ee, eff);
        for (int k = 0; k < 3; k++) {
            R w = eff * (R)dx[k];
            pi.f[k] -= w;
            pj.f[k] += w;
        }
        double bm = std::fabs((double)eff) * std::sqrt((double)r2);
        pi.fmag += bm;
        pj.fmag += bm;
        epot += ee;
        e.virial += -(double)eff * (double)r2;
    }
    e.epot_bond = epot;
}

// angle_eval (tfAngle.cpp:90-382).
template <typename R> static void eval_angles(Engine<R> &e) {
    R epot = 0;
    for (size_t aid = 0; aid < e.angles.size(); aid++) {
        const AngleRec &A = e.angles[aid];
        const Pot<R> &pot = e.bpots[A.slot];
        if (!pot.set) continue;
        Part<R> &pi = part_of(e, A.i), &pj = part_of(e, A.j), &pk = part_of(e, A.k);
        const int *li = e.cells[e.where_cell[A.i]].loc, *lj = e.cells[e.where_cell[A.j]].loc,
                  *lk = e.cells[e.where_cell[A.k]].loc;
        float xi[3], xj[3], xk[3];
        for (int k = 0; k < 3; k++) {
            xj[k] = pj.x[k];
            int s = li[k] - lj[k];
            if (s > 1) s = -1;
            else if (s < -1) s = 1;
            xi[k] = pi.x[k] + s * e.h[k];
            s = lk[k] - lj[k];
            if (s > 1) s = -1;
            else if (s < -1) s = 1;
            xk[k] = pk.x[k] + s * e.h[k];
        }
        float rji[3], rjk[3];
        for (int k = 0; k < 3; k++) { rji[k] = xi[k] - xj[k]; rjk[k] = xk[k] - xj[k]; }
        float dprod = rji[0] * rjk[0] + rji[1] * rjk[1] + rji[2] * rjk[2];
        float inji = 1.0f / std::sqrt(rji[0] * rji[0] + rji[1] * rji[1] + rji[2] * rji[2]);
        float injk = 1.0f / std::sqrt(rjk[0] * rjk[0] + rjk[1] * rjk[1] + rjk[2] * rjk[2]);
        float ctheta = std::fmax(-1.0f, std::fmin(1.0f, dprod * inji * injk));
        float dxi[3], dxk[3];
        if (ctheta == 0 || ctheta == -1) {
            // The reference draws this plane from the global mt19937; here a Philox stream.
            e.straight_angles++;
            U4 r = philox({(uint32_t)e.time, (uint32_t)aid, 0u, STREAM_ANGLE},
                          (uint32_t)e.d.seed, (uint32_t)(e.d.seed >> 32));
            float x[3] = {2.f * u01(r.x) - 1.f, 2.f * u01(r.y) - 1.f, 2.f * u01(r.z) - 1.f};
            float vik[3] = {xi[0] - xk[0], xi[1] - xk[1], xi[2] - xk[2]};
            float dd = x[0] * vik[0] + x[1] * vik[1] + x[2] * vik[2];
            for (int k = 0; k < 3; k++) x[k] = x[k] - dd * vik[k];
            float len = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
            for (int k = 0; k < 3; k++) dxi[k] = dxk[k] = x[k] / len;
        } else {
            for (int k = 0; k < 3; k++) {
                dxi[k] = (rjk[k] * injk - ctheta * rji[k] * inji) * inji;
                dxk[k] = (rji[k] * inji - ctheta * rjk[k] * injk) * injk;
            }
        }
        if (ctheta > pot.b) continue;
        R ee, eff;
        if (!pot_eval_r(pot, std::fmax(ctheta, pot.a), ee, eff)) continue;
        double mi = 0, mk = 0;
        for (int k = 0; k < 3; k++) {
            R wi = eff * (R)dxi[k], wk = eff * (R)dxk[k];
            pi.f[k] -= wi;
            pk.f[k] -= wk;
            pj.f[k] += wi + wk;
            mi += (double)wi * wi;
            mk += (double)wk * wk;
        }
        pi.fmag += std::sqrt(mi);
        pk.fmag += std::sqrt(mk);
        pj.fmag += std::sqrt(mi) + std::sqrt(mk);
        epot += ee;
    }
    e.epot_angle = epot;
}

// space_prepare: f = force_i, number density = W(0).
template <typename R> static void prepare(Engine<R> &e) {
    const float self_nd = Wdens<R>(0.f, e.cutoff);
    for (auto &c : e.cells) {
        c.epot = 0;
        c.computed_volume = 0;
        c.virial = 0;
        for (auto &p : c.parts) {
            for (int k = 0; k < 3; k++) p.f[k] = p.fi[k];
            p.f[3] = self_nd;
            p.fmag = std::sqrt((double)p.fi[0] * p.fi[0] + (double)p.fi[1] * p.fi[1] + (double)p.fi[2] * p.fi[2]);
        }
    }
    e.epot_nonbond = e.epot_bond = e.epot_angle = 0;
    e.virial = 0;
    e.sig_cnt.assign(e.nparts, 0);
    e.sig_hash.assign(e.nparts, 0u);
}

// space_shuffle_local + space_cell_welcome.
template <typename R> static void shuffle(Engine<R> &e) {
    for (int cid = 0; cid < e.ncells; cid++) {
        Cell<R> &c = e.cells[cid];
        size_t pid = 0;
        while (pid < c.parts.size()) {
            Part<R> &p = c.parts[pid];
            int delta[3];
            for (int k = 0; k < 3; k++)
                delta[k] = std::isgreaterequal(p.x[k], e.h[k]) - std::isless(p.x[k], 0.0f);
            if (delta[0] || delta[1] || delta[2]) {
                for (int k = 0; k < 3; k++) p.x[k] -= delta[k] * e.h[k];
                int dest = cellid(e, (c.loc[0] + delta[0] + e.cdim[0]) % e.cdim[0],
                                  (c.loc[1] + delta[1] + e.cdim[1]) % e.cdim[1],
                                  (c.loc[2] + delta[2] + e.cdim[2]) % e.cdim[2]);
                e.cells[dest].incoming.push_back(p);
                c.parts[pid] = c.parts.back();
                c.parts.pop_back();
            } else {
                pid++;
            }
        }
    }
    for (auto &c : e.cells) {
        for (auto &p : c.incoming) c.parts.push_back(p);
        c.incoming.clear();
    }
}

// Parallel for over [0, n) with `threads` workers taking chunks of `chunk` items.
template <typename F> static void par_for(int threads, size_t n, size_t chunk, F fn) {
    if (threads <= 1 || n <= chunk) {
        for (size_t k = 0; k < n; k++) fn(k);
        return;
    }
    std::atomic<size_t> next(0);
    std::vector<std::thread> th;
    int nt = (int)std::min<size_t>(threads, (n + chunk - 1) / chunk);
    for (int t = 0; t < nt; t++)
        th.emplace_back([&]() {
            for (;;) {
                size_t k0 = next.fetch_add(chunk);
                if (k0 >= n) return;
                size_t k1 = std::min(n, k0 + chunk);
                for (size_t k = k0; k < k1; k++) fn(k);
            }
        });
    for (auto &t : th) t.join();
}

// Colour of a coordinate: residue mod 3 for the first 3*floor(n/3) cells, unique colours
// for the (at most two) trailing cells, so that equal colours are >= 3 apart with wrap.
static inline int axis_colour(int x, int n) {
    int m = 3 * (n / 3);
    return x < m ? x % 3 : 3 + (x - m);
}

// Nonbonded pass.  A pair task's owner is its cell_i (the cell whose shift to cell_j is
// lexicographically positive); an owner touches itself and its 13 forward neighbours,
// i.e. x in [x, x+1], y and z in [-1, +1].  Owners of one colour class therefore touch
// disjoint cells and run concurrently without locks; classes run one after another.
// This gives the reference runners' per-cell exclusion (tfRunner.cpp:204-380) with a
// deterministic task order.
template <typename R> static void nonbond(Engine<R> &e) {
    // sort tasks run only while a Verlet rebuild is due (tfRunner.cpp:314; without the
    // Verlet flag verlet_rebuild stays set); between rebuilds the windows of the last sort
    // are widened by 2 maxdx
    if (!e.verlet || e.verlet_rebuild)
        par_for(e.nthreads, (size_t)e.ncells, 64, [&](size_t cid) { do_sort(e, (int)cid); });
    if (e.owned.empty()) {
        e.owned.assign(e.ncells, std::vector<int>());
        for (size_t k = 0; k < e.tasks.size(); k++) e.owned[e.tasks[k].i].push_back((int)k);
        std::vector<std::vector<int>> cls(125);
        for (int c = 0; c < e.ncells; c++) {
            const int *l = e.cells[c].loc;
            int col = (axis_colour(l[0], e.cdim[0]) * 5 + axis_colour(l[1], e.cdim[1])) * 5 +
                      axis_colour(l[2], e.cdim[2]);
            cls[col].push_back(c);
        }
        for (auto &v : cls)
            if (!v.empty()) e.colour_classes.push_back(v);
    }
    std::vector<R> cell_epot(e.ncells, (R)0);
    for (const auto &cls : e.colour_classes) {
        par_for(e.nthreads, cls.size(), 8, [&](size_t q) {
            int owner = cls[q];
            R ep = 0;
            for (int k : e.owned[owner]) {
                const Task &t = e.tasks[k];
                if (t.type == 0) do_self(e, t.i, ep);
                else do_pair(e, t.i, t.j, ep);
            }
            cell_epot[owner] = ep;
        });
    }
    R epot = 0;
    for (R v : cell_epot) epot += v;
    e.epot_nonbond = epot;
    for (auto &c : e.cells) e.virial += c.virial;
}

// cell_advance_forward_euler for one cell; migrating particles go to the incoming list
// of their destination (tf_engine_advance.cpp:140-247), then Fluxes_integrate (tfFlux.cpp:188).
template <typename R> static void advance_cell(Engine<R> &e, int cid, const float *maxv, const float *maxv2,
                                              const float *maxx, const float *maxx2, int *err) {
    Cell<R> &c = e.cells[cid];
    float dt = e.dt;
    float h2[3] = {(float)(2. * e.h[0]), (float)(2. * e.h[1]), (float)(2. * e.h[2])};
    size_t pid = 0;
    R cv = 0;
    while (pid < c.parts.size()) {
        Part<R> &p = c.parts[pid];
        if ((p.flags & TFG_PARTICLE_FROZEN_X) && (p.flags & TFG_PARTICLE_FROZEN_Y) &&
            (p.flags & TFG_PARTICLE_FROZEN_Z)) {
            pid++;
            continue;
        }
        float mask[3] = {(p.flags & TFG_PARTICLE_FROZEN_X) ? 0.0f : 1.0f,
                         (p.flags & TFG_PARTICLE_FROZEN_Y) ? 0.0f : 1.0f,
                         (p.flags & TFG_PARTICLE_FROZEN_Z) ? 0.0f : 1.0f};
        int delta[3];
        float fx[3] = {(float)p.f[0], (float)p.f[1], (float)p.f[2]};
        if (e.dyn[p.type] == TFG_NEWTONIAN) {
            for (int k = 0; k < 3; k++) {
                float v = mask[k] * (p.v[k] + dt * fx[k] * p.imass);
                p.v[k] = v * v <= maxv2[k] ? v : v / std::fabs(v) * maxv[k];
                p.x[k] += dt * p.v[k];
                delta[k] = std::isgreaterequal(p.x[k], e.h[k]) - std::isless(p.x[k], 0.0f);
            }
        } else {
            for (int k = 0; k < 3; k++) {
                float dx = mask[k] * (dt * fx[k] * p.imass);
                dx = dx * dx <= maxx2[k] ? dx : dx / std::fabs(dx) * maxx[k];
                p.v[k] = dx / dt;
                p.x[k] += dx;
                delta[k] = std::isgreaterequal(p.x[k], e.h[k]) - std::isless(p.x[k], 0.0f);
            }
        }
        float nd = (float)p.f[3];
        p.v[3] = nd > 0.f ? 1.f / nd : 0.f;
        if (delta[0] || delta[1] || delta[2]) {
            // apply_update_pos_vel (tf_boundary_eval.h:46-134): reflect at FREESLIP / VELOCITY walls
            bool enforced = false;
            for (int w = 0; w < 6; w++) {
                const tfg_boundary &bw = e.walls[w];
                if (!(bw.kind & (TFG_BOUNDARY_FREESLIP | TFG_BOUNDARY_VELOCITY)) || !on_wall(e, w, c.loc)) continue;
                const int ax = w >> 1;
                const bool high = (w & 1) != 0;
                if (high ? !(p.x[ax] >= e.h[ax]) : !(p.x[ax] <= 0)) continue;
                const bool slip = (bw.kind & TFG_BOUNDARY_FREESLIP) != 0;
                const float rest = slip ? 1.0f : bw.restore;
                if (high) p.x[ax] = e.h[ax] - std::max<float>((p.x[ax] - e.h[ax]) * rest, FLT_EPSILON);
                else p.x[ax] = std::max<float>(-p.x[ax] * rest, 0.0f);
                if (slip) {
                    p.v[ax] *= -1.0f;
                } else {
                    for (int k = 0; k < 3; k++) p.v[k] = bw.velocity[k] - ((p.v[k] - bw.velocity[k]) * rest);
                }
                enforced = true;
            }
            if (enforced)
                for (int k = 0; k < 3; k++)
                    delta[k] = std::isgreaterequal(p.x[k], e.h[k]) - std::isless(p.x[k], 0.0f);
        }
        if (delta[0] || delta[1] || delta[2]) {
            for (int k = 0; k < 3; k++) {
                if (p.x[k] >= h2[k] || p.x[k] <= -e.h[k]) { *err = TFG_E_TOOFAST; break; }
                float dx = -delta[k] * e.h[k];
                p.x[k] += dx;
            }
            int dest = cellid(e, (c.loc[0] + delta[0] + e.cdim[0]) % e.cdim[0],
                              (c.loc[1] + delta[1] + e.cdim[1]) % e.cdim[1],
                              (c.loc[2] + delta[2] + e.cdim[2]) % e.cdim[2]);
            Cell<R> &cd = e.cells[dest];
            // apply_boundary_particle_crossing (tfBoundaryConditions.cpp:676-735)
            if (e.nspec > 0 && crossing_resets(e, c.loc, cd.loc))
                for (int s = 0; s < e.nspec; s++) e.svec[(size_t)p.id * e.nspec + s] = e.species_reset[s];
            {
                std::lock_guard<std::mutex> g(cd.mtx);
                cd.incoming.push_back(p);
                cd.computed_volume += p.v[3];
            }
            e.migrated[p.id] = 1;
            c.parts[pid] = c.parts.back();
            c.parts.pop_back();
        } else {
            cv += p.v[3];
            pid++;
        }
    }
    c.computed_volume = cv;
    // Fluxes_integrate over the particles now in the cell (migrants are deferred).
    if (e.nspec > 0) {
        for (auto &p : c.parts) {
            for (int s = 0; s < e.nspec; s++) {
                float konst = (e.species_flags[s] & 1u) ? 0.f : 1.f;
                float &fv = e.svec[(size_t)p.id * e.nspec + s];
                R &q = e.sq[(size_t)p.id * e.nspec + s];
                fv = std::fmax(0.0f, fv + e.dt_flux * (float)q * konst);
                q = 0;
            }
        }
    }
}

template <typename R> static int advance(Engine<R> &e) {
    float maxx[3], maxx2[3], maxv[3], maxv2[3];
    for (int k = 0; k < 3; k++) {
        maxx[k] = e.h[k] * e.d.particle_max_dist_fraction;
        maxx2[k] = maxx[k] * maxx[k];
        maxv[k] = maxx[k] / e.dt;
        maxv2[k] = maxv[k] * maxv[k];
    }
    e.migrated.assign(e.nparts, 0);
    int err = TFG_OK;
    // 3x3x3-staggered cell order (tf_engine_advance.cpp:122-136); within one stagger
    // class no two cells share a neighbour, so they may run concurrently.
    for (int ii = 0; ii < 3; ii++)
        for (int jj = 0; jj < 3; jj++)
            for (int kk = 0; kk < 3; kk++) {
                std::vector<int> ids;
                for (int i = ii; i < e.cdim[0]; i += 3)
                    for (int j = jj; j < e.cdim[1]; j += 3)
                        for (int k = kk; k < e.cdim[2]; k += 3) ids.push_back(cellid(e, i, j, k));
                if (e.nthreads <= 1) {
                    for (int cid : ids) advance_cell(e, cid, maxv, maxv2, maxx, maxx2, &err);
                } else {
                    std::atomic<size_t> next(0);
                    std::vector<int> errs(e.nthreads, TFG_OK);
                    std::vector<std::thread> th;
                    for (int t = 0; t < e.nthreads; t++)
                        th.emplace_back([&, t]() {
                            for (;;) {
                                size_t k = next.fetch_add(16);
                                if (k >= ids.size()) return;
                                size_t lim = std::min(ids.size(), k + 16);
                                for (size_t q = k; q < lim; q++)
                                    advance_cell(e, ids[q], maxv, maxv2, maxx, maxx2, &errs[t]);
                            }
                        });
                    for (auto &t : th) t.join();
                    for (int v : errs) if (v != TFG_OK) err = v;
                }
            }
    int64_t mig = 0;
    double cvol = 0;
    for (auto &c : e.cells) {
        mig += (int64_t)c.incoming.size();
        for (auto &p : c.incoming) c.parts.push_back(p);
        c.incoming.clear();
        cvol += (double)c.computed_volume;
    }
    e.migrations = mig;
    e.computed_volume = cvol;
    return err;
}

template <typename R> static void kinetic(Engine<R> &e) {
    double ke = 0;
    for (auto &c : e.cells)
        for (auto &p : c.parts)
            ke += 0.5 * e.mass[p.type] * ((double)p.v[0] * p.v[0] + (double)p.v[1] * p.v[1] + (double)p.v[2] * p.v[2]);
    e.kinetic = ke;
}

template <typename R> static int force_all(Engine<R> &e, bool bonded) {
    nonbond(e);
    if (bonded && (!e.bonds.empty() || !e.angles.empty())) {
        rebuild_index(e);
        if (!e.bonds.empty()) eval_bonds(e);
        if (!e.angles.empty()) eval_angles(e);
    }
    return TFG_OK;
}

// Flux substeps of engine_advance_forward_euler (tf_engine_advance.cpp:314-323): before the
// step's force evaluation, nr_fluxsteps-1 times a flux-only pass over the same tasks
// (engine_fluxonly_eval, tfEngine.cpp:1358-1376; runner_dopair_fluxonly / runner_doself_fluxonly,
// tf_runner_dopair.cpp:334-419, 760-819) followed by Fluxes_integrate over every cell.
template <typename R> static void flux_substeps(Engine<R> &e) {
    if (e.nr_fluxsteps <= 1 || e.nspec == 0) return;
    for (int sub = 0; sub < e.nr_fluxsteps - 1; sub++) {
        e.flux_only = true;
        const R ep = e.epot_nonbond;
        const double vir = e.virial;
        nonbond(e);
        e.epot_nonbond = ep;
        e.virial = vir;
        e.flux_only = false;
        for (auto &c : e.cells)
            for (auto &p : c.parts)
                for (int s = 0; s < e.nspec; s++) {
                    float konst = (e.species_flags[s] & 1u) ? 0.f : 1.f;
                    float &fv = e.svec[(size_t)p.id * e.nspec + s];
                    R &q = e.sq[(size_t)p.id * e.nspec + s];
                    fv = std::fmax(0.0f, fv + e.dt_flux * (float)q * konst);
                    q = 0;
                }
    }
}

// engine_verlet_update (tfEngine.cpp:214-354): unless a rebuild is already due, the largest
// displacement since the last rebuild, measured as the OpenMP branch does (:239-252; the
// default branch sums into a shadowing int and so always finds 0); rebuild when twice it
// exceeds the skin, by re-binning (engine_shuffle) and storing the reference positions.
template <typename R> static void verlet_update(Engine<R> &e) {
    if (!e.verlet_rebuild) {
        float m2 = 0.f;
        for (auto &c : e.cells)
            for (auto &p : c.parts) {
                float dx = 0.0f;
                for (int k = 0; k < 3; k++) {
                    const float w = p.x[k] - p.ox[k];
                    dx += w * w;
                }
                m2 = std::fmax(dx, m2);
            }
        const float m = std::sqrt(m2);
        e.verlet_rebuild = 2.0 * m > e.skin;
        e.verlet_maxdx = m;
    }
    if (e.verlet_rebuild) {
        shuffle(e);
        for (auto &c : e.cells)
            for (auto &p : c.parts)
                for (int k = 0; k < 3; k++) p.ox[k] = p.x[k];
        e.verlet_maxdx = 0.f;
        e.verlet_rebuilds++;
    }
}

// The Verlet branch of engine_advance_forward_euler (tf_engine_advance.cpp:367-427): no
// frozen mask, velocity clamp, wall reflection, migration or flux integration; the
// computed volume sums the cells' values, which space_prepare zeroed.
template <typename R> static int advance_verlet(Engine<R> &e) {
    const float dt = e.dt;
    for (auto &c : e.cells)
        for (auto &p : c.parts) {
            const float fx[3] = {(float)p.f[0], (float)p.f[1], (float)p.f[2]};
            if (e.dyn[p.type] == TFG_NEWTONIAN) {
                for (int k = 0; k < 3; k++) {
                    p.v[k] += fx[k] * dt * p.imass;
                    p.x[k] += p.v[k] * dt;
                }
            } else {
                for (int k = 0; k < 3; k++) {
                    p.v[k] = fx[k] * p.imass;
                    p.x[k] += p.v[k] * dt;
                }
            }
        }
    e.migrations = 0;
    e.computed_volume = 0;
    return TFG_OK;
}

template <typename R> static int step(Engine<R> &e) {
    e.time += 1;
    kinetic(e);
    prepare(e);
    if (e.verlet) verlet_update(e);
    else shuffle(e);
    flux_substeps(e);
    force_all(e, true);
    if (e.verlet) {
        e.verlet_rebuild = false;   // engine_force, tfEngine.cpp:1539-1540
        return advance_verlet(e);
    }
    return advance(e);
}

// ---------------- type-erased handle ----------------
struct Handle {
    bool fp64 = false;
    Engine<float> *f32 = nullptr;
    Engine<double> *f64 = nullptr;
    std::string err;
};

template <typename R> static int load_common(Engine<R> &e, int n, const float *v, const int32_t *type,
                                             const float *radius, const float *imass, const uint32_t *flags,
                                             const float *species, const float *force_i,
                                             const int32_t *cellv, const float *xrel) {
    e.nparts = n;
    e.svec.assign((size_t)n * e.nspec, 0.0f);
    e.sq.assign((size_t)n * e.nspec, (R)0);
    for (auto &c : e.cells) c.parts.clear();
    for (int i = 0; i < n; i++) {
        Part<R> p;
        std::memset(&p, 0, sizeof(p));
        p.id = i;
        p.type = type ? type[i] : 0;
        if (p.type < 0 || p.type >= e.max_type) return TFG_E_INVAL;
        p.radius = radius ? radius[i] : 1.0f;
        p.imass = imass ? imass[i] : 1.0f;
        p.flags = flags ? flags[i] : 0u;
        for (int k = 0; k < 3; k++) {
            p.v[k] = v ? v[3 * i + k] : 0.f;
            p.fi[k] = force_i ? force_i[3 * i + k] : 0.f;
            p.x[k] = xrel[3 * i + k];
        }
        if (species)
            for (int s = 0; s < e.nspec; s++) e.svec[(size_t)i * e.nspec + s] = species[(size_t)i * e.nspec + s];
        int c = cellv[i];
        if (c < 0 || c >= e.ncells) return TFG_E_RANGE;
        e.cells[c].parts.push_back(p);
    }
    e.time = 0;
    e.verlet_rebuild = true;   // engine_start (tfEngine.cpp:1238-1263)
    e.verlet_maxdx = 0.f;
    e.verlet_rebuilds = 0;
    return TFG_OK;
}

// space_setpartp: clamp into the domain, bin, make the position cell-relative.
template <typename R> static int bin_global(const Engine<R> &e, int n, const float *x, std::vector<int32_t> &cell,
                                           std::vector<float> &xrel) {
    cell.resize(n);
    xrel.resize((size_t)3 * n);
    for (int i = 0; i < n; i++) {
        int ind[3];
        float xx[3];
        for (int k = 0; k < 3; k++) {
            xx[k] = std::max<float>(e.origin[k] * (1.0 + FLT_EPSILON),
                                    std::min<float>((e.dim[k] + e.origin[k]) * (1.0 - FLT_EPSILON), x[3 * i + k]));
            ind[k] = (xx[k] - e.origin[k]) * e.ih[k];
            if (ind[k] < 0 || ind[k] >= e.cdim[k]) return TFG_E_RANGE;
        }
        int c = cellid(e, ind[0], ind[1], ind[2]);
        cell[i] = c;
        for (int k = 0; k < 3; k++) xrel[3 * i + k] = xx[k] - e.cells[c].origin[k];
    }
    return TFG_OK;
}

template <typename R> static void download(Engine<R> &e, float *x, float *xrel, int32_t *cell, float *v, float *f,
                                           float *dens, float *species, float *q) {
    for (int c = 0; c < e.ncells; c++)
        for (auto &p : e.cells[c].parts) {
            int i = p.id;
            for (int k = 0; k < 3; k++) {
                if (x) x[3 * i + k] = e.cells[c].origin[k] + p.x[k];
                if (xrel) xrel[3 * i + k] = p.x[k];
                if (v) v[3 * i + k] = p.v[k];
                if (f) f[3 * i + k] = (float)p.f[k];
            }
            if (cell) cell[i] = c;
            if (dens) dens[i] = (float)p.f[3];
        }
    if (species) for (size_t k = 0; k < e.svec.size(); k++) species[k] = e.svec[k];
    if (q) for (size_t k = 0; k < e.sq.size(); k++) q[k] = (float)e.sq[k];
}

}  // namespace

#define DISPATCH(h, call) ((h)->fp64 ? call(*(h)->f64) : call(*(h)->f32))

extern "C" {

typedef struct tfo_engine tfo_engine;

// mode bits: 1 = FP64 evaluation, 2 = brute-force pairs, 4 = reference DPD random term,
// 8 = no number density
TFG_API int tfo_create(const tfg_engine_desc *d, int mode, int nthreads, tfo_engine **out) {
    if (!d || !out) return TFG_E_INVAL;
    Handle *h = new Handle();
    h->fp64 = (mode & 1) != 0;
    int rc;
    auto setup = [&](auto &e) {
        rc = init_space(e, d);
        e.nthreads = std::max(1, nthreads);
        e.brute = (mode & 2) != 0;
        e.ref_dpd_random = (mode & 4) != 0 || (d->flags & TFG_ENGINE_DPD_REFERENCE_RANDOM) != 0;
        e.density = (mode & 8) == 0 && (d->flags & TFG_ENGINE_NO_DENSITY) == 0;
    };
    if (h->fp64) { h->f64 = new Engine<double>(); setup(*h->f64); }
    else { h->f32 = new Engine<float>(); setup(*h->f32); }
    if (rc != TFG_OK) { delete h->f32; delete h->f64; delete h; return rc; }
    *out = reinterpret_cast<tfo_engine *>(h);
    return TFG_OK;
}

TFG_API void tfo_destroy(tfo_engine *eh) {
    Handle *h = reinterpret_cast<Handle *>(eh);
    if (!h) return;
    delete h->f32;
    delete h->f64;
    delete h;
}

TFG_API int tfo_set_type(tfo_engine *eh, int type, int dynamics, float mass) {
    Handle *h = reinterpret_cast<Handle *>(eh);
    auto go = [&](auto &e) {
        if (type < 0 || type >= e.max_type) return TFG_E_INVAL;
        e.dyn[type] = dynamics; e.mass[type] = mass; return TFG_OK;
    };
    return DISPATCH(h, go);
}

TFG_API int tfo_set_potential(tfo_engine *eh, int ti, int tj, const tfg_potential *p) {
    Handle *h = reinterpret_cast<Handle *>(eh);
    auto go = [&](auto &e) {
        if (!p || ti < 0 || tj < 0 || ti >= e.max_type || tj >= e.max_type) return TFG_E_INVAL;
        copy_pot(e.pots[ti * e.max_type + tj], p);
        copy_pot(e.pots[tj * e.max_type + ti], p);
        return TFG_OK;
    };
    return DISPATCH(h, go);
}

TFG_API int tfo_set_boundary(tfo_engine *eh, int wall, const tfg_boundary *bc) {
    Handle *h = reinterpret_cast<Handle *>(eh);
    auto go = [&](auto &e) {
        if (!bc || wall < 0 || wall > 5) return TFG_E_INVAL;
        tfg_boundary b = *bc;
        if (b.kind & TFG_BOUNDARY_NO_SLIP) {   // BoundaryCondition::init, tfBoundaryConditions.cpp:151-158
            b.kind = (b.kind & ~TFG_BOUNDARY_NO_SLIP) | TFG_BOUNDARY_VELOCITY;
            b.velocity[0] = b.velocity[1] = b.velocity[2] = 0.f;
        }
        e.walls_set[wall] = b;
        // check_periodicy (tfBoundaryConditions.cpp:192-216) on the current settings
        e.periodic = 0;
        for (int w = 0; w < 6; w++) e.walls[w] = e.walls_set[w];
        for (int ax = 0; ax < 3; ax++) {
            tfg_boundary &lo = e.walls[2 * ax], &hi = e.walls[2 * ax + 1];
            const bool pl = lo.kind & TFG_BOUNDARY_PERIODIC, ph = hi.kind & TFG_BOUNDARY_PERIODIC;
            // only one of the two periodic: both become exactly PERIODIC; both periodic:
            // their other bits (RESETTING) stay
            if (pl != ph) lo.kind = hi.kind = TFG_BOUNDARY_PERIODIC;
            if (pl || ph) e.periodic |= 1u << ax;
        }
        build_tasks(e);
        e.verlet_rebuild = true;
        return TFG_OK;
    };
    return DISPATCH(h, go);
}

TFG_API int tfo_set_boundary_potential(tfo_engine *eh, int wall, int type, const tfg_potential *p) {
    Handle *h = reinterpret_cast<Handle *>(eh);
    auto go = [&](auto &e) {
        if (wall < -1 || wall > 5 || type < 0 || type >= e.max_type) return TFG_E_INVAL;
        for (int w = (wall < 0 ? 0 : wall); w <= (wall < 0 ? 5 : wall); w++) {
            if (p) copy_pot(e.wpots[w * e.max_type + type], p);
            else e.wpots[w * e.max_type + type].set = false;
        }
        return TFG_OK;
    };
    return DISPATCH(h, go);
}

TFG_API int tfo_add_flux(tfo_engine *eh, int ti, int tj, const tfg_flux *f) {
    Handle *h = reinterpret_cast<Handle *>(eh);
    auto go = [&](auto &e) {
        if (!f || ti < 0 || tj < 0 || ti >= e.max_type || tj >= e.max_type) return TFG_E_INVAL;
        auto &L = e.fluxes[ti * e.max_type + tj];
        if ((int)L.size() >= TFG_MAX_FLUX_PER_PAIR - 1) return TFG_E_OVERFLOW;
        L.push_back(*f);
        if (ti != tj) e.fluxes[tj * e.max_type + ti] = L;
        return TFG_OK;
    };
    return DISPATCH(h, go);
}

TFG_API int tfo_set_species_reset(tfo_engine *eh, int nr, const float *values) {
    Handle *h = reinterpret_cast<Handle *>(eh);
    auto go = [&](auto &e) {
        for (int s = 0; s < nr && s < (int)e.species_reset.size(); s++) e.species_reset[s] = values[s];
        return TFG_OK;
    };
    return DISPATCH(h, go);
}

TFG_API int tfo_set_species_flags(tfo_engine *eh, int nr, const uint32_t *flags) {
    Handle *h = reinterpret_cast<Handle *>(eh);
    auto go = [&](auto &e) {
        for (int s = 0; s < nr && s < (int)e.species_flags.size(); s++) e.species_flags[s] = flags[s];
        return TFG_OK;
    };
    return DISPATCH(h, go);
}

TFG_API int tfo_set_random_force(tfo_engine *eh, int type, float mean, float std_, int dur) {
    Handle *h = reinterpret_cast<Handle *>(eh);
    auto go = [&](auto &e) {
        if (type < 0 || type >= e.max_type || dur < 1) return TFG_E_INVAL;
        e.rf_mean[type] = mean; e.rf_std[type] = std_; e.rf_dur[type] = dur; return TFG_OK;
    };
    return DISPATCH(h, go);
}

TFG_API int tfo_load_particles(tfo_engine *eh, int n, const float *x, const float *v, const int32_t *type,
                               const float *radius, const float *imass, const uint32_t *flags,
                               const float *species, const float *force_i) {
    Handle *h = reinterpret_cast<Handle *>(eh);
    auto go = [&](auto &e) {
        std::vector<int32_t> cell;
        std::vector<float> xrel;
        int rc = bin_global(e, n, x, cell, xrel);
        if (rc != TFG_OK) return rc;
        return load_common(e, n, v, type, radius, imass, flags, species, force_i, cell.data(), xrel.data());
    };
    return DISPATCH(h, go);
}

TFG_API int tfo_load_particles_binned(tfo_engine *eh, int n, const int32_t *cell, const float *xrel,
                                      const float *v, const int32_t *type, const float *radius,
                                      const float *imass, const uint32_t *flags, const float *species,
                                      const float *force_i) {
    Handle *h = reinterpret_cast<Handle *>(eh);
    auto go = [&](auto &e) {
        return load_common(e, n, v, type, radius, imass, flags, species, force_i, cell, xrel);
    };
    return DISPATCH(h, go);
}

TFG_API int tfo_bin(tfo_engine *eh, int n, const float *x, int32_t *cell, float *xrel) {
    Handle *h = reinterpret_cast<Handle *>(eh);
    auto go = [&](auto &e) {
        std::vector<int32_t> c;
        std::vector<float> xr;
        int rc = bin_global(e, n, x, c, xr);
        if (rc != TFG_OK) return rc;
        std::memcpy(cell, c.data(), sizeof(int32_t) * n);
        std::memcpy(xrel, xr.data(), sizeof(float) * 3 * n);
        return TFG_OK;
    };
    return DISPATCH(h, go);
}

TFG_API int tfo_set_bonded_potential(tfo_engine *eh, int slot, const tfg_potential *p) {
    Handle *h = reinterpret_cast<Handle *>(eh);
    auto go = [&](auto &e) {
        if (slot < 0 || slot > 255 || !p) return TFG_E_INVAL;
        if ((int)e.bpots.size() <= slot) e.bpots.resize(slot + 1);
        copy_pot(e.bpots[slot], p);
        return TFG_OK;
    };
    return DISPATCH(h, go);
}

TFG_API int tfo_load_bonds(tfo_engine *eh, int n, const int32_t *i, const int32_t *j, const int32_t *slot) {
    Handle *h = reinterpret_cast<Handle *>(eh);
    auto go = [&](auto &e) {
        e.bonds.clear();
        for (int k = 0; k < n; k++) e.bonds.push_back({i[k], j[k], slot ? slot[k] : 0});
        return TFG_OK;
    };
    return DISPATCH(h, go);
}

TFG_API int tfo_load_angles(tfo_engine *eh, int n, const int32_t *i, const int32_t *j, const int32_t *k,
                            const int32_t *slot) {
    Handle *h = reinterpret_cast<Handle *>(eh);
    auto go = [&](auto &e) {
        e.angles.clear();
        for (int q = 0; q < n; q++) e.angles.push_back({i[q], j[q], k[q], slot ? slot[q] : 0});
        return TFG_OK;
    };
    return DISPATCH(h, go);
}

TFG_API int tfo_step(tfo_engine *eh, int nsteps) {
    Handle *h = reinterpret_cast<Handle *>(eh);
    auto go = [&](auto &e) {
        for (int s = 0; s < nsteps; s++) {
            int rc = step(e);
            if (rc != TFG_OK) return rc;
        }
        return TFG_OK;
    };
    return DISPATCH(h, go);
}

// engine_force_prep + engine_force at the current time (no advance).  The time
// counter is advanced first, as engine_step does before its force pass.
TFG_API int tfo_force_only(tfo_engine *eh, int with_bonded) {
    Handle *h = reinterpret_cast<Handle *>(eh);
    auto go = [&](auto &e) {
        e.time += 1;
        kinetic(e);
        prepare(e);
        if (e.verlet) verlet_update(e);
        else shuffle(e);
        const int rc = force_all(e, with_bonded != 0);
        e.verlet_rebuild = false;
        return rc;
    };
    return DISPATCH(h, go);
}

// Test hook (Verlet mode): take the current cells and positions as the last rebuild's, so
// that the next step or force pass does not re-bin.  The sorted windows are only valid for
// positions inside their cells; for others use brute-force pair enumeration (mode bit 2).
TFG_API int tfo_verlet_hold(tfo_engine *eh) {
    Handle *h = reinterpret_cast<Handle *>(eh);
    auto go = [&](auto &e) {
        for (auto &c : e.cells)
            for (auto &p : c.parts)
                for (int k = 0; k < 3; k++) p.ox[k] = p.x[k];
        for (int cid = 0; cid < e.ncells; cid++) do_sort(e, cid);
        e.verlet_rebuild = false;
        e.verlet_maxdx = 0.f;
        return TFG_OK;
    };
    return DISPATCH(h, go);
}

TFG_API int tfo_download(tfo_engine *eh, float *x, float *xrel, int32_t *cell, float *v, float *f, float *dens,
                         float *species, float *q) {
    Handle *h = reinterpret_cast<Handle *>(eh);
    auto go = [&](auto &e) { download(e, x, xrel, cell, v, f, dens, species, q); return TFG_OK; };
    return DISPATCH(h, go);
}

// Per-particle sum of contribution magnitudes (by id).
TFG_API int tfo_download_fmag(tfo_engine *eh, double *out) {
    Handle *h = reinterpret_cast<Handle *>(eh);
    auto go = [&](auto &e) {
        for (auto &c : e.cells)
            for (auto &p : c.parts) out[p.id] = p.fmag;
        return TFG_OK;
    };
    return DISPATCH(h, go);
}

// Forces in full precision (FP64 mode keeps double accumulators).
TFG_API int tfo_download_forces_f64(tfo_engine *eh, double *f) {
    Handle *h = reinterpret_cast<Handle *>(eh);
    auto go = [&](auto &e) {
        for (auto &c : e.cells)
            for (auto &p : c.parts)
                for (int k = 0; k < 4; k++) f[4 * p.id + k] = (double)p.f[k];
        return TFG_OK;
    };
    return DISPATCH(h, go);
}

TFG_API int tfo_get_reductions(tfo_engine *eh, tfg_reductions *out) {
    Handle *h = reinterpret_cast<Handle *>(eh);
    auto go = [&](auto &e) {
        std::memset(out, 0, sizeof(*out));
        out->epot_nonbond = (double)e.epot_nonbond;
        out->epot_bond = (double)e.epot_bond;
        out->epot_angle = (double)e.epot_angle;
        out->epot = out->epot_nonbond + out->epot_bond + out->epot_angle;
        out->kinetic = e.kinetic;
        out->virial = e.virial;
        out->computed_volume = e.computed_volume;
        for (int s = 0; s < e.nspec && s < 8; s++) {
            double t = 0;
            for (int i = 0; i < e.nparts; i++) t += e.svec[(size_t)i * e.nspec + s];
            out->species_total[s] = t;
        }
        out->steps = e.time;
        out->migrations = e.migrations;
        return TFG_OK;
    };
    return DISPATCH(h, go);
}

TFG_API int tfo_get_verlet(tfo_engine *eh, int64_t *rebuilds, float *maxdx) {
    Handle *h = reinterpret_cast<Handle *>(eh);
    auto go = [&](auto &e) {
        if (rebuilds) *rebuilds = e.verlet_rebuilds;
        if (maxdx) *maxdx = e.verlet_maxdx;
        return TFG_OK;
    };
    return DISPATCH(h, go);
}

TFG_API int tfo_enable_signature(tfo_engine *eh, int on) {
    Handle *h = reinterpret_cast<Handle *>(eh);
    auto go = [&](auto &e) { e.want_sig = on != 0; return TFG_OK; };
    return DISPATCH(h, go);
}

// Per-particle pair signature of the last force pass (count, hash of partner ids).
TFG_API int tfo_signature(tfo_engine *eh, int32_t *count, uint32_t *hash) {
    Handle *h = reinterpret_cast<Handle *>(eh);
    auto go = [&](auto &e) {
        if ((int)e.sig_cnt.size() != e.nparts) return TFG_E_STATE;
        std::memcpy(count, e.sig_cnt.data(), sizeof(int32_t) * e.nparts);
        std::memcpy(hash, e.sig_hash.data(), sizeof(uint32_t) * e.nparts);
        return TFG_OK;
    };
    return DISPATCH(h, go);
}

// Diagnostics: [0] cell pairs skipped by the unsigned sorted-window wrap,
// [1] straight/perpendicular angles that took the random plane, [2] tasks.
TFG_API int tfo_get_stats(tfo_engine *eh, int64_t *out3) {
    Handle *h = reinterpret_cast<Handle *>(eh);
    auto go = [&](auto &e) {
        out3[0] = e.window_skips.load(); out3[1] = e.straight_angles; out3[2] = (int64_t)e.tasks.size();
        return TFG_OK;
    };
    return DISPATCH(h, go);
}

// Record the interacting pair set of the next force pass.  tfo_get_pairs copies up to
// cap (lo, hi) id pairs (sorted) and returns the total count.
TFG_API int tfo_record_pairs(tfo_engine *eh, int on) {
    Handle *h = reinterpret_cast<Handle *>(eh);
    auto go = [&](auto &e) { e.record_pairs = on != 0; e.pairs.clear(); return TFG_OK; };
    return DISPATCH(h, go);
}

TFG_API int64_t tfo_get_pairs(tfo_engine *eh, int32_t *out, int64_t cap) {
    Handle *h = reinterpret_cast<Handle *>(eh);
    auto go = [&](auto &e) -> int64_t {
        std::sort(e.pairs.begin(), e.pairs.end());
        int64_t n = (int64_t)e.pairs.size();
        for (int64_t k = 0; k < n && k < cap; k++) { out[2 * k] = e.pairs[k].first; out[2 * k + 1] = e.pairs[k].second; }
        return n;
    };
    return h->fp64 ? go(*h->f64) : go(*h->f32);
}

TFG_API uint32_t tfo_philox_probe(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1,
                                  uint32_t *out4) {
    U4 r = philox({c0, c1, c2, c3}, k0, k1);
    out4[0] = r.x; out4[1] = r.y; out4[2] = r.z; out4[3] = r.w;
    return r.x;
}

}  // extern "C"
