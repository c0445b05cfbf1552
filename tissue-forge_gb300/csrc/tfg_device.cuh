// Device-side data layout and per-pair arithmetic of the GB300 engine.
//
// Particles are stored structure-of-arrays in cell order (re-binned every step by a
// counting sort).  All pair arithmetic that decides WHICH pairs interact is done with
// explicitly rounded FP32 intrinsics (__fadd_rn / __fsub_rn / __fmul_rn), so that it is
// bit-identical to the reference's scalar build (-mavx -msse4.2, no FMA contraction,
// CMakeLists.txt:78,91-95): cell-relative coordinates, per-pair shift from the cell
// origins (space_getsid, tfSpace.cpp:79-114) and r2 = dx.dx (fptype_r2,
// include/tf_fptype.h:204-210).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "tfg.h"

namespace tfg {

constexpr int kChunk = TFG_POTENTIAL_CHUNK;
constexpr int kMaxTypes = 16;
constexpr int kMaxFluxPerPair = TFG_MAX_FLUX_PER_PAIR;
constexpr int kMaxSpecies = 8;
constexpr int kMaxBondSlots = 16;

// Error bits set by kernels; the host maps them to TFG_E_* at sync.
enum : uint32_t {
    ERR_TOOFAST = 1u << 0,
    ERR_NAN = 1u << 1,
    ERR_OVERFLOW = 1u << 2,
    ERR_RANGE = 1u << 3,
};

// Random streams (Philox4x32-10 counter word 3).
enum : uint32_t { STREAM_DPD = 0xD0D0u, STREAM_FORCE = 0xF0F0u, STREAM_ANGLE = 0xA0A0u, STREAM_WALL = 0xB0B0u };

// One potential as consumed by the kernels (struct Potential, tfPotential.h:213-253).
// 64 bytes, 16-byte aligned: a descriptor is read with four 128-bit loads.
struct __align__(16) PotDev {
    uint32_t kind;       // 0 none, 1 table, 2 dpd  (internal encoding, see engine)
    uint32_t flags;
    float alpha0, alpha1, alpha2;
    float r0_plusone, a, b;
    int32_t n;
    int32_t offset;      // float offset of the table in the table blob (a multiple of 8)
    float dpd_alpha, dpd_gamma, dpd_sigma;
    float pad_[3];
};
static_assert(sizeof(PotDev) == 64, "PotDev layout");
enum : uint32_t { POT_NONE = 0, POT_TABLE = 1, POT_DPD = 2 };

struct FluxDev {
    int32_t kind, type_a, type_b, index_a, index_b;
    float coef, half_decay, target, cutoff;
};

struct FluxSet {
    int32_t count;
    FluxDev f[kMaxFluxPerPair];
};

// Per-step kernel parameters of one simulation.  An engine holds one or more
// simulations in one device arena: their cells and particles are concatenated, so a
// simulation owns global cells [cell_off, cell_off + ncells) and global particle ids
// [id_off, id_off + n).  Per-simulation tables sit at pot_base (potentials and fluxes,
// max_type^2 entries) and type_base (per-type arrays); its FP64 totals at red_base.
struct SimParams {
    float h[3], dim[3];
    int32_t cdim[3];
    int32_t ncells;
    int32_t cell_off, id_off, angle_off;
    int32_t pot_base, type_base, red_base, spec_base;
    float cutoff, cutoff2;
    float dt, dt_flux;
    float maxx[3], maxx2[3], maxv[3], maxv2[3], h2[3];
    float inv_cutoff;        // 1/cutoff in FP32
    float self_density;      // W(0, cutoff)
    float dpd_delta;         // 1/sqrt(dt) in FP32
    int32_t max_type, nspec;
    int32_t nr_fluxsteps;    // flux substeps per step (dt_flux = dt / nr_fluxsteps)
    uint32_t flags;          // TFG_ENGINE_*
    uint64_t seed;
    int64_t time;            // engine time of the step being computed
    const float *corig[3];   // cell origin per axis, cdim[k] entries
    // boundary conditions: walls 0..5 = x low, x high, y low, y high, z low, z high
    uint32_t periodic;       // bit k: axis k is periodic
    uint32_t walls_active;   // bit w: wall w is FREESLIP, VELOCITY or POTENTIAL
    uint32_t walls_reflect;  // bit w: wall w is FREESLIP or VELOCITY
    uint32_t wall_kind[6];
    float4 wall_vel[6];      // wall velocity; w = restore
    float wall_radius[6];
    int32_t wpot_base;       // (wall 0, type 0) in the wall-potential array; walls x types
    float species_reset[kMaxSpecies];  // species values after crossing a RESETTING wall
    // A simulation may be told to stop at an engine time: k_tick sets `stopped` once time has
    // reached stop_at, and every kernel of the step then leaves the simulation (and its
    // totals) alone, so a batch can step on while some members are already done.
    int64_t stop_at;         // -1: no stop
    int32_t stopped;         // device: this step does not advance the simulation
    // Verlet mode (TFG_ENGINE_VERLET; engine_verlet_update, tfEngine.cpp:214-354).  The
    // device fields are written by k_tick and k_advance; the host writes 2 to
    // verlet_rebuild to force a rebuild at the next step.
    float skin;              // min(h) - cutoff
    float rlist2;            // (cutoff + skin)^2 with a relative margin: pair-list radius
    int32_t verlet_rebuild;  // device: this step re-bins and rebuilds the pair lists
    uint32_t verlet_maxdx2;  // device: max |x - oldx|^2 after the last advance (float bits)
    float verlet_maxdx;      // device: largest displacement at the last check (0 on a rebuild)
    int64_t verlet_rebuilds; // device: rebuilds so far
};

// Does a particle that moves by delta[] from the cell at loc[] cross a RESETTING wall?
// apply_boundary_particle_crossing (tfBoundaryConditions.cpp:676-735): along each axis in
// order x, y, z whose cell index changes, on a periodic axis, both cells must carry the
// periodic wall flag of their side (space_init: a cell at index 0 takes the low wall's flag
// when that wall is PERIODIC, else a cell at index cdim-1 the high wall's), and the
// destination's wall must be RESETTING.
__host__ __device__ inline bool crosses_resetting_wall(const SimParams &P, const int loc[3], const int delta[3]) {
    for (int k = 0; k < 3; k++) {
        if (delta[k] == 0 || !((P.periodic >> k) & 1u)) continue;
        const int n = P.cdim[k];
        const int src = loc[k], dst = (loc[k] + delta[k] + n) % n;
        auto side = [&](int l) {   // 0 low wall flag, 1 high wall flag, -1 none
            if (l == 0 && (P.wall_kind[2 * k] & TFG_BOUNDARY_PERIODIC)) return 0;
            if (l + 1 == n && (P.wall_kind[2 * k + 1] & TFG_BOUNDARY_PERIODIC)) return 1;
            return -1;
        };
        const int ss = side(src), ds = side(dst);
        if (ss < 0 || ds < 0) continue;
        if (P.wall_kind[2 * k + ds] & TFG_BOUNDARY_RESETTING) return true;
    }
    return false;
}

// Is wall w of this simulation active and is cell location (a, b, c) on it?
__host__ __device__ inline bool on_wall(const SimParams &P, int w, int a, int b, int c) {
    if (!(P.walls_active & (1u << w))) return false;
    const int l = w < 2 ? a : (w < 4 ? b : c), ax = w >> 1;
    return (w & 1) ? l + 1 == P.cdim[ax] : l == 0;
}

// ---------------- Philox4x32-10 (Salmon et al., SC'11) ----------------
struct U4 { uint32_t x, y, z, w; };

__device__ __forceinline__ U4 philox(U4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        U4 n = {hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
        c = n;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

// (0,1) uniform from the 24 high bits.
__device__ __forceinline__ float u01(uint32_t u) {
    return __fadd_rn(__fmul_rn((float)(u >> 8), 5.9604644775390625e-8f), 2.98023223876953125e-8f);
}

__device__ __forceinline__ float gauss_pair(uint64_t seed, int64_t step, int ida, int idb) {
    int lo = min(ida, idb), hi = max(ida, idb);
    U4 r = philox({(uint32_t)step, (uint32_t)lo, (uint32_t)hi, STREAM_DPD}, (uint32_t)seed, (uint32_t)(seed >> 32));
    float u1 = u01(r.x), u2 = u01(r.y);
    return sqrtf(-2.0f * logf(u1)) * cosf(6.283185307179586f * u2);
}

// Normal deviate of the DPD wall random term, keyed on (step, particle, wall).
__device__ __forceinline__ float gauss_wall(uint64_t seed, int64_t step, int id, int wall) {
    U4 r = philox({(uint32_t)step, (uint32_t)id, (uint32_t)wall, STREAM_WALL}, (uint32_t)seed, (uint32_t)(seed >> 32));
    float u1 = u01(r.x), u2 = u01(r.y);
    return sqrtf(-2.0f * logf(u1)) * cosf(6.283185307179586f * u2);
}

// ---------------- geometry ----------------
// Does the neighbour at offset o of location l exist along axis ax?  Always on a periodic
// axis; on a non-periodic one only inside the box (space_init, tfSpace.cpp:913-970).
__device__ __forceinline__ bool nb_exists(const SimParams &P, int ax, int l, int o) {
    const int v = l + o;
    return ((P.periodic >> ax) & 1u) || (v >= 0 && v < P.cdim[ax]);
}

// Global cell index of the simulation's cell at grid location (i, j, k).
__device__ __forceinline__ int cell_index(const SimParams &P, int i, int j, int k) {
    return P.cell_off + (i * P.cdim[1] + j) * P.cdim[2] + k;
}

// Grid location of global cell c.
__device__ __forceinline__ void cell_loc(const SimParams &P, int c, int &i, int &j, int &k) {
    c -= P.cell_off;
    k = c % P.cdim[2];
    int t = c / P.cdim[2];
    j = t % P.cdim[1];
    i = t / P.cdim[1];
}

// Shift from cell at loc a to cell at loc b along axis k, wrapped into (-dim/2, dim/2]
// exactly as space_getsid computes it.
__device__ __forceinline__ float cell_shift(const SimParams &P, int k, int la, int lb) {
    float s = __fsub_rn(P.corig[k][lb], P.corig[k][la]);
    float s2 = __fmul_rn(s, 2.0f);
    if (s2 > P.dim[k]) s = __fsub_rn(s, P.dim[k]);
    else if (s2 < -P.dim[k]) s = __fadd_rn(s, P.dim[k]);
    return s;
}

// r2 = dx.dx with dx = (xi - shift) - xj, no contraction.
__device__ __forceinline__ float pair_r2(float3 xi, float3 sh, float3 xj, float3 &dx) {
    dx.x = __fsub_rn(__fsub_rn(xi.x, sh.x), xj.x);
    dx.y = __fsub_rn(__fsub_rn(xi.y, sh.y), xj.y);
    dx.z = __fsub_rn(__fsub_rn(xi.z, sh.z), xj.z);
    return __fadd_rn(__fadd_rn(__fmul_rn(dx.x, dx.x), __fmul_rn(dx.y, dx.y)), __fmul_rn(dx.z, dx.z));
}

__device__ __forceinline__ float pair_r2_self(float3 xi, float3 xj, float3 &dx) {
    dx.x = __fsub_rn(xi.x, xj.x);
    dx.y = __fsub_rn(xi.y, xj.y);
    dx.z = __fsub_rn(xi.z, xj.z);
    return __fadd_rn(__fadd_rn(__fmul_rn(dx.x, dx.x), __fmul_rn(dx.y, dx.y)), __fmul_rn(dx.z, dx.z));
}

// ---------------- per-pair physics ----------------
// Cubic-spline number density W(r2, h) (tf_smoothing_kernel.h:49-67).  The reference's
// x86 build takes r from a 12-bit rsqrt estimate; this uses the correctly rounded sqrt
// (computed once per pair by the caller), r/h as r*(1/h) and y/(pi h^3) as y*norm.
__device__ __forceinline__ float density_w(float r, float inv_h, float norm) {
    float x = r * inv_h;
    float y;
    if (x < 1.f) {
        float x2 = __fmul_rn(x, x);
        y = __fadd_rn(__fsub_rn(1.f, __fmul_rn(1.5f, x2)), __fmul_rn(__fmul_rn(0.75f, x2), x));
    } else if (x < 2.f) {
        float arg = __fsub_rn(2.f, x);
        y = __fmul_rn(__fmul_rn(__fmul_rn(0.25f, arg), arg), arg);
    } else {
        y = 0.f;
    }
    return y * norm;   // norm = 1 / (pi h^3)
}

// One interval of a table (potential_eval_ex's polynomial, tf_potential_eval.h:128-139):
// x = (r - c0) c1, ee and eff by the Horner recurrence over c2..c7.  The row is 8 floats,
// 32-byte aligned (table offsets are multiples of 8), read as two 128-bit loads.
__device__ __forceinline__ void table_row_eval(const float *row, float r, float &ee, float &eff, float &c1) {
    const float4 *c4 = reinterpret_cast<const float4 *>(row);
    const float4 ca = c4[0], cb = c4[1];
    const float x = (r - ca.x) * ca.y;
    ee = fmaf(ca.z, x, ca.w);
    eff = ca.z;
    eff = fmaf(eff, x, ee);
    ee = fmaf(ee, x, cb.x);
    eff = fmaf(eff, x, ee);
    ee = fmaf(ee, x, cb.y);
    eff = fmaf(eff, x, ee);
    ee = fmaf(ee, x, cb.z);
    eff = fmaf(eff, x, ee);
    ee = fmaf(ee, x, cb.w);
    c1 = ca.y;
}

// Tabulated potential (potential_eval_ex, tf_potential_eval.h:104-146).  Returns false
// when out of range.  The interval index is computed with the reference's unfused FP32
// arithmetic so the same interval is chosen; the Horner recurrence uses FMA.
__device__ __forceinline__ bool table_eval(const PotDev &p, const float *__restrict__ blob, float ri, float rj,
                                           float r2, float &e, float &f) {
    float r = __fsqrt_rn(r2);
    float ro = r < 1.1920928955078125e-7f ? 1.1920928955078125e-7f : r;
    if (p.flags & TFG_POTENTIAL_SCALED) r = __fdiv_rn(r, __fadd_rn(ri, rj));
    else if (p.flags & TFG_POTENTIAL_SHIFTED) r = __fadd_rn(__fsub_rn(r, __fadd_rn(ri, rj)), p.r0_plusone);
    r = r < p.a ? p.a : r;
    float t = __fadd_rn(p.alpha0, __fmul_rn(r, __fadd_rn(p.alpha1, __fmul_rn(r, p.alpha2))));
    unsigned ind = (unsigned)fmaxf(0.0f, t);
    if (r > p.b || ind > (unsigned)p.n) return false;
    float ee, eff, c1;
    table_row_eval(blob + p.offset + ind * kChunk, r, ee, eff, c1);
    e = ee;
    f = __fdividef(eff * c1, ro);   // within 2 ulp of eff*c1/ro; the interval is already chosen
    return true;
}

// Wall potentials of one particle in a cell on active walls (boundary_eval,
// tf_boundary_eval.h:192-254, with boundary_potential_eval_ex :146-188 and dpd_boundary_eval,
// tf_dpd_eval.h:78-120).  x is cell-relative; the distance to a wall is x (low walls) or
// h - x (high walls).  Adds the force to f and the energy to epot.
__device__ __forceinline__ void wall_eval(const SimParams &P, const PotDev *wpots, const float *blob, int type,
                                          float3 x, float radius, float4 vel, int lid, int la, int lb, int lc,
                                          float3 &f, float &epot) {
    for (int w = 0; w < 6; w++) {
        if (!on_wall(P, w, la, lb, lc)) continue;
        const PotDev pot = wpots[P.wpot_base + w * P.max_type + type];
        if (pot.kind == POT_NONE) continue;
        const int ax = w >> 1;
        const float xa = ax == 0 ? x.x : (ax == 1 ? x.y : x.z);
        const float r = (w & 1) ? __fsub_rn(P.h[ax], xa) : xa;
        if (!(r <= pot.b)) continue;
        const float dxa = (w & 1) ? -r : r;
        const float r2 = __fmul_rn(r, r);
        float fa = 0.f;
        if (pot.kind == POT_TABLE) {
            float e, fv;
            if (table_eval(pot, blob, radius, P.wall_radius[w], r2, e, fv)) {
                fa = -fv * dxa;   // part->f -= f * dx
                epot += e;
            }
        } else if (pot.kind == POT_DPD) {
            float rr = __fsqrt_rn(r2);
            const float ro = rr < 1.1920928955078125e-7f ? 1.1920928955078125e-7f : rr;
            if (pot.flags & TFG_POTENTIAL_SHIFTED) rr = __fsub_rn(rr, __fadd_rn(radius, P.wall_radius[w]));
            if (rr > pot.b) continue;
            rr = rr >= pot.a ? rr : pot.a;
            const float ea = __fdividef(dxa, ro);
            const float4 U = P.wall_vel[w];
            const float va = ax == 0 ? vel.x - U.x : (ax == 1 ? vel.y - U.y : vel.z - U.z);
            const float omega_c = rr < 0.f ? 1.f : 1.f - __fdividef(rr, pot.b);
            float xi_r = 1.0f;
            if (!(P.flags & TFG_ENGINE_DPD_REFERENCE_RANDOM)) xi_r = gauss_wall(P.seed, P.time, lid, w);
            const float ftot = pot.dpd_alpha * omega_c - pot.dpd_gamma * omega_c * omega_c * (ea * va) +
                               pot.dpd_sigma * omega_c * xi_r * P.dpd_delta;
            fa = ftot * ea;   // part->f += f * e
        }
        if (ax == 0) f.x += fa;
        else if (ax == 1) f.y += fa;
        else f.z += fa;
    }
}

}  // namespace tfg
