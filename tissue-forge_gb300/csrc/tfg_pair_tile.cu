// Tiled nonbonded pair pass (Newton's third law, warp-level compaction).
//
// Reference path replaced: runner_dopair / runner_doself (tf_runner_dopair.cpp:72-758)
// with potential_eval_super_ex (tf_potential_eval.h:207-272), dpd_eval
// (tf_dpd_eval.h:32-76), flux_eval_ex (tf_flux_eval.h:48-103) and the number density W
// (tf_smoothing_kernel.h:49-67).
//
// Work unit: one warp owns a home cell and runs the reference's 14 tasks of that cell
// (the self task and the 13 pair tasks whose cell_i it is: a neighbour at offset d is
// task-partner of the home cell with the home as cell_i exactly when d is
// lexicographically positive, space_getsid / space_init tfSpace.cpp:79-114, 893-1019).
// The home cell and then each neighbour cell are staged into the warp's shared memory;
// a neighbour particle is staged only if it lies within the cutoff of the box holding the
// home particles.  All 32 lanes test candidate pairs (r2 with the reference's unfused FP32
// arithmetic, so the pair set is bit-identical), hits go to a warp-private ring queue, and
// the queue is evaluated 32 pairs at a time so the force arithmetic runs with full lanes.
// Each evaluated pair adds the force, number density and flux increments of both partners
// to the particle arrays with global vector atomics.  Home cells above kHomeCap particles
// are listed and handled by k_pair_overflow.
#include <algorithm>

#include "tfg_internal.h"

namespace tfg {

namespace {

constexpr int kWarps = 8;
constexpr int kCapT = 200;          // staged particles per warp (table variants)
constexpr int kCapX = 120;          // staged particles per warp (DPD and flux variants)
constexpr int kHomeCap = 96;        // largest home cell handled by the tiled kernel
constexpr int kUnroll = 2;          // home particles tested per pass of the table variants' candidate loop
static_assert(kHomeCap + kUnroll <= kCapT, "the unrolled candidate loop reads up to kUnroll - 1 past the home cell");
constexpr int kQ = 128;             // candidate ring queue entries per warp (power of two, >= 31 + 32 kUnroll)
static_assert(kQ >= 31 + 32 * kUnroll, "a pass queues up to 32 kUnroll hits onto at most 31 waiting ones");
constexpr int kMaxSmemTable = 4096; // floats of potential table staged per CTA
constexpr int kMaxSmemPots = 64;    // potential descriptors staged per CTA (all simulations)
constexpr size_t kFourCtaBytes = 228 * 1024 / 4 - 1024;   // dynamic shared memory of a CTA, four per SM

// One warp's staging area.  The DPD and flux variants (EXTRA) also stage each particle's
// velocity, id and species value, with fewer particles per warp, so that every variant fits
// four CTAs per SM.  Force variants add each pair's increments straight to the particle
// arrays; only the signature variant (SIG) keeps per-particle sums in shared memory.
template <int CAP, bool EXTRA, bool SIG> struct StagedT {
    static constexpr int cap = CAP;
    float4 pos[CAP];        // cell-relative position; w = type bits
    float4 acc[SIG ? CAP : 1];   // signature: partner count, id hash (bits)
    int32_t gslot[CAP];     // global slot of the staged particle
    float rad[CAP];         // radius
    float sh[27][3];        // shift of each task's partner cell (space_getsid)
    uint32_t q[kQ];         // packed hit (i | k << 16), staged indices
    float4 vel[EXTRA ? CAP : 1];
    int32_t id[EXTRA ? CAP : 1];
    float sv[EXTRA ? CAP : 1];   // species 0 value
    float4 box[2];          // box holding every home particle (lo, hi); lo.w: squared pruning distance
    int32_t toff[13];       // flat staging: offset of forward task 14 + L's particles in the flat list
    int32_t tg0[13];        // flat staging: first slot of forward task 14 + L's cell
    uint8_t seg[CAP];       // task of the staged particle's cell: its shift is sh[seg]
};

// Shift of staged particle k's cell as seen from the home cell, with its radius in w.
template <class ST> __device__ __forceinline__ float4 staged_shift(const ST &S, int k) {
    const float *s = S.sh[S.seg[k]];
    return make_float4(s[0], s[1], s[2], S.rad[k]);
}
template <bool kDPD, bool kFlux, bool kSig> struct TileOf {
    using S = StagedT<(kDPD || kFlux) ? kCapX : kCapT, kDPD || kFlux, kSig>;
};
static_assert(sizeof(TileOf<false, false, false>::S) * kWarps <= kFourCtaBytes, "table variants: four CTAs per SM");
static_assert(sizeof(TileOf<true, true, false>::S) * kWarps <= kFourCtaBytes, "DPD and flux variants: four CTAs per SM");

// v in [-1, n] wrapped into [0, n): (v + n) % n for a neighbour offset of at most one cell.
__device__ __forceinline__ int wrap1(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Pair lists are stored in groups of 128 entries, interleaved so that one 16-byte load per
// lane fetches four batches of 32: sequential entry p of a list sits at list_slot(p), and
// component c of lane L's load is entry 32 c + L of the group.  Each staged chunk's
// entries end with a kListEnd marker and the next chunk starts at the next group.
__device__ __forceinline__ int list_slot(int p) { return (p & ~127) | ((p & 31) << 2) | ((p >> 5) & 3); }

struct TileArgs {
    PairKernelArgs a;
    int *overflow_list;    // home cells handed to the overflow kernel
    int *overflow_count;   // [0] overflow cells, [1] work counter of the tiled pass
    int split;             // warps per home cell: the 14 tasks are divided into `split` groups
    int grab;              // work items a warp takes from the shared counter at a time
    int stage_floats;      // table floats and descriptors staged per CTA (TilePlan)
    int stage_pots;
    int prune;             // stage only neighbour particles within the cutoff of the home cell's bounding box
};

// Evaluate one candidate pair, reference orientation I = part_i (home), K = part_j.  Returns
// false when the reference's test puts it beyond the cutoff; otherwise adds the I-side and
// K-side increments (force xyz, density) to fI / fK and the flux increments to qI / qK.
template <bool kDPD, bool kFlux, bool kDensity, class ST>
__device__ __forceinline__ bool eval_pair(const TileArgs &T, const SimParams &P, ST &S, const PotDev *pots,
                                          const float *blob, int I, int K, float &epot, float &vir, float4 &fI,
                                          float4 &fK, float &qI, float &qK) {
    const PairKernelArgs &a = T.a;
    const float4 pi = S.pos[I], pk = S.pos[K];
    const float4 s4 = staged_shift(S, K);
    const float3 sh = make_float3(s4.x, s4.y, s4.z);
    float3 dx;
    const float r2 = pair_r2(make_float3(pi.x, pi.y, pi.z), sh, make_float3(pk.x, pk.y, pk.z), dx);
    if (r2 > P.cutoff2) return false;   // a candidate that only the table loop's looser filter passed
    const float r = __fsqrt_rn(r2);
    const bool flux_only = kFlux && a.flux_sub >= 0;
    if (kDensity && !flux_only) {
        const float w = density_w(r, P.inv_cutoff, P.self_density);
        fI.w += w;
        fK.w += w;
    }
    const int ti = __float_as_int(pi.w), tk = __float_as_int(pk.w);
    const int pidx = P.pot_base + ti * a.max_type + tk;
    if (kFlux) {
        const FluxSet &fs = a.fluxes[pidx];
        for (int f = 0; f < fs.count; f++) {
            const FluxDev &F = fs.f[f];
            if (r > F.cutoff) continue;
            float term = __fsub_rn(1.0f, __fdividef(r, F.cutoff));
            term = __fmul_rn(term, term);
            const bool a_is_I = (ti == F.type_a);
            const bool b_is_K = (tk == F.type_b);
            // staged indices of the flux's "a" and "b" particles; one species is staged, more
            // are read from the particle arrays and their increments added there directly
            const int sa = a_is_I ? I : K, sb = b_is_K ? K : I;
            const bool one = a.nspec == 1;
            const size_t ga = (size_t)F.index_a * a.cap + S.gslot[sa], gb = (size_t)F.index_b * a.cap + S.gslot[sb];
            const float ssi = one ? S.sv[sa] : a.sval[ga], ssj = one ? S.sv[sb] : a.sval[gb];
            float q = term;
            if (F.kind == TFG_FLUX_FICK) {
                q = __fmul_rn(q, __fmul_rn(F.coef, __fsub_rn(ssi, ssj)));
            } else if (F.kind == TFG_FLUX_SECRETE) {
                const float qq = __fmul_rn(F.coef, __fsub_rn(ssi, F.target));
                q = __fmul_rn(q, qq > 0.f ? qq : 0.f);
            } else {
                const float qq = __fmul_rn(__fmul_rn(F.coef, __fsub_rn(F.target, ssj)), ssi);
                q = __fmul_rn(q, qq > 0.f ? qq : 0.f);
            }
            const float da = -q - F.half_decay * ssi, db = q - F.half_decay * ssj;
            if (one) {
                if (a_is_I) qI += da; else qK += da;
                if (b_is_K) qK += db; else qI += db;
            } else {
                atomicAdd(&a.sq[ga], da);
                atomicAdd(&a.sq[gb], db);
            }
        }
    }
    if (flux_only) return true;
    const PotDev pot = pots[pidx];
    if (pot.kind == POT_TABLE) {
        float e, f;
        // radii ride in the staged shift's w component
        if (table_eval(pot, blob, S.rad[I], s4.w, r2, e, f)) {
            const float wx = f * dx.x, wy = f * dx.y, wz = f * dx.z;
            fI.x -= wx; fI.y -= wy; fI.z -= wz;
            fK.x += wx; fK.y += wy; fK.z += wz;
            epot += e;
            vir -= f * r2;
        }
    } else if (kDPD && pot.kind == POT_DPD) {
        float rr = r;
        const float ro = r < 1.1920928955078125e-7f ? 1.1920928955078125e-7f : r;
        if (pot.flags & TFG_POTENTIAL_SHIFTED) rr = __fsub_rn(rr, __fadd_rn(S.rad[I], s4.w));
        if (rr <= pot.b) {
            rr = rr >= pot.a ? rr : pot.a;
            const float4 vi = S.vel[I], vk = S.vel[K];
            const float inv_ro = __fdividef(1.0f, ro);
            const float ex = dx.x * inv_ro, ey = dx.y * inv_ro, ez = dx.z * inv_ro;
            const float omega_c = rr < 0.f ? 1.f : 1.f - __fdividef(rr, pot.b);
            const float edv = ex * (vi.x - vk.x) + ey * (vi.y - vk.y) + ez * (vi.z - vk.z);
            float xi_r = 1.0f;
            if (!(P.flags & TFG_ENGINE_DPD_REFERENCE_RANDOM))
                xi_r = gauss_pair(P.seed, P.time, S.id[I] - P.id_off, S.id[K] - P.id_off);
            const float ftot = pot.dpd_alpha * omega_c - pot.dpd_gamma * omega_c * omega_c * edv +
                               pot.dpd_sigma * omega_c * xi_r * P.dpd_delta;
            const float wx = ftot * ex, wy = ftot * ey, wz = ftot * ez;
            // part_i.f += F e ; part_j.f -= F e
            fI.x += wx; fI.y += wy; fI.z += wz;
            fK.x -= wx; fK.y -= wy; fK.z -= wz;
            vir += ftot * ro;
        }
    }
    return true;
}

// Evaluate the queued hits held by the active lanes, one pair per lane.  Both partners'
// increments (force, number density, and the flux increment of a single staged species) are
// added straight to the particle arrays with global atomics: a batch holds up to 32 pairs
// whose partners repeat in no fixed pattern, and the L2 atomics cost less than grouping
// equal partners within the warp (a segmented scan and match_any) and flushing shared sums.
// The signature variant counts partners and hashes their ids in the staged sums instead.
template <bool kDPD, bool kFlux, bool kDensity, bool kSig, class ST>
__device__ __forceinline__ void eval_batch(const TileArgs &T, const SimParams &P, ST &S, const PotDev *pots,
                                           const float *blob, bool active, uint32_t e, float &epot, float &vir) {
    if (!active) return;
    const int I = e & 0xffff, K = e >> 16;
    if constexpr (kSig) {
        // the pair decision proper (the table loop queues candidates with a looser filter)
        const float4 pi = S.pos[I], pk = S.pos[K], s4 = staged_shift(S, K);
        float3 dx;
        if (pair_r2(make_float3(pi.x, pi.y, pi.z), make_float3(s4.x, s4.y, s4.z), make_float3(pk.x, pk.y, pk.z), dx) >
            P.cutoff2)
            return;
        atomicAdd(reinterpret_cast<int *>(&S.acc[I].x), 1);
        atomicAdd(reinterpret_cast<int *>(&S.acc[K].x), 1);
        const uint32_t idi = (uint32_t)__float_as_int(T.a.aux[S.gslot[I]].w);
        const uint32_t idk = (uint32_t)__float_as_int(T.a.aux[S.gslot[K]].w);
        atomicAdd(reinterpret_cast<unsigned *>(&S.acc[I].y), sig_mix(idk));
        atomicAdd(reinterpret_cast<unsigned *>(&S.acc[K].y), sig_mix(idi));
        record_pair(T.a, (int)idi, (int)idk);
    } else {
        float4 fI = make_float4(0.f, 0.f, 0.f, 0.f), fK = make_float4(0.f, 0.f, 0.f, 0.f);
        float qI = 0.f, qK = 0.f;   // species 0 flux increments (flux variants, one species)
        if (!eval_pair<kDPD, kFlux, kDensity>(T, P, S, pots, blob, I, K, epot, vir, fI, fK, qI, qK)) return;
        const int gI = S.gslot[I], gK = S.gslot[K];
        if (!(kFlux && T.a.flux_sub >= 0)) {   // a flux-only substep adds no force
            atomicAdd(&T.a.force[gI], fI);
            atomicAdd(&T.a.force[gK], fK);
        }
        if (kFlux && T.a.nspec == 1) {
            if (qI != 0.f) atomicAdd(&T.a.sq[gI], qI);
            if (qK != 0.f) atomicAdd(&T.a.sq[gK], qK);
        }
    }
}

// Add a warp's FP32 energy and virial partials to a simulation's FP64 totals.
__device__ __forceinline__ void flush_red(double *red, int rb, float &epot, float &vir, int lane) {
    double de = epot, dv = vir;
    for (int o = 16; o > 0; o >>= 1) {
        de += __shfl_down_sync(0xffffffffu, de, o);
        dv += __shfl_down_sync(0xffffffffu, dv, o);
    }
    if (lane == 0 && rb >= 0) {
        if (de != 0.0) atomicAdd(&red[rb + RED_EPOT_NONBOND], de);
        if (dv != 0.0) atomicAdd(&red[rb + RED_VIRIAL], dv);
    }
    epot = 0.f;
    vir = 0.f;
}

// Stage the home cell's particles [g0, g0 + n) at staged indices 0 .. n-1 (task 13: no shift).
template <bool kDPD, bool kFlux, bool kSig, class ST>
__device__ __forceinline__ void stage_home_body(const PairKernelArgs &a, ST &S, int g0, int n, int lane) {
#pragma unroll 1
    for (int k = lane; k < n; k += 32) {
        const int g = g0 + k;
        const float4 ax = a.aux[g];
        S.pos[k] = a.pos[g];
        if (kSig) S.acc[k] = make_float4(0.f, 0.f, 0.f, 0.f);
        S.gslot[k] = g;
        S.rad[k] = ax.x;
        S.seg[k] = 13;
        if (!kSig && kDPD) {
            S.vel[k] = a.vel[g];
            S.id[k] = __float_as_int(ax.w);
        }
        if (!kSig && kFlux) S.sv[k] = a.sval[g];
    }
}

// Signature variant: add the staged partner counts and id hashes to the per-id totals.
template <class ST>
__device__ __forceinline__ void flush_sig(const PairKernelArgs &a, ST &S, int b0, int b1, int lane) {
#pragma unroll 1
    for (int k = b0 + lane; k < b1; k += 32) {
        const float4 v = S.acc[k];
        const int c = __float_as_int(v.x);
        if (c) {
            const int id = __float_as_int(a.aux[S.gslot[k]].w);
            atomicAdd(&a.sig_count[id], c);
            atomicAdd(&a.sig_hash[id], (uint32_t)__float_as_int(v.y));
        }
    }
}

// Stage entries [f0, f1) of the flat list of this work item's neighbour particles (the
// forward tasks' offsets and first slots are in S.toff / S.tg0) at staged index base on, in
// passes of 64 whose loads are in flight together.  When pruning, a particle is staged only
// when its position in the home frame (x + its task's shift) lies within sqrt(S.box[0].w) of
// the box S.box that holds every home particle: any other one is farther than the cutoff
// from every home particle, so no pair is lost.  Staged particles keep the list order.
// Returns the number staged.
template <bool kDPD, bool kFlux, bool kSig, class ST>
__device__ __forceinline__ int stage_flat_body(const PairKernelArgs &a, ST &S, int base, int f0, int f1, int lane,
                                               bool prune) {
    int kept = 0;
#pragma unroll 1
    for (int b0 = f0; b0 < f1; b0 += 64) {
        // two lanes' worth of particles per pass: both loads issue before either is used
        int g[2], tk[2];
        float4 p[2], ax[2];
        bool keep[2];
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int idx = b0 + 32 * h + lane;
            keep[h] = idx < f1;
            int L = 0;   // the last forward task whose flat offset is <= idx
#pragma unroll
            for (int st = 8; st > 0; st >>= 1)
                if (L + st < 13 && S.toff[L + st] <= idx) L += st;
            tk[h] = 14 + L;
            g[h] = keep[h] ? S.tg0[L] + (idx - S.toff[L]) : 0;   // slot 0 exists: the pass has particles
            p[h] = a.pos[g[h]];
            ax[h] = a.aux[g[h]];
        }
#pragma unroll
        for (int h = 0; h < 2; h++) {
            if (prune && keep[h]) {
                const float4 lo = S.box[0], hi = S.box[1];
                const float *sh = S.sh[tk[h]];
                const float xs = p[h].x + sh[0], ys = p[h].y + sh[1], zs = p[h].z + sh[2];
                const float dx = fmaxf(fmaxf(lo.x - xs, xs - hi.x), 0.f);
                const float dy = fmaxf(fmaxf(lo.y - ys, ys - hi.y), 0.f);
                const float dz = fmaxf(fmaxf(lo.z - zs, zs - hi.z), 0.f);
                keep[h] = fmaf(dx, dx, fmaf(dy, dy, dz * dz)) <= lo.w;
            }
            const uint32_t m = __ballot_sync(0xffffffffu, keep[h]);
            if (keep[h]) {
                const int d = base + kept + __popc(m & lanemask_lt());
                S.pos[d] = p[h];
                if (kSig) S.acc[d] = make_float4(0.f, 0.f, 0.f, 0.f);
                S.gslot[d] = g[h];
                S.rad[d] = ax[h].x;
                S.seg[d] = (uint8_t)tk[h];
                if (!kSig && kDPD) {
                    S.vel[d] = a.vel[g[h]];
                    S.id[d] = __float_as_int(ax[h].w);
                }
                if (!kSig && kFlux) S.sv[d] = a.sval[g[h]];
            }
            kept += __popc(m);
        }
    }
    return kept;
}

// Staging runs once per work item, not per pair.  Out of line it keeps the hot candidate and
// evaluation loop of the table variants small in instruction cache; the DPD and flux
// variants, whose evaluation is inlined once, run faster with it inline.
template <bool kDPD, bool kFlux, bool kSig, class ST>
__device__ __noinline__ void stage_home_call(const PairKernelArgs &a, ST &S, int g0, int n, int lane) {
    stage_home_body<kDPD, kFlux, kSig>(a, S, g0, n, lane);
}
template <bool kDPD, bool kFlux, bool kSig, class ST>
__device__ __noinline__ int stage_flat_call(const PairKernelArgs &a, ST &S, int base, int f0, int f1, int lane,
                                            bool prune) {
    return stage_flat_body<kDPD, kFlux, kSig>(a, S, base, f0, f1, lane, prune);
}
template <bool kDPD, bool kFlux, bool kSig, class ST>
__device__ __forceinline__ int stage_flat(const PairKernelArgs &a, ST &S, int base, int f0, int f1, int lane,
                                          bool prune) {
    if constexpr (kDPD || kFlux) return stage_flat_body<kDPD, kFlux, kSig>(a, S, base, f0, f1, lane, prune);
    else return stage_flat_call<kDPD, kFlux, kSig>(a, S, base, f0, f1, lane, prune);
}
template <bool kDPD, bool kFlux, bool kSig, class ST>
__device__ __forceinline__ void stage_home(const PairKernelArgs &a, ST &S, int g0, int n, int lane) {
    if constexpr (kDPD || kFlux) stage_home_body<kDPD, kFlux, kSig>(a, S, g0, n, lane);
    else stage_home_call<kDPD, kFlux, kSig>(a, S, g0, n, lane);
}

// kVerlet (table variants): simulations in Verlet mode record, on their rebuild steps, the
// pairs within the list radius of every staged chunk, and on the other steps evaluate
// those lists instead of testing every candidate pair (engine_flag_verlet; the reference
// keeps its sorted windows between rebuilds instead, tf_runner_dopair.cpp:115-117).
template <bool kDPD, bool kFlux, bool kDensity, bool kSig, bool kVerlet = false, int kW = kWarps>
__global__ void __launch_bounds__(kW * 32, 32 / kW) k_pair_tile(TileArgs T) {
    using Staged = typename TileOf<kDPD, kFlux, kSig>::S;
    constexpr int kCap = Staged::cap;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Staged *L = reinterpret_cast<Staged *>(smem_raw);
    PotDev *spot_smem = reinterpret_cast<PotDev *>(smem_raw + sizeof(Staged) * kW);
    float *sblob = reinterpret_cast<float *>(spot_smem + T.stage_pots);
    const PairKernelArgs &a = T.a;

    // potential descriptors and tables in shared memory when they fit (TilePlan), else
    // read through L1
    const int npots = a.nsims * a.max_type * a.max_type;
    const bool staged = a.blob_floats <= T.stage_floats && npots <= T.stage_pots;
    if (staged) {
        for (int k = threadIdx.x; k < a.blob_floats; k += blockDim.x) sblob[k] = a.blob[k];
        for (int k = threadIdx.x; k < npots; k += blockDim.x) spot_smem[k] = a.pots[k];
    }
    __syncthreads();
    const float *blob = staged ? sblob : a.blob;
    const PotDev *spots = staged ? spot_smem : a.pots;

    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    Staged &S = L[wid];
    float epot = 0.f, vir = 0.f;
    int cur_rb = -1;
    const int per = 14 / T.split;
    const int nitems = a.ncells * T.split;

    // warps take items (home cell x task group) from a shared counter, T.grab at a time, so
    // that uneven cells (empty ones, droplet interiors) balance dynamically
    const int grab = T.grab;
    int base = 0;
    if (lane == 0) base = atomicAdd(T.overflow_count + 1, grab);
    base = __shfl_sync(0xffffffffu, base, 0);
    for (; base < nitems;) {
    // the next items are reserved now and read after these, so the atomic's round trip
    // overlaps this work instead of adding to it
    int nxt = 0;
    if (lane == 0) nxt = atomicAdd(T.overflow_count + 1, grab);
#pragma unroll 1
    for (int item = base; item < base + grab && item < nitems; item++) {
        const int home = T.split == 1 ? item : item / T.split, grp = item - home * T.split;
        const int h0 = a.start[home], nh = a.start[home + 1] - h0;
        if (nh == 0) continue;
        const SimParams &P = a.sims[a.cell_sim[home]];
        if (!kSig && P.stopped) continue;
        if (kFlux && a.flux_sub >= 0 && a.flux_sub >= P.nr_fluxsteps - 1) continue;
        if (!kSig && P.red_base != cur_rb) {
            flush_red(a.red, cur_rb, epot, vir, lane);
            cur_rb = P.red_base;
        }
        const float cutoff2 = P.cutoff2;
        // pair list of this item: 1 = build it (candidate tests record the pairs within the
        // list radius), 2 = walk it, 0 = candidate tests only
        int lmode = 0, lcount = 0, lvalid = 0;
        uint32_t *lst = nullptr;
        float rlist2 = 0.f;
        if (kVerlet && (P.flags & TFG_ENGINE_VERLET)) {
            lvalid = a.vlen[item];
            lmode = P.verlet_rebuild ? 1 : (lvalid >= 0 ? 2 : 0);
            lst = a.vlist + (size_t)item * a.list_k;
            rlist2 = P.rlist2;
        }
        const int t0 = 13 + grp * per, t1 = t0 + per;
        int li, lj, lk;
        cell_loc(P, home, li, lj, lk);
        // lane L (< 13) describes forward task 14+L: partner cell start, count and shift
        int my_g0 = 0, my_n = 0;
        if (lane < 13) {
            const int d = 14 + lane;
            const int ox = d / 9 - 1, oy = (d / 3) % 3 - 1, oz = d % 3 - 1;
            // periodic wrap of a +-1 offset, without an integer division
            const int mi = wrap1(li + ox, P.cdim[0]);
            const int mj = wrap1(lj + oy, P.cdim[1]);
            const int mk = wrap1(lk + oz, P.cdim[2]);
            const int c = cell_index(P, mi, mj, mk);
            my_g0 = a.start[c];
            my_n = a.start[c + 1] - my_g0;
            // no cell pair across the edge of a non-periodic axis
            if (!(nb_exists(P, 0, li, ox) && nb_exists(P, 1, lj, oy) && nb_exists(P, 2, lk, oz))) my_n = 0;
            S.sh[d][0] = cell_shift(P, 0, li, mi);
            S.sh[d][1] = cell_shift(P, 1, lj, mj);
            S.sh[d][2] = cell_shift(P, 2, lk, mk);
        }
        if (lane == 13) { S.sh[13][0] = 0.f; S.sh[13][1] = 0.f; S.sh[13][2] = 0.f; }
        __syncwarp();
        // capacity: a home cell above kHomeCap goes to the overflow pass (every group of the
        // cell takes the same decision); neighbour cells of any size are staged in chunks
        if (nh > kHomeCap) {
            if (lane == 0 && grp == 0) {
                const int k = atomicAdd(T.overflow_count, 1);
                T.overflow_list[k] = home;
            }
            if (kVerlet && lmode == 1 && lane == 0) a.vlen[item] = -1;
            continue;
        }
        stage_home<kDPD, kFlux, kSig>(a, S, h0, nh, lane);
        __syncwarp();
        // the box that holds every home particle, for the neighbour staging's pruning, with the
        // squared cutoff and a 1e-4 relative margin (far above the few-ulp difference between
        // this box distance and the reference's r2)
        const bool prune = !kVerlet && T.prune && t1 > 14;
        if (prune) {
            float4 blo = make_float4(3.0e38f, 3.0e38f, 3.0e38f, cutoff2 * 1.0001f);
            float4 bhi = make_float4(-3.0e38f, -3.0e38f, -3.0e38f, 0.f);
#pragma unroll 1
            for (int k = lane; k < nh; k += 32) {
                const float4 p4 = S.pos[k];
                blo.x = fminf(blo.x, p4.x); blo.y = fminf(blo.y, p4.y); blo.z = fminf(blo.z, p4.z);
                bhi.x = fmaxf(bhi.x, p4.x); bhi.y = fmaxf(bhi.y, p4.y); bhi.z = fmaxf(bhi.z, p4.z);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                blo.x = fminf(blo.x, __shfl_xor_sync(0xffffffffu, blo.x, o));
                blo.y = fminf(blo.y, __shfl_xor_sync(0xffffffffu, blo.y, o));
                blo.z = fminf(blo.z, __shfl_xor_sync(0xffffffffu, blo.z, o));
                bhi.x = fmaxf(bhi.x, __shfl_xor_sync(0xffffffffu, bhi.x, o));
                bhi.y = fmaxf(bhi.y, __shfl_xor_sync(0xffffffffu, bhi.y, o));
                bhi.z = fmaxf(bhi.z, __shfl_xor_sync(0xffffffffu, bhi.z, o));
            }
            if (lane == 0) {
                S.box[0] = blo;
                S.box[1] = bhi;
            }
            __syncwarp();
        }
        // wall potentials of the home particles, once per home cell (runner_doself's
        // boundary_eval, tf_runner_dopair.cpp:594-596)
        if (!kSig && t0 == 13 && a.has_wall_pots && P.walls_active && !(kFlux && a.flux_sub >= 0)) {
#pragma unroll 1
            for (int k = lane; k < nh; k += 32) {
                const float4 p4 = S.pos[k];
                const int g = S.gslot[k];
                float3 fw = make_float3(0.f, 0.f, 0.f);
                float ew = 0.f;
                wall_eval(P, a.wpots, blob, __float_as_int(p4.w), make_float3(p4.x, p4.y, p4.z), S.rad[k],
                          a.vel[g], __float_as_int(a.aux[g].w) - P.id_off, li, lj, lk, fw, ew);
                if (fw.x != 0.f || fw.y != 0.f || fw.z != 0.f) atomicAdd(&a.force[g], make_float4(fw.x, fw.y, fw.z, 0.f));
                epot += ew;
            }
            __syncwarp();
        }

        // The neighbour cells of this work item form one flat list (task order, cell order);
        // each chunk stages as much of it as fits after the home cell.
        const int tf = t0 < 14 ? 14 : t0;     // first neighbour task of this item
        bool with_self = (t0 == 13);
        int total = 0;
        if (tf < t1) {
            const bool inc = lane >= tf - 14 && lane < t1 - 14;
            const int cnt = inc ? my_n : 0;
            int incl = cnt;
#pragma unroll
            for (int o = 1; o < 16; o <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += v;
            }
            total = __shfl_sync(0xffffffffu, incl, 15);
            if (lane < 13) {
                S.toff[lane] = lane < tf - 14 ? -1 : (inc ? incl - cnt : 0x7fffffff);
                S.tg0[lane] = my_g0;
            }
            __syncwarp();
        }
        int fpos = 0;   // next flat entry to stage
        while (with_self || fpos < total) {
            // walk: the chunk's first group of list entries loads while its particles are staged
            uint4 gnext = make_uint4(kListEnd, kListEnd, kListEnd, kListEnd);
            if (kVerlet && lmode == 2 && lcount + 4 * lane < lvalid)
                gnext = *reinterpret_cast<const uint4 *>(lst + lcount + 4 * lane);
            int end = nh;
            if (fpos < total) {   // nh <= kHomeCap < kCap, so every chunk takes at least one entry
                const int take = min(total - fpos, kCap - end);
                end += stage_flat<kDPD, kFlux, kSig>(a, S, end, fpos, fpos + take, lane, prune);
                fpos += take;
            }
            __syncwarp();
            const int tbeg = with_self ? 0 : nh;
            const int ntgt = end - tbeg;
            with_self = false;
            int qhead = 0, qtail = 0;
            if (kVerlet && lmode == 2) {
                // the list entries of this chunk, up to its marker: re-test each pair at the
                // cutoff with the current positions, queue the hits, evaluate 32 at a time
                bool done = false;
                int c = 0;              // batch of 32 within the current group
                uint4 gcur = gnext;
                for (;;) {
                    if (!done) {
                        if (c == 0) {   // the next group loads while this one is tested
                            const bool end_here =
                                __any_sync(0xffffffffu, gcur.x == kListEnd || gcur.y == kListEnd ||
                                                            gcur.z == kListEnd || gcur.w == kListEnd);
                            gnext = make_uint4(kListEnd, kListEnd, kListEnd, kListEnd);
                            if (!end_here && lcount + 128 + 4 * lane < lvalid)
                                gnext = *reinterpret_cast<const uint4 *>(lst + lcount + 128 + 4 * lane);
                        }
                        const uint32_t e = c == 0 ? gcur.x : (c == 1 ? gcur.y : (c == 2 ? gcur.z : gcur.w));
                        const uint32_t mm = __ballot_sync(0xffffffffu, e == kListEnd);
                        const int fm = mm ? __ffs(mm) - 1 : 32;
                        const int I = e & 0xffff, K = e >> 16;
                        bool hit = false;
                        if (lane < fm && I < end && K < end) {
                            const float4 pi4 = S.pos[I], pk = S.pos[K], s4 = staged_shift(S, K);
                            float3 dx;
                            const float r2 = pair_r2(make_float3(pi4.x, pi4.y, pi4.z), make_float3(s4.x, s4.y, s4.z),
                                                     make_float3(pk.x, pk.y, pk.z), dx);
                            hit = r2 <= cutoff2;
                        }
                        const uint32_t m = __ballot_sync(0xffffffffu, hit);
                        if (hit) S.q[(qtail + __popc(m & lanemask_lt())) & (kQ - 1)] = e;
                        qtail += __popc(m);
                        done = fm < 32;
                        if (++c == 4 || done) {
                            c = 0;
                            lcount += 128;
                            gcur = gnext;
                        }
                        __syncwarp();
                    }
                    const int avail = qtail - qhead;
                    if (avail >= 32 || (done && avail > 0)) {
                        const int take = avail < 32 ? avail : 32;
                        const bool act = lane < take;
                        const uint32_t e = act ? S.q[(qhead + lane) & (kQ - 1)] : 0u;
                        eval_batch<kDPD, kFlux, kDensity, kSig>(T, P, S, spots, blob, act, e, epot, vir);
                        qhead += take;
                        __syncwarp();
                    } else if (done) {
                        break;
                    }
                }
            } else if (ntgt > 0) {
                if constexpr (kDPD || kFlux) {
                    // The DPD and flux evaluations are long: the candidate walk over (block of 32
                    // targets, i) pauses whenever 32 hits are queued, so the evaluation has a
                    // single call site (a second inlined copy costs more in instruction fetch
                    // than the resumable walk costs in instructions).
                    int kb = tbeg, i = 0, k = 0, ilim = 0, iend = 0;
                    float3 xk = make_float3(0.f, 0.f, 0.f), shk = xk;
                    for (;;) {
                        while (kb < end && qtail - qhead < 32) {
                            if (i == 0) {
                                k = kb + lane;
                                float4 pk = make_float4(0.f, 0.f, 0.f, 0.f), s4 = pk;
                                if (k < end) {
                                    pk = S.pos[k];
                                    s4 = staged_shift(S, k);
                                }
                                ilim = k < end ? (k < nh ? k : nh) : 0;
                                iend = kb + 31 < nh ? kb + 31 : nh;
                                xk = make_float3(pk.x, pk.y, pk.z);
                                shk = make_float3(s4.x, s4.y, s4.z);
                            }
                            const float4 pi4 = S.pos[i];
                            float3 dx;
                            const float r2 = pair_r2(make_float3(pi4.x, pi4.y, pi4.z), shk, xk, dx);
                            const bool hit = i < ilim && r2 <= cutoff2;
                            const uint32_t m = __ballot_sync(0xffffffffu, hit);
                            if (hit)
                                S.q[(qtail + __popc(m & lanemask_lt())) & (kQ - 1)] = (uint32_t)i | ((uint32_t)k << 16);
                            qtail += __popc(m);
                            if (++i >= iend) {
                                i = 0;
                                kb += 32;
                            }
                        }
                        __syncwarp();
                        const int avail = qtail - qhead;
                        if (avail == 0) break;
                        const int take = avail < 32 ? avail : 32;
                        const bool act = lane < take;
                        const uint32_t e = act ? S.q[(qhead + lane) & (kQ - 1)] : 0u;
                        eval_batch<kDPD, kFlux, kDensity, kSig>(T, P, S, spots, blob, act, e, epot, vir);
                        qhead += take;
                        __syncwarp();
                    }
                } else {
                    // each lane keeps one target k in registers; the home particles i are
                    // broadcast to all lanes.  Self targets (k < nh) pair only with i < k.
                    // Candidates are queued by a cheaper test, x_i - (x_k + shift) with FMA
                    // against the squared cutoff plus 1e-5 relative (far above the few-ulp
                    // difference to the reference's (x_i - shift) - x_k); the evaluation and
                    // the signature then apply the reference's test, so the pair set is exact.
                    for (int kb = tbeg; kb < end; kb += 32) {
                        const int k = kb + lane;
                        float4 pk = make_float4(0.f, 0.f, 0.f, 0.f), s4 = pk;
                        if (k < end) {
                            pk = S.pos[k];
                            s4 = staged_shift(S, k);
                        }
                        const int ilim = k < end ? (k < nh ? k : nh) : 0;
                        const int iend = kb + 31 < nh ? kb + 31 : nh;
                        const float xs = pk.x + s4.x, ys = pk.y + s4.y, zs = pk.z + s4.z;
                        const float cut_f = cutoff2 * 1.00001f;
                        if constexpr (kVerlet) {
                            for (int i = 0; i < iend; i++) {
                                const float4 pi4 = S.pos[i];
                                const float ddx = pi4.x - xs, ddy = pi4.y - ys, ddz = pi4.z - zs;
                                const float r2 = fmaf(ddx, ddx, fmaf(ddy, ddy, ddz * ddz));
                                const bool hit = i < ilim && r2 <= cut_f;
                                if (lmode == 1) {
                                    const bool lh = i < ilim && r2 <= rlist2;
                                    const uint32_t lm = __ballot_sync(0xffffffffu, lh);
                                    if (lh) {
                                        const int lp = lcount + __popc(lm & lanemask_lt());
                                        if (lp < a.list_k) lst[list_slot(lp)] = (uint32_t)i | ((uint32_t)k << 16);
                                    }
                                    lcount += __popc(lm);
                                }
                                const uint32_t m = __ballot_sync(0xffffffffu, hit);
                                if (hit)
                                    S.q[(qtail + __popc(m & lanemask_lt())) & (kQ - 1)] = (uint32_t)i | ((uint32_t)k << 16);
                                qtail += __popc(m);
                                __syncwarp();
                                if (qtail - qhead >= 32) {
                                    const uint32_t e = S.q[(qhead + lane) & (kQ - 1)];
                                    eval_batch<kDPD, kFlux, kDensity, kSig>(T, P, S, spots, blob, true, e, epot, vir);
                                    qhead += 32;
                                    __syncwarp();
                                }
                            }
                        } else {
                            // kUnroll home particles per pass share the queue bookkeeping; i < ilim
                            // implies i < iend, so the reads past iend (still inside pos[]) are
                            // never queued
                            const uint32_t lt = lanemask_lt();
                            for (int i = 0; i < iend; i += kUnroll) {
                                int add = 0;
#pragma unroll
                                for (int u = 0; u < kUnroll; u++) {
                                    const int ii = i + u;
                                    const float4 pi4 = S.pos[ii];
                                    const float ddx = pi4.x - xs, ddy = pi4.y - ys, ddz = pi4.z - zs;
                                    const float r2 = fmaf(ddx, ddx, fmaf(ddy, ddy, ddz * ddz));
                                    const bool hit = ii < ilim && r2 <= cut_f;
                                    const uint32_t m = __ballot_sync(0xffffffffu, hit);
                                    if (hit)
                                        S.q[(qtail + add + __popc(m & lt)) & (kQ - 1)] = (uint32_t)ii | ((uint32_t)k << 16);
                                    add += __popc(m);
                                }
                                qtail += add;
                                __syncwarp();
                                while (qtail - qhead >= 32) {
                                    const uint32_t e = S.q[(qhead + lane) & (kQ - 1)];
                                    eval_batch<kDPD, kFlux, kDensity, kSig>(T, P, S, spots, blob, true, e, epot, vir);
                                    qhead += 32;
                                    __syncwarp();
                                }
                            }
                        }
                    }
                    if (qtail > qhead) {
                        const bool act = lane < qtail - qhead;
                        const uint32_t e = act ? S.q[(qhead + lane) & (kQ - 1)] : 0u;
                        eval_batch<kDPD, kFlux, kDensity, kSig>(T, P, S, spots, blob, act, e, epot, vir);
                    }
                }
                __syncwarp();
            }
            if (kVerlet && lmode == 1) {   // end of this chunk's entries; the next starts a group
                if (lane == 0 && lcount < a.list_k) lst[list_slot(lcount)] = kListEnd;
                lcount = (lcount + 128) & ~127;
            }
            if (kSig) flush_sig(a, S, nh, end, lane);
            __syncwarp();
        }
        if (kSig) flush_sig(a, S, 0, nh, lane);
        if (kVerlet && lmode == 1 && lane == 0) {
            a.vlen[item] = lcount <= a.list_k ? lcount : -1;
            atomicMax(a.list_need, lcount);
        }
        __syncwarp();
    }
    base = __shfl_sync(0xffffffffu, nxt, 0);
    }
    if (kSig) return;
    flush_red(a.red, cur_rb, epot, vir, lane);
}

// Home cells above the tiled kernel's home capacity (crowded clusters): candidates read
// from global memory, accumulation with global atomics, same orientation and arithmetic as
// the tiled kernel.  The work of one listed cell is spread over 14 x kOverflowParts warps
// (task, and a share of the task's candidate pairs), so that one crowded cell does not
// leave a single warp working while the rest of the GPU waits.
constexpr int kOverflowParts = 8;
template <bool kDPD, bool kFlux, bool kDensity, bool kSig>
__global__ void __launch_bounds__(256) k_pair_overflow(TileArgs T) {
    const PairKernelArgs &a = T.a;
    const int lane = threadIdx.x & 31;
    const int nlist = *T.overflow_count;
    float epot = 0.f, vir = 0.f;
    const long long nwork = (long long)nlist * 14 * kOverflowParts;
    for (long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; w < nwork;
         w += ((long long)gridDim.x * blockDim.x) >> 5) {
        const int home = T.overflow_list[w / (14 * kOverflowParts)];
        const int d = 13 + (int)((w / kOverflowParts) % 14);   // this warp's task
        const int part = (int)(w % kOverflowParts);             // and its share of the pairs
        const int h0 = a.start[home], nh = a.start[home + 1] - h0;
        const SimParams &P = a.sims[a.cell_sim[home]];
        if (!kSig && P.stopped) continue;
        const bool flux_only = kFlux && a.flux_sub >= 0;
        if (flux_only && a.flux_sub >= P.nr_fluxsteps - 1) continue;
        int li, lj, lk;
        cell_loc(P, home, li, lj, lk);
        if (!kSig && !flux_only && a.has_wall_pots && P.walls_active && d == 13 && part == 0) {
            for (int i = lane; i < nh; i += 32) {
                const int g = h0 + i;
                const float4 p4 = a.pos[g], ax4 = a.aux[g];
                float3 fw = make_float3(0.f, 0.f, 0.f);
                float ew = 0.f;
                wall_eval(P, a.wpots, a.blob, __float_as_int(p4.w), make_float3(p4.x, p4.y, p4.z), ax4.x, a.vel[g],
                          __float_as_int(ax4.w) - P.id_off, li, lj, lk, fw, ew);
                if (fw.x != 0.f || fw.y != 0.f || fw.z != 0.f) atomicAdd(&a.force[g], make_float4(fw.x, fw.y, fw.z, 0.f));
                epot += ew;
            }
        }
        do {   // this warp's task (the continue below leaves it)
            const int ox = d / 9 - 1, oy = (d / 3) % 3 - 1, oz = d % 3 - 1;
            const bool self = d == 13;
            const int mi = (li + ox + P.cdim[0]) % P.cdim[0];
            const int mj = (lj + oy + P.cdim[1]) % P.cdim[1];
            const int mk = (lk + oz + P.cdim[2]) % P.cdim[2];
            if (!(nb_exists(P, 0, li, ox) && nb_exists(P, 1, lj, oy) && nb_exists(P, 2, lk, oz))) continue;
            const int c = cell_index(P, mi, mj, mk);
            const int g0 = a.start[c], nn = a.start[c + 1] - g0;
            float3 sh = make_float3(0.f, 0.f, 0.f);
            if (!self) {
                sh.x = cell_shift(P, 0, li, mi);
                sh.y = cell_shift(P, 1, lj, mj);
                sh.z = cell_shift(P, 2, lk, mk);
            }
            const long long total = (long long)nh * nn;
            for (long long p = 32 * part + lane; p < total; p += 32 * kOverflowParts) {
                const int i = (int)(p / nn), j = (int)(p % nn);
                if (self && i >= j) continue;
                const int gi = h0 + i, gj = g0 + j;
                const float4 pi = a.pos[gi], pj = a.pos[gj];
                float3 dx;
                const float r2 = pair_r2(make_float3(pi.x, pi.y, pi.z), sh, make_float3(pj.x, pj.y, pj.z), dx);
                if (r2 > P.cutoff2) continue;
                const float4 axi = a.aux[gi], axj = a.aux[gj];
                if (kSig) {
                    atomicAdd(&a.sig_count[__float_as_int(axi.w)], 1);
                    atomicAdd(&a.sig_count[__float_as_int(axj.w)], 1);
                    atomicAdd(&a.sig_hash[__float_as_int(axi.w)], sig_mix((uint32_t)__float_as_int(axj.w)));
                    atomicAdd(&a.sig_hash[__float_as_int(axj.w)], sig_mix((uint32_t)__float_as_int(axi.w)));
                    record_pair(a, __float_as_int(axi.w), __float_as_int(axj.w));
                    continue;
                }
                const float r = __fsqrt_rn(r2);
                float4 fi = make_float4(0.f, 0.f, 0.f, 0.f), fj = make_float4(0.f, 0.f, 0.f, 0.f);
                if (kDensity && !flux_only) {
                    const float wd = density_w(r, P.inv_cutoff, P.self_density);
                    fi.w = wd;
                    fj.w = wd;
                }
                const int ti = __float_as_int(pi.w), tj = __float_as_int(pj.w);
                const int pidx = P.pot_base + ti * a.max_type + tj;
                if (kFlux) {
                    const FluxSet &fs = a.fluxes[pidx];
                    for (int k = 0; k < fs.count; k++) {
                        const FluxDev &F = fs.f[k];
                        if (r > F.cutoff) continue;
                        float term = __fsub_rn(1.0f, __fdividef(r, F.cutoff));
                        term = __fmul_rn(term, term);
                        const int sa = (ti == F.type_a) ? gi : gj, sb = (tj == F.type_b) ? gj : gi;
                        const float ssi = a.sval[F.index_a * a.cap + sa], ssj = a.sval[F.index_b * a.cap + sb];
                        float q = term;
                        if (F.kind == TFG_FLUX_FICK) {
                            q = __fmul_rn(q, __fmul_rn(F.coef, __fsub_rn(ssi, ssj)));
                        } else if (F.kind == TFG_FLUX_SECRETE) {
                            const float qq = __fmul_rn(F.coef, __fsub_rn(ssi, F.target));
                            q = __fmul_rn(q, qq > 0.f ? qq : 0.f);
                        } else {
                            const float qq = __fmul_rn(__fmul_rn(F.coef, __fsub_rn(F.target, ssj)), ssi);
                            q = __fmul_rn(q, qq > 0.f ? qq : 0.f);
                        }
                        atomicAdd(&a.sq[F.index_a * a.cap + sa], -q - F.half_decay * ssi);
                        atomicAdd(&a.sq[F.index_b * a.cap + sb], q - F.half_decay * ssj);
                    }
                }
                if (flux_only) continue;
                const PotDev &pot = a.pots[pidx];
                if (pot.kind == POT_TABLE) {
                    float e, f;
                    if (table_eval(pot, a.blob, axi.x, axj.x, r2, e, f)) {
                        fi.x -= f * dx.x; fi.y -= f * dx.y; fi.z -= f * dx.z;
                        fj.x += f * dx.x; fj.y += f * dx.y; fj.z += f * dx.z;
                        epot += e;
                        vir -= f * r2;
                    }
                } else if (kDPD && pot.kind == POT_DPD) {
                    float rr = r;
                    const float ro = r < 1.1920928955078125e-7f ? 1.1920928955078125e-7f : r;
                    if (pot.flags & TFG_POTENTIAL_SHIFTED) rr = __fsub_rn(rr, __fadd_rn(axi.x, axj.x));
                    if (rr <= pot.b) {
                        rr = rr >= pot.a ? rr : pot.a;
                        const float4 vi = a.vel[gi], vj = a.vel[gj];
                        const float inv_ro = __fdividef(1.0f, ro);
                        const float ex = dx.x * inv_ro, ey = dx.y * inv_ro, ez = dx.z * inv_ro;
                        const float omega_c = rr < 0.f ? 1.f : 1.f - __fdividef(rr, pot.b);
                        const float edv = ex * (vi.x - vj.x) + ey * (vi.y - vj.y) + ez * (vi.z - vj.z);
                        float xi_r = 1.0f;
                        if (!(P.flags & TFG_ENGINE_DPD_REFERENCE_RANDOM))
                            xi_r = gauss_pair(P.seed, P.time, __float_as_int(axi.w) - P.id_off,
                                              __float_as_int(axj.w) - P.id_off);
                        const float ftot = pot.dpd_alpha * omega_c - pot.dpd_gamma * omega_c * omega_c * edv +
                                           pot.dpd_sigma * omega_c * xi_r * P.dpd_delta;
                        fi.x += ftot * ex; fi.y += ftot * ey; fi.z += ftot * ez;
                        fj.x -= ftot * ex; fj.y -= ftot * ey; fj.z -= ftot * ez;
                        vir += ftot * ro;
                    }
                }
                atomicAdd(&a.force[gi], fi);
                atomicAdd(&a.force[gj], fj);
            }
        } while (0);
        if (!kSig) flush_red(a.red, P.red_base, epot, vir, lane);
    }
}

template <bool kDPD, bool kFlux, bool kDensity, bool kSig, bool kVerlet = false, int kW = kWarps>
void launch_variant(const TileArgs &T0, cudaStream_t s, int sms) {
    const size_t base = sizeof(typename TileOf<kDPD, kFlux, kSig>::S) * kW;
    const size_t smem_max = base + sizeof(float) * kMaxSmemTable + sizeof(PotDev) * kMaxSmemPots;
    // Tables and descriptors are staged only while a CTA still fits 32 / kW per SM (four of 8
    // warps): those CTAs are worth more than shared-memory tables (the table variants' staging
    // alone takes 56 KB per 8 warps, so their tables are always read through L1)
    const size_t cta_budget = kFourCtaBytes * kW / kWarps;
    TileArgs T = T0;
    if (base + sizeof(PotDev) * T.stage_pots + sizeof(float) * ((T.stage_floats + 3) & ~3) > cta_budget) {
        T.stage_floats = 0;
        T.stage_pots = 0;
    }
    const size_t smem = base + sizeof(PotDev) * T.stage_pots + sizeof(float) * ((T.stage_floats + 3) & ~3);
    static bool configured = false;
    static size_t occ_smem = 0;
    static int per_sm = 1;
    if (!configured) {
        cudaFuncSetAttribute(k_pair_tile<kDPD, kFlux, kDensity, kSig, kVerlet, kW>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max);
        configured = true;
    }
    if (occ_smem != smem) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pair_tile<kDPD, kFlux, kDensity, kSig, kVerlet, kW>,
                                                      kW * 32, smem);
        if (per_sm < 1) per_sm = 1;
        occ_smem = smem;
    }
    const int want = (T.a.ncells * T.split + kW - 1) / kW;
    const int grid = std::max(1, std::min(want, sms * per_sm));
    k_pair_tile<kDPD, kFlux, kDensity, kSig, kVerlet, kW><<<grid, kW * 32, smem, s>>>(T);
    k_pair_overflow<kDPD, kFlux, kDensity, kSig><<<sms, 256, 0, s>>>(T);
}

}  // namespace

int pair_tile_capacity() { return kCapT; }

void launch_pair_overflow(const PairKernelArgs &a, int *overflow_list, int *overflow_count, bool signature, int sms,
                          cudaStream_t s) {
    TileArgs T;
    T.a = a;
    T.overflow_list = overflow_list;
    T.overflow_count = overflow_count;
    T.split = 1;
    T.grab = 1;
    T.stage_floats = 0;
    T.stage_pots = 0;
    T.prune = 0;
    if (signature) k_pair_overflow<false, false, false, true><<<sms, 256, 0, s>>>(T);
    else if (!(a.flags & TFG_ENGINE_NO_DENSITY)) k_pair_overflow<false, false, true, false><<<sms, 256, 0, s>>>(T);
    else k_pair_overflow<false, false, false, false><<<sms, 256, 0, s>>>(T);
}

void launch_pair_fluxonly(const PairKernelArgs &a, const TilePlan &plan, int *overflow_list, int *overflow_count,
                          int sms, bool tile, cudaStream_t s) {
    if (!tile) {
        launch_pair_stencil_fluxonly(a, s);
        return;
    }
    TileArgs T;
    T.a = a;
    T.overflow_list = overflow_list;
    T.overflow_count = overflow_count;
    T.split = 1;
    T.grab = 1;
    T.stage_floats = plan.stage_floats;
    T.stage_pots = plan.stage_pots;
    T.prune = 1;
    cudaMemsetAsync(overflow_count, 0, 2 * sizeof(int), s);
    if (a.n <= 0) return;
    launch_variant<false, true, false, false>(T, s, sms);
}

TilePlan plan_pair_tile(int nsims, int max_type, int blob_floats) {
    TilePlan p;
    if (blob_floats <= kMaxSmemTable && nsims * max_type * max_type <= kMaxSmemPots) {
        p.stage_floats = blob_floats;
        p.stage_pots = nsims * max_type * max_type;
    }
    return p;
}

void launch_pair_tile(const PairKernelArgs &a, const TilePlan &plan, int *overflow_list, int *overflow_count, int sms,
                      bool signature, const TileTune &tune, cudaStream_t s) {
    const int split = tune.split;
    TileArgs T;
    T.a = a;
    T.overflow_list = overflow_list;
    T.overflow_count = overflow_count;
    T.split = (split == 1 || split == 2 || split == 7 || split == 14) ? split : 1;
    T.grab = tune.grab >= 1 && tune.grab <= 8 ? tune.grab : 1;
    T.stage_floats = plan.stage_floats;
    T.stage_pots = plan.stage_pots;
    T.prune = 1;
    cudaMemsetAsync(overflow_count, 0, 2 * sizeof(int), s);
    if (a.n <= 0) return;
    const bool dpd = a.has_dpd, flux = a.nspec > 0 && a.has_flux;
    const bool dens = !(a.flags & TFG_ENGINE_NO_DENSITY);
    if (split == TFG_PAIR_HOME_OUTER && pair_home_eligible(a)) {
        launch_pair_home(a, overflow_list, overflow_count, sms, signature, s);
        return;
    }
    if (signature) {
        if (a.vlist) launch_variant<false, false, false, true, true>(T, s, sms);
        else launch_variant<false, false, false, true>(T, s, sms);
        return;
    }
    if (a.vlist && !dpd && !flux) {   // Verlet pair lists (some simulation in Verlet mode)
        if (dens) launch_variant<false, false, true, false, true>(T, s, sms);
        else launch_variant<false, false, false, false, true>(T, s, sms);
        return;
    }
    if (!dpd && !flux && tune.warps == 4) {   // the table variants also come in CTAs of 4 warps
        if (dens) launch_variant<false, false, true, false, false, 4>(T, s, sms);
        else launch_variant<false, false, false, false, false, 4>(T, s, sms);
        return;
    }
#define TFG_PAIR_DISPATCH(D, F)                                          \
    if (dens) launch_variant<D, F, true, false>(T, s, sms);              \
    else launch_variant<D, F, false, false>(T, s, sms);
    if (dpd && flux) { TFG_PAIR_DISPATCH(true, true) }
    else if (dpd) { TFG_PAIR_DISPATCH(true, false) }
    else if (flux) { TFG_PAIR_DISPATCH(false, true) }
    else { TFG_PAIR_DISPATCH(false, false) }
#undef TFG_PAIR_DISPATCH
}

}  // namespace tfg
