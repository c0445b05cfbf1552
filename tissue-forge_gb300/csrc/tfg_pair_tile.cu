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
// all 32 lanes test candidate pairs (r2 with the reference's unfused FP32 arithmetic, so
// the pair set is bit-identical), hits go to a warp-private ring queue, and the queue is
// evaluated 32 pairs at a time so the force arithmetic runs with full lanes.  Forces,
// number densities and flux increments of both partners accumulate in shared memory and
// each staged particle is flushed once to global memory with a vector atomic add.
// Cells above the staging capacity are listed and handled by k_pair_overflow.
#include <algorithm>

#include "tfg_internal.h"

namespace tfg {

namespace {

constexpr int kWarps = 8;
constexpr int kCap = 64;            // particles of one cell staged per warp (home and neighbour)
constexpr int kQ = 64;              // candidate ring queue entries per warp (power of two)
constexpr int kMaxSmemTable = 4096; // floats of potential table staged per CTA

struct Staged {
    float4 pos[2 * kCap];   // [0,kCap): home, [kCap,2kCap): neighbour ; w = type bits
    float4 acc[2 * kCap];   // fx, fy, fz, number density
    float2 rid[2 * kCap];   // radius, id bits
    uint32_t q[kQ];         // packed (i | j << 16), indices into the staged arrays
};

struct StagedDyn {         // DPD and flux extras
    float4 vel[2 * kCap];
    float sval[2 * kCap];  // species 0 (flux supports one species in the tiled path)
    float sq[2 * kCap];
};

template <bool kDPD, bool kFlux> struct SmemLayout {
    Staged st[kWarps];
    StagedDyn dyn[(kDPD || kFlux) ? kWarps : 1];
};

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

struct TileArgs {
    PairKernelArgs a;
    int *overflow_list;    // home cells handed to the overflow kernel
    int *overflow_count;
    int split;             // warps per home cell: the 14 tasks are divided into `split` groups
};

// Evaluate one interacting pair (reference orientation: I = part_i, J = part_j) and
// accumulate into the staged accumulators of both.
template <bool kDPD, bool kFlux, bool kDensity, bool kSig>
__device__ __forceinline__ void eval_pair(const TileArgs &T, Staged &S, StagedDyn &D, const PotDev *pots,
                                          const float *blob, int I, int J, float3 sh, float &epot, float &vir,
                                          float4 &fI) {
    const PairKernelArgs &a = T.a;
    const SimParams &P = a.P;
    const float4 pi = S.pos[I], pj = S.pos[J];
    float3 dx;
    const float r2 = pair_r2(make_float3(pi.x, pi.y, pi.z), sh, make_float3(pj.x, pj.y, pj.z), dx);
    if (kSig) {
        // counters live in the accumulator bits: x = count, y = hash (integer atomics)
        atomicAdd(reinterpret_cast<int *>(&S.acc[I].x), 1);
        atomicAdd(reinterpret_cast<int *>(&S.acc[J].x), 1);
        atomicAdd(reinterpret_cast<unsigned *>(&S.acc[I].y), sig_mix((uint32_t)__float_as_int(S.rid[J].y)));
        atomicAdd(reinterpret_cast<unsigned *>(&S.acc[J].y), sig_mix((uint32_t)__float_as_int(S.rid[I].y)));
        return;
    }
    const float r = __fsqrt_rn(r2);
    if (kDensity) {
        const float w = density_w(r, 1.0f / P.cutoff, P.self_density);
        fI.w += w;
        atomicAdd(&S.acc[J].w, w);
    }
    const int ti = __float_as_int(pi.w), tj = __float_as_int(pj.w);
    const int pidx = ti * P.max_type + tj;
    if (kFlux) {
        const FluxSet &fs = a.fluxes[pidx];
        for (int k = 0; k < fs.count; k++) {
            const FluxDev &F = fs.f[k];
            if (r > F.cutoff) continue;
            float term = __fsub_rn(1.0f, __fdiv_rn(r, F.cutoff));
            term = __fmul_rn(term, term);
            const bool a_is_I = (ti == F.type_a);
            const bool b_is_J = (tj == F.type_b);
            const int sa = a_is_I ? I : J, sb = b_is_J ? J : I;
            const float ssi = D.sval[sa], ssj = D.sval[sb];
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
            atomicAdd(&D.sq[sa], -q - F.half_decay * ssi);
            atomicAdd(&D.sq[sb], q - F.half_decay * ssj);
        }
    }
    const PotDev &pot = pots[pidx];
    if (pot.kind == POT_TABLE) {
        float e, f;
        if (table_eval(pot, blob, S.rid[I].x, S.rid[J].x, r2, e, f)) {
            const float wx = f * dx.x, wy = f * dx.y, wz = f * dx.z;
            fI.x -= wx;
            fI.y -= wy;
            fI.z -= wz;
            atomicAdd(&S.acc[J].x, wx);
            atomicAdd(&S.acc[J].y, wy);
            atomicAdd(&S.acc[J].z, wz);
            epot += e;
            vir -= f * r2;
        }
    } else if (kDPD && pot.kind == POT_DPD) {
        float rr = r;
        const float ro = r < 1.1920928955078125e-7f ? 1.1920928955078125e-7f : r;
        if (pot.flags & TFG_POTENTIAL_SHIFTED) rr = __fsub_rn(rr, __fadd_rn(S.rid[I].x, S.rid[J].x));
        if (rr <= pot.b) {
            rr = rr >= pot.a ? rr : pot.a;
            const float4 vi = D.vel[I], vj = D.vel[J];
            const float inv_ro = 1.0f / ro;
            const float ex = dx.x * inv_ro, ey = dx.y * inv_ro, ez = dx.z * inv_ro;
            const float omega_c = rr < 0.f ? 1.f : 1.f - rr / pot.b;
            const float edv = ex * (vi.x - vj.x) + ey * (vi.y - vj.y) + ez * (vi.z - vj.z);
            float xi_r = 1.0f;
            if (!(P.flags & TFG_ENGINE_DPD_REFERENCE_RANDOM))
                xi_r = gauss_pair(P.seed, P.time, __float_as_int(S.rid[I].y), __float_as_int(S.rid[J].y));
            const float ftot = pot.dpd_alpha * omega_c - pot.dpd_gamma * omega_c * omega_c * edv +
                               pot.dpd_sigma * omega_c * xi_r * P.dpd_delta;
            const float wx = ftot * ex, wy = ftot * ey, wz = ftot * ez;
            // part_i.f += F e ; part_j.f -= F e
            fI.x += wx;
            fI.y += wy;
            fI.z += wz;
            atomicAdd(&S.acc[J].x, -wx);
            atomicAdd(&S.acc[J].y, -wy);
            atomicAdd(&S.acc[J].z, -wz);
            vir += ftot * ro;
        }
    }
}

// Evaluate the queued pairs held by the active lanes (entries in enumeration order, so
// equal I form contiguous runs).  The I side is reduced over each run with a segmented
// warp scan and written once per distinct I by the run's last lane; the J side (rarely
// repeated inside a batch) uses shared-memory atomics.
template <bool kDPD, bool kFlux, bool kDensity, bool kSig>
__device__ __forceinline__ void eval_batch(const TileArgs &T, Staged &S, StagedDyn &D, const PotDev *pots,
                                           const float *blob, bool active, uint32_t e, float3 sh, int lane,
                                           float &epot, float &vir) {
    const int I = e & 0xffff, J = e >> 16;
    float4 fI = make_float4(0.f, 0.f, 0.f, 0.f);
    if (active) eval_pair<kDPD, kFlux, kDensity, kSig>(T, S, D, pots, blob, I, J, sh, epot, vir, fI);
    if (kSig) return;
    const int key = active ? I : 1024 + lane;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int k2 = __shfl_up_sync(0xffffffffu, key, o);
        const float x = __shfl_up_sync(0xffffffffu, fI.x, o);
        const float y = __shfl_up_sync(0xffffffffu, fI.y, o);
        const float z = __shfl_up_sync(0xffffffffu, fI.z, o);
        const float w = __shfl_up_sync(0xffffffffu, fI.w, o);
        if (lane >= o && k2 == key) {
            fI.x += x; fI.y += y; fI.z += z; fI.w += w;
        }
    }
    const int knext = __shfl_down_sync(0xffffffffu, key, 1);
    if (active && (lane == 31 || knext != key)) {
        float4 v = S.acc[I];
        v.x += fI.x; v.y += fI.y; v.z += fI.z; v.w += fI.w;
        S.acc[I] = v;
    }
}

// Stage `n` particles of global slots [g0, g0+n) into staged index base..base+n.
template <bool kDPD, bool kFlux, bool kSig>
__device__ __forceinline__ void stage(const PairKernelArgs &a, Staged &S, StagedDyn &D, int base, int g0, int n,
                                      int lane) {
    for (int k = lane; k < n; k += 32) {
        const int g = g0 + k;
        S.pos[base + k] = a.pos[g];
        const float4 ax = a.aux[g];
        S.rid[base + k] = make_float2(ax.x, ax.w);
        S.acc[base + k] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (!kSig && kDPD) D.vel[base + k] = a.vel[g];
        if (!kSig && kFlux) {
            D.sval[base + k] = a.sval[g];
            D.sq[base + k] = 0.f;
        }
    }
}

// Flush staged accumulators of [base, base+n) to the particles at global slots g0...
template <bool kFlux, bool kSig>
__device__ __forceinline__ void flush(const PairKernelArgs &a, Staged &S, StagedDyn &D, int base, int g0, int n,
                                      int lane) {
    for (int k = lane; k < n; k += 32) {
        const float4 v = S.acc[base + k];
        if (kSig) {
            const int id = __float_as_int(S.rid[base + k].y);
            const int c = __float_as_int(v.x);
            if (c) {
                atomicAdd(&a.sig_count[id], c);
                atomicAdd(&a.sig_hash[id], (uint32_t)__float_as_int(v.y));
            }
            continue;
        }
        if (v.x != 0.f || v.y != 0.f || v.z != 0.f || v.w != 0.f) atomicAdd(&a.force[g0 + k], v);
        if (kFlux) {
            const float q = D.sq[base + k];
            if (q != 0.f) atomicAdd(&a.sq[g0 + k], q);
        }
    }
}

template <bool kDPD, bool kFlux, bool kDensity, bool kSig>
__global__ void __launch_bounds__(kWarps * 32) k_pair_tile(TileArgs T) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    using Layout = SmemLayout<kDPD, kFlux>;
    Layout &L = *reinterpret_cast<Layout *>(smem_raw);
    float *sblob = reinterpret_cast<float *>(smem_raw + sizeof(Layout));
    const PairKernelArgs &a = T.a;
    const SimParams &P = a.P;

    // potential tables and descriptors, shared by the CTA
    const int nb = a.blob_floats <= kMaxSmemTable ? a.blob_floats : 0;
    for (int k = threadIdx.x; k < nb; k += blockDim.x) sblob[k] = a.blob[k];
    PotDev *spots = reinterpret_cast<PotDev *>(sblob + ((nb + 3) & ~3));
    const int npots = P.max_type * P.max_type;
    for (int k = threadIdx.x; k < npots; k += blockDim.x) spots[k] = a.pots[k];
    __syncthreads();
    const float *blob = nb ? sblob : a.blob;

    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    Staged &S = L.st[wid];
    StagedDyn &D = L.dyn[(kDPD || kFlux) ? wid : 0];
    float epot = 0.f, vir = 0.f;
    const int nwarps_total = gridDim.x * kWarps;

    const int per = 14 / T.split;                       // tasks per work item
    const int nitems = P.ncells * T.split;
    for (int item = blockIdx.x * kWarps + wid; item < nitems; item += nwarps_total) {
        const int home = item / T.split, grp = item - home * T.split;
        const int h0 = a.start[home], nh = a.start[home + 1] - h0;
        if (nh == 0) continue;
        int li, lj, lk;
        cell_loc(P, home, li, lj, lk);
        // capacity check over the home cell and its forward neighbours
        bool over = nh > kCap;
        for (int d = 14 + lane; d < 27 && !over; d += 32) {
            const int ox = d / 9 - 1, oy = (d / 3) % 3 - 1, oz = d % 3 - 1;
            const int c = cell_index(P, (li + ox + P.cdim[0]) % P.cdim[0], (lj + oy + P.cdim[1]) % P.cdim[1],
                                     (lk + oz + P.cdim[2]) % P.cdim[2]);
            if (a.start[c + 1] - a.start[c] > kCap) over = true;
        }
        if (__any_sync(0xffffffffu, over)) {
            if (lane == 0 && grp == 0) {
                const int k = atomicAdd(T.overflow_count, 1);
                T.overflow_list[k] = home;
            }
            continue;
        }
        stage<kDPD, kFlux, kSig>(a, S, D, 0, h0, nh, lane);
        __syncwarp();

        // 14 tasks: offsets 13 (self) and 14..26 (the lexicographically positive ones);
        // this work item runs tasks [13 + grp*per, 13 + (grp+1)*per)
        for (int d = 13 + grp * per; d < 13 + (grp + 1) * per; d++) {
            const int ox = d / 9 - 1, oy = (d / 3) % 3 - 1, oz = d % 3 - 1;
            const bool self = (d == 13);
            int g0 = h0, nn = nh, base = 0;
            float3 sh = make_float3(0.f, 0.f, 0.f);
            if (!self) {
                const int mi = (li + ox + P.cdim[0]) % P.cdim[0];
                const int mj = (lj + oy + P.cdim[1]) % P.cdim[1];
                const int mk = (lk + oz + P.cdim[2]) % P.cdim[2];
                const int c = cell_index(P, mi, mj, mk);
                g0 = a.start[c];
                nn = a.start[c + 1] - g0;
                if (nn == 0) continue;
                base = kCap;
                sh.x = cell_shift(P, 0, li, mi);
                sh.y = cell_shift(P, 1, lj, mj);
                sh.z = cell_shift(P, 2, lk, mk);
                stage<kDPD, kFlux, kSig>(a, S, D, kCap, g0, nn, lane);
                __syncwarp();
            } else if (nh < 2) {
                continue;
            }
            // candidates (i in home, j in partner); self: i < j
            const int total = nh * nn;
            const float inv_nn = 1.0f / (float)nn;
            int qhead = 0, qtail = 0;   // warp-uniform ring indices
            for (int p0 = 0; p0 < total; p0 += 32) {
                const int p = p0 + lane;
                bool hit = false;
                int i = 0, j = 0;
                if (p < total) {
                    i = (int)(((float)p + 0.5f) * inv_nn);
                    j = p - i * nn;
                    if (!self || i < j) {
                        float3 dx;
                        const float4 pi = S.pos[i], pj = S.pos[base + j];
                        const float r2 = pair_r2(make_float3(pi.x, pi.y, pi.z), sh, make_float3(pj.x, pj.y, pj.z), dx);
                        hit = r2 <= P.cutoff2;
                    }
                }
                const uint32_t m = __ballot_sync(0xffffffffu, hit);
                if (hit) S.q[(qtail + __popc(m & lanemask_lt())) & (kQ - 1)] = (uint32_t)i | ((uint32_t)(base + j) << 16);
                qtail += __popc(m);
                __syncwarp();
                if (qtail - qhead >= 32) {
                    const uint32_t e = S.q[(qhead + lane) & (kQ - 1)];
                    eval_batch<kDPD, kFlux, kDensity, kSig>(T, S, D, spots, blob, true, e, sh, lane, epot, vir);
                    qhead += 32;
                    __syncwarp();
                }
            }
            if (qtail > qhead) {
                const bool act = lane < qtail - qhead;
                const uint32_t e = act ? S.q[(qhead + lane) & (kQ - 1)] : 0u;
                eval_batch<kDPD, kFlux, kDensity, kSig>(T, S, D, spots, blob, act, e, sh, lane, epot, vir);
            }
            __syncwarp();
            if (!self) {
                flush<kFlux, kSig>(a, S, D, kCap, g0, nn, lane);
                __syncwarp();
            }
        }
        flush<kFlux, kSig>(a, S, D, 0, h0, nh, lane);
        __syncwarp();
    }
    if (kSig) return;
    double de = epot, dv = vir;
    for (int o = 16; o > 0; o >>= 1) {
        de += __shfl_down_sync(0xffffffffu, de, o);
        dv += __shfl_down_sync(0xffffffffu, dv, o);
    }
    if (lane == 0) {
        if (de != 0.0) atomicAdd(&a.red[RED_EPOT_NONBOND], de);
        if (dv != 0.0) atomicAdd(&a.red[RED_VIRIAL], dv);
    }
}

// Home cells whose own or neighbour population exceeds the staging capacity: one warp
// per listed home cell, candidates read from global memory, accumulation with global
// atomics.  Same orientation and arithmetic as the tiled kernel.
template <bool kDPD, bool kFlux, bool kDensity, bool kSig>
__global__ void __launch_bounds__(256) k_pair_overflow(TileArgs T) {
    const PairKernelArgs &a = T.a;
    const SimParams &P = a.P;
    const int lane = threadIdx.x & 31;
    const int nlist = *T.overflow_count;
    float epot = 0.f, vir = 0.f;
    for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nlist; w += (gridDim.x * blockDim.x) >> 5) {
        const int home = T.overflow_list[w];
        const int h0 = a.start[home], nh = a.start[home + 1] - h0;
        int li, lj, lk;
        cell_loc(P, home, li, lj, lk);
        for (int d = 13; d < 27; d++) {
            const int ox = d / 9 - 1, oy = (d / 3) % 3 - 1, oz = d % 3 - 1;
            const bool self = d == 13;
            const int mi = (li + ox + P.cdim[0]) % P.cdim[0];
            const int mj = (lj + oy + P.cdim[1]) % P.cdim[1];
            const int mk = (lk + oz + P.cdim[2]) % P.cdim[2];
            const int c = cell_index(P, mi, mj, mk);
            const int g0 = a.start[c], nn = a.start[c + 1] - g0;
            float3 sh = make_float3(0.f, 0.f, 0.f);
            if (!self) {
                sh.x = cell_shift(P, 0, li, mi);
                sh.y = cell_shift(P, 1, lj, mj);
                sh.z = cell_shift(P, 2, lk, mk);
            }
            const long long total = (long long)nh * nn;
            for (long long p = lane; p < total; p += 32) {
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
                    continue;
                }
                const float r = __fsqrt_rn(r2);
                float4 fi = make_float4(0.f, 0.f, 0.f, 0.f), fj = make_float4(0.f, 0.f, 0.f, 0.f);
                if (kDensity) {
                    const float wd = density_w(r, 1.0f / P.cutoff, P.self_density);
                    fi.w = wd;
                    fj.w = wd;
                }
                const int ti = __float_as_int(pi.w), tj = __float_as_int(pj.w);
                const int pidx = ti * P.max_type + tj;
                if (kFlux) {
                    const FluxSet &fs = a.fluxes[pidx];
                    for (int k = 0; k < fs.count; k++) {
                        const FluxDev &F = fs.f[k];
                        if (r > F.cutoff) continue;
                        float term = __fsub_rn(1.0f, __fdiv_rn(r, F.cutoff));
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
                        const float inv_ro = 1.0f / ro;
                        const float ex = dx.x * inv_ro, ey = dx.y * inv_ro, ez = dx.z * inv_ro;
                        const float omega_c = rr < 0.f ? 1.f : 1.f - rr / pot.b;
                        const float edv = ex * (vi.x - vj.x) + ey * (vi.y - vj.y) + ez * (vi.z - vj.z);
                        float xi_r = 1.0f;
                        if (!(P.flags & TFG_ENGINE_DPD_REFERENCE_RANDOM))
                            xi_r = gauss_pair(P.seed, P.time, __float_as_int(axi.w), __float_as_int(axj.w));
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
        }
    }
    if (kSig) return;
    double de = epot, dv = vir;
    for (int o = 16; o > 0; o >>= 1) {
        de += __shfl_down_sync(0xffffffffu, de, o);
        dv += __shfl_down_sync(0xffffffffu, dv, o);
    }
    if (lane == 0) {
        if (de != 0.0) atomicAdd(&a.red[RED_EPOT_NONBOND], de);
        if (dv != 0.0) atomicAdd(&a.red[RED_VIRIAL], dv);
    }
}

template <bool kDPD, bool kFlux, bool kDensity, bool kSig>
void launch_variant(const TileArgs &T, cudaStream_t s, int sms) {
    using Layout = SmemLayout<kDPD, kFlux>;
    const size_t smem_max = sizeof(Layout) + sizeof(float) * kMaxSmemTable + sizeof(PotDev) * kMaxTypes * kMaxTypes;
    const int nb = T.a.blob_floats <= kMaxSmemTable ? T.a.blob_floats : 0;
    const size_t smem = sizeof(Layout) + sizeof(float) * ((nb + 3) & ~3) +
                        sizeof(PotDev) * T.a.P.max_type * T.a.P.max_type;
    static bool configured = false;
    static size_t occ_smem = 0;
    static int per_sm = 1;
    if (!configured) {
        cudaFuncSetAttribute(k_pair_tile<kDPD, kFlux, kDensity, kSig>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem_max);
        configured = true;
    }
    if (occ_smem != smem) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pair_tile<kDPD, kFlux, kDensity, kSig>, kWarps * 32,
                                                      smem);
        if (per_sm < 1) per_sm = 1;
        occ_smem = smem;
    }
    const int want = (T.a.P.ncells * T.split + kWarps - 1) / kWarps;
    const int grid = std::max(1, std::min(want, sms * per_sm));
    k_pair_tile<kDPD, kFlux, kDensity, kSig><<<grid, kWarps * 32, smem, s>>>(T);
    k_pair_overflow<kDPD, kFlux, kDensity, kSig><<<sms, 256, 0, s>>>(T);
}

}  // namespace

int pair_tile_capacity() { return kCap; }

void launch_pair_tile(const PairKernelArgs &a, int *overflow_list, int *overflow_count, int sms, bool signature,
                      int split, cudaStream_t s) {
    TileArgs T;
    T.a = a;
    T.overflow_list = overflow_list;
    T.overflow_count = overflow_count;
    T.split = (split == 1 || split == 2 || split == 7 || split == 14) ? split : 1;
    cudaMemsetAsync(overflow_count, 0, sizeof(int), s);
    if (a.n <= 0) return;
    const bool dpd = a.has_dpd, flux = a.P.nspec > 0 && a.has_flux;
    const bool dens = !(a.P.flags & TFG_ENGINE_NO_DENSITY);
    if (signature) {
        launch_variant<false, false, false, true>(T, s, sms);
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
