// Nonbonded pair pass for tabulated potentials, home-particle-outer form.
//
// Reference path replaced: runner_dopair / runner_doself (tf_runner_dopair.cpp:72-758)
// with potential_eval_super_ex (tf_potential_eval.h:207-272) and the number density W
// (tf_smoothing_kernel.h:49-67), for simulations without DPD potentials or fluxes.
//
// Work unit: one warp owns a home cell and runs the reference's 14 tasks of that cell (the
// self task and the 13 pair tasks whose cell_i it is: a neighbour at offset d is the
// partner with the home as cell_i exactly when d is lexicographically positive,
// space_getsid / space_init, tfSpace.cpp:79-114, 893-1019), so every interacting pair is
// evaluated once, in the reference's orientation (Newton's third law).
//
// The home cell and its 13 forward neighbours are staged into the warp's shared memory
// (up to kHCap particles; larger neighbourhoods are staged in chunks).  Every lane keeps
// one target of each block of 32 staged particles in registers, as x + shift.  The home
// particles are then taken one at a time: all lanes test the home particle against their
// targets with a cheap FMA distance (squared cutoff plus 1e-5 relative, far above its few
// ulps of difference to the reference's unfused (x_i - shift) - x_k), and the hits of that
// one home particle are compacted into a queue and evaluated 32 at a time.  Because one
// batch holds a single home particle and distinct targets:
//   - the target side is added to the target's shared-memory accumulator with plain
//     read-modify-writes (no two lanes share a target),
//   - the home side accumulates in registers and is reduced once per home particle.
// The evaluation applies the reference's exact pair test ((x_i - shift) - x_k, unfused),
// so the pair set is bit-identical to the reference's.  Each staged particle is flushed
// once to global memory with a vector atomic add.  Home cells whose neighbourhood does
// not fit are handled by the overflow kernel of the tiled pass.
#include <algorithm>

#include "tfg_internal.h"

namespace tfg {

namespace {

constexpr int kHW = 8;                 // warps per CTA
constexpr int kHCap = 320;             // staged particles per warp (home cell first)
constexpr int kHBlk = kHCap / 32;      // target blocks held in registers

struct HStage {
    float4 pos[kHCap];      // cell-relative position; w = type bits
    float4 acc[kHCap];      // fx, fy, fz, number density (signature: count, hash bits)
    int32_t gslot[kHCap];   // global slot
    float rad[kHCap];       // radius
    uint16_t q[kHCap];      // targets hit by the current home particle
    uint8_t seg[kHCap];     // task (13..26) of the staged particle's cell
    float sh[27][3];        // shift of each task's cell as seen from the home cell
};

struct HomeArgs {
    PairKernelArgs a;
    int *overflow_list;     // home cells handed to the overflow kernel
    int *overflow_count;    // [0] overflow cells, [1] work counter
};

__device__ __forceinline__ uint32_t lanemask_lt_h() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__device__ __forceinline__ void flush_red_h(double *red, int rb, float &epot, float &vir, int lane) {
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

template <bool kSig>
__device__ __noinline__ void stage_h(const PairKernelArgs &a, HStage &S, int base, int g0, int n, int task, int lane) {
#pragma unroll 1
    for (int k = lane; k < n; k += 32) {
        const int g = g0 + k;
        S.pos[base + k] = a.pos[g];
        S.acc[base + k] = make_float4(0.f, 0.f, 0.f, 0.f);
        S.gslot[base + k] = g;
        S.rad[base + k] = a.aux[g].x;
        S.seg[base + k] = (uint8_t)task;
    }
}

template <bool kSig>
__device__ __noinline__ void flush_h(const PairKernelArgs &a, HStage &S, int b0, int b1, int lane) {
#pragma unroll 1
    for (int k = b0 + lane; k < b1; k += 32) {
        const float4 v = S.acc[k];
        const int g = S.gslot[k];
        if (kSig) {
            const int c = __float_as_int(v.x);
            if (c) {
                const int id = __float_as_int(a.aux[g].w);
                atomicAdd(&a.sig_count[id], c);
                atomicAdd(&a.sig_hash[id], (uint32_t)__float_as_int(v.y));
            }
            continue;
        }
        if (v.x != 0.f || v.y != 0.f || v.z != 0.f || v.w != 0.f) atomicAdd(&a.force[g], v);
    }
}

template <bool kDensity, bool kSig>
__global__ void __launch_bounds__(kHW * 32, 2) k_pair_home(HomeArgs T) {
    extern __shared__ __align__(16) unsigned char smem_h[];
    HStage *Lw = reinterpret_cast<HStage *>(smem_h);
    const PairKernelArgs &a = T.a;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    HStage &S = Lw[wid];
    const uint32_t lt = lanemask_lt_h();
    const float *blob = a.blob;
    const PotDev *pots = a.pots;
    float epot = 0.f, vir = 0.f;
    int cur_rb = -1;

    for (;;) {
        // warps take home cells from a shared counter, one at a time
        int home = 0;
        if (lane == 0) home = atomicAdd(T.overflow_count + 1, 1);
        home = __shfl_sync(0xffffffffu, home, 0);
        if (home >= a.ncells) break;
        const int h0 = a.start[home], nh = a.start[home + 1] - h0;
        if (nh == 0) continue;
        const SimParams &P = a.sims[a.cell_sim[home]];
        if (!kSig && P.stopped) continue;
        if (!kSig && P.red_base != cur_rb) {
            flush_red_h(a.red, cur_rb, epot, vir, lane);
            cur_rb = P.red_base;
        }
        int li, lj, lk;
        cell_loc(P, home, li, lj, lk);
        // lane L (< 13) describes forward task 14+L: partner cell start, count and shift
        int my_g0 = 0, my_n = 0;
        if (lane < 13) {
            const int d = 14 + lane;
            const int ox = d / 9 - 1, oy = (d / 3) % 3 - 1, oz = d % 3 - 1;
            const int mi = (li + ox + P.cdim[0]) % P.cdim[0];
            const int mj = (lj + oy + P.cdim[1]) % P.cdim[1];
            const int mk = (lk + oz + P.cdim[2]) % P.cdim[2];
            const int c = cell_index(P, mi, mj, mk);
            my_g0 = a.start[c];
            my_n = a.start[c + 1] - my_g0;
            // no cell pair across the edge of a non-periodic axis
            if (!(nb_exists(P, 0, li, ox) && nb_exists(P, 1, lj, oy) && nb_exists(P, 2, lk, oz))) my_n = 0;
            S.sh[d][0] = cell_shift(P, 0, li, mi);
            S.sh[d][1] = cell_shift(P, 1, lj, mj);
            S.sh[d][2] = cell_shift(P, 2, lk, mk);
        }
        if (lane == 13) {
            S.sh[13][0] = 0.f;
            S.sh[13][1] = 0.f;
            S.sh[13][2] = 0.f;
        }
        __syncwarp();
        // every neighbour segment must fit beside the home cell
        const bool over = nh >= kHCap || (lane < 13 && nh + my_n > kHCap);
        if (__any_sync(0xffffffffu, over)) {
            if (lane == 0) {
                const int k = atomicAdd(T.overflow_count, 1);
                T.overflow_list[k] = home;
            }
            continue;
        }
        stage_h<kSig>(a, S, 0, h0, nh, 13, lane);
        __syncwarp();
        // wall potentials of the home particles (runner_doself's boundary_eval,
        // tf_runner_dopair.cpp:594-596)
        if (!kSig && a.has_wall_pots && P.walls_active) {
#pragma unroll 1
            for (int k = lane; k < nh; k += 32) {
                const float4 p4 = S.pos[k];
                const int g = S.gslot[k];
                float3 fw = make_float3(0.f, 0.f, 0.f);
                float ew = 0.f;
                wall_eval(P, a.wpots, blob, __float_as_int(p4.w), make_float3(p4.x, p4.y, p4.z), S.rad[k], a.vel[g],
                          __float_as_int(a.aux[g].w) - P.id_off, li, lj, lk, fw, ew);
                S.acc[k].x += fw.x;
                S.acc[k].y += fw.y;
                S.acc[k].z += fw.z;
                epot += ew;
            }
            __syncwarp();
        }
        const float cutoff2 = P.cutoff2;
        const float cutf = cutoff2 * 1.00001f;
        int t = 14;          // next neighbour task to stage
        bool first = true;   // the first chunk also holds the self task
        while (first || t < 27) {
            int end = nh;
            while (t < 27) {
                const int g0 = __shfl_sync(0xffffffffu, my_g0, t - 14);
                const int nn = __shfl_sync(0xffffffffu, my_n, t - 14);
                if (end + nn > kHCap) break;
                if (nn > 0) stage_h<kSig>(a, S, end, g0, nn, t, lane);
                end += nn;
                t++;
            }
            __syncwarp();
            const int tbeg = first ? 0 : nh;
            first = false;
            const int nb = (end - tbeg + 31) >> 5;
            // targets of this chunk in registers, one per lane and block, as x + shift.  A
            // target pairs with home particle i when its staged index exceeds i: the self
            // task's pairs (k > i) and every neighbour (k >= nh > i).
            float tx[kHBlk], ty[kHBlk], tz[kHBlk];
#pragma unroll
            for (int b = 0; b < kHBlk; b++) {
                const int k = tbeg + 32 * b + lane;
                tx[b] = 3.0e18f;
                ty[b] = 0.f;
                tz[b] = 0.f;
                if (b < nb && k < end) {
                    const float4 p = S.pos[k];
                    const float *s = S.sh[S.seg[k]];
                    tx[b] = p.x + s[0];
                    ty[b] = p.y + s[1];
                    tz[b] = p.z + s[2];
                }
            }
            const int kl = tbeg + lane;
#pragma unroll 1
            for (int i = 0; i < nh; i++) {
                const float4 xi = S.pos[i];
                int qn = 0;
#pragma unroll
                for (int b = 0; b < kHBlk; b++) {
                    if (b < nb) {
                        const float dx = xi.x - tx[b], dy = xi.y - ty[b], dz = xi.z - tz[b];
                        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                        const bool hit = r2 <= cutf && kl + 32 * b > i;
                        const uint32_t m = __ballot_sync(0xffffffffu, hit);
                        if (hit) S.q[qn + __popc(m & lt)] = (uint16_t)(tbeg + 32 * b + lane);
                        qn += __popc(m);
                    }
                }
                if (qn == 0) continue;
                __syncwarp();
                const float ri = S.rad[i];
                const int pbase = P.pot_base + __float_as_int(xi.w) * a.max_type;
                uint32_t idi = 0;
                if (kSig) idi = (uint32_t)__float_as_int(a.aux[S.gslot[i]].w);
                float4 fI = make_float4(0.f, 0.f, 0.f, 0.f);
                int cI = 0;
                uint32_t hI = 0;
#pragma unroll 1
                for (int base = 0; base < qn; base += 32) {
                    if (base + lane < qn) {
                        const int k = S.q[base + lane];
                        const float4 pk = S.pos[k];
                        const float *s = S.sh[S.seg[k]];
                        float3 dx;
                        // the reference's pair decision: (x_i - shift) - x_k, unfused
                        const float r2 = pair_r2(make_float3(xi.x, xi.y, xi.z), make_float3(s[0], s[1], s[2]),
                                                 make_float3(pk.x, pk.y, pk.z), dx);
                        if (r2 <= cutoff2) {
                            if (kSig) {
                                const uint32_t idk = (uint32_t)__float_as_int(a.aux[S.gslot[k]].w);
                                cI += 1;
                                hI += sig_mix(idk);
                                int *ck = reinterpret_cast<int *>(&S.acc[k].x);
                                uint32_t *hk2 = reinterpret_cast<uint32_t *>(&S.acc[k].y);
                                *ck += 1;
                                *hk2 += sig_mix(idi);
                                record_pair(a, (int)idi, (int)idk);
                            } else {
                                float4 fK = make_float4(0.f, 0.f, 0.f, 0.f);
                                if (kDensity) {
                                    const float w = density_w(__fsqrt_rn(r2), P.inv_cutoff, P.self_density);
                                    fI.w += w;
                                    fK.w = w;
                                }
                                const PotDev pot = pots[pbase + __float_as_int(pk.w)];
                                if (pot.kind == POT_TABLE) {
                                    float e, f;
                                    if (table_eval(pot, blob, ri, S.rad[k], r2, e, f)) {
                                        // part_i.f -= f dx ; part_k.f += f dx
                                        const float wx = f * dx.x, wy = f * dx.y, wz = f * dx.z;
                                        fI.x -= wx;
                                        fI.y -= wy;
                                        fI.z -= wz;
                                        fK.x = wx;
                                        fK.y = wy;
                                        fK.z = wz;
                                        epot += e;
                                        vir -= f * r2;
                                    }
                                }
                                float4 v = S.acc[k];
                                v.x += fK.x;
                                v.y += fK.y;
                                v.z += fK.z;
                                v.w += fK.w;
                                S.acc[k] = v;
                            }
                        }
                    }
                }
                // the home particle's side, reduced over the warp once
                if (kSig) {
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) {
                        cI += __shfl_xor_sync(0xffffffffu, cI, o);
                        hI += __shfl_xor_sync(0xffffffffu, hI, o);
                    }
                    if (lane == 0) {
                        *reinterpret_cast<int *>(&S.acc[i].x) += cI;
                        *reinterpret_cast<uint32_t *>(&S.acc[i].y) += hI;
                    }
                } else {
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) {
                        fI.x += __shfl_xor_sync(0xffffffffu, fI.x, o);
                        fI.y += __shfl_xor_sync(0xffffffffu, fI.y, o);
                        fI.z += __shfl_xor_sync(0xffffffffu, fI.z, o);
                        if (kDensity) fI.w += __shfl_xor_sync(0xffffffffu, fI.w, o);
                    }
                    if (lane == 0) {
                        float4 v = S.acc[i];
                        v.x += fI.x;
                        v.y += fI.y;
                        v.z += fI.z;
                        v.w += fI.w;
                        S.acc[i] = v;
                    }
                }
                __syncwarp();
            }
            __syncwarp();
            flush_h<kSig>(a, S, nh, end, lane);
            __syncwarp();
        }
        flush_h<kSig>(a, S, 0, nh, lane);
        __syncwarp();
    }
    if (!kSig) flush_red_h(a.red, cur_rb, epot, vir, lane);
}

template <bool kDensity, bool kSig>
void launch_home_variant(const HomeArgs &T, int sms, cudaStream_t s) {
    const size_t smem = sizeof(HStage) * kHW;
    static bool configured = false;
    static int per_sm = 1;
    if (!configured) {
        cudaFuncSetAttribute(k_pair_home<kDensity, kSig>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pair_home<kDensity, kSig>, kHW * 32, smem);
        if (per_sm < 1) per_sm = 1;
        configured = true;
    }
    const int want = (T.a.ncells + kHW - 1) / kHW;
    const int grid = std::max(1, std::min(want, sms * per_sm));
    k_pair_home<kDensity, kSig><<<grid, kHW * 32, smem, s>>>(T);
}

}  // namespace

void launch_pair_home(const PairKernelArgs &a, int *overflow_list, int *overflow_count, int sms, bool signature,
                      cudaStream_t s) {
    HomeArgs T;
    T.a = a;
    T.overflow_list = overflow_list;
    T.overflow_count = overflow_count;
    const bool dens = !(a.flags & TFG_ENGINE_NO_DENSITY);
    if (signature) launch_home_variant<false, true>(T, sms, s);
    else if (dens) launch_home_variant<true, false>(T, sms, s);
    else launch_home_variant<false, false>(T, sms, s);
    launch_pair_overflow(a, overflow_list, overflow_count, signature, sms, s);
}

}  // namespace tfg
