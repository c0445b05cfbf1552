// Engine state, re-binning, bonded forces, forward-Euler advance, reductions and the
// C-ABI of libtfg.
//
// Per step (engine_step, tfEngine.cpp:1378-1429), all on the engine's stream:
//   bin      space_shuffle_local re-check + counting sort into cell order
//            (tfSpace.cpp:274-391; the reference keeps particles in per-cell arrays)
//   pair     fused nonbonded pass (tfg_pair.cu)
//   bonded   bond_eval / angle_eval (tfBond.cpp:97-345, tfAngle.cpp:90-382)
//   advance  cell_advance_forward_euler + Fluxes_integrate (tf_engine_advance.cpp:140-247,
//            tfFlux.cpp:175-202) with FP64 reductions
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "tfg_internal.h"

using namespace tfg;

struct tfg_engine {
    tfg_engine_desc desc{};
    SimParams P{};
    int n = 0, cap = 0;
    int nb = 0, na = 0, bcap = 0, acap = 0;
    int cur = 0;
    ParticleArrays A[2];
    float4 *force = nullptr;
    int32_t *count = nullptr, *start = nullptr, *lidx = nullptr, *tmp_id = nullptr, *tmp_src = nullptr,
            *dest = nullptr, *slot_of_id = nullptr, *scan_sums = nullptr;
    float *corig = nullptr;          // 3 axes, cdim[k] entries each
    PotDev *pots = nullptr;
    float *blob = nullptr;
    int blob_cap = 0, blob_floats = 0;
    FluxSet *fluxes = nullptr;
    float4 *rforce = nullptr;        // per type: mean, std, duration, enabled
    float *type_mass = nullptr;
    int32_t *type_dyn = nullptr;
    int2 *bonds = nullptr;
    int32_t *bond_slot = nullptr;
    int4 *angles = nullptr;          // i, j, k, slot
    PotDev *bpots = nullptr;
    float *bblob = nullptr;
    int bblob_cap = 0;
    double *red = nullptr;
    uint32_t *err = nullptr;
    int *overflow_list = nullptr, *overflow_count = nullptr;
    int sms = 1;
    int split = 0;          // warps per home cell of the tiled pair kernel (0 = not tuned yet)
    bool has_dpd = false, has_flux = false;
    uint32_t *species_flags = nullptr;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    cudaEvent_t ev[5] = {};
    float phase_ms[4] = {0, 0, 0, 0};
    std::string last_error;
    int64_t time = 0;
    // host mirrors
    std::vector<PotDev> h_pots;
    std::vector<std::vector<float>> h_tables;   // per type pair
    std::vector<FluxSet> h_fluxes;
    std::vector<float4> h_rforce;
    std::vector<float> h_mass;
    std::vector<int32_t> h_dyn;
    std::vector<PotDev> h_bpots;
    std::vector<std::vector<float>> h_btables;
    std::vector<uint32_t> h_species_flags;
    bool tables_dirty = true;
};

namespace {

constexpr int kThreads = 256;

inline float bits_to_float(int32_t v) {
    float f;
    std::memcpy(&f, &v, sizeof(f));
    return f;
}

inline int blocks_for(int n, int t = kThreads) { return (n + t - 1) / t; }

int fail(tfg_engine *e, int code, const std::string &msg) {
    if (e) e->last_error = msg;
    return code;
}

#define CK(call)                                                                              \
    do {                                                                                      \
        cudaError_t _e = (call);                                                              \
        if (_e != cudaSuccess)                                                                \
            return fail(eng, TFG_E_CUDA, std::string(#call ": ") + cudaGetErrorString(_e));   \
    } while (0)

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

// ------------------------------------------------------------------ kernels

// space_setpartp (tfSpace.cpp:432-475): clamp, bin, make cell-relative.
__global__ void k_setpartp(int n, const float *__restrict__ xg, SimParams P, float3 lo, float3 hi, float3 org,
                           float3 ih, int32_t *cell, float4 *pos, const int32_t *__restrict__ type,
                           uint32_t *err) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float x[3] = {xg[3 * i], xg[3 * i + 1], xg[3 * i + 2]};
    const float l3[3] = {lo.x, lo.y, lo.z}, h3[3] = {hi.x, hi.y, hi.z}, o3[3] = {org.x, org.y, org.z},
                i3[3] = {ih.x, ih.y, ih.z};
    int ind[3];
    for (int k = 0; k < 3; k++) {
        x[k] = fmaxf(l3[k], fminf(h3[k], x[k]));
        ind[k] = (int)__fmul_rn(__fsub_rn(x[k], o3[k]), i3[k]);
        if (ind[k] < 0 || ind[k] >= P.cdim[k]) {
            atomicOr(err, ERR_RANGE);
            ind[k] = ind[k] < 0 ? 0 : P.cdim[k] - 1;
        }
    }
    cell[i] = cell_index(P, ind[0], ind[1], ind[2]);
    pos[i] = make_float4(__fsub_rn(x[0], P.corig[0][ind[0]]), __fsub_rn(x[1], P.corig[1][ind[1]]),
                         __fsub_rn(x[2], P.corig[2][ind[2]]), __int_as_float(type ? type[i] : 0));
}

// Re-check of the cell-relative position (space_shuffle_local) and per-cell counting.
__global__ void k_bin_count(int n, SimParams P, float4 *pos, int32_t *cell, int32_t *count, int32_t *lidx,
                            int shuffle) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int c = cell[i];
    if (shuffle) {
        float4 p = pos[i];
        int d0 = (p.x >= P.h[0]) - (p.x < 0.f);
        int d1 = (p.y >= P.h[1]) - (p.y < 0.f);
        int d2 = (p.z >= P.h[2]) - (p.z < 0.f);
        if (d0 | d1 | d2) {
            p.x = __fsub_rn(p.x, __fmul_rn((float)d0, P.h[0]));
            p.y = __fsub_rn(p.y, __fmul_rn((float)d1, P.h[1]));
            p.z = __fsub_rn(p.z, __fmul_rn((float)d2, P.h[2]));
            pos[i] = p;
            int a, b, k;
            cell_loc(P, c, a, b, k);
            c = cell_index(P, (a + d0 + P.cdim[0]) % P.cdim[0], (b + d1 + P.cdim[1]) % P.cdim[1],
                           (k + d2 + P.cdim[2]) % P.cdim[2]);
            cell[i] = c;
        }
    }
    lidx[i] = atomicAdd(&count[c], 1);
}

// Exclusive scan of the cell counts: per-block scan, scan of block sums, add.
__device__ __forceinline__ int block_exclusive_scan(int v, int *tot) {
    __shared__ int ws[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[w] = x;
    __syncthreads();
    if (w == 0) {
        int s = lane < (int)(blockDim.x >> 5) ? ws[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        ws[lane] = s;
    }
    __syncthreads();
    int excl = x - v + (w > 0 ? ws[w - 1] : 0);
    if (tot) *tot = ws[(blockDim.x >> 5) - 1];
    __syncthreads();
    return excl;
}

__global__ void k_scan_local(const int32_t *count, int n, int32_t *start, int32_t *sums) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int v = i < n ? count[i] : 0;
    int tot;
    int ex = block_exclusive_scan(v, &tot);
    if (i < n) start[i] = ex;
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void k_scan_sums(int32_t *sums, int nb) {
    // one block of 1024 threads, each owning a contiguous run of block sums
    const int per = (nb + blockDim.x - 1) / blockDim.x;
    const int b0 = threadIdx.x * per;
    int local = 0;
    for (int k = 0; k < per; k++) if (b0 + k < nb) local += sums[b0 + k];
    int ex = block_exclusive_scan(local, nullptr);
    int run = ex;
    for (int k = 0; k < per; k++)
        if (b0 + k < nb) {
            int s = sums[b0 + k];
            sums[b0 + k] = run;
            run += s;
        }
}

__global__ void k_scan_add(int32_t *start, const int32_t *sums, const int32_t *count, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        int s = start[i] + sums[blockIdx.x];
        start[i] = s;
        if (i == n - 1) start[n] = s + count[i];
    }
}

__global__ void k_place(int n, const int32_t *cell, const int32_t *lidx, const int32_t *start, const float4 *aux,
                        int32_t *tmp_id, int32_t *tmp_src) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int p = start[cell[i]] + lidx[i];
    tmp_id[p] = __float_as_int(aux[i].w);
    tmp_src[p] = i;
}

// Deterministic order inside a cell: rank by particle id (one warp per cell).  Cells of
// up to 32 particles rank in registers (one id per lane, compared through shuffles);
// larger cells compare against global memory.
__global__ void k_rank(int ncells, const int32_t *start, const int32_t *tmp_id, const int32_t *tmp_src,
                       int32_t *dest) {
    int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (w >= ncells) return;
    int s0 = start[w], s1 = start[w + 1];
    const int n = s1 - s0;
    if (n == 0) return;
    if (n <= 32) {
        const int my = lane < n ? tmp_id[s0 + lane] : 0x7fffffff;
        int r = 0;
        for (int o = 0; o < n; o++) r += __shfl_sync(0xffffffffu, my, o) < my;
        if (lane < n) dest[tmp_src[s0 + lane]] = s0 + r;
        return;
    }
    for (int e = s0 + lane; e < s1; e += 32) {
        int my = tmp_id[e];
        int r = 0;
        for (int o = s0; o < s1; o++) r += tmp_id[o] < my;
        dest[tmp_src[e]] = s0 + r;
    }
}

// Scatter into cell order and initialise the force of the coming pair pass: f = force_i
// plus the Gaussian persistent force (gaussian_force, tfForce.cpp:211-223, redrawn when
// (time + id) % duration == 0 from a Philox stream) and f[3] = W(0) (space_prepare,
// tfSpace.cpp:182-201).
__global__ void k_scatter(int n, int cap, int nspec, const int32_t *dest, ParticleArrays src, ParticleArrays dst,
                          const int32_t *cell_src, int32_t *slot_of_id, SimParams P, const float4 *rforce,
                          float4 *force) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int d = dest[i];
    float4 ax = src.aux[i];
    const float4 p = src.pos[i];
    const float4 fe = src.fext[i];
    float4 pf = src.pforce[i];
    const int id = __float_as_int(ax.w);
    const float4 rf = rforce[__float_as_int(p.w)];
    if (rf.w != 0.f) {
        const int dur = (int)rf.z;
        if ((P.time + id) % dur == 0) {
            U4 r = philox({(uint32_t)P.time, (uint32_t)id, 0u, STREAM_FORCE}, (uint32_t)P.seed, (uint32_t)(P.seed >> 32));
            const float theta = 6.283185307179586f * u01(r.x);
            const float phi = acosf(1.f - 2.f * u01(r.y));
            const float g = sqrtf(-2.0f * logf(u01(r.z))) * cosf(6.283185307179586f * u01(r.w));
            const float rr = rf.x + rf.y * g;
            pf.x = rr * sinf(phi) * cosf(theta);
            pf.y = rr * sinf(phi) * sinf(theta);
            pf.z = rr * cosf(phi);
        }
        force[d] = make_float4(fe.x + pf.x, fe.y + pf.y, fe.z + pf.z, P.self_density);
    } else {
        force[d] = make_float4(fe.x, fe.y, fe.z, P.self_density);
    }
    dst.pos[d] = p;
    dst.vel[d] = src.vel[i];
    dst.aux[d] = ax;
    dst.fext[d] = fe;
    dst.pforce[d] = pf;
    dst.cell[d] = cell_src[i];
    for (int s = 0; s < nspec; s++) {
        dst.sval[s * cap + d] = src.sval[s * cap + i];
        dst.sq[s * cap + d] = src.sq[s * cap + i];
    }
    slot_of_id[__float_as_int(ax.w)] = d;
}

__device__ __forceinline__ int wrap_shift(int s) { return s > 1 ? -1 : (s < -1 ? 1 : s); }

// Block reduction of a per-thread FP32 partial into an FP64 global total: FP32 sums over
// each warp, FP64 across the warps of the block, one FP64 atomic per block.  Every
// thread of the block must call it (it synchronises the block).
__device__ __forceinline__ void block_add(double *dst, float v) {
    __shared__ double part[32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) part[w] = (double)v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < nw; k++) t += part[k];
        if (t != 0.0) atomicAdd(dst, t);
    }
}

// bond_eval (tfBond.cpp:97-345) for table potentials; one thread per bond.
__global__ void k_bonds(int nb, SimParams P, const int2 *bonds, const int32_t *bslot, const PotDev *bpots,
                        const float *bblob, const int32_t *slot_of_id, const float4 *pos, const float4 *aux,
                        const int32_t *cell, float4 *force, double *red) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    float epot = 0.f, vir = 0.f;
    if (b < nb) {
        int2 bd = bonds[b];
        const PotDev &pot = bpots[bslot[b]];
        int si = slot_of_id[bd.x], sj = slot_of_id[bd.y];
        if (pot.kind == POT_TABLE && si >= 0 && sj >= 0) {
            float4 pi = pos[si], pj = pos[sj];
            int ai, bi, ci, aj, bj, cj;
            cell_loc(P, cell[si], ai, bi, ci);
            cell_loc(P, cell[sj], aj, bj, cj);
            int s0 = wrap_shift(ai - aj), s1 = wrap_shift(bi - bj), s2 = wrap_shift(ci - cj);
            float pix = __fadd_rn(pi.x, __fmul_rn(P.h[0], (float)s0));
            float piy = __fadd_rn(pi.y, __fmul_rn(P.h[1], (float)s1));
            float piz = __fadd_rn(pi.z, __fmul_rn(P.h[2], (float)s2));
            float dx = __fsub_rn(pix, pj.x), dy = __fsub_rn(piy, pj.y), dz = __fsub_rn(piz, pj.z);
            float r2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
            // potential_eval_adjust_distance2
            float r = __fsqrt_rn(r2);
            if (pot.flags & TFG_POTENTIAL_SCALED) r = __fdiv_rn(r, __fadd_rn(aux[si].x, aux[sj].x));
            else if (pot.flags & TFG_POTENTIAL_SHIFTED)
                r = __fadd_rn(__fsub_rn(r, __fadd_rn(aux[si].x, aux[sj].x)), pot.r0_plusone);
            float rr2 = __fmul_rn(r, r);
            if (!(rr2 > __fmul_rn(pot.b, pot.b))) {
                rr2 = fmaxf(rr2, __fmul_rn(pot.a, pot.a));
                // potential_eval (tf_potential_eval.h:74-102)
                float rb = __fsqrt_rn(rr2);
                float t = __fadd_rn(pot.alpha0, __fmul_rn(rb, __fadd_rn(pot.alpha1, __fmul_rn(rb, pot.alpha2))));
                int ind = (int)fmaxf(0.0f, t);
                if (ind > pot.n) ind = pot.n;
                const float *c = bblob + pot.offset + ind * kChunk;
                float x = (rb - c[0]) * c[1];
                float ee = fmaf(c[2], x, c[3]), eff = c[2];
#pragma unroll
                for (int k = 4; k < kChunk; k++) {
                    eff = fmaf(eff, x, ee);
                    ee = fmaf(ee, x, c[k]);
                }
                float f = eff * c[1] / rb;
                atomicAdd(&force[si], make_float4(-f * dx, -f * dy, -f * dz, 0.f));
                atomicAdd(&force[sj], make_float4(f * dx, f * dy, f * dz, 0.f));
                epot = ee;
                vir = -f * r2;
            }
        }
    }
    block_add(&red[RED_EPOT_BOND], epot);
    block_add(&red[RED_VIRIAL], vir);
}

// angle_eval (tfAngle.cpp:90-382); one thread per angle, j is the vertex.
__global__ void k_angles(int na, SimParams P, const int4 *angles, const PotDev *bpots, const float *bblob,
                         const int32_t *slot_of_id, const float4 *pos, const int32_t *cell, float4 *force,
                         double *red) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    float epot = 0.f;
    if (q < na) {
        int4 A = angles[q];
        const PotDev &pot = bpots[A.w];
        int si = slot_of_id[A.x], sj = slot_of_id[A.y], sk = slot_of_id[A.z];
        if (pot.kind == POT_TABLE && si >= 0 && sj >= 0 && sk >= 0) {
            float4 pi = pos[si], pj = pos[sj], pk = pos[sk];
            int li[3], lj[3], lk[3];
            cell_loc(P, cell[si], li[0], li[1], li[2]);
            cell_loc(P, cell[sj], lj[0], lj[1], lj[2]);
            cell_loc(P, cell[sk], lk[0], lk[1], lk[2]);
            float xi[3] = {pi.x, pi.y, pi.z}, xj[3] = {pj.x, pj.y, pj.z}, xk[3] = {pk.x, pk.y, pk.z};
            float rji[3], rjk[3];
            for (int k = 0; k < 3; k++) {
                xi[k] = __fadd_rn(xi[k], __fmul_rn((float)wrap_shift(li[k] - lj[k]), P.h[k]));
                xk[k] = __fadd_rn(xk[k], __fmul_rn((float)wrap_shift(lk[k] - lj[k]), P.h[k]));
                rji[k] = __fsub_rn(xi[k], xj[k]);
                rjk[k] = __fsub_rn(xk[k], xj[k]);
            }
            float dprod = __fadd_rn(__fadd_rn(__fmul_rn(rji[0], rjk[0]), __fmul_rn(rji[1], rjk[1])),
                                    __fmul_rn(rji[2], rjk[2]));
            float nji = __fadd_rn(__fadd_rn(__fmul_rn(rji[0], rji[0]), __fmul_rn(rji[1], rji[1])),
                                  __fmul_rn(rji[2], rji[2]));
            float njk = __fadd_rn(__fadd_rn(__fmul_rn(rjk[0], rjk[0]), __fmul_rn(rjk[1], rjk[1])),
                                  __fmul_rn(rjk[2], rjk[2]));
            float inji = __fdiv_rn(1.0f, __fsqrt_rn(nji));
            float injk = __fdiv_rn(1.0f, __fsqrt_rn(njk));
            float ctheta = fmaxf(-1.0f, fminf(1.0f, __fmul_rn(__fmul_rn(dprod, inji), injk)));
            float dxi[3], dxk[3];
            if (ctheta == 0.f || ctheta == -1.f) {
                // Random derivative plane: the reference draws from the global mt19937
                // (tfAngle.cpp:210-223); here a Philox stream keyed on (step, angle).
                U4 r = philox({(uint32_t)P.time, (uint32_t)q, 0u, STREAM_ANGLE}, (uint32_t)P.seed,
                              (uint32_t)(P.seed >> 32));
                float x[3] = {2.f * u01(r.x) - 1.f, 2.f * u01(r.y) - 1.f, 2.f * u01(r.z) - 1.f};
                float vik[3] = {xi[0] - xk[0], xi[1] - xk[1], xi[2] - xk[2]};
                float dd = x[0] * vik[0] + x[1] * vik[1] + x[2] * vik[2];
                for (int k = 0; k < 3; k++) x[k] = x[k] - dd * vik[k];
                float len = sqrtf(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
                for (int k = 0; k < 3; k++) dxi[k] = dxk[k] = x[k] / len;
            } else {
                for (int k = 0; k < 3; k++) {
                    dxi[k] = (rjk[k] * injk - ctheta * rji[k] * inji) * inji;
                    dxk[k] = (rji[k] * inji - ctheta * rjk[k] * injk) * injk;
                }
            }
            if (!(ctheta > pot.b)) {
                float rr = fmaxf(ctheta, pot.a);
                float t = __fadd_rn(pot.alpha0, __fmul_rn(rr, __fadd_rn(pot.alpha1, __fmul_rn(rr, pot.alpha2))));
                int ind = (int)fmaxf(0.0f, t);
                if (ind <= pot.n) {
                    const float *c = bblob + pot.offset + ind * kChunk;
                    float x = (rr - c[0]) * c[1];
                    float ee = fmaf(c[2], x, c[3]), eff = c[2];
#pragma unroll
                    for (int k = 4; k < kChunk; k++) {
                        eff = fmaf(eff, x, ee);
                        ee = fmaf(ee, x, c[k]);
                    }
                    eff = eff * c[1];
                    float wi[3], wk[3];
                    for (int k = 0; k < 3; k++) { wi[k] = eff * dxi[k]; wk[k] = eff * dxk[k]; }
                    atomicAdd(&force[si], make_float4(-wi[0], -wi[1], -wi[2], 0.f));
                    atomicAdd(&force[sk], make_float4(-wk[0], -wk[1], -wk[2], 0.f));
                    atomicAdd(&force[sj], make_float4(wi[0] + wk[0], wi[1] + wk[1], wi[2] + wk[2], 0.f));
                    epot = ee;
                }
            }
        }
    }
    block_add(&red[RED_EPOT_ANGLE], epot);
}

// cell_advance_forward_euler + Fluxes_integrate; one thread per particle.
__global__ void k_advance(int n, int cap, SimParams P, float4 *pos, float4 *vel, const float4 *aux,
                          const float4 *force, int32_t *cell, float *sval, float *sq, const float *type_mass,
                          const int32_t *type_dyn, const uint32_t *species_flags, double *red, uint32_t *err) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    float ke = 0.f, vol = 0.f, mig = 0.f;
    float stot[kMaxSpecies];
#pragma unroll
    for (int s = 0; s < kMaxSpecies; s++) stot[s] = 0.f;
    if (i < n) {
        float4 p = pos[i], v = vel[i];
        const float4 ax = aux[i];
        const float4 f = force[i];
        const int type = __float_as_int(p.w);
        const uint32_t flags = (uint32_t)__float_as_int(ax.z);
        const float imass = ax.y;
        ke = 0.5f * type_mass[type] * (v.x * v.x + v.y * v.y + v.z * v.z);
        bool migrated = false;
        const bool frozen_all = (flags & TFG_PARTICLE_FROZEN_X) && (flags & TFG_PARTICLE_FROZEN_Y) &&
                                (flags & TFG_PARTICLE_FROZEN_Z);
        if (!frozen_all) {
            const float mask[3] = {(flags & TFG_PARTICLE_FROZEN_X) ? 0.0f : 1.0f,
                                   (flags & TFG_PARTICLE_FROZEN_Y) ? 0.0f : 1.0f,
                                   (flags & TFG_PARTICLE_FROZEN_Z) ? 0.0f : 1.0f};
            float x[3] = {p.x, p.y, p.z}, vv[3] = {v.x, v.y, v.z};
            const float fv[3] = {f.x, f.y, f.z};
            int delta[3];
            const float dt = P.dt;
            if (type_dyn[type] == TFG_NEWTONIAN) {
                for (int k = 0; k < 3; k++) {
                    float a = __fmul_rn(__fmul_rn(dt, fv[k]), imass);
                    float nv = __fmul_rn(mask[k], __fadd_rn(vv[k], a));
                    vv[k] = __fmul_rn(nv, nv) <= P.maxv2[k] ? nv : __fmul_rn(__fdiv_rn(nv, fabsf(nv)), P.maxv[k]);
                    x[k] = __fadd_rn(x[k], __fmul_rn(dt, vv[k]));
                    delta[k] = (x[k] >= P.h[k]) - (x[k] < 0.0f);
                }
            } else {
                for (int k = 0; k < 3; k++) {
                    float dx = __fmul_rn(mask[k], __fmul_rn(__fmul_rn(dt, fv[k]), imass));
                    dx = __fmul_rn(dx, dx) <= P.maxx2[k] ? dx : __fmul_rn(__fdiv_rn(dx, fabsf(dx)), P.maxx[k]);
                    vv[k] = __fdiv_rn(dx, dt);
                    x[k] = __fadd_rn(x[k], dx);
                    delta[k] = (x[k] >= P.h[k]) - (x[k] < 0.0f);
                }
            }
            const float nd = f.w;
            const float inv_nd = nd > 0.f ? __fdiv_rn(1.f, nd) : 0.f;
            vol = inv_nd;
            if (delta[0] | delta[1] | delta[2]) {
                for (int k = 0; k < 3; k++) {
                    if (x[k] >= P.h2[k] || x[k] <= -P.h[k]) { atomicOr(err, ERR_TOOFAST); break; }
                    x[k] = __fadd_rn(x[k], -__fmul_rn((float)delta[k], P.h[k]));
                }
                int a, b, c;
                cell_loc(P, cell[i], a, b, c);
                cell[i] = cell_index(P, (a + delta[0] + P.cdim[0]) % P.cdim[0], (b + delta[1] + P.cdim[1]) % P.cdim[1],
                                     (c + delta[2] + P.cdim[2]) % P.cdim[2]);
                migrated = true;
                mig = 1.f;
            }
            if (!(isfinite(x[0]) && isfinite(x[1]) && isfinite(x[2]))) atomicOr(err, ERR_NAN);
            pos[i] = make_float4(x[0], x[1], x[2], p.w);
            vel[i] = make_float4(vv[0], vv[1], vv[2], inv_nd);
        }
        // Fluxes_integrate runs over the particles still in their cell: migrants keep their
        // flux increment for the next step (they sit in the destination's incoming list).
        for (int s = 0; s < P.nspec; s++) {
            float sv = sval[s * cap + i];
            if (!migrated) {
                float konst = (species_flags[s] & 1u) ? 0.f : 1.f;
                float q = sq[s * cap + i];
                sv = fmaxf(0.0f, __fadd_rn(sv, __fmul_rn(__fmul_rn(P.dt_flux, q), konst)));
                sval[s * cap + i] = sv;
                sq[s * cap + i] = 0.f;
            }
            stot[s] = sv;
        }
    }
    block_add(&red[RED_KINETIC], ke);
    block_add(&red[RED_VOLUME], vol);
    block_add(&red[RED_MIGRATIONS], mig);
    for (int s = 0; s < P.nspec; s++) block_add(&red[RED_SPECIES0 + s], stot[s]);
}

__global__ void k_gather(int n, int cap, int nspec, SimParams P, ParticleArrays A, const float4 *force, float *x,
                         float *xrel, int32_t *cellout, float *v, float *f, float *dens, float *species, float *q) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = A.pos[i];
    const int id = __float_as_int(A.aux[i].w);
    const int c = A.cell[i];
    int l0, l1, l2;
    cell_loc(P, c, l0, l1, l2);
    if (x) {
        x[3 * id] = __fadd_rn(P.corig[0][l0], p.x);
        x[3 * id + 1] = __fadd_rn(P.corig[1][l1], p.y);
        x[3 * id + 2] = __fadd_rn(P.corig[2][l2], p.z);
    }
    if (xrel) { xrel[3 * id] = p.x; xrel[3 * id + 1] = p.y; xrel[3 * id + 2] = p.z; }
    if (cellout) cellout[id] = c;
    if (v) { float4 w = A.vel[i]; v[3 * id] = w.x; v[3 * id + 1] = w.y; v[3 * id + 2] = w.z; }
    if (f || dens) {
        float4 w = force[i];
        if (f) { f[3 * id] = w.x; f[3 * id + 1] = w.y; f[3 * id + 2] = w.z; }
        if (dens) dens[id] = w.w;
    }
    for (int s = 0; s < nspec; s++) {
        if (species) species[id * nspec + s] = A.sval[s * cap + i];
        if (q) q[id * nspec + s] = A.sq[s * cap + i];
    }
}

// ------------------------------------------------------------------ host helpers

int alloc_particles(tfg_engine *eng, int cap) {
    int rc;
    for (int b = 0; b < 2; b++) {
        ParticleArrays &A = eng->A[b];
        if ((rc = dalloc(eng, &A.pos, cap)) || (rc = dalloc(eng, &A.vel, cap)) || (rc = dalloc(eng, &A.aux, cap)) ||
            (rc = dalloc(eng, &A.fext, cap)) || (rc = dalloc(eng, &A.pforce, cap)) ||
            (rc = dalloc(eng, &A.cell, cap)) ||
            (rc = dalloc(eng, &A.sval, (size_t)cap * std::max(1, eng->P.nspec))) ||
            (rc = dalloc(eng, &A.sq, (size_t)cap * std::max(1, eng->P.nspec))))
            return rc;
    }
    if ((rc = dalloc(eng, &eng->force, cap)) || (rc = dalloc(eng, &eng->lidx, cap)) ||
        (rc = dalloc(eng, &eng->tmp_id, cap)) || (rc = dalloc(eng, &eng->tmp_src, cap)) ||
        (rc = dalloc(eng, &eng->dest, cap)) || (rc = dalloc(eng, &eng->slot_of_id, cap)))
        return rc;
    eng->cap = cap;
    return TFG_OK;
}

int upload_tables(tfg_engine *eng) {
    if (!eng->tables_dirty) return TFG_OK;
    const int T = eng->P.max_type;
    eng->has_dpd = false;
    eng->has_flux = false;
    for (int k = 0; k < T * T; k++) {
        if (eng->h_pots[k].kind == POT_DPD) eng->has_dpd = true;
        if (eng->h_fluxes[k].count > 0) eng->has_flux = true;
    }
    // nonbonded blob
    std::vector<float> blob;
    std::vector<PotDev> pots = eng->h_pots;
    for (int k = 0; k < T * T; k++) {
        if (pots[k].kind == POT_TABLE) {
            pots[k].offset = (int)blob.size();
            blob.insert(blob.end(), eng->h_tables[k].begin(), eng->h_tables[k].end());
        }
    }
    if (blob.empty()) blob.push_back(0.f);
    if ((int)blob.size() > eng->blob_cap) {
        int rc = dalloc(eng, &eng->blob, blob.size());
        if (rc) return rc;
        eng->blob_cap = (int)blob.size();
    }
    eng->blob_floats = (int)blob.size();
    cudaStream_t s = eng->stream;
    CK(cudaMemcpyAsync(eng->blob, blob.data(), sizeof(float) * blob.size(), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(eng->pots, pots.data(), sizeof(PotDev) * pots.size(), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(eng->fluxes, eng->h_fluxes.data(), sizeof(FluxSet) * eng->h_fluxes.size(),
                       cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(eng->rforce, eng->h_rforce.data(), sizeof(float4) * T, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(eng->type_mass, eng->h_mass.data(), sizeof(float) * T, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(eng->type_dyn, eng->h_dyn.data(), sizeof(int32_t) * T, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(eng->species_flags, eng->h_species_flags.data(), sizeof(uint32_t) * kMaxSpecies,
                       cudaMemcpyHostToDevice, s));
    // bonded blob
    std::vector<float> bblob;
    std::vector<PotDev> bp = eng->h_bpots;
    for (int k = 0; k < kMaxBondSlots; k++) {
        if (bp[k].kind == POT_TABLE) {
            bp[k].offset = (int)bblob.size();
            bblob.insert(bblob.end(), eng->h_btables[k].begin(), eng->h_btables[k].end());
        }
    }
    if (bblob.empty()) bblob.push_back(0.f);
    if ((int)bblob.size() > eng->bblob_cap) {
        int rc = dalloc(eng, &eng->bblob, bblob.size());
        if (rc) return rc;
        eng->bblob_cap = (int)bblob.size();
    }
    CK(cudaMemcpyAsync(eng->bblob, bblob.data(), sizeof(float) * bblob.size(), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(eng->bpots, bp.data(), sizeof(PotDev) * kMaxBondSlots, cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));
    eng->tables_dirty = false;
    return TFG_OK;
}

PotDev to_dev(const tfg_potential *p) {
    PotDev d;
    std::memset(&d, 0, sizeof(d));
    d.kind = p->kind == TFG_POTENTIAL_KIND_DPD ? POT_DPD : POT_TABLE;
    d.flags = p->flags;
    d.alpha0 = p->alpha[0];
    d.alpha1 = p->alpha[1];
    d.alpha2 = p->alpha[2];
    d.r0_plusone = p->r0_plusone;
    d.a = p->a;
    d.b = p->b;
    d.n = p->n;
    d.dpd_alpha = p->dpd_alpha;
    d.dpd_gamma = p->dpd_gamma;
    d.dpd_sigma = p->dpd_sigma;
    return d;
}

int bin(tfg_engine *eng, int shuffle) {
    const int n = eng->n;
    const int nc = eng->P.ncells;
    cudaStream_t s = eng->stream;
    ParticleArrays &S = eng->A[eng->cur], &D = eng->A[eng->cur ^ 1];
    CK(cudaMemsetAsync(eng->count, 0, sizeof(int32_t) * nc, s));
    if (n > 0) k_bin_count<<<blocks_for(n), kThreads, 0, s>>>(n, eng->P, S.pos, S.cell, eng->count, eng->lidx, shuffle);
    const int nbs = blocks_for(nc, 1024);
    k_scan_local<<<nbs, 1024, 0, s>>>(eng->count, nc, eng->start, eng->scan_sums);
    k_scan_sums<<<1, 1024, 0, s>>>(eng->scan_sums, nbs);
    k_scan_add<<<nbs, 1024, 0, s>>>(eng->start, eng->scan_sums, eng->count, nc);
    if (n > 0) {
        k_place<<<blocks_for(n), kThreads, 0, s>>>(n, S.cell, eng->lidx, eng->start, S.aux, eng->tmp_id, eng->tmp_src);
        k_rank<<<blocks_for(nc * 32), kThreads, 0, s>>>(nc, eng->start, eng->tmp_id, eng->tmp_src, eng->dest);
        k_scatter<<<blocks_for(n), kThreads, 0, s>>>(n, eng->cap, eng->P.nspec, eng->dest, S, D, S.cell,
                                                     eng->slot_of_id, eng->P, eng->rforce, eng->force);
    }
    eng->cur ^= 1;
    return TFG_OK;
}

int check_launch(tfg_engine *eng) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(eng, TFG_E_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    return TFG_OK;
}

PairKernelArgs pair_args(tfg_engine *eng) {
    ParticleArrays &A = eng->A[eng->cur];
    PairKernelArgs a;
    std::memset(&a, 0, sizeof(a));
    a.P = eng->P;
    a.n = eng->n;
    a.pos = A.pos;
    a.vel = A.vel;
    a.aux = A.aux;
    a.fext = A.fext;
    a.pforce = A.pforce;
    a.cell = A.cell;
    a.start = eng->start;
    a.sval = A.sval;
    a.sq = A.sq;
    a.cap = eng->cap;
    a.force = eng->force;
    a.pots = eng->pots;
    a.blob = eng->blob;
    a.blob_floats = eng->blob_floats;
    a.fluxes = eng->fluxes;
    a.rforce = eng->rforce;
    a.pforce_out = A.pforce;
    a.red = eng->red;
    a.err = eng->err;
    a.has_dpd = eng->has_dpd;
    a.has_flux = eng->has_flux;
    return a;
}

// The tiled half-shell kernel handles at most one species; more go to the stencil kernel.
bool use_tile(const tfg_engine *eng) { return !(eng->has_flux && eng->P.nspec > 1); }

int force_pass(tfg_engine *eng, bool bonded, bool timed) {
    cudaStream_t s = eng->stream;
    ParticleArrays &A = eng->A[eng->cur];
    PairKernelArgs a = pair_args(eng);
    if (use_tile(eng)) launch_pair_tile(a, eng->overflow_list, eng->overflow_count, eng->sms, false, eng->split, s);
    else launch_pair(a, s);
    if (timed) cudaEventRecord(eng->ev[2], s);
    if (bonded) {
        if (eng->nb > 0)
            k_bonds<<<blocks_for(eng->nb), kThreads, 0, s>>>(eng->nb, eng->P, eng->bonds, eng->bond_slot, eng->bpots,
                                                            eng->bblob, eng->slot_of_id, A.pos, A.aux, A.cell,
                                                            eng->force, eng->red);
        if (eng->na > 0)
            k_angles<<<blocks_for(eng->na), kThreads, 0, s>>>(eng->na, eng->P, eng->angles, eng->bpots, eng->bblob,
                                                             eng->slot_of_id, A.pos, A.cell, eng->force, eng->red);
    }
    if (timed) cudaEventRecord(eng->ev[3], s);
    return check_launch(eng);
}

// Pick the tiled pair kernel's work split (warps per home cell) by timing each choice on
// the current binned state.  Every trial re-initialises the forces with a non-shuffling
// re-bin (idempotent on sorted data); the flux increments the trials add are saved and
// restored, so the engine state is unchanged.
int autotune(tfg_engine *eng) {
    if (!use_tile(eng) || eng->n == 0) {
        eng->split = 1;
        return TFG_OK;
    }
    cudaStream_t s = eng->stream;
    const size_t nq = (size_t)eng->cap * std::max(1, eng->P.nspec);
    float *save = nullptr;
    int rc = dalloc(eng, &save, nq);
    if (rc) return rc;
    CK(cudaMemcpyAsync(save, eng->A[eng->cur].sq, sizeof(float) * nq, cudaMemcpyDeviceToDevice, s));
    const int cand[4] = {1, 2, 7, 14};
    float best = 1e30f;
    int best_split = 1;
    for (int c = 0; c < 4; c++) {
        float tmin = 1e30f;
        for (int rep = 0; rep < 3; rep++) {
            rc = bin(eng, 0);
            if (rc) { cudaFree(save); return rc; }
            PairKernelArgs a = pair_args(eng);
            cudaEventRecord(eng->ev[0], s);
            launch_pair_tile(a, eng->overflow_list, eng->overflow_count, eng->sms, false, cand[c], s);
            cudaEventRecord(eng->ev[1], s);
            CK(cudaEventSynchronize(eng->ev[1]));
            float ms = 0.f;
            cudaEventElapsedTime(&ms, eng->ev[0], eng->ev[1]);
            tmin = std::min(tmin, ms);
        }
        if (tmin < best) { best = tmin; best_split = cand[c]; }
    }
    CK(cudaMemcpyAsync(eng->A[eng->cur].sq, save, sizeof(float) * nq, cudaMemcpyDeviceToDevice, s));
    CK(cudaStreamSynchronize(s));
    cudaFree(save);
    rc = bin(eng, 0);
    if (rc) return rc;
    CK(cudaStreamSynchronize(s));
    eng->split = best_split;
    return check_launch(eng);
}

int one_step(tfg_engine *eng, bool advance, bool timed) {
    cudaStream_t s = eng->stream;
    eng->time += 1;
    eng->P.time = eng->time;
    CK(cudaMemsetAsync(eng->red, 0, sizeof(double) * RED_COUNT, s));
    if (timed) cudaEventRecord(eng->ev[0], s);
    int rc = bin(eng, 1);
    if (rc) return rc;
    if (timed) cudaEventRecord(eng->ev[1], s);
    rc = force_pass(eng, true, timed);
    if (rc) return rc;
    if (advance) {
        ParticleArrays &A = eng->A[eng->cur];
        if (eng->n > 0)
            k_advance<<<blocks_for(eng->n), kThreads, 0, s>>>(eng->n, eng->cap, eng->P, A.pos, A.vel, A.aux, eng->force,
                                                             A.cell, A.sval, A.sq, eng->type_mass, eng->type_dyn,
                                                             eng->species_flags, eng->red, eng->err);
    }
    if (timed) cudaEventRecord(eng->ev[4], s);
    return check_launch(eng);
}

int read_err(tfg_engine *eng) {
    uint32_t flags = 0;
    CK(cudaMemcpyAsync(&flags, eng->err, sizeof(uint32_t), cudaMemcpyDeviceToHost, eng->stream));
    CK(cudaStreamSynchronize(eng->stream));
    if (flags) {
        CK(cudaMemsetAsync(eng->err, 0, sizeof(uint32_t), eng->stream));
        CK(cudaStreamSynchronize(eng->stream));
        if (flags & ERR_NAN) return fail(eng, TFG_E_NAN, "non-finite particle position");
        if (flags & ERR_RANGE) return fail(eng, TFG_E_RANGE, "particle outside the space");
        if (flags & ERR_TOOFAST) return fail(eng, TFG_E_TOOFAST, "particle moved more than one cell in a step");
        if (flags & ERR_OVERFLOW) return fail(eng, TFG_E_OVERFLOW, "capacity exceeded");
    }
    return TFG_OK;
}

}  // namespace

// ------------------------------------------------------------------ C ABI

extern "C" {

TFG_API const char *tfg_build_info(void) {
    return "libtfg: GB300 (sm_103a) engine for Tissue Forge's per-step particle path";
}

TFG_API const char *tfg_last_error(const tfg_engine *eng) { return eng ? eng->last_error.c_str() : "null engine"; }

TFG_API int tfg_engine_create(const tfg_engine_desc *d, tfg_engine **out) {
    if (!d || !out) return TFG_E_INVAL;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return TFG_E_NODEVICE;
    if (d->device < 0 || d->device >= ndev) return TFG_E_INVAL;
    if (d->max_type < 1 || d->max_type > kMaxTypes || d->nr_species < 0 || d->nr_species > kMaxSpecies ||
        !(d->cutoff > 0) || !(d->dt > 0))
        return TFG_E_INVAL;
    for (int k = 0; k < 3; k++) {
        if (d->cells[k] < 3 || !(d->dim[k] > 0)) return TFG_E_INVAL;
        float h = d->dim[k] / d->cells[k];
        float ih = 1.0 / h;
        if ((int)std::ceil(d->cutoff * ih) != 1) return TFG_E_INVAL;   // span 1 stencil only
    }
    tfg_engine *eng = new (std::nothrow) tfg_engine();
    if (!eng) return TFG_E_OOM;
    eng->desc = *d;
    if (cudaSetDevice(d->device) != cudaSuccess) { delete eng; return TFG_E_CUDA; }
    cudaDeviceGetAttribute(&eng->sms, cudaDevAttrMultiProcessorCount, d->device);
    SimParams &P = eng->P;
    for (int k = 0; k < 3; k++) {
        P.dim[k] = d->dim[k];
        P.cdim[k] = d->cells[k];
        P.h[k] = P.dim[k] / P.cdim[k];
    }
    P.ncells = P.cdim[0] * P.cdim[1] * P.cdim[2];
    P.cutoff = d->cutoff;
    P.cutoff2 = d->cutoff * d->cutoff;
    P.dt = d->dt;
    P.dt_flux = d->dt;
    const float frac = d->particle_max_dist_fraction > 0 ? d->particle_max_dist_fraction : 0.05f;
    for (int k = 0; k < 3; k++) {
        P.h2[k] = 2. * P.h[k];
        P.maxx[k] = P.h[k] * frac;
        P.maxx2[k] = P.maxx[k] * P.maxx[k];
        P.maxv[k] = P.maxx[k] / P.dt;
        P.maxv2[k] = P.maxv[k] * P.maxv[k];
    }
    P.self_density = (float)(1.0 / (3.14159265358979323846 * (double)P.cutoff * P.cutoff * P.cutoff));
    P.dpd_delta = 1.f / std::sqrt(P.dt);
    P.max_type = d->max_type;
    P.nspec = d->nr_species;
    P.flags = d->flags;
    P.seed = d->seed;
    P.time = 0;

    int rc = TFG_OK;
    if (cudaStreamCreateWithFlags(&eng->stream, cudaStreamNonBlocking) != cudaSuccess) { delete eng; return TFG_E_CUDA; }
    eng->own_stream = true;
    for (int k = 0; k < 5; k++) cudaEventCreate(&eng->ev[k]);
    // cell origins: o = origin + l*h (space_init, tfSpace.cpp:772-777)
    int maxc = std::max(P.cdim[0], std::max(P.cdim[1], P.cdim[2]));
    std::vector<float> orig(3 * maxc, 0.f);
    for (int k = 0; k < 3; k++)
        for (int l = 0; l < P.cdim[k]; l++) orig[k * maxc + l] = d->origin[k] + l * P.h[k];
    const int T = d->max_type;
    if ((rc = dalloc(eng, &eng->corig, 3 * maxc)) || (rc = dalloc(eng, &eng->count, P.ncells)) ||
        (rc = dalloc(eng, &eng->start, P.ncells + 1)) || (rc = dalloc(eng, &eng->scan_sums, blocks_for(P.ncells, 1024))) ||
        (rc = dalloc(eng, &eng->pots, T * T)) || (rc = dalloc(eng, &eng->fluxes, T * T)) ||
        (rc = dalloc(eng, &eng->rforce, T)) || (rc = dalloc(eng, &eng->type_mass, T)) ||
        (rc = dalloc(eng, &eng->type_dyn, T)) || (rc = dalloc(eng, &eng->bpots, kMaxBondSlots)) ||
        (rc = dalloc(eng, &eng->red, RED_COUNT)) || (rc = dalloc(eng, &eng->err, 1)) ||
        (rc = dalloc(eng, &eng->species_flags, kMaxSpecies)) || (rc = dalloc(eng, &eng->overflow_list, P.ncells)) ||
        (rc = dalloc(eng, &eng->overflow_count, 1))) {
        tfg_engine_destroy(eng);
        return rc;
    }
    cudaMemcpy(eng->corig, orig.data(), sizeof(float) * orig.size(), cudaMemcpyHostToDevice);
    for (int k = 0; k < 3; k++) P.corig[k] = eng->corig + k * maxc;
    cudaMemset(eng->err, 0, sizeof(uint32_t));
    cudaMemset(eng->red, 0, sizeof(double) * RED_COUNT);
    eng->h_pots.assign(T * T, PotDev{});
    for (auto &p : eng->h_pots) std::memset(&p, 0, sizeof(p));
    eng->h_tables.assign(T * T, std::vector<float>());
    FluxSet empty;
    std::memset(&empty, 0, sizeof(empty));
    eng->h_fluxes.assign(T * T, empty);
    eng->h_rforce.assign(T, make_float4(0, 0, 1, 0));
    eng->h_mass.assign(T, 1.0f);
    eng->h_dyn.assign(T, TFG_NEWTONIAN);
    eng->h_bpots.assign(kMaxBondSlots, PotDev{});
    for (auto &p : eng->h_bpots) std::memset(&p, 0, sizeof(p));
    eng->h_btables.assign(kMaxBondSlots, std::vector<float>());
    eng->h_species_flags.assign(kMaxSpecies, 0u);
    if (d->capacity > 0) {
        if ((rc = alloc_particles(eng, d->capacity))) { tfg_engine_destroy(eng); return rc; }
    }
    if (cudaDeviceSynchronize() != cudaSuccess) { tfg_engine_destroy(eng); return TFG_E_CUDA; }
    *out = eng;
    return TFG_OK;
}

TFG_API int tfg_engine_destroy(tfg_engine *eng) {
    if (!eng) return TFG_E_INVAL;
    if (eng->stream) cudaStreamSynchronize(eng->stream);
    for (int b = 0; b < 2; b++) {
        ParticleArrays &A = eng->A[b];
        cudaFree(A.pos); cudaFree(A.vel); cudaFree(A.aux); cudaFree(A.fext); cudaFree(A.pforce);
        cudaFree(A.cell); cudaFree(A.sval); cudaFree(A.sq);
    }
    void *bufs[] = {eng->force, eng->count, eng->start, eng->lidx, eng->tmp_id, eng->tmp_src, eng->dest,
                    eng->slot_of_id, eng->scan_sums, eng->corig, eng->pots, eng->blob, eng->fluxes, eng->rforce,
                    eng->type_mass, eng->type_dyn, eng->bonds, eng->bond_slot, eng->angles, eng->bpots, eng->bblob,
                    eng->red, eng->err, eng->species_flags, eng->overflow_list, eng->overflow_count};
    for (void *p : bufs) cudaFree(p);
    for (int k = 0; k < 5; k++) if (eng->ev[k]) cudaEventDestroy(eng->ev[k]);
    if (eng->own_stream && eng->stream) cudaStreamDestroy(eng->stream);
    delete eng;
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
    return TFG_OK;
}

TFG_API int tfg_set_type(tfg_engine *eng, int type, int dynamics, float mass) {
    if (!eng || type < 0 || type >= eng->P.max_type) return TFG_E_INVAL;
    if (dynamics != TFG_NEWTONIAN && dynamics != TFG_OVERDAMPED) return fail(eng, TFG_E_INVAL, "bad dynamics");
    eng->h_dyn[type] = dynamics;
    eng->h_mass[type] = mass;
    eng->tables_dirty = true;
    return TFG_OK;
}

TFG_API int tfg_set_potential(tfg_engine *eng, int ti, int tj, const tfg_potential *p) {
    if (!eng) return TFG_E_INVAL;
    const int T = eng->P.max_type;
    if (ti < 0 || tj < 0 || ti >= T || tj >= T) return fail(eng, TFG_E_INVAL, "type out of range");
    for (int pass = 0; pass < 2; pass++) {
        int k = pass == 0 ? ti * T + tj : tj * T + ti;
        if (!p) {
            std::memset(&eng->h_pots[k], 0, sizeof(PotDev));
            eng->h_tables[k].clear();
            continue;
        }
        if (p->kind == TFG_POTENTIAL_KIND_POTENTIAL) {
            if (!p->c || p->n < 1 || p->n > TFG_POTENTIAL_IVALSMAX) return fail(eng, TFG_E_INVAL, "bad table");
            eng->h_tables[k].assign(p->c, p->c + (size_t)(p->n + 1) * kChunk);
        } else if (p->kind != TFG_POTENTIAL_KIND_DPD) {
            return fail(eng, TFG_E_INVAL, "unsupported potential kind");
        }
        eng->h_pots[k] = to_dev(p);
    }
    eng->tables_dirty = true;
    return TFG_OK;
}

TFG_API int tfg_add_flux(tfg_engine *eng, int ti, int tj, const tfg_flux *f) {
    if (!eng || !f) return TFG_E_INVAL;
    const int T = eng->P.max_type;
    if (ti < 0 || tj < 0 || ti >= T || tj >= T) return fail(eng, TFG_E_INVAL, "type out of range");
    if (f->index_a < 0 || f->index_a >= eng->P.nspec || f->index_b < 0 || f->index_b >= eng->P.nspec)
        return fail(eng, TFG_E_INVAL, "species index out of range");
    FluxSet &fs = eng->h_fluxes[ti * T + tj];
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
    F.cutoff = f->cutoff > 0 ? f->cutoff : eng->P.cutoff;
    if (ti != tj) eng->h_fluxes[tj * T + ti] = fs;
    eng->tables_dirty = true;
    return TFG_OK;
}

TFG_API int tfg_set_species_flags(tfg_engine *eng, int nr, const uint32_t *flags) {
    if (!eng || nr < 0 || nr > kMaxSpecies || (nr && !flags)) return TFG_E_INVAL;
    for (int s = 0; s < nr; s++) eng->h_species_flags[s] = flags[s];
    eng->tables_dirty = true;
    return TFG_OK;
}

TFG_API int tfg_set_random_force(tfg_engine *eng, int type, float mean, float std_, int duration_steps) {
    if (!eng || type < 0 || type >= eng->P.max_type || duration_steps < 1) return TFG_E_INVAL;
    eng->h_rforce[type] = make_float4(mean, std_, (float)duration_steps, std_ > 0.f ? 1.f : 0.f);
    eng->tables_dirty = true;
    return TFG_OK;
}

static int load_impl(tfg_engine *eng, int n, const float *xg, const int32_t *cellv, const float *xrel, const float *v,
                     const int32_t *type, const float *radius, const float *imass, const uint32_t *flags,
                     const float *species, const float *force_i) {
    if (!eng || n < 0 || (n > 0 && !xg && !(cellv && xrel))) return TFG_E_INVAL;
    const int T = eng->P.max_type;
    if (type)
        for (int i = 0; i < n; i++)
            if (type[i] < 0 || type[i] >= T) return fail(eng, TFG_E_INVAL, "particle type out of range");
    if (n > eng->cap) {
        int rc = alloc_particles(eng, std::max(n, eng->desc.capacity));
        if (rc) return rc;
    }
    eng->cur = 0;
    ParticleArrays &A = eng->A[0];
    const int ns = eng->P.nspec;
    cudaStream_t s = eng->stream;
    // host staging of the per-particle records
    std::vector<float4> vel(n), aux(n), fext(n), pf(n, make_float4(0, 0, 0, 0));
    for (int i = 0; i < n; i++) {
        vel[i] = make_float4(v ? v[3 * i] : 0.f, v ? v[3 * i + 1] : 0.f, v ? v[3 * i + 2] : 0.f, 0.f);
        aux[i] = make_float4(radius ? radius[i] : 1.0f, imass ? imass[i] : 1.0f,
                             bits_to_float((int32_t)(flags ? flags[i] : 0u)), bits_to_float(i));
        fext[i] = make_float4(force_i ? force_i[3 * i] : 0.f, force_i ? force_i[3 * i + 1] : 0.f,
                              force_i ? force_i[3 * i + 2] : 0.f, 0.f);
    }
    std::vector<float> sv((size_t)std::max(1, ns) * eng->cap, 0.f);
    if (species)
        for (int i = 0; i < n; i++)
            for (int k = 0; k < ns; k++) sv[(size_t)k * eng->cap + i] = species[(size_t)i * ns + k];
    CK(cudaMemcpyAsync(A.vel, vel.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(A.aux, aux.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(A.fext, fext.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(A.pforce, pf.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(A.sval, sv.data(), sizeof(float) * sv.size(), cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(A.sq, 0, sizeof(float) * sv.size(), s));
    int32_t *dtype = nullptr;
    int rc = dalloc(eng, &dtype, std::max(1, n));
    if (rc) return rc;
    std::vector<int32_t> tt(n, 0);
    if (type) std::memcpy(tt.data(), type, sizeof(int32_t) * n);
    CK(cudaMemcpyAsync(dtype, tt.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, s));
    if (xg) {
        float *dx = nullptr;
        rc = dalloc(eng, &dx, (size_t)3 * std::max(1, n));
        if (rc) { cudaFree(dtype); return rc; }
        CK(cudaMemcpyAsync(dx, xg, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, s));
        float3 lo, hi, org, ih;
        float *plo = &lo.x, *phi = &hi.x, *porg = &org.x, *pih = &ih.x;
        for (int k = 0; k < 3; k++) {
            const float o = eng->desc.origin[k], dm = eng->desc.dim[k];
            plo[k] = (float)(o * (1.0 + FLT_EPSILON));
            phi[k] = (float)((dm + o) * (1.0 - FLT_EPSILON));
            porg[k] = o;
            pih[k] = (float)(1.0 / eng->P.h[k]);
        }
        if (n > 0)
            k_setpartp<<<blocks_for(n), kThreads, 0, s>>>(n, dx, eng->P, lo, hi, org, ih, A.cell, A.pos, dtype, eng->err);
        CK(cudaStreamSynchronize(s));
        cudaFree(dx);
    } else {
        std::vector<float4> pos(n);
        for (int i = 0; i < n; i++) {
            if (cellv[i] < 0 || cellv[i] >= eng->P.ncells) { cudaFree(dtype); return fail(eng, TFG_E_RANGE, "cell out of range"); }
            pos[i] = make_float4(xrel[3 * i], xrel[3 * i + 1], xrel[3 * i + 2], bits_to_float(tt[i]));
        }
        CK(cudaMemcpyAsync(A.pos, pos.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(A.cell, cellv, sizeof(int32_t) * n, cudaMemcpyHostToDevice, s));
        CK(cudaStreamSynchronize(s));
    }
    cudaFree(dtype);
    eng->n = n;
    eng->time = 0;
    rc = read_err(eng);
    if (rc) return rc;
    // sort into cell order without the shuffle re-check
    rc = bin(eng, 0);
    if (rc) return rc;
    CK(cudaStreamSynchronize(s));
    return check_launch(eng);
}

TFG_API int tfg_load_particles(tfg_engine *eng, int n, const float *x, const float *v, const int32_t *type,
                               const float *radius, const float *imass, const uint32_t *flags, const float *species,
                               const float *force_i) {
    if (!x && n > 0) return TFG_E_INVAL;
    return load_impl(eng, n, x, nullptr, nullptr, v, type, radius, imass, flags, species, force_i);
}

TFG_API int tfg_load_particles_binned(tfg_engine *eng, int n, const int32_t *cell, const float *xrel, const float *v,
                                      const int32_t *type, const float *radius, const float *imass,
                                      const uint32_t *flags, const float *species, const float *force_i) {
    if ((!cell || !xrel) && n > 0) return TFG_E_INVAL;
    return load_impl(eng, n, nullptr, cell, xrel, v, type, radius, imass, flags, species, force_i);
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
    if (!eng || n < 0 || (n > 0 && (!i || !j))) return TFG_E_INVAL;
    std::vector<int2> b(n);
    std::vector<int32_t> sl(n, 0);
    for (int k = 0; k < n; k++) {
        if (i[k] < 0 || j[k] < 0 || i[k] >= eng->n || j[k] >= eng->n) return fail(eng, TFG_E_INVAL, "bond id out of range");
        b[k] = make_int2(i[k], j[k]);
        if (slot) {
            if (slot[k] < 0 || slot[k] >= kMaxBondSlots) return fail(eng, TFG_E_INVAL, "bond slot out of range");
            sl[k] = slot[k];
        }
    }
    if (n > eng->bcap) {
        int rc;
        if ((rc = dalloc(eng, &eng->bonds, n)) || (rc = dalloc(eng, &eng->bond_slot, n))) return rc;
        eng->bcap = n;
    }
    if (n) {
        CK(cudaMemcpyAsync(eng->bonds, b.data(), sizeof(int2) * n, cudaMemcpyHostToDevice, eng->stream));
        CK(cudaMemcpyAsync(eng->bond_slot, sl.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, eng->stream));
        CK(cudaStreamSynchronize(eng->stream));
    }
    eng->nb = n;
    return TFG_OK;
}

TFG_API int tfg_load_angles(tfg_engine *eng, int n, const int32_t *i, const int32_t *j, const int32_t *k,
                            const int32_t *slot) {
    if (!eng || n < 0 || (n > 0 && (!i || !j || !k))) return TFG_E_INVAL;
    std::vector<int4> a(n);
    for (int q = 0; q < n; q++) {
        if (i[q] < 0 || j[q] < 0 || k[q] < 0 || i[q] >= eng->n || j[q] >= eng->n || k[q] >= eng->n)
            return fail(eng, TFG_E_INVAL, "angle id out of range");
        int s = slot ? slot[q] : 0;
        if (s < 0 || s >= kMaxBondSlots) return fail(eng, TFG_E_INVAL, "angle slot out of range");
        a[q] = make_int4(i[q], j[q], k[q], s);
    }
    if (n > eng->acap) {
        int rc = dalloc(eng, &eng->angles, n);
        if (rc) return rc;
        eng->acap = n;
    }
    if (n) {
        CK(cudaMemcpyAsync(eng->angles, a.data(), sizeof(int4) * n, cudaMemcpyHostToDevice, eng->stream));
        CK(cudaStreamSynchronize(eng->stream));
    }
    eng->na = n;
    return TFG_OK;
}

TFG_API int tfg_autotune(tfg_engine *eng, int *split) {
    if (!eng) return TFG_E_INVAL;
    if (eng->cap == 0) return fail(eng, TFG_E_STATE, "no particles loaded");
    int rc = upload_tables(eng);
    if (rc) return rc;
    rc = autotune(eng);
    if (split) *split = eng->split;
    return rc;
}

TFG_API int tfg_set_split(tfg_engine *eng, int split) {
    if (!eng || !(split == 1 || split == 2 || split == 7 || split == 14)) return TFG_E_INVAL;
    eng->split = split;
    return TFG_OK;
}

TFG_API int tfg_step(tfg_engine *eng, int nsteps) {
    if (!eng || nsteps < 0) return TFG_E_INVAL;
    if (eng->cap == 0) return fail(eng, TFG_E_STATE, "no particles loaded");
    int rc = upload_tables(eng);
    if (rc) return rc;
    if (eng->split == 0 && (rc = autotune(eng))) return rc;
    for (int k = 0; k < nsteps; k++) {
        rc = one_step(eng, true, k == nsteps - 1);
        if (rc) return rc;
    }
    return TFG_OK;
}

TFG_API int tfg_force_only(tfg_engine *eng, int with_bonded) {
    if (!eng) return TFG_E_INVAL;
    if (eng->cap == 0) return fail(eng, TFG_E_STATE, "no particles loaded");
    int rc = upload_tables(eng);
    if (rc) return rc;
    if (eng->split == 0 && (rc = autotune(eng))) return rc;
    cudaStream_t s = eng->stream;
    eng->time += 1;
    eng->P.time = eng->time;
    CK(cudaMemsetAsync(eng->red, 0, sizeof(double) * RED_COUNT, s));
    rc = bin(eng, 1);
    if (rc) return rc;
    return force_pass(eng, with_bonded != 0, false);
}

TFG_API int tfg_pair_signature(tfg_engine *eng, int32_t *count, uint32_t *hash) {
    if (!eng || !count || !hash) return TFG_E_INVAL;
    const int n = eng->n;
    if (n == 0) return TFG_OK;
    int rc = upload_tables(eng);
    if (rc) return rc;
    if (eng->split == 0) eng->split = 1;
    int32_t *dbuf = nullptr;
    rc = dalloc(eng, &dbuf, (size_t)2 * n);
    if (rc) return rc;
    PairKernelArgs a = pair_args(eng);
    a.sig_count = dbuf;
    a.sig_hash = reinterpret_cast<uint32_t *>(dbuf + n);
    cudaMemsetAsync(dbuf, 0, sizeof(int32_t) * 2 * n, eng->stream);
    if (use_tile(eng))
        launch_pair_tile(a, eng->overflow_list, eng->overflow_count, eng->sms, true, eng->split, eng->stream);
    else launch_pair_signature(a, eng->stream);
    cudaMemcpyAsync(count, a.sig_count, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, eng->stream);
    cudaMemcpyAsync(hash, a.sig_hash, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, eng->stream);
    cudaError_t e = cudaStreamSynchronize(eng->stream);
    cudaFree(dbuf);
    if (e != cudaSuccess) return fail(eng, TFG_E_CUDA, cudaGetErrorString(e));
    return check_launch(eng);
}

TFG_API int tfg_sync(tfg_engine *eng) {
    if (!eng) return TFG_E_INVAL;
    CK(cudaStreamSynchronize(eng->stream));
    int rc = check_launch(eng);
    if (rc) return rc;
    return read_err(eng);
}

TFG_API int tfg_get_count(const tfg_engine *eng, int *n) {
    if (!eng || !n) return TFG_E_INVAL;
    *n = eng->n;
    return TFG_OK;
}

TFG_API int tfg_download(tfg_engine *eng, float *x, float *xrel, int32_t *cell, float *v, float *f, float *density,
                         float *species, float *q) {
    if (!eng) return TFG_E_INVAL;
    const int n = eng->n, ns = eng->P.nspec;
    if (n == 0) return TFG_OK;
    cudaStream_t s = eng->stream;
    // one staging buffer on the device, gathered by id
    const size_t nf = (size_t)n * (3 + 3 + 3 + 3 + 1 + 2 * ns) + n;
    float *stage = nullptr;
    int rc = dalloc(eng, &stage, nf);
    if (rc) return rc;
    float *dx = stage, *dxr = dx + 3 * n, *dv = dxr + 3 * n, *df = dv + 3 * n, *dd = df + 3 * n;
    float *dsp = dd + n, *dq = dsp + (size_t)n * ns;
    int32_t *dc = reinterpret_cast<int32_t *>(dq + (size_t)n * ns);
    k_gather<<<blocks_for(n), kThreads, 0, s>>>(n, eng->cap, ns, eng->P, eng->A[eng->cur], eng->force, dx, dxr, dc, dv,
                                                df, dd, ns ? dsp : nullptr, ns ? dq : nullptr);
    auto cp = [&](void *dst, const void *src, size_t bytes) {
        if (dst) cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s);
    };
    cp(x, dx, sizeof(float) * 3 * n);
    cp(xrel, dxr, sizeof(float) * 3 * n);
    cp(v, dv, sizeof(float) * 3 * n);
    cp(f, df, sizeof(float) * 3 * n);
    cp(density, dd, sizeof(float) * n);
    if (ns) {
        cp(species, dsp, sizeof(float) * n * ns);
        cp(q, dq, sizeof(float) * n * ns);
    }
    cp(cell, dc, sizeof(int32_t) * n);
    cudaError_t e = cudaStreamSynchronize(s);
    cudaFree(stage);
    if (e != cudaSuccess) return fail(eng, TFG_E_CUDA, cudaGetErrorString(e));
    return read_err(eng);
}

TFG_API int tfg_get_reductions(tfg_engine *eng, tfg_reductions *out) {
    if (!eng || !out) return TFG_E_INVAL;
    double r[RED_COUNT];
    CK(cudaMemcpyAsync(r, eng->red, sizeof(r), cudaMemcpyDeviceToHost, eng->stream));
    CK(cudaStreamSynchronize(eng->stream));
    std::memset(out, 0, sizeof(*out));
    out->epot_nonbond = r[RED_EPOT_NONBOND];
    out->epot_bond = r[RED_EPOT_BOND];
    out->epot_angle = r[RED_EPOT_ANGLE];
    out->epot = out->epot_nonbond + out->epot_bond + out->epot_angle;
    out->kinetic = r[RED_KINETIC];
    out->virial = r[RED_VIRIAL];
    out->computed_volume = r[RED_VOLUME];
    for (int s = 0; s < kMaxSpecies; s++) out->species_total[s] = r[RED_SPECIES0 + s];
    out->steps = eng->time;
    out->migrations = (int64_t)r[RED_MIGRATIONS];
    return read_err(eng);
}

TFG_API int tfg_get_phase_ms(tfg_engine *eng, float ms[4]) {
    if (!eng || !ms) return TFG_E_INVAL;
    CK(cudaStreamSynchronize(eng->stream));
    for (int k = 0; k < 4; k++) {
        float t = 0.f;
        if (cudaEventElapsedTime(&t, eng->ev[k], eng->ev[k + 1]) != cudaSuccess) t = -1.f;
        ms[k] = t;
    }
    cudaGetLastError();
    return TFG_OK;
}

}  // extern "C"
