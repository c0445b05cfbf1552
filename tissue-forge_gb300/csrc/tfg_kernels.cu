// Per-particle, per-cell, per-bond and per-angle kernels of the engine (everything but
// the pair pass).  Every kernel serves an arena of one or more simulations: a particle's
// simulation is cell_sim[cell], and its parameters are sims[that index].
//
//   bin      space_shuffle_local re-check (tfSpace.cpp:274-391) + counting sort into
//            cell order (count, scan, place, rank by id, scatter)
//   scatter  also initialises the pair pass's force: force_i + Gaussian persistent force
//            (gaussian_force, tfForce.cpp:211-223) and W(0) (space_prepare, tfSpace.cpp:182-201)
//   bonded   bond_eval / angle_eval (tfBond.cpp:97-345, tfAngle.cpp:90-382)
//   advance  cell_advance_forward_euler + Fluxes_integrate (tf_engine_advance.cpp:140-247,
//            tfFlux.cpp:175-202) with FP64 per-simulation totals
#include "tfg_kernels.h"

namespace tfg {

namespace {

__device__ __forceinline__ int wrap_shift(int s) { return s > 1 ? -1 : (s < -1 ? 1 : s); }

// Add per-thread FP32 partials into per-simulation FP64 totals.  When the whole block
// belongs to one simulation: FP32 over each warp, FP64 across warps, one atomic per
// block.  Otherwise each warp whose lanes share a simulation adds once, and mixed warps
// add lane by lane.  Every thread of the block must call it.
__device__ __forceinline__ void keyed_add(double *red, int rb, int slot, float v) {
    __shared__ double part[32];
    const int rb0 = __shfl_sync(0xffffffffu, rb, 0);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    __shared__ int block_rb;
    if (threadIdx.x == 0) block_rb = rb;
    __syncthreads();
    const bool uniform = __syncthreads_and(rb == block_rb || rb < 0);
    if (uniform) {
        float s = v;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) part[w] = (double)s;
        __syncthreads();
        if (threadIdx.x == 0 && block_rb >= 0) {
            double t = 0.0;
            for (int k = 0; k < nw; k++) t += part[k];
            if (t != 0.0) atomicAdd(&red[block_rb + slot], t);
        }
        __syncthreads();
        return;
    }
    if (__all_sync(0xffffffffu, rb == rb0 || rb < 0)) {
        float s = v;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0 && rb0 >= 0 && s != 0.f) atomicAdd(&red[rb0 + slot], (double)s);
    } else if (rb >= 0 && v != 0.f) {
        atomicAdd(&red[rb + slot], (double)v);
    }
}

// keyed_add of three values to three slots of the same simulation, under one set of block
// barriers.
__device__ __forceinline__ void keyed_add3(double *red, int rb, int s0, float v0, int s1, float v1, int s2, float v2) {
    __shared__ double part3[3][32];
    const int rb0 = __shfl_sync(0xffffffffu, rb, 0);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    __shared__ int block_rb3;
    if (threadIdx.x == 0) block_rb3 = rb;
    __syncthreads();
    const bool uniform = __syncthreads_and(rb == block_rb3 || rb < 0);
    float a = v0, b = v1, c = v2;
    if (uniform || __all_sync(0xffffffffu, rb == rb0 || rb < 0)) {
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_down_sync(0xffffffffu, a, o);
            b += __shfl_down_sync(0xffffffffu, b, o);
            c += __shfl_down_sync(0xffffffffu, c, o);
        }
    }
    if (uniform) {
        if (lane == 0) {
            part3[0][w] = (double)a;
            part3[1][w] = (double)b;
            part3[2][w] = (double)c;
        }
        __syncthreads();
        if (threadIdx.x < 3 && block_rb3 >= 0) {
            double t = 0.0;
            for (int k = 0; k < nw; k++) t += part3[threadIdx.x][k];
            const int slot = threadIdx.x == 0 ? s0 : (threadIdx.x == 1 ? s1 : s2);
            if (t != 0.0) atomicAdd(&red[block_rb3 + slot], t);
        }
        __syncthreads();
        return;
    }
    if (__all_sync(0xffffffffu, rb == rb0 || rb < 0)) {
        if (lane == 0 && rb0 >= 0) {
            if (a != 0.f) atomicAdd(&red[rb0 + s0], (double)a);
            if (b != 0.f) atomicAdd(&red[rb0 + s1], (double)b);
            if (c != 0.f) atomicAdd(&red[rb0 + s2], (double)c);
        }
    } else if (rb >= 0) {
        if (v0 != 0.f) atomicAdd(&red[rb + s0], (double)v0);
        if (v1 != 0.f) atomicAdd(&red[rb + s1], (double)v1);
        if (v2 != 0.f) atomicAdd(&red[rb + s2], (double)v2);
    }
}

__global__ void k_stamp(unsigned long long *t, int k) {
    unsigned long long v;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(v));
    t[k] = v;
}

// time += 1 (engine_step, tfEngine.cpp:1387) and, in Verlet mode, the rebuild decision of
// engine_verlet_update (tfEngine.cpp:234-290): rebuild when 2 * maxdx > skin, maxdx being
// the largest displacement since the last rebuild, measured after the previous advance.
// One step's start for every simulation: stop it if it has reached its stop time, else
// advance its clock and clear its FP64 totals (a stopped simulation keeps the totals of its
// last step).
__global__ void k_tick(int nsims, SimParams *sims, double *red) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nsims) return;
    SimParams &P = sims[k];
    if (P.stop_at >= 0 && P.time >= P.stop_at) {
        P.stopped = 1;
        if (P.verlet_rebuild == 1) P.verlet_rebuild = 0;
        return;
    }
    P.stopped = 0;
    P.time += 1;
    for (int r = 0; r < RED_COUNT; r++) red[P.red_base + r] = 0.0;
    if (P.flags & TFG_ENGINE_VERLET) {
        int rb = P.verlet_rebuild == 2;
        float m = 0.f;
        if (!rb) {
            m = __fsqrt_rn(__uint_as_float(P.verlet_maxdx2));
            rb = __fmul_rn(2.0f, m) > P.skin;
        }
        P.verlet_maxdx = rb ? 0.f : m;
        P.verlet_rebuild = rb;
        P.verlet_maxdx2 = 0u;
        if (rb) P.verlet_rebuilds += 1;
    }
}

// space_setpartp (tfSpace.cpp:432-475) for one simulation's particles, written to arena
// slots [slot0, slot0+n) with global cell indices and ids.
__global__ void k_setpartp(int n, const float *__restrict__ xg, SimParams P, float3 lo, float3 hi, float3 org,
                           float3 ih, int slot0, int32_t *cell, float4 *pos, float4 *aux,
                           const int32_t *__restrict__ type, uint32_t *err) {
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
            atomicOr(err + 1 + P.red_base / RED_COUNT, ERR_RANGE);
            ind[k] = ind[k] < 0 ? 0 : P.cdim[k] - 1;
        }
    }
    const int s = slot0 + i;
    cell[s] = cell_index(P, ind[0], ind[1], ind[2]);
    pos[s] = make_float4(__fsub_rn(x[0], P.corig[0][ind[0]]), __fsub_rn(x[1], P.corig[1][ind[1]]),
                         __fsub_rn(x[2], P.corig[2][ind[2]]), __int_as_float(type ? type[i] : 0));
    float4 a = aux[s];
    a.w = __int_as_float(P.id_off + i);
    aux[s] = a;
}

// Copy one simulation's particle records from one arena layout to another, moving its
// ids and cells by the change of its offsets.
__global__ void k_relocate(int n, int src0, int dst0, int cap_src, int cap_dst, int nspec, int did, int dcell,
                           ParticleArrays src, ParticleArrays dst) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int a = src0 + i, b = dst0 + i;
    dst.pos[b] = src.pos[a];
    dst.vel[b] = src.vel[a];
    float4 ax = src.aux[a];
    ax.w = __int_as_float(__float_as_int(ax.w) + did);
    dst.aux[b] = ax;
    dst.fext[b] = src.fext[a];
    dst.pforce[b] = src.pforce[a];
    dst.cell[b] = src.cell[a] + dcell;
    for (int s = 0; s < nspec; s++) {
        dst.sval[s * cap_dst + b] = src.sval[s * cap_src + a];
        dst.sq[s * cap_dst + b] = src.sq[s * cap_src + a];
    }
}

// Re-check of the cell-relative position (space_shuffle_local) and per-cell counting.
__global__ void k_bin_count(int n, const SimParams *sims, const int32_t *cell_sim, float4 *pos, int32_t *cell,
                            int32_t *count, int32_t *lidx, int shuffle) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int c = cell[i];
    if (shuffle) {
        const SimParams &P = sims[cell_sim[c]];
        // Verlet mode re-bins only on rebuild steps (engine_verlet_update -> engine_shuffle);
        // a stopped simulation stays as it is
        if (P.stopped || ((P.flags & TFG_ENGINE_VERLET) && !P.verlet_rebuild)) {
            lidx[i] = atomicAdd(&count[c], 1);
            return;
        }
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
    int tot;
    int ex = block_exclusive_scan(i < n ? count[i] : 0, &tot);
    if (i < n) start[i] = ex;
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void k_scan_sums(int32_t *sums, int nb) {
    const int per = (nb + blockDim.x - 1) / blockDim.x;
    const int b0 = threadIdx.x * per;
    int local = 0;
    for (int k = 0; k < per; k++) if (b0 + k < nb) local += sums[b0 + k];
    int run = block_exclusive_scan(local, nullptr);
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
// up to 32 particles rank in registers; larger cells compare against global memory.
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

__global__ void k_scatter(int n, int cap, int nspec, const int32_t *dest, ParticleArrays src, ParticleArrays dst,
                          int32_t *slot_of_id, const SimParams *sims, const int32_t *cell_sim, const float4 *rforce,
                          float4 *force, float4 *oldx) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int d = dest[i];
    const float4 ax = src.aux[i];
    const float4 p = src.pos[i];
    const float4 fe = src.fext[i];
    const int c = src.cell[i];
    float4 pf = src.pforce[i];
    const int id = __float_as_int(ax.w);
    const SimParams &P = sims[cell_sim[c]];
    const float4 rf = rforce[P.type_base + __float_as_int(p.w)];
    if (rf.w != 0.f) {
        const int lid = id - P.id_off;
        const int dur = (int)rf.z;
        if ((P.time + lid) % dur == 0) {
            U4 r = philox({(uint32_t)P.time, (uint32_t)lid, 0u, STREAM_FORCE}, (uint32_t)P.seed,
                          (uint32_t)(P.seed >> 32));
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
    // Verlet reference positions, stored after the rebuild's re-binning (tfEngine.cpp:308-335)
    if (oldx && (P.flags & TFG_ENGINE_VERLET) && P.verlet_rebuild) oldx[d] = make_float4(p.x, p.y, p.z, 0.f);
    dst.vel[d] = src.vel[i];
    dst.aux[d] = ax;
    dst.fext[d] = fe;
    dst.pforce[d] = pf;
    dst.cell[d] = c;
    for (int s = 0; s < nspec; s++) {
        dst.sval[s * cap + d] = src.sval[s * cap + i];
        dst.sq[s * cap + d] = src.sq[s * cap + i];
    }
    slot_of_id[id] = d;
}

// bond_eval (tfBond.cpp:97-345) for table potentials; one thread per bond.
__global__ void k_bonds(int nb, const SimParams *sims, const int32_t *cell_sim, const int2 *bonds,
                        const int32_t *bslot, const PotDev *bpots, const float *bblob, const int32_t *slot_of_id,
                        const float4 *pos, const float4 *aux, const int32_t *cell, float4 *force, double *red) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    float epot = 0.f, vir = 0.f;
    int rb = -1;
    if (b < nb) {
        const int2 bd = bonds[b];
        const PotDev &pot = bpots[bslot[b]];
        const int si = slot_of_id[bd.x], sj = slot_of_id[bd.y];
        const SimParams *Pp = (si >= 0) ? &sims[cell_sim[cell[si]]] : nullptr;
        if (pot.kind == POT_TABLE && si >= 0 && sj >= 0 && !Pp->stopped) {
            const SimParams &P = *Pp;
            rb = P.red_base;
            const float4 pi = pos[si], pj = pos[sj];
            int ai, bi, ci, aj, bj, cj;
            cell_loc(P, cell[si], ai, bi, ci);
            cell_loc(P, cell[sj], aj, bj, cj);
            const int s0 = wrap_shift(ai - aj), s1 = wrap_shift(bi - bj), s2 = wrap_shift(ci - cj);
            const float pix = __fadd_rn(pi.x, __fmul_rn(P.h[0], (float)s0));
            const float piy = __fadd_rn(pi.y, __fmul_rn(P.h[1], (float)s1));
            const float piz = __fadd_rn(pi.z, __fmul_rn(P.h[2], (float)s2));
            const float dx = __fsub_rn(pix, pj.x), dy = __fsub_rn(piy, pj.y), dz = __fsub_rn(piz, pj.z);
            const float r2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
            // potential_eval_adjust_distance2
            float r = __fsqrt_rn(r2);
            if (pot.flags & TFG_POTENTIAL_SCALED) r = __fdiv_rn(r, __fadd_rn(aux[si].x, aux[sj].x));
            else if (pot.flags & TFG_POTENTIAL_SHIFTED)
                r = __fadd_rn(__fsub_rn(r, __fadd_rn(aux[si].x, aux[sj].x)), pot.r0_plusone);
            float rr2 = __fmul_rn(r, r);
            if (!(rr2 > __fmul_rn(pot.b, pot.b))) {
                rr2 = fmaxf(rr2, __fmul_rn(pot.a, pot.a));
                // potential_eval (tf_potential_eval.h:74-102)
                const float rb_ = __fsqrt_rn(rr2);
                const float t = __fadd_rn(pot.alpha0, __fmul_rn(rb_, __fadd_rn(pot.alpha1, __fmul_rn(rb_, pot.alpha2))));
                int ind = (int)fmaxf(0.0f, t);
                if (ind > pot.n) ind = pot.n;
                float ee, eff, c1;
                table_row_eval(bblob + pot.offset + ind * kChunk, rb_, ee, eff, c1);
                const float f = eff * c1 / rb_;
                atomicAdd(&force[si], make_float4(-f * dx, -f * dy, -f * dz, 0.f));
                atomicAdd(&force[sj], make_float4(f * dx, f * dy, f * dz, 0.f));
                epot = ee;
                vir = -f * r2;
            }
        }
    }
    keyed_add3(red, rb, RED_EPOT_BOND, epot, RED_VIRIAL, vir, RED_VIRIAL, 0.f);
}

// angle_eval (tfAngle.cpp:90-382); one thread per angle, j is the vertex.
__global__ void k_angles(int na, const SimParams *sims, const int32_t *cell_sim, const int4 *angles,
                         const PotDev *bpots, const float *bblob, const int32_t *slot_of_id, const float4 *pos,
                         const int32_t *cell, float4 *force, double *red) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    float epot = 0.f;
    int rb = -1;
    if (q < na) {
        const int4 A = angles[q];
        const PotDev &pot = bpots[A.w];
        const int si = slot_of_id[A.x], sj = slot_of_id[A.y], sk = slot_of_id[A.z];
        const SimParams *Pp = (sj >= 0) ? &sims[cell_sim[cell[sj]]] : nullptr;
        if (pot.kind == POT_TABLE && si >= 0 && sj >= 0 && sk >= 0 && !Pp->stopped) {
            const SimParams &P = *Pp;
            rb = P.red_base;
            const float4 pi = pos[si], pj = pos[sj], pk = pos[sk];
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
            const float dprod = __fadd_rn(__fadd_rn(__fmul_rn(rji[0], rjk[0]), __fmul_rn(rji[1], rjk[1])),
                                          __fmul_rn(rji[2], rjk[2]));
            const float nji = __fadd_rn(__fadd_rn(__fmul_rn(rji[0], rji[0]), __fmul_rn(rji[1], rji[1])),
                                        __fmul_rn(rji[2], rji[2]));
            const float njk = __fadd_rn(__fadd_rn(__fmul_rn(rjk[0], rjk[0]), __fmul_rn(rjk[1], rjk[1])),
                                        __fmul_rn(rjk[2], rjk[2]));
            const float inji = __fdiv_rn(1.0f, __fsqrt_rn(nji));
            const float injk = __fdiv_rn(1.0f, __fsqrt_rn(njk));
            const float ctheta = fmaxf(-1.0f, fminf(1.0f, __fmul_rn(__fmul_rn(dprod, inji), injk)));
            float dxi[3], dxk[3];
            if (ctheta == 0.f || ctheta == -1.f) {
                // Random derivative plane: the reference draws from the global mt19937
                // (tfAngle.cpp:210-223); here a Philox stream keyed on (step, angle).
                U4 r = philox({(uint32_t)P.time, (uint32_t)(q - P.angle_off), 0u, STREAM_ANGLE}, (uint32_t)P.seed,
                              (uint32_t)(P.seed >> 32));
                float x[3] = {2.f * u01(r.x) - 1.f, 2.f * u01(r.y) - 1.f, 2.f * u01(r.z) - 1.f};
                const float vik[3] = {xi[0] - xk[0], xi[1] - xk[1], xi[2] - xk[2]};
                const float dd = x[0] * vik[0] + x[1] * vik[1] + x[2] * vik[2];
                for (int k = 0; k < 3; k++) x[k] = x[k] - dd * vik[k];
                const float len = sqrtf(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
                for (int k = 0; k < 3; k++) dxi[k] = dxk[k] = x[k] / len;
            } else {
                for (int k = 0; k < 3; k++) {
                    dxi[k] = (rjk[k] * injk - ctheta * rji[k] * inji) * inji;
                    dxk[k] = (rji[k] * inji - ctheta * rjk[k] * injk) * injk;
                }
            }
            if (!(ctheta > pot.b)) {
                const float rr = fmaxf(ctheta, pot.a);
                const float t = __fadd_rn(pot.alpha0, __fmul_rn(rr, __fadd_rn(pot.alpha1, __fmul_rn(rr, pot.alpha2))));
                const int ind = (int)fmaxf(0.0f, t);
                if (ind <= pot.n) {
                    float ee, eff, c1;
                    table_row_eval(bblob + pot.offset + ind * kChunk, rr, ee, eff, c1);
                    eff = eff * c1;
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
    keyed_add(red, rb, RED_EPOT_ANGLE, epot);
}

// Verlet mode: the integrator branch of engine_advance_forward_euler for Verlet lists
// (tf_engine_advance.cpp:367-427), plus the squared displacement from the reference
// position that engine_verlet_update takes the maximum of (tfEngine.cpp:239-252).
__device__ __forceinline__ float advance_verlet(const SimParams &P, bool newtonian, const float4 &f, float imass,
                                                float4 &p, float4 &v, const float4 &ox) {
    const float dt = P.dt;
    const float fv[3] = {f.x, f.y, f.z};
    float x[3] = {p.x, p.y, p.z}, vv[3] = {v.x, v.y, v.z};
    for (int k = 0; k < 3; k++) {
        if (newtonian) vv[k] = __fadd_rn(vv[k], __fmul_rn(__fmul_rn(fv[k], dt), imass));
        else vv[k] = __fmul_rn(fv[k], imass);
        x[k] = __fadd_rn(x[k], __fmul_rn(vv[k], dt));
    }
    p = make_float4(x[0], x[1], x[2], p.w);
    v = make_float4(vv[0], vv[1], vv[2], v.w);
    const float w0 = __fsub_rn(x[0], ox.x), w1 = __fsub_rn(x[1], ox.y), w2 = __fsub_rn(x[2], ox.z);
    return __fadd_rn(__fadd_rn(__fmul_rn(w0, w0), __fmul_rn(w1, w1)), __fmul_rn(w2, w2));
}

// cell_advance_forward_euler + Fluxes_integrate; one thread per particle.
__global__ void k_advance(int n, int cap, int nspec, SimParams *sims, const int32_t *cell_sim, float4 *pos,
                          float4 *vel, const float4 *aux, const float4 *force, int32_t *cell, float *sval, float *sq,
                          const float *type_mass, const int32_t *type_dyn, const uint32_t *species_flags,
                          const float4 *oldx, double *red, uint32_t *err) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    float ke = 0.f, vol = 0.f, mig = 0.f;
    float stot[kMaxSpecies];
#pragma unroll
    for (int s = 0; s < kMaxSpecies; s++) stot[s] = 0.f;
    int rb = -1;
    int vsim = -1;          // Verlet simulation of this particle
    uint32_t dx2 = 0u;      // its squared displacement (float bits)
    if (i < n && !sims[cell_sim[cell[i]]].stopped) {
        const int c0 = cell[i];
        const SimParams &P = sims[cell_sim[c0]];
        rb = P.red_base;
        float4 p = pos[i], v = vel[i];
        const float4 ax = aux[i];
        const float4 f = force[i];
        const int type = __float_as_int(p.w);
        const uint32_t flags = (uint32_t)__float_as_int(ax.z);
        const float imass = ax.y;
        ke = 0.5f * type_mass[P.type_base + type] * (v.x * v.x + v.y * v.y + v.z * v.z);
        bool migrated = false;
        if (P.flags & TFG_ENGINE_VERLET) {
            const float d2 = advance_verlet(P, type_dyn[P.type_base + type] == TFG_NEWTONIAN, f, imass, p, v, oldx[i]);
            if (!(isfinite(p.x) && isfinite(p.y) && isfinite(p.z))) {
                atomicOr(err, ERR_NAN);
                atomicOr(err + 1 + rb / RED_COUNT, ERR_NAN);
            }
            pos[i] = p;
            vel[i] = v;
            vsim = cell_sim[c0];
            dx2 = __float_as_uint(d2);
            for (int s = 0; s < nspec; s++) stot[s] = sval[s * cap + i];
            goto reduce;
        }
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
            if (type_dyn[P.type_base + type] == TFG_NEWTONIAN) {
                for (int k = 0; k < 3; k++) {
                    const float a = __fmul_rn(__fmul_rn(dt, fv[k]), imass);
                    const float nv = __fmul_rn(mask[k], __fadd_rn(vv[k], a));
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
            if ((delta[0] | delta[1] | delta[2]) && P.walls_reflect) {
                // reflection at FREESLIP / VELOCITY walls (apply_update_pos_vel,
                // tf_boundary_eval.h:46-134), walls in the reference's order
                int la, lb, lc;
                cell_loc(P, c0, la, lb, lc);
                bool enforced = false;
                for (int w = 0; w < 6; w++) {
                    if (!(P.walls_reflect & (1u << w)) || !on_wall(P, w, la, lb, lc)) continue;
                    const int ax = w >> 1;
                    const bool high = (w & 1) != 0;
                    if (high ? !(x[ax] >= P.h[ax]) : !(x[ax] <= 0.f)) continue;
                    const bool slip = (P.wall_kind[w] & TFG_BOUNDARY_FREESLIP) != 0;
                    const float rest = slip ? 1.0f : P.wall_vel[w].w;
                    if (high)
                        x[ax] = __fsub_rn(P.h[ax], fmaxf(__fmul_rn(__fsub_rn(x[ax], P.h[ax]), rest), 1.1920928955078125e-7f));
                    else
                        x[ax] = fmaxf(__fmul_rn(-x[ax], rest), 0.0f);
                    if (slip) {
                        vv[ax] = -vv[ax];
                    } else {
                        const float U[3] = {P.wall_vel[w].x, P.wall_vel[w].y, P.wall_vel[w].z};
                        for (int k = 0; k < 3; k++) vv[k] = __fsub_rn(U[k], __fmul_rn(__fsub_rn(vv[k], U[k]), rest));
                    }
                    enforced = true;
                }
                if (enforced)
                    for (int k = 0; k < 3; k++) delta[k] = (x[k] >= P.h[k]) - (x[k] < 0.0f);
            }
            if (delta[0] | delta[1] | delta[2]) {
                for (int k = 0; k < 3; k++) {
                    if (x[k] >= P.h2[k] || x[k] <= -P.h[k]) {
                        atomicOr(err, ERR_TOOFAST);
                        atomicOr(err + 1 + rb / RED_COUNT, ERR_TOOFAST);
                        break;
                    }
                    x[k] = __fadd_rn(x[k], -__fmul_rn((float)delta[k], P.h[k]));
                }
                int a, b, c;
                cell_loc(P, c0, a, b, c);
                cell[i] = cell_index(P, (a + delta[0] + P.cdim[0]) % P.cdim[0], (b + delta[1] + P.cdim[1]) % P.cdim[1],
                                     (c + delta[2] + P.cdim[2]) % P.cdim[2]);
                migrated = true;
                mig = 1.f;
                if (nspec > 0) {
                    const int loc[3] = {a, b, c};
                    if (crosses_resetting_wall(P, loc, delta))
                        for (int s = 0; s < nspec; s++) sval[s * cap + i] = P.species_reset[s];
                }
            }
            if (!(isfinite(x[0]) && isfinite(x[1]) && isfinite(x[2]))) {
                atomicOr(err, ERR_NAN);
                atomicOr(err + 1 + rb / RED_COUNT, ERR_NAN);
            }
            pos[i] = make_float4(x[0], x[1], x[2], p.w);
            vel[i] = make_float4(vv[0], vv[1], vv[2], inv_nd);
        }
        // Fluxes_integrate runs over the particles still in their cell: migrants keep their
        // flux increment for the next step (they sit in the destination's incoming list).
        for (int s = 0; s < nspec; s++) {
            float sv = sval[s * cap + i];
            if (!migrated) {
                const float konst = (species_flags[P.spec_base + s] & 1u) ? 0.f : 1.f;
                const float q = sq[s * cap + i];
                sv = fmaxf(0.0f, __fadd_rn(sv, __fmul_rn(__fmul_rn(P.dt_flux, q), konst)));
                sval[s * cap + i] = sv;
                sq[s * cap + i] = 0.f;
            }
            stot[s] = sv;
        }
    }
reduce:
    {
        // largest displacement per Verlet simulation: one atomic per warp when the warp's
        // particles share a simulation
        const int first = __shfl_sync(0xffffffffu, vsim, 0);
        if (__all_sync(0xffffffffu, vsim == first)) {
            const uint32_t m = __reduce_max_sync(0xffffffffu, dx2);
            if (first >= 0 && (threadIdx.x & 31) == 0) atomicMax(&sims[first].verlet_maxdx2, m);
        } else if (vsim >= 0) {
            atomicMax(&sims[vsim].verlet_maxdx2, dx2);
        }
    }
    keyed_add3(red, rb, RED_KINETIC, ke, RED_VOLUME, vol, RED_MIGRATIONS, mig);
    for (int s = 0; s < nspec; s++) keyed_add(red, rb, RED_SPECIES0 + s, stot[s]);
}

__global__ void k_flux_integrate(int n, int cap, int nspec, int sub, const SimParams *sims, const int32_t *cell_sim,
                                 const int32_t *cell, float *sval, float *sq, const uint32_t *species_flags) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const SimParams &P = sims[cell_sim[cell[i]]];
    if (P.stopped || sub >= P.nr_fluxsteps - 1) return;
    for (int s = 0; s < nspec; s++) {
        const float konst = (species_flags[P.spec_base + s] & 1u) ? 0.f : 1.f;
        const float q = sq[s * cap + i];
        sval[s * cap + i] = fmaxf(0.0f, __fadd_rn(sval[s * cap + i], __fmul_rn(__fmul_rn(P.dt_flux, q), konst)));
        sq[s * cap + i] = 0.f;
    }
}

// Per-particle state of slots [slot0, slot0+n) gathered by local id (id - id_off).
__global__ void k_gather(int n, int slot0, int cap, int nspec, SimParams P, ParticleArrays A, const float4 *force,
                         float *x, float *xrel, int32_t *cellout, float *v, float *f, float *dens, float *species,
                         float *q) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int i = slot0 + k;
    const float4 p = A.pos[i];
    const int id = __float_as_int(A.aux[i].w) - P.id_off;
    if (id < 0 || id >= n) return;
    const int c = A.cell[i];
    int l0, l1, l2;
    cell_loc(P, c, l0, l1, l2);
    if (x) {
        x[3 * id] = __fadd_rn(P.corig[0][l0], p.x);
        x[3 * id + 1] = __fadd_rn(P.corig[1][l1], p.y);
        x[3 * id + 2] = __fadd_rn(P.corig[2][l2], p.z);
    }
    if (xrel) { xrel[3 * id] = p.x; xrel[3 * id + 1] = p.y; xrel[3 * id + 2] = p.z; }
    if (cellout) cellout[id] = c - P.cell_off;
    if (v) { const float4 w = A.vel[i]; v[3 * id] = w.x; v[3 * id + 1] = w.y; v[3 * id + 2] = w.z; }
    if (f || dens) {
        const float4 w = force[i];
        if (f) { f[3 * id] = w.x; f[3 * id + 1] = w.y; f[3 * id + 2] = w.z; }
        if (dens) dens[id] = w.w;
    }
    for (int s = 0; s < nspec; s++) {
        if (species) species[id * nspec + s] = A.sval[s * cap + i];
        if (q) q[id * nspec + s] = A.sq[s * cap + i];
    }
}

inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }

}  // namespace

void launch_stamp(unsigned long long *t, int k, cudaStream_t s) { k_stamp<<<1, 1, 0, s>>>(t, k); }

void launch_tick(int nsims, SimParams *sims, double *red, cudaStream_t s) {
    if (nsims > 0) k_tick<<<nblk(nsims, 128), 128, 0, s>>>(nsims, sims, red);
}

void launch_setpartp(int n, const float *xg, const SimParams &P, float3 lo, float3 hi, float3 org, float3 ih,
                     int slot0, int32_t *cell, float4 *pos, float4 *aux, const int32_t *type, uint32_t *err,
                     cudaStream_t s) {
    if (n > 0)
        k_setpartp<<<nblk(n, kThreads), kThreads, 0, s>>>(n, xg, P, lo, hi, org, ih, slot0, cell, pos, aux, type, err);
}

void launch_relocate(int n, int src0, int dst0, int cap_src, int cap_dst, int nspec, int did, int dcell,
                     const ParticleArrays &src, const ParticleArrays &dst, cudaStream_t s) {
    if (n > 0)
        k_relocate<<<nblk(n, kThreads), kThreads, 0, s>>>(n, src0, dst0, cap_src, cap_dst, nspec, did, dcell, src,
                                                          dst);
}

void launch_bin(const BinArgs &b, cudaStream_t s) {
    cudaMemsetAsync(b.count, 0, sizeof(int32_t) * b.ncells, s);
    if (b.n > 0)
        k_bin_count<<<nblk(b.n, kThreads), kThreads, 0, s>>>(b.n, b.sims, b.cell_sim, b.src.pos, b.src.cell, b.count,
                                                            b.lidx, b.shuffle);
    const int nbs = nblk(b.ncells, 1024);
    k_scan_local<<<nbs, 1024, 0, s>>>(b.count, b.ncells, b.start, b.scan_sums);
    k_scan_sums<<<1, 1024, 0, s>>>(b.scan_sums, nbs);
    k_scan_add<<<nbs, 1024, 0, s>>>(b.start, b.scan_sums, b.count, b.ncells);
    if (b.n > 0) {
        k_place<<<nblk(b.n, kThreads), kThreads, 0, s>>>(b.n, b.src.cell, b.lidx, b.start, b.src.aux, b.tmp_id,
                                                        b.tmp_src);
        k_rank<<<nblk((long long)b.ncells * 32, kThreads), kThreads, 0, s>>>(b.ncells, b.start, b.tmp_id, b.tmp_src,
                                                                             b.dest);
        k_scatter<<<nblk(b.n, kThreads), kThreads, 0, s>>>(b.n, b.cap, b.nspec, b.dest, b.src, b.dst, b.slot_of_id,
                                                          b.sims, b.cell_sim, b.rforce, b.force, b.oldx);
    }
}

void launch_bonds(int nb, const SimParams *sims, const int32_t *cell_sim, const int2 *bonds, const int32_t *bslot,
                  const PotDev *bpots, const float *bblob, const int32_t *slot_of_id, const float4 *pos,
                  const float4 *aux, const int32_t *cell, float4 *force, double *red, cudaStream_t s) {
    if (nb > 0)
        k_bonds<<<nblk(nb, kThreads), kThreads, 0, s>>>(nb, sims, cell_sim, bonds, bslot, bpots, bblob, slot_of_id, pos,
                                                       aux, cell, force, red);
}

void launch_angles(int na, const SimParams *sims, const int32_t *cell_sim, const int4 *angles, const PotDev *bpots,
                   const float *bblob, const int32_t *slot_of_id, const float4 *pos, const int32_t *cell,
                   float4 *force, double *red, cudaStream_t s) {
    if (na > 0)
        k_angles<<<nblk(na, kThreads), kThreads, 0, s>>>(na, sims, cell_sim, angles, bpots, bblob, slot_of_id, pos, cell,
                                                        force, red);
}

void launch_advance(int n, int cap, int nspec, SimParams *sims, const int32_t *cell_sim,
                    const ParticleArrays &A, const float4 *force, const float *type_mass, const int32_t *type_dyn,
                    const uint32_t *species_flags, const float4 *oldx, double *red, uint32_t *err, cudaStream_t s) {
    if (n > 0)
        k_advance<<<nblk(n, kThreads), kThreads, 0, s>>>(n, cap, nspec, sims, cell_sim, A.pos, A.vel, A.aux, force,
                                                        A.cell, A.sval, A.sq, type_mass, type_dyn, species_flags, oldx,
                                                        red, err);
}

void launch_flux_integrate(int n, int cap, int nspec, int sub, const SimParams *sims, const int32_t *cell_sim,
                           const int32_t *cell, float *sval, float *sq, const uint32_t *species_flags,
                           cudaStream_t s) {
    if (n > 0 && nspec > 0)
        k_flux_integrate<<<nblk(n, kThreads), kThreads, 0, s>>>(n, cap, nspec, sub, sims, cell_sim, cell, sval, sq,
                                                                species_flags);
}

void launch_gather(int n, int slot0, int cap, int nspec, const SimParams &P, const ParticleArrays &A,
                   const float4 *force, float *x, float *xrel, int32_t *cell, float *v, float *f, float *dens,
                   float *species, float *q, cudaStream_t s) {
    if (n > 0)
        k_gather<<<nblk(n, kThreads), kThreads, 0, s>>>(n, slot0, cap, nspec, P, A, force, x, xrel, cell, v, f, dens,
                                                       species, q);
}

}  // namespace tfg
