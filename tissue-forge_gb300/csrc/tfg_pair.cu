// Nonbonded pair pass: number density, Fickian/secrete/uptake flux, tabulated potentials
// and DPD, fused into one kernel over the 27-cell stencil.
//
// Reference path replaced: runner_dopair / runner_doself (tf_runner_dopair.cpp:72-758)
// with potential_eval_super_ex (tf_potential_eval.h:207-272), dpd_eval
// (tf_dpd_eval.h:32-76), flux_eval_ex (tf_flux_eval.h:48-103) and W
// (tf_smoothing_kernel.h:49-67); the reference GPU offload computes the same in
// runner_run_cuda_do_{self,pair_left,pair_right}_kernel (tfRunner_cuda.cu:2487-2845).
//
// One thread owns one particle i and visits every particle j of the 27 surrounding
// cells.  Each pair is evaluated in the reference's orientation: the cell whose shift
// to the other is lexicographically positive plays `cell_i` (space_getsid), so
// dx = (x_i - shift) - x_j and r2 are bit-identical to the reference and the pair set
// {r2 <= cutoff^2} matches exactly.  The thread accumulates only its own force, density
// and flux increment, so no atomics are needed and results are deterministic.
#include "tfg_internal.h"

namespace tfg {

namespace {

constexpr int kPairThreads = 128;
constexpr int kMaxSmemBlob = 8 * 1024;    // floats of table blob staged in shared memory (32 KB)

struct Accum {
    float fx, fy, fz, dens;
    float q[kMaxSpecies];
    float epot, vir;     // per-thread partial sums; FP64 only in the block reduction
};

template <bool kHasFlux>
__device__ __forceinline__ void pair_flux(const PairKernelArgs &a, const FluxSet &fs, bool i_is_pi,
                                          int ti, int tj, int si, int sj, float r, Accum &acc) {
    // flux_eval_ex: orient (a,b) by the flux's type ids, starting from the reference's
    // (part_i, part_j) = i_is_pi ? (i, j) : (j, i).
    for (int k = 0; k < fs.count; k++) {
        const FluxDev &F = fs.f[k];
        if (r > F.cutoff) continue;
        float term = __fsub_rn(1.0f, __fdiv_rn(r, F.cutoff));
        term = __fmul_rn(term, term);
        // reference particles: P = part_i, Q = part_j
        int tP = i_is_pi ? ti : tj, tQ = i_is_pi ? tj : ti;
        int sP = i_is_pi ? si : sj, sQ = i_is_pi ? sj : si;
        // pi = P if type(P)==a else Q ; pj = Q if type(Q)==b else P
        bool a_is_P = (tP == F.type_a);
        bool b_is_Q = (tQ == F.type_b);
        int sa = a_is_P ? sP : sQ;          // slot of the "a" particle
        int sb = b_is_Q ? sQ : sP;          // slot of the "b" particle
        float ssi = a.sval[F.index_a * a.cap + sa];
        float ssj = a.sval[F.index_b * a.cap + sb];
        float q = term;
        if (F.kind == TFG_FLUX_FICK) {
            q = __fmul_rn(q, __fmul_rn(F.coef, __fsub_rn(ssi, ssj)));
        } else if (F.kind == TFG_FLUX_SECRETE) {
            float qq = __fmul_rn(F.coef, __fsub_rn(ssi, F.target));
            q = __fmul_rn(q, qq > 0.f ? qq : 0.f);
        } else {
            float qq = __fmul_rn(__fmul_rn(F.coef, __fsub_rn(F.target, ssj)), ssi);
            q = __fmul_rn(q, qq > 0.f ? qq : 0.f);
        }
        int me = si;
        if (sa == me) acc.q[F.index_a] = __fsub_rn(__fsub_rn(acc.q[F.index_a], q), __fmul_rn(F.half_decay, ssi));
        if (sb == me) acc.q[F.index_b] = __fsub_rn(__fadd_rn(acc.q[F.index_b], q), __fmul_rn(F.half_decay, ssj));
    }
}

template <bool kHasFlux, bool kDensity, bool kSig = false, bool kFluxOnly = false>
__global__ void __launch_bounds__(kPairThreads) k_pair_stencil(PairKernelArgs a) {
    extern __shared__ float sblob[];
    const int nb = a.blob_floats <= kMaxSmemBlob ? a.blob_floats : 0;
    for (int k = threadIdx.x; k < nb; k += blockDim.x) sblob[k] = a.blob[k];
    __syncthreads();
    const float *blob = nb ? sblob : a.blob;

    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double red_epot = 0.0, red_vir = 0.0;
    int red_base = -1;
    if (i < a.n) {

    const float4 pi4 = a.pos[i];
    const float3 xi = make_float3(pi4.x, pi4.y, pi4.z);
    const int ti = __float_as_int(pi4.w);
    const float4 vi4 = a.vel[i];
    const float4 axi = a.aux[i];
    const float ri = axi.x;
    const int idi = __float_as_int(axi.w);
    const int ci = a.cell[i];
    const SimParams &P = a.sims[a.cell_sim[ci]];
    red_base = P.red_base;
    // flux-only substep pass: only simulations with a substep of this number take part
    if ((kSig || !P.stopped) && (!kFluxOnly || a.flux_sub < P.nr_fluxsteps - 1)) {
    int li, lj, lk;
    cell_loc(P, ci, li, lj, lk);

    Accum acc;
    {
        // initial force: external + random force and the self density W(0), set by the scatter
        const float4 f0 = a.force[i];
        acc.fx = f0.x; acc.fy = f0.y; acc.fz = f0.z;
        acc.dens = f0.w;
    }
#pragma unroll
    for (int s = 0; s < kMaxSpecies; s++) acc.q[s] = 0.f;
    acc.epot = 0.f;
    acc.vir = 0.f;
    const float inv_cut = 1.0f / P.cutoff;

    int sig_n = 0;
    uint32_t sig_h = 0;
    if (!kSig && !kFluxOnly && a.has_wall_pots && P.walls_active) {
        float3 fw = make_float3(0.f, 0.f, 0.f);
        float ew = 0.f;
        wall_eval(P, a.wpots, blob, ti, xi, ri, vi4, idi - P.id_off, li, lj, lk, fw, ew);
        acc.fx += fw.x;
        acc.fy += fw.y;
        acc.fz += fw.z;
        acc.epot += ew;
    }
    for (int d = 0; d < 27; d++) {
        const int ox = d / 9 - 1, oy = (d / 3) % 3 - 1, oz = d % 3 - 1;
        const int mi = li + ox < 0 ? li + ox + P.cdim[0] : (li + ox >= P.cdim[0] ? li + ox - P.cdim[0] : li + ox);
        const int mj = lj + oy < 0 ? lj + oy + P.cdim[1] : (lj + oy >= P.cdim[1] ? lj + oy - P.cdim[1] : lj + oy);
        const int mk = lk + oz < 0 ? lk + oz + P.cdim[2] : (lk + oz >= P.cdim[2] ? lk + oz - P.cdim[2] : lk + oz);
        if (!(nb_exists(P, 0, li, ox) && nb_exists(P, 1, lj, oy) && nb_exists(P, 2, lk, oz))) continue;
        const int cj = cell_index(P, mi, mj, mk);
        const int j0 = a.start[cj], j1 = a.start[cj + 1];
        const bool self = (d == 13);
        // Orientation: offset (ox,oy,oz) lexicographically positive -> this cell is cell_i.
        const bool fwd = (ox > 0) || (ox == 0 && (oy > 0 || (oy == 0 && oz > 0)));
        float3 sh;
        if (!self) {
            if (fwd) {
                sh.x = cell_shift(P, 0, li, mi);
                sh.y = cell_shift(P, 1, lj, mj);
                sh.z = cell_shift(P, 2, lk, mk);
            } else {
                sh.x = cell_shift(P, 0, mi, li);
                sh.y = cell_shift(P, 1, mj, lj);
                sh.z = cell_shift(P, 2, mk, lk);
            }
        }
        for (int j = j0; j < j1; j++) {
            if (self && j == i) continue;
            const float4 pj4 = a.pos[j];
            const float3 xj = make_float3(pj4.x, pj4.y, pj4.z);
            float3 dx;
            float r2;
            bool i_is_pi;
            if (self) {
                // runner_doself pairs (i<j) with dx = x_first - x_second; the first is part_i.
                i_is_pi = i < j;
                r2 = i_is_pi ? pair_r2_self(xi, xj, dx) : pair_r2_self(xj, xi, dx);
            } else if (fwd) {
                i_is_pi = true;
                r2 = pair_r2(xi, sh, xj, dx);
            } else {
                i_is_pi = false;
                r2 = pair_r2(xj, sh, xi, dx);
            }
            if (r2 > P.cutoff2) continue;
            if (kSig) {
                sig_n++;
                const int idj = __float_as_int(a.aux[j].w);
                sig_h += sig_mix((uint32_t)idj);
                if (idi < idj) record_pair(a, idi, idj);
                continue;
            }
            const float r = __fsqrt_rn(r2);
            if (kDensity && !kFluxOnly) acc.dens += density_w(r, inv_cut, P.self_density);
            const int tj = __float_as_int(pj4.w);
            const int pidx = P.pot_base + ti * a.max_type + tj;
            if (kHasFlux) {
                const FluxSet &fs = a.fluxes[pidx];
                if (fs.count) pair_flux<kHasFlux>(a, fs, i_is_pi, ti, tj, i, j, r, acc);
            }
            if (kFluxOnly) continue;
            const PotDev &pot = a.pots[pidx];
            if (pot.kind == POT_TABLE) {
                const float rj = a.aux[j].x;
                float e, f;
                if (table_eval(pot, blob, i_is_pi ? ri : rj, i_is_pi ? rj : ri, r2, e, f)) {
                    // part_i.f -= f*dx ; part_j.f += f*dx
                    const float sgn = i_is_pi ? -1.f : 1.f;
                    acc.fx += sgn * (f * dx.x);
                    acc.fy += sgn * (f * dx.y);
                    acc.fz += sgn * (f * dx.z);
                    acc.epot += 0.5f * e;
                    acc.vir -= 0.5f * f * r2;
                }
            } else if (pot.kind == POT_DPD) {
                const float4 axj = a.aux[j];
                const float rj = axj.x;
                float rr = r;
                const float ro = r < 1.1920928955078125e-7f ? 1.1920928955078125e-7f : r;
                if (pot.flags & TFG_POTENTIAL_SHIFTED) rr = __fsub_rn(rr, __fadd_rn(ri, rj));
                if (rr <= pot.b) {
                    rr = rr >= pot.a ? rr : pot.a;
                    const float4 vj4 = a.vel[j];
                    // v = v(part_i) - v(part_j); e = dx/ro
                    const float3 v = i_is_pi ? make_float3(vi4.x - vj4.x, vi4.y - vj4.y, vi4.z - vj4.z)
                                             : make_float3(vj4.x - vi4.x, vj4.y - vi4.y, vj4.z - vi4.z);
                    const float3 ev = make_float3(__fdiv_rn(dx.x, ro), __fdiv_rn(dx.y, ro), __fdiv_rn(dx.z, ro));
                    const float omega_c = rr < 0.f ? 1.f : 1.f - rr / pot.b;
                    const float fc = pot.dpd_alpha * omega_c;
                    const float omega_d = omega_c * omega_c;
                    const float edv = ev.x * v.x + ev.y * v.y + ev.z * v.z;
                    const float fd = -pot.dpd_gamma * omega_d * edv;
                    float xi_r = 1.0f;
                    if (!(P.flags & TFG_ENGINE_DPD_REFERENCE_RANDOM))
                        xi_r = gauss_pair(P.seed, P.time, idi - P.id_off, __float_as_int(axj.w) - P.id_off);
                    const float fr = pot.dpd_sigma * omega_c * xi_r * P.dpd_delta;
                    const float ftot = fc + fd + fr;
                    // part_i.f += F e ; part_j.f -= F e
                    const float sgn = i_is_pi ? 1.f : -1.f;
                    acc.fx += sgn * (ftot * ev.x);
                    acc.fy += sgn * (ftot * ev.y);
                    acc.fz += sgn * (ftot * ev.z);
                    acc.vir += 0.5f * ftot * ro;
                }
            }
        }
    }

    if (kSig) {
        a.sig_count[idi] = sig_n;
        a.sig_hash[idi] = sig_h;
    } else {
        if (!kFluxOnly) a.force[i] = make_float4(acc.fx, acc.fy, acc.fz, acc.dens);
        if (kHasFlux) {
            for (int s = 0; s < a.nspec; s++) a.sq[s * a.cap + i] += acc.q[s];
        }
        red_epot = (double)acc.epot;
        red_vir = (double)acc.vir;
    }
    }  // this simulation takes part
    }  // i < n
    if (kSig) return;

    // FP64 warp reduction of energy and virial into each simulation's totals: one atomic
    // per warp when the warp's particles belong to one simulation, else one per lane.
    const int rb0 = __shfl_sync(0xffffffffu, red_base, 0);
    if (__all_sync(0xffffffffu, red_base == rb0 || red_base < 0)) {
        for (int o = 16; o > 0; o >>= 1) {
            red_epot += __shfl_down_sync(0xffffffffu, red_epot, o);
            red_vir += __shfl_down_sync(0xffffffffu, red_vir, o);
        }
        if ((threadIdx.x & 31) == 0 && rb0 >= 0) {
            if (red_epot != 0.0) atomicAdd(&a.red[rb0 + RED_EPOT_NONBOND], red_epot);
            if (red_vir != 0.0) atomicAdd(&a.red[rb0 + RED_VIRIAL], red_vir);
        }
    } else if (red_base >= 0) {
        if (red_epot != 0.0) atomicAdd(&a.red[red_base + RED_EPOT_NONBOND], red_epot);
        if (red_vir != 0.0) atomicAdd(&a.red[red_base + RED_VIRIAL], red_vir);
    }
}

}  // namespace

void launch_pair_stencil_fluxonly(const PairKernelArgs &a, cudaStream_t s) {
    if (a.n <= 0) return;
    const int blocks = (a.n + kPairThreads - 1) / kPairThreads;
    const size_t smem = (a.blob_floats <= kMaxSmemBlob ? a.blob_floats : 0) * sizeof(float);
    k_pair_stencil<true, false, false, true><<<blocks, kPairThreads, smem, s>>>(a);
}

void launch_pair_signature(const PairKernelArgs &a, cudaStream_t s) {
    if (a.n <= 0) return;
    const int blocks = (a.n + kPairThreads - 1) / kPairThreads;
    const size_t smem = (a.blob_floats <= kMaxSmemBlob ? a.blob_floats : 0) * sizeof(float);
    k_pair_stencil<false, false, true><<<blocks, kPairThreads, smem, s>>>(a);
}

void launch_pair(const PairKernelArgs &a, cudaStream_t s) {
    if (a.n <= 0) return;
    const int blocks = (a.n + kPairThreads - 1) / kPairThreads;
    const size_t smem = (a.blob_floats <= kMaxSmemBlob ? a.blob_floats : 0) * sizeof(float);
    const bool flux = a.nspec > 0 && a.has_flux;
    const bool dens = !(a.flags & TFG_ENGINE_NO_DENSITY);
    if (flux) {
        if (dens) k_pair_stencil<true, true><<<blocks, kPairThreads, smem, s>>>(a);
        else k_pair_stencil<true, false><<<blocks, kPairThreads, smem, s>>>(a);
    } else {
        if (dens) k_pair_stencil<false, true><<<blocks, kPairThreads, smem, s>>>(a);
        else k_pair_stencil<false, false><<<blocks, kPairThreads, smem, s>>>(a);
    }
}

}  // namespace tfg
