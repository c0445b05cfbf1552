// Cell binning that allocates nothing.
//
// Some callers of this library cannot allocate device memory: code that runs inside a
// CUDA graph being captured by someone else, plugins handed a fixed memory pool by their
// host application, or real-time loops where a cudaMalloc/cudaFree would stall the whole
// device.  tfg_bin_noalloc gives them the cell binning of an engine load (the reference's
// space_setpartp, source/mdcore/src/tfSpace.cpp:432-475, followed by a sort into cell
// order) with every temporary buffer taken from one statically allocated device array
// instead of cudaMalloc.
//
// The scratch array below is a file-scope __device__ variable: every GPU that loads this
// library holds it (TFG_NOALLOC_SCRATCH_BYTES) until the process exits.  Its host-side
// name is only a stand-in for the device variable, so host code never passes `scratch`
// to a kernel; the device address is looked up with cudaGetSymbolAddress, with the
// device current, once per CUDA context (the address belongs to the context that loaded
// the module: a host application's own context, or a primary context re-created after
// cudaDeviceReset, gets its own lookup).
//
// The cell order is a stable least-significant-digit radix sort of the particle indices
// on their cell (8-bit digits, one to three passes), so its work is linear in n whatever
// the distribution: all particles in one cell cost the same as a uniform spread.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <cstdint>
#include <mutex>

#include "tfg_internal.h"

using namespace tfg;

namespace {

constexpr int kNoAllocMaxParticles = TFG_NOALLOC_MAX_PARTICLES;
constexpr int kNoAllocMaxCells = TFG_NOALLOC_MAX_CELLS;
constexpr int kScanBlock = 1024;
constexpr int kTile = 1024;                                   // radix-sort tile (one element per thread)
constexpr int kMaxTiles = (kNoAllocMaxParticles + kTile - 1) / kTile;
constexpr int kRadix = 256;                                   // 8-bit digits
constexpr int kHistWords = kRadix * kMaxTiles;                // digit-major per-tile digit counts
constexpr int kMaxScanBlocks = (kNoAllocMaxCells > kHistWords ? kNoAllocMaxCells : kHistWords) / kScanBlock;

// Layout of the scratch array, in 32-bit words:
//   counts [kNoAllocMaxCells]      particles per cell (cleared at the start of every call)
//   hist   [kHistWords]            digit counts per radix tile, digit-major
//   hoff   [kHistWords + 1]        exclusive prefix of hist: where a tile's digit run starts
//   ia, ib [kNoAllocMaxParticles]  ping-pong particle orders between radix passes
//   sums   [kMaxScanBlocks]        per-block totals of the scans
constexpr size_t kOffCounts = 0;
constexpr size_t kOffHist = kOffCounts + kNoAllocMaxCells;
constexpr size_t kOffHoff = kOffHist + kHistWords;
constexpr size_t kOffA = kOffHoff + kHistWords + 1;
constexpr size_t kOffB = kOffA + kNoAllocMaxParticles;
constexpr size_t kOffSums = kOffB + kNoAllocMaxParticles;
constexpr size_t kScratchWords = kOffSums + kMaxScanBlocks;
static_assert(kScratchWords * 4 == TFG_NOALLOC_SCRATCH_BYTES, "scratch size must match the header");
static_assert(kHistWords <= kScanBlock * kScanBlock && kNoAllocMaxCells <= kScanBlock * kScanBlock,
              "the three-pass scan covers at most 1024 blocks of 1024");

static __device__ __align__(256) int32_t scratch[kScratchWords];

__global__ void k_na_clear(int32_t *counts, int ncells) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ncells) counts[i] = 0;
}

// space_setpartp: clamp into the domain, bin, make the position cell-relative; count.
__global__ void k_na_setpartp(int n, const float *__restrict__ xg, int3 cdim, float3 lo, float3 hi, float3 org,
                              float3 ih, float3 h, int32_t *cell, float *xrel, int32_t *counts) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float l3[3] = {lo.x, lo.y, lo.z}, h3[3] = {hi.x, hi.y, hi.z}, o3[3] = {org.x, org.y, org.z};
    const float i3[3] = {ih.x, ih.y, ih.z}, e3[3] = {h.x, h.y, h.z};
    const int c3[3] = {cdim.x, cdim.y, cdim.z};
    int ind[3];
    float x[3];
    for (int k = 0; k < 3; k++) {
        x[k] = fmaxf(l3[k], fminf(h3[k], xg[3 * i + k]));
        ind[k] = (int)__fmul_rn(__fsub_rn(x[k], o3[k]), i3[k]);
        ind[k] = ind[k] < 0 ? 0 : (ind[k] >= c3[k] ? c3[k] - 1 : ind[k]);
    }
    const int c = (ind[0] * c3[1] + ind[1]) * c3[2] + ind[2];
    cell[i] = c;
    for (int k = 0; k < 3; k++) {
        // cell origin o = origin + l*h, as space_init computes it
        const float oc = __fadd_rn(o3[k], __fmul_rn((float)ind[k], e3[k]));
        xrel[3 * i + k] = __fsub_rn(x[k], oc);
    }
    atomicAdd(&counts[c], 1);
}

__device__ __forceinline__ int na_block_scan(int v, int *tot) {
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

// Exclusive scan of in[0..n) into out[0..n], out[n] = total (three passes).
__global__ void k_na_scan_local(const int32_t *in, int n, int32_t *out, int32_t *sums) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int tot;
    int ex = na_block_scan(i < n ? in[i] : 0, &tot);
    if (i < n) out[i] = ex;
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void k_na_scan_sums(int32_t *sums, int nb) {
    const int per = (nb + blockDim.x - 1) / blockDim.x;
    const int b0 = threadIdx.x * per;
    int local = 0;
    for (int k = 0; k < per; k++) if (b0 + k < nb) local += sums[b0 + k];
    int run = na_block_scan(local, nullptr);
    for (int k = 0; k < per; k++)
        if (b0 + k < nb) {
            int s = sums[b0 + k];
            sums[b0 + k] = run;
            run += s;
        }
}

__global__ void k_na_scan_add(int32_t *out, const int32_t *sums, const int32_t *in, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        int s = out[i] + sums[blockIdx.x];
        out[i] = s;
        if (i == n - 1) out[n] = s + in[i];
    }
}

// Radix pass, step 1: how many elements of each tile carry each digit of the cell index.
// `src` is the order left by the previous pass (nullptr: the identity, particle index order).
__global__ void __launch_bounds__(kTile) k_na_radix_hist(int n, int ntiles, int shift, const int32_t *cell,
                                                         const int32_t *src, int32_t *hist) {
    __shared__ int h[kRadix];
    const int t = threadIdx.x, tile = blockIdx.x;
    if (t < kRadix) h[t] = 0;
    __syncthreads();
    const int e = tile * kTile + t;
    if (e < n) {
        const int v = src ? src[e] : e;
        atomicAdd(&h[(cell[v] >> shift) & (kRadix - 1)], 1);
    }
    __syncthreads();
    if (t < kRadix) hist[t * ntiles + tile] = h[t];
}

// Radix pass, step 2: stable scatter.  An element's destination is where its tile's run
// of its digit starts (hoff), plus the elements of that digit in earlier warps of the tile,
// plus those in earlier lanes of its own warp: the relative order of equal digits is kept.
__global__ void __launch_bounds__(kTile) k_na_radix_scatter(int n, int ntiles, int shift, const int32_t *cell,
                                                            const int32_t *src, const int32_t *hoff,
                                                            int32_t *dst) {
    __shared__ int wh[kTile / 32][kRadix];
    __shared__ int boff[kRadix];
    const int t = threadIdx.x, tile = blockIdx.x, w = t >> 5, lane = t & 31;
    for (int k = t; k < (kTile / 32) * kRadix; k += kTile) (&wh[0][0])[k] = 0;
    if (t < kRadix) boff[t] = hoff[t * ntiles + tile];
    __syncthreads();
    const int e = tile * kTile + t;
    const bool valid = e < n;
    int v = 0, d = kRadix;  // lanes past the end carry a digit no real element has
    if (valid) {
        v = src ? src[e] : e;
        d = (cell[v] >> shift) & (kRadix - 1);
    }
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int r = __popc(peers & ((1u << lane) - 1u));
    if (valid && r == 0) wh[w][d] = __popc(peers);
    __syncthreads();
    if (t < kRadix) {
        int run = 0;
        for (int k = 0; k < kTile / 32; k++) {
            const int c = wh[k][t];
            wh[k][t] = run;
            run += c;
        }
    }
    __syncthreads();
    if (valid) dst[boff[d] + wh[w][d] + r] = v;
}

// ---- device address of the scratch array, per CUDA context ----
typedef CUresult (*PfnCtxGetCurrent)(CUcontext *);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long *);

struct CtxScratch {
    unsigned long long ctx_id;  // cuCtxGetId: unique for the life of the process
    int32_t *ptr;
};
constexpr int kMaxContexts = 64;
std::mutex g_setup_mutex;
CtxScratch g_ctx[kMaxContexts] = {};
int g_nctx = 0, g_next_slot = 0;
bool g_entry_points_tried = false;
PfnCtxGetCurrent g_get_current = nullptr;
PfnCtxGetId g_get_id = nullptr;

bool current_context_id(unsigned long long *id) {
    if (!g_get_current || !g_get_id) return false;
    CUcontext ctx = nullptr;
    if (g_get_current(&ctx) != CUDA_SUCCESS || !ctx) return false;
    return g_get_id(ctx, id) == CUDA_SUCCESS;
}

// The scratch array's address in the calling thread's current context.  The first call
// in a context looks it up with cudaGetSymbolAddress (which also makes the device's
// primary context current when none is); later calls in that context reuse it.  Without
// the driver's context-id entry points every call looks the address up.
int scratch_for_current_context(int32_t **out) {
    std::lock_guard<std::mutex> g(g_setup_mutex);
    if (!g_entry_points_tried) {
        g_entry_points_tried = true;
        cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
        void *f1 = nullptr, *f2 = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
            q1 == cudaDriverEntryPointSuccess && q2 == cudaDriverEntryPointSuccess) {
            g_get_current = (PfnCtxGetCurrent)f1;
            g_get_id = (PfnCtxGetId)f2;
        }
    }
    unsigned long long id = 0;
    if (current_context_id(&id))
        for (int k = 0; k < g_nctx; k++)
            if (g_ctx[k].ctx_id == id) {
                *out = g_ctx[k].ptr;
                return TFG_OK;
            }
    int32_t *ptr = nullptr;
    if (cudaGetSymbolAddress((void **)&ptr, scratch) != cudaSuccess || !ptr) return TFG_E_CUDA;
    if (current_context_id(&id)) {
        // ids are never reused, so an entry of a destroyed context is only dead weight
        int slot = g_nctx < kMaxContexts ? g_nctx++ : (g_next_slot++ % kMaxContexts);
        g_ctx[slot] = {id, ptr};
    }
    *out = ptr;
    return TFG_OK;
}

template <typename... KArgs, typename... Args>
cudaError_t launch(void (*kernel)(KArgs...), int grid, int block, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.stream = s;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// Exclusive scan of in[0..n) into out[0..n] using the scratch's block sums.
cudaError_t scan(const int32_t *in, int n, int32_t *out, int32_t *sums, cudaStream_t s) {
    const int nb = (n + kScanBlock - 1) / kScanBlock;
    cudaError_t e = launch(k_na_scan_local, nb, kScanBlock, s, in, n, out, sums);
    if (e == cudaSuccess) e = launch(k_na_scan_sums, 1, kScanBlock, s, sums, nb);
    if (e == cudaSuccess) e = launch(k_na_scan_add, nb, kScanBlock, s, out, (const int32_t *)sums, in, n);
    return e;
}

}  // namespace

extern "C" TFG_API int tfg_bin_noalloc(const tfg_engine_desc *desc, int n, const float *x_dev, int32_t *cell_dev,
                                       float *xrel_dev, int32_t *order_dev, int32_t *cell_start_dev, void *stream) {
    if (!desc || n < 0) return TFG_E_INVAL;
    for (int k = 0; k < 3; k++)
        if (desc->cells[k] < 1 || !(desc->dim[k] > 0)) return TFG_E_INVAL;
    // sizes first, each axis on its own so that the product below cannot overflow:
    // requests beyond the static scratch are refused before anything runs
    for (int k = 0; k < 3; k++)
        if (desc->cells[k] > kNoAllocMaxCells) return TFG_E_OVERFLOW;
    const long long ncells = (long long)desc->cells[0] * desc->cells[1] * desc->cells[2];
    if (n > kNoAllocMaxParticles || ncells > kNoAllocMaxCells) return TFG_E_OVERFLOW;
    if ((n > 0 && (!x_dev || !cell_dev || !xrel_dev || !order_dev)) || !cell_start_dev) return TFG_E_INVAL;
    int32_t *base = nullptr;
    int rc = scratch_for_current_context(&base);
    if (rc != TFG_OK) return rc;
    int32_t *counts = base + kOffCounts, *hist = base + kOffHist, *hoff = base + kOffHoff, *ia = base + kOffA,
            *ib = base + kOffB, *sums = base + kOffSums;
    cudaStream_t s = (cudaStream_t)stream;
    const int nc = (int)ncells;

    // geometry exactly as engine creation and space_setpartp compute it
    float3 lo, hi, org, ih, h;
    float *plo = &lo.x, *phi = &hi.x, *porg = &org.x, *pih = &ih.x, *ph = &h.x;
    for (int k = 0; k < 3; k++) {
        const float o = desc->origin[k], dm = desc->dim[k];
        const float hk = dm / desc->cells[k];
        plo[k] = (float)(o * (1.0 + FLT_EPSILON));
        phi[k] = (float)((dm + o) * (1.0 - FLT_EPSILON));
        porg[k] = o;
        pih[k] = (float)(1.0 / hk);
        ph[k] = hk;
    }
    const int3 cdim = make_int3(desc->cells[0], desc->cells[1], desc->cells[2]);
    const int T = 256;
    cudaError_t e = launch(k_na_clear, (nc + T - 1) / T, T, s, counts, nc);
    if (e == cudaSuccess && n > 0)
        e = launch(k_na_setpartp, (n + T - 1) / T, T, s, n, x_dev, cdim, lo, hi, org, ih, h, cell_dev, xrel_dev,
                   counts);
    if (e == cudaSuccess) e = scan(counts, nc, cell_start_dev, sums, s);
    if (e == cudaSuccess && n > 0) {
        int bits = 0;
        while ((1LL << bits) < ncells) bits++;
        const int passes = bits > 8 ? (bits + 7) / 8 : 1;
        const int ntiles = (n + kTile - 1) / kTile;
        const int32_t *src = nullptr;  // the first pass starts from particle index order
        for (int p = 0; p < passes && e == cudaSuccess; p++) {
            int32_t *dst = p == passes - 1 ? order_dev : (p % 2 == 0 ? ia : ib);
            e = launch(k_na_radix_hist, ntiles, kTile, s, n, ntiles, 8 * p, (const int32_t *)cell_dev, src, hist);
            if (e == cudaSuccess) e = scan(hist, kRadix * ntiles, hoff, sums, s);
            if (e == cudaSuccess)
                e = launch(k_na_radix_scatter, ntiles, kTile, s, n, ntiles, 8 * p, (const int32_t *)cell_dev, src,
                           (const int32_t *)hoff, dst);
            src = dst;
        }
    }
    return e == cudaSuccess ? TFG_OK : TFG_E_CUDA;
}
