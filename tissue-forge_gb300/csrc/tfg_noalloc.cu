// Cell binning that allocates nothing.
//
// Some callers of this library cannot allocate device memory: code that runs inside a
// CUDA graph being captured by someone else, plugins handed a fixed memory pool by their
// host application, or real-time loops where a cudaMalloc/cudaFree would stall the whole
// device.  tfg_bin_noalloc gives them the cell binning of an engine load (the reference's
// space_setpartp, source/mdcore/src/tfSpace.cpp:432-475, followed by a counting sort into
// cell order) with every temporary buffer taken from one statically allocated device
// array instead of cudaMalloc.
//
// The scratch array below is a file-scope __device__ variable: every GPU that loads this
// library holds it (TFG_NOALLOC_SCRATCH_BYTES) until the process exits.  Its host-side
// name is only a stand-in for the device variable, so host code never passes `scratch`
// to a kernel; the device address is looked up once per device with
// cudaGetSymbolAddress (with that device current) on the first call made on it.
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
constexpr int kMaxScanBlocks = (kNoAllocMaxCells + kScanBlock - 1) / kScanBlock;

// Layout of the scratch array, in 32-bit words:
//   counts   [kNoAllocMaxCells]     particles per cell (must start at zero every call)
//   lidx     [kNoAllocMaxParticles] arrival index of each particle inside its cell
//   unsorted [kNoAllocMaxParticles] particle indices placed by cell, unordered in a cell
//   sums     [kMaxScanBlocks]       per-block totals of the cell-count scan
constexpr size_t kOffCounts = 0;
constexpr size_t kOffLidx = kOffCounts + kNoAllocMaxCells;
constexpr size_t kOffUnsorted = kOffLidx + kNoAllocMaxParticles;
constexpr size_t kOffSums = kOffUnsorted + kNoAllocMaxParticles;
constexpr size_t kScratchWords = kOffSums + kMaxScanBlocks;
static_assert(kScratchWords * 4 == TFG_NOALLOC_SCRATCH_BYTES, "scratch size must match the header");

static __device__ __align__(256) int32_t scratch[kScratchWords];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
int32_t *g_scratch_ptr[kMaxDevices] = {};

__global__ void k_na_clear(int32_t *counts, int ncells) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ncells) counts[i] = 0;
}

// space_setpartp: clamp into the domain, bin, make the position cell-relative; count.
__global__ void k_na_setpartp(int n, const float *__restrict__ xg, int3 cdim, float3 lo, float3 hi, float3 org,
                              float3 ih, float3 h, int32_t *cell, float *xrel, int32_t *counts, int32_t *lidx) {
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
    lidx[i] = atomicAdd(&counts[c], 1);
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

__global__ void k_na_scan_local(const int32_t *counts, int n, int32_t *start, int32_t *sums) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int tot;
    int ex = na_block_scan(i < n ? counts[i] : 0, &tot);
    if (i < n) start[i] = ex;
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

__global__ void k_na_scan_add(int32_t *start, const int32_t *sums, const int32_t *counts, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        int s = start[i] + sums[blockIdx.x];
        start[i] = s;
        if (i == n - 1) start[n] = s + counts[i];
    }
}

__global__ void k_na_place(int n, const int32_t *cell, const int32_t *lidx, const int32_t *start, int32_t *unsorted) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsorted[start[cell[i]] + lidx[i]] = i;
}

// Order each cell by particle index (one warp per cell), the order an engine load uses.
__global__ void k_na_rank(int ncells, const int32_t *start, const int32_t *unsorted, int32_t *order) {
    int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (w >= ncells) return;
    const int s0 = start[w], s1 = start[w + 1];
    for (int e = s0 + lane; e < s1; e += 32) {
        const int my = unsorted[e];
        int r = 0;
        for (int o = s0; o < s1; o++) r += unsorted[o] < my;
        order[s0 + r] = my;
    }
}

// Device address of the scratch array on the current device; set up once per device.
int scratch_for_device(int32_t **out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return TFG_E_CUDA;
    std::lock_guard<std::mutex> g(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
        int32_t *ptr = nullptr;
        if (cudaGetSymbolAddress((void **)&ptr, scratch) != cudaSuccess || !ptr) return TFG_E_CUDA;
        g_scratch_ptr[dev] = ptr;
    }
    *out = g_scratch_ptr[dev];
    return TFG_OK;
}

}  // namespace

extern "C" TFG_API int tfg_bin_noalloc(const tfg_engine_desc *desc, int n, const float *x_dev, int32_t *cell_dev,
                                       float *xrel_dev, int32_t *order_dev, int32_t *cell_start_dev, void *stream) {
    if (!desc || n < 0) return TFG_E_INVAL;
    for (int k = 0; k < 3; k++)
        if (desc->cells[k] < 1 || !(desc->dim[k] > 0)) return TFG_E_INVAL;
    const long long ncells = (long long)desc->cells[0] * desc->cells[1] * desc->cells[2];
    // sizes first: requests beyond the static scratch are refused before anything runs
    if (n > kNoAllocMaxParticles || ncells > kNoAllocMaxCells) return TFG_E_OVERFLOW;
    if ((n > 0 && (!x_dev || !cell_dev || !xrel_dev || !order_dev)) || !cell_start_dev) return TFG_E_INVAL;
    int32_t *base = nullptr;
    int rc = scratch_for_device(&base);
    if (rc != TFG_OK) return rc;
    int32_t *counts = base + kOffCounts, *lidx = base + kOffLidx, *unsorted = base + kOffUnsorted,
            *sums = base + kOffSums;
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
    k_na_clear<<<(nc + T - 1) / T, T, 0, s>>>(counts, nc);
    if (n > 0)
        k_na_setpartp<<<(n + T - 1) / T, T, 0, s>>>(n, x_dev, cdim, lo, hi, org, ih, h, cell_dev, xrel_dev, counts,
                                                    lidx);
    const int nbs = (nc + kScanBlock - 1) / kScanBlock;
    k_na_scan_local<<<nbs, kScanBlock, 0, s>>>(counts, nc, cell_start_dev, sums);
    k_na_scan_sums<<<1, kScanBlock, 0, s>>>(sums, nbs);
    k_na_scan_add<<<nbs, kScanBlock, 0, s>>>(cell_start_dev, sums, counts, nc);
    if (n > 0) {
        k_na_place<<<(n + T - 1) / T, T, 0, s>>>(n, cell_dev, lidx, cell_start_dev, unsorted);
        k_na_rank<<<(int)(((long long)nc * 32 + T - 1) / T), T, 0, s>>>(nc, cell_start_dev, unsorted, order_dev);
    }
    return cudaGetLastError() == cudaSuccess ? TFG_OK : TFG_E_CUDA;
}
