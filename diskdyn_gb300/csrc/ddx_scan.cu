// Device-wide exclusive scan of 32-bit counts, in three launches: per-tile sums, one block
// scanning the tile sums, and the per-tile scan plus its offset.  The spatial-hash grid uses
// it for the bucket starts (the scan of the bucket sizes) and for the output slots of the
// pair list (the scan of the partner counts).
#include "ddx_scan.cuh"

namespace ddx {
namespace {

constexpr int kThreads = 256;
constexpr int kScanTile = 1024;   // elements per block of the scan (256 threads x 4)

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    return v;
}

// Block-wide exclusive scan of one value per thread; returns the block total in *total.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* total) {
    __shared__ uint32_t ws[kThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t inc = warp_incl_scan(v);
    if (lane == 31) ws[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const uint32_t x = lane < kThreads / 32 ? ws[lane] : 0u;
        const uint32_t y = warp_incl_scan(x);
        if (lane < kThreads / 32) ws[lane] = y - x;
        if (lane == kThreads / 32 - 1) *total = y;
    }
    __syncthreads();
    const uint32_t r = ws[warp] + inc - v;
    __syncthreads();
    return r;
}

// Element k of a strided array: a[k * stride].
__global__ void scan_sums_kernel(const uint32_t* __restrict__ in, int is, int n, uint32_t* __restrict__ sums) {
    const int base = blockIdx.x * kScanTile + threadIdx.x * 4;
    uint32_t s = 0;
    for (int k = 0; k < 4; ++k)
        if (base + k < n) s += in[(size_t)(base + k) * is];
    __shared__ uint32_t tot;
    block_excl_scan(s, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

// One block scans the block sums (sequential chunks per thread).
__global__ void scan_top_kernel(uint32_t* __restrict__ sums, int nb, uint32_t* __restrict__ total) {
    const int per = (nb + kThreads - 1) / kThreads;
    const int b0 = threadIdx.x * per;
    uint32_t s = 0;
    for (int k = 0; k < per; ++k)
        if (b0 + k < nb) s += sums[b0 + k];
    __shared__ uint32_t tot;
    uint32_t off = block_excl_scan(s, &tot);
    for (int k = 0; k < per; ++k)
        if (b0 + k < nb) { const uint32_t x = sums[b0 + k]; sums[b0 + k] = off; off += x; }
    if (threadIdx.x == 0 && total) *total = tot;
}

__global__ void scan_apply_kernel(const uint32_t* __restrict__ in, int is, int n, const uint32_t* __restrict__ sums,
                                  uint32_t* __restrict__ out, int os, uint32_t* __restrict__ copy) {
    const int base = blockIdx.x * kScanTile + threadIdx.x * 4;
    uint32_t v[4], s = 0;
    for (int k = 0; k < 4; ++k) { v[k] = base + k < n ? in[(size_t)(base + k) * is] : 0u; s += v[k]; }
    __shared__ uint32_t tot;
    uint32_t off = block_excl_scan(s, &tot) + sums[blockIdx.x];
    for (int k = 0; k < 4; ++k)
        if (base + k < n) {
            out[(size_t)(base + k) * os] = off;
            if (copy) copy[(size_t)(base + k) * os] = v[k];
            off += v[k];
        }
}

}  // namespace

size_t scan_temp_words(int n) { return (size_t)(n + kScanTile - 1) / kScanTile + 1; }

cudaError_t exclusive_scan_strided(const uint32_t* in, int is, uint32_t* out, int os, int n, uint32_t* temp,
                                   uint32_t* total, cudaStream_t st, uint32_t* copy) {
    if (n <= 0) {
        return total ? cudaMemsetAsync(total, 0, sizeof(uint32_t), st) : cudaSuccess;
    }
    const int nb = (n + kScanTile - 1) / kScanTile;
    scan_sums_kernel<<<nb, kThreads, 0, st>>>(in, is, n, temp);
    scan_top_kernel<<<1, kThreads, 0, st>>>(temp, nb, total);
    scan_apply_kernel<<<nb, kThreads, 0, st>>>(in, is, n, temp, out, os, copy);
    return cudaGetLastError();
}

cudaError_t exclusive_scan(const uint32_t* in, uint32_t* out, int n, uint32_t* temp, uint32_t* total,
                           cudaStream_t st) {
    return exclusive_scan_strided(in, 1, out, 1, n, temp, total, st, nullptr);
}

}  // namespace ddx
