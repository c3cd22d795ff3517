// Device-wide primitives for the spatial-hash grid: a stable LSD radix sort of
// (32-bit key, 32-bit value) pairs and an exclusive scan of 32-bit counts.
//
// Radix sort, per 8-bit digit pass:
//   hist    : every block counts the digits of its tile of kSortTile keys and writes the
//             counts digit-major, hist[d * nblocks + b];
//   scan    : an exclusive scan of hist gives every (digit, block) its first output slot,
//             in digit order and, within a digit, in block order (so the pass is stable);
//   scatter : every block walks its tile again in kItems rounds of 256 keys; inside a round
//             __match_any_sync groups the lanes of a warp by digit, which gives each key
//             its rank among the equal digits of lower lanes; a per-(warp, digit) count in
//             shared memory, scanned over the warps and accumulated over the rounds, orders
//             the warps and the rounds.  Keys move in their original order within a digit.
#include "ddx_sort.cuh"

namespace ddx {
namespace {

constexpr int kThreads = 256;
constexpr int kItems = 8;
constexpr int kSortTile = kThreads * kItems;
constexpr int kScanTile = 1024;   // elements per block of the scan (256 threads x 4)

__global__ void hist_kernel(const uint32_t* __restrict__ keys, int n, int shift, uint32_t* __restrict__ hist,
                            int nblocks) {
    __shared__ uint32_t cnt[256];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const int base = blockIdx.x * kSortTile;
    for (int r = 0; r < kItems; ++r) {
        const int e = base + r * kThreads + threadIdx.x;
        if (e < n) atomicAdd(&cnt[(keys[e] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * nblocks + blockIdx.x] = cnt[threadIdx.x];
}

__global__ void scatter_kernel(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                               uint32_t* __restrict__ kout, uint32_t* __restrict__ vout, int n, int shift,
                               const uint32_t* __restrict__ offs, int nblocks) {
    __shared__ uint32_t wcnt[kThreads / 32][257];
    __shared__ uint32_t run[256];
    __shared__ uint32_t gofs[256];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    run[t] = 0;
    gofs[t] = offs[t * nblocks + blockIdx.x];
    for (int w = 0; w < kThreads / 32; ++w) wcnt[w][t] = 0;
    __syncthreads();
    const int base = blockIdx.x * kSortTile;
    for (int r = 0; r < kItems; ++r) {
        const int e = base + r * kThreads + t;
        const bool valid = e < n;
        uint32_t key = 0, val = 0, d = 256;
        if (valid) { key = kin[e]; val = vin[e]; d = (key >> shift) & 255u; }
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const unsigned rank = __popc(peers & ((1u << lane) - 1u));
        if (valid && rank == 0) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        {   // thread t owns digit t: exclusive offsets over the warps, then the running total
            uint32_t acc = run[t];
            for (int w = 0; w < kThreads / 32; ++w) {
                const uint32_t c = wcnt[w][t];
                wcnt[w][t] = acc;
                acc += c;
            }
            run[t] = acc;
        }
        __syncthreads();
        if (valid) {
            const uint32_t pos = gofs[d] + wcnt[warp][d] + rank;
            kout[pos] = key;
            vout[pos] = val;
        }
        __syncthreads();
        for (int w = 0; w < kThreads / 32; ++w) wcnt[w][t] = 0;
        __syncthreads();
    }
}

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

__global__ void scan_sums_kernel(const uint32_t* __restrict__ in, int n, uint32_t* __restrict__ sums) {
    const int base = blockIdx.x * kScanTile + threadIdx.x * 4;
    uint32_t s = 0;
    for (int k = 0; k < 4; ++k)
        if (base + k < n) s += in[base + k];
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

__global__ void scan_apply_kernel(const uint32_t* __restrict__ in, int n, const uint32_t* __restrict__ sums,
                                  uint32_t* __restrict__ out) {
    const int base = blockIdx.x * kScanTile + threadIdx.x * 4;
    uint32_t v[4], s = 0;
    for (int k = 0; k < 4; ++k) { v[k] = base + k < n ? in[base + k] : 0u; s += v[k]; }
    __shared__ uint32_t tot;
    uint32_t off = block_excl_scan(s, &tot) + sums[blockIdx.x];
    for (int k = 0; k < 4; ++k)
        if (base + k < n) { out[base + k] = off; off += v[k]; }
}

}  // namespace

size_t scan_temp_words(int n) { return (size_t)(n + kScanTile - 1) / kScanTile + 1; }

cudaError_t exclusive_scan(const uint32_t* in, uint32_t* out, int n, uint32_t* temp, uint32_t* total,
                           cudaStream_t st) {
    if (n <= 0) {
        return total ? cudaMemsetAsync(total, 0, sizeof(uint32_t), st) : cudaSuccess;
    }
    const int nb = (n + kScanTile - 1) / kScanTile;
    scan_sums_kernel<<<nb, kThreads, 0, st>>>(in, n, temp);
    scan_top_kernel<<<1, kThreads, 0, st>>>(temp, nb, total);
    scan_apply_kernel<<<nb, kThreads, 0, st>>>(in, n, temp, out);
    return cudaGetLastError();
}

size_t sort_temp_words(int n) {
    const int nb = (n + kSortTile - 1) / kSortTile;
    const int nh = 256 * (nb > 0 ? nb : 1);
    return 2 * (size_t)nh + scan_temp_words(nh) + 2 * (size_t)n + 16;
}

cudaError_t radix_sort_pairs(uint32_t* keys, uint32_t* vals, int n, int key_bits, uint32_t* temp,
                             cudaStream_t st) {
    if (n <= 1) return cudaSuccess;
    const int nb = (n + kSortTile - 1) / kSortTile;
    const int nh = 256 * nb;
    uint32_t* hist = temp;
    uint32_t* offs = hist + nh;
    uint32_t* stmp = offs + nh;
    uint32_t* k2 = stmp + scan_temp_words(nh);
    uint32_t* v2 = k2 + n;
    uint32_t *ka = keys, *va = vals, *kb = k2, *vb = v2;
    int passes = 0;
    for (int shift = 0; shift < key_bits; shift += 8, ++passes) {
        hist_kernel<<<nb, kThreads, 0, st>>>(ka, n, shift, hist, nb);
        cudaError_t e = exclusive_scan(hist, offs, nh, stmp, nullptr, st);
        if (e != cudaSuccess) return e;
        scatter_kernel<<<nb, kThreads, 0, st>>>(ka, va, kb, vb, n, shift, offs, nb);
        uint32_t* tk = ka; ka = kb; kb = tk;
        uint32_t* tv = va; va = vb; vb = tv;
    }
    if (passes & 1) {   // the result is in the temporary buffers; move it home
        cudaMemcpyAsync(keys, ka, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(vals, va, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, st);
    }
    return cudaGetLastError();
}

}  // namespace ddx
