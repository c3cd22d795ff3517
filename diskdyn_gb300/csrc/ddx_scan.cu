// Device-wide exclusive scan of 32-bit counts, in three launches: per-tile sums, one block
// scanning the tile sums, and the per-tile scan plus its offset.  The spatial-hash grid uses
// it for the bucket starts (the scan of the bucket sizes, written straight into the bucket
// table) and for the output slots of the pair list (the scan of the partner counts); the
// tracer order uses it for its cell starts.
//
// Item layout in a tile of 4,096 items: warp w owns items [512 w, 512 w + 512), and lane l of
// it holds, for k = 0..3, the four items at 512 w + 128 k + 4 l + e (e = 0..3).  Each load
// and store instruction of a warp then covers 512 contiguous bytes of the counts (one 16-byte
// vector per lane) or 2,048 contiguous bytes of the bucket table, every sector written in
// full.
#include "ddx_scan.cuh"

namespace ddx {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kTile = kThreads * 16;   // items per block

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    return v;
}

// First item of lane l's group k in the tile starting at t0.
__device__ __forceinline__ long long group_base(long long t0, int k) {
    return t0 + 512 * (threadIdx.x >> 5) + 128 * k + 4 * (threadIdx.x & 31);
}

// The lane's 16 items (0 past n); vec: in is 16-byte aligned.
__device__ __forceinline__ void load_items(const uint32_t* __restrict__ in, long long n, long long t0, bool vec,
                                           uint32_t v[16]) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const long long b = group_base(t0, k);
        if (vec && b + 3 < n) {
            const uint4 q = __ldg(reinterpret_cast<const uint4*>(in + b));
            v[4 * k] = q.x;
            v[4 * k + 1] = q.y;
            v[4 * k + 2] = q.z;
            v[4 * k + 3] = q.w;
        } else {
#pragma unroll
            for (int e = 0; e < 4; ++e) v[4 * k + e] = b + e < n ? in[b + e] : 0u;
        }
    }
}

__global__ void scan_sums_kernel(const uint32_t* __restrict__ in, long long n, bool vec, uint32_t* __restrict__ sums) {
    uint32_t v[16];
    load_items(in, n, (long long)blockIdx.x * kTile, vec, v);
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < 16; ++k) s += v[k];
    s = __reduce_add_sync(0xffffffffu, s);
    __shared__ uint32_t ws[kWarps];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
#pragma unroll
        for (int w = 0; w < kWarps; ++w) t += ws[w];
        sums[blockIdx.x] = t;
    }
}

// One block scans the tile sums (a sequential chunk per thread).
__global__ void scan_top_kernel(uint32_t* __restrict__ sums, int nb, uint32_t* __restrict__ total) {
    const int per = (nb + kThreads - 1) / kThreads;
    const int b0 = threadIdx.x * per;
    uint32_t s = 0;
    for (int k = 0; k < per; ++k)
        if (b0 + k < nb) s += sums[b0 + k];
    __shared__ uint32_t ws[kWarps];
    const uint32_t inc = warp_incl_scan(s);
    if ((threadIdx.x & 31) == 31) ws[threadIdx.x >> 5] = inc;
    __syncthreads();
    uint32_t off = inc - s;
    for (int w = 0; w < (int)(threadIdx.x >> 5); ++w) off += ws[w];
    for (int k = 0; k < per; ++k)
        if (b0 + k < nb) {
            const uint32_t x = sums[b0 + k];
            sums[b0 + k] = off;
            off += x;
        }
    if (threadIdx.x == kThreads - 1 && total) *total = off;
}

// TABLE: out holds 16-byte entries {start, size, 0, 0}; else out[i] = start (vec: out is
// 16-byte aligned).
template <bool TABLE>
__global__ void scan_apply_kernel(const uint32_t* __restrict__ in, long long n, bool vec,
                                  const uint32_t* __restrict__ sums, void* __restrict__ out) {
    const long long t0 = (long long)blockIdx.x * kTile;
    uint32_t v[16];
    load_items(in, n, t0, vec, v);
    // exclusive offsets of the lane's four groups within its warp
    uint32_t off[4], carry = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint32_t s = v[4 * k] + v[4 * k + 1] + v[4 * k + 2] + v[4 * k + 3];
        const uint32_t inc = warp_incl_scan(s);
        off[k] = carry + inc - s;
        carry += __shfl_sync(0xffffffffu, inc, 31);
    }
    __shared__ uint32_t ws[kWarps];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = carry;
    __syncthreads();
    uint32_t base = sums[blockIdx.x];
    for (int w = 0; w < (int)(threadIdx.x >> 5); ++w) base += ws[w];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const long long b = group_base(t0, k);
        uint32_t st[4];
        st[0] = base + off[k];
        st[1] = st[0] + v[4 * k];
        st[2] = st[1] + v[4 * k + 1];
        st[3] = st[2] + v[4 * k + 2];
        if (TABLE) {
            uint4* tab = static_cast<uint4*>(out);
#pragma unroll
            for (int e = 0; e < 4; ++e)
                if (b + e < n) tab[b + e] = make_uint4(st[e], v[4 * k + e], 0u, 0u);
        } else {
            uint32_t* o = static_cast<uint32_t*>(out);
            if (vec && b + 3 < n) {
                *reinterpret_cast<uint4*>(o + b) = make_uint4(st[0], st[1], st[2], st[3]);
            } else {
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (b + e < n) o[b + e] = st[e];
            }
        }
    }
}

bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

cudaError_t scan(const uint32_t* in, void* out, bool table, int n, uint32_t* temp, uint32_t* total,
                 cudaStream_t st) {
    if (n <= 0) return total ? cudaMemsetAsync(total, 0, sizeof(uint32_t), st) : cudaSuccess;
    const int nb = (n + kTile - 1) / kTile;
    const bool vin = aligned16(in);
    scan_sums_kernel<<<nb, kThreads, 0, st>>>(in, n, vin, temp);
    scan_top_kernel<<<1, kThreads, 0, st>>>(temp, nb, total);
    if (table)
        scan_apply_kernel<true><<<nb, kThreads, 0, st>>>(in, n, vin, temp, out);
    else
        scan_apply_kernel<false><<<nb, kThreads, 0, st>>>(in, n, vin && aligned16(out), temp, out);
    return cudaGetLastError();
}

}  // namespace

size_t scan_temp_words(int n) { return (size_t)(n + kTile - 1) / kTile + 1; }

cudaError_t exclusive_scan(const uint32_t* in, uint32_t* out, int n, uint32_t* temp, uint32_t* total,
                           cudaStream_t st) {
    return scan(in, out, false, n, temp, total, st);
}

cudaError_t exclusive_scan_table(const uint32_t* in, uint4* table, int n, uint32_t* temp, uint32_t* total,
                                 cudaStream_t st) {
    return scan(in, table, true, n, temp, total, st);
}

}  // namespace ddx
