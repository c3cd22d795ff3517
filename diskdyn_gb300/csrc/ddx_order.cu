// Cell order of a set of bodies (no counterpart in the reference).  The mixed dust kernel
// reads its FP32 sources, and visits its tracers, in this order, so that the sources of a
// span of pair records and the tracers of a warp each lie in a small region, and a tracer
// far from a span can take the separation from the high parts alone.
//
// The order: the bodies' bounding box (in FP32), a cell per body on a 2^bits grid over it,
// and a code per cell that puts cells close on the curve close in space, in one of two forms:
//  - the Hilbert index on cubic cells (the box's largest extent cut into 2^bits on every
//    axis, so a thin disk is not cut into slabs), for DDX_PREC_MIXED.  Against the Morton
//    form the spans of 32 dusty-ring planetesimals shrank from a median radius of 37 AU to
//    12 AU, 89 % of the tracer-span pairs were far instead of 81 %, and the dust kernel went
//    from 8.02 to 7.75 ms (cubic Morton cells alone: 7.79 ms);
//  - the Morton code (x, y, z bits interleaved) on cells stretched to the box per axis, for
//    DDX_PREC_COMPENSATED.  Its longer spans take more sources into the float-float form per
//    span test: over 1,000 steps of four 16,384-grain shards its worst grains were 6.0e-10,
//    2.0e-9, 5.0e-10 and 4.7e-10 from FP64 at 24.8 ms a step, where the Hilbert order gave
//    1.5e-9, 1.9e-9, 6.3e-10 and 8.9e-10 at 21.8 ms, and needed the float-float radius doubled
//    (30.6 ms) to come to 8.6e-10, 1.8e-9, 8.6e-10 and 8.6e-10.
// The codes are sorted in one of two ways:
//  - counting sort (the tracers: 6 bits per axis): an atomic increment gives each body its
//    rank in its cell, an exclusive scan of the cell counts the cells' first positions, and
//    perm[start + rank] = body.  The order inside a cell follows the atomics, which is
//    fine for the tracers: each tracer's result depends on its own data and the sources;
//  - sorted by (code, index) (the sources: 5 bits per axis).  The sources' order is the
//    order of the FP32 sums over them, so it must not depend on timing: equal codes keep
//    their index order.  Up to 8,192 bodies one block does it all (box, keys, a bitonic sort
//    of code << 13 | index in shared memory, the slots), in one launch; beyond that a stable
//    LSD radix sort of (code, index) with 8-bit digits: per digit pass every block counts the
//    digits of its tile, digit-major; an exclusive scan gives every (digit, block) its first
//    output slot; the scatter ranks equal digits inside a warp with __match_any_sync and
//    orders warps and rounds by counts in shared memory.  Both give the same order.
#include "ddx_internal.cuh"
#include "ddx_scan.cuh"

namespace ddx {
namespace {

constexpr int kThreads = 256;
constexpr int kItems = 8;                       // keys per thread in a radix pass
constexpr int kSortTile = kThreads * kItems;

// Floats as ints with the same order (for atomicMin / atomicMax), and back.
__device__ __forceinline__ int ord_of(float f) {
    const int b = __float_as_int(f);
    return b >= 0 ? b : b ^ 0x7FFFFFFF;
}
__device__ __forceinline__ float float_of(int k) { return __int_as_float(k >= 0 ? k : k ^ 0x7FFFFFFF); }

__device__ __forceinline__ bool removed(const ddx_state& s, int i) {
    return (((unsigned long long)__double_as_longlong(s.N[i])) << 1) == 0ull;   // N == +-0
}

__global__ void order_init_kernel(uint32_t* __restrict__ count, int* __restrict__ box) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k <= kOrderBins) count[k] = 0;
    if (k < 3) {
        box[k] = ord_of(INFINITY);
        box[3 + k] = ord_of(-INFINITY);
    }
}

// Bounding box of the bodies' FP32 positions (NaN left out): a block reduction, then one
// atomic per block and bound.
__global__ void order_box_kernel(ddx_state s, int first, int n, bool dead_last, int* __restrict__ box) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    if (k < n && !(dead_last && removed(s, first + k))) {
        const float v[3] = {d2f_toward0(s.x[first + k]), d2f_toward0(s.y[first + k]), d2f_toward0(s.z[first + k])};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            lo[a] = fminf(lo[a], v[a]);
            hi[a] = fmaxf(hi[a], v[a]);
        }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
        }
    __shared__ float red[kThreads / 32][6];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0)
        for (int a = 0; a < 3; ++a) { red[warp][a] = lo[a]; red[warp][3 + a] = hi[a]; }
    __syncthreads();
    if (threadIdx.x < 6) {
        float v = red[0][threadIdx.x];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
            v = threadIdx.x < 3 ? fminf(v, red[w][threadIdx.x]) : fmaxf(v, red[w][threadIdx.x]);
        if (threadIdx.x < 3) atomicMin(&box[threadIdx.x], ord_of(v));
        else atomicMax(&box[threadIdx.x], ord_of(v));
    }
}

// Hilbert index (3 bits per level, most significant first) of cell c of a (1 << bits)^3
// grid: Skilling's transform of the axes to the transposed index ("Programming the Hilbert
// curve", AIP Conf. Proc. 707, 2004), then its bits interleaved.
__device__ __forceinline__ uint32_t hilbert_index(uint32_t c0, uint32_t c1, uint32_t c2, int bits) {
    uint32_t X[3] = {c0, c1, c2};
    const uint32_t M = 1u << (bits - 1);
    for (uint32_t Q = M; Q > 1; Q >>= 1) {   // inverse undo
        const uint32_t P = Q - 1;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            if (X[i] & Q) {
                X[0] ^= P;                      // invert
            } else {
                const uint32_t t = (X[0] ^ X[i]) & P;   // exchange
                X[0] ^= t;
                X[i] ^= t;
            }
        }
    }
    X[1] ^= X[0];                               // Gray encode
    X[2] ^= X[1];
    uint32_t t = 0;
    for (uint32_t Q = M; Q > 1; Q >>= 1)
        if (X[2] & Q) t ^= Q - 1;
    X[0] ^= t;
    X[1] ^= t;
    X[2] ^= t;
    uint32_t key = 0;
    for (int b = bits - 1; b >= 0; --b)
#pragma unroll
        for (int i = 0; i < 3; ++i) key = key << 1 | ((X[i] >> b) & 1u);
    return key;
}

__device__ __forceinline__ uint32_t spread3(uint32_t v) {   // bit b of v to bit 3b
    uint32_t r = 0;
#pragma unroll
    for (int b = 0; b < kOrderBits; ++b) r |= ((v >> b) & 1u) << (3 * b);
    return r;
}

// Code of the cell of v on a (1 << bits)^3 grid over the box [lo, hi]: hilbert, the Hilbert
// index on cubic cells (the largest extent sets the cell size on every axis); else the
// Morton code on cells stretched to the box per axis.
__device__ __forceinline__ uint32_t cell_code(const float* v, const float* lo, const float* hi, int bits,
                                              bool hilbert) {
    const int cells = 1 << bits;
    const float ext = fmaxf(fmaxf(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]);
    uint32_t c[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float e = hilbert ? ext : hi[a] - lo[a];
        const float scale = e > 0.0f ? (float)cells / e : 0.0f;
        // NaN, or a span too wide for FP32, gives cell 0 or the last: any cell is valid
        const float u = fminf(fmaxf((v[a] - lo[a]) * scale, 0.0f), (float)(cells - 1));
        c[a] = (uint32_t)(u == u ? (int)u : 0);
    }
    return hilbert ? hilbert_index(c[0], c[1], c[2], bits) : spread3(c[0]) << 2 | spread3(c[1]) << 1 | spread3(c[2]);
}

// The whole stable order of up to kSmallOrder bodies in one block.
constexpr int kSmallOrder = 8192;        // index < 2^13 below the 15-bit code + removed bit
constexpr int kSmallThreads = 1024;
__global__ void __launch_bounds__(kSmallThreads)
order_small_kernel(ddx_state s, int first, int n, bool dead_last, bool hilbert, int* __restrict__ perm,
                   int* __restrict__ inv) {
    __shared__ uint32_t keys[kSmallOrder];
    __shared__ float red[kSmallThreads / 32][6];
    __shared__ float box[6];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    constexpr int kBits = kOrderBits - 1;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int k = t; k < n; k += kSmallThreads) {
        if (dead_last && removed(s, first + k)) continue;
        const float v[3] = {d2f_toward0(s.x[first + k]), d2f_toward0(s.y[first + k]), d2f_toward0(s.z[first + k])};
#pragma unroll
        for (int a = 0; a < 3; ++a) { lo[a] = fminf(lo[a], v[a]); hi[a] = fmaxf(hi[a], v[a]); }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
        }
    if (lane == 0)
        for (int a = 0; a < 3; ++a) { red[warp][a] = lo[a]; red[warp][3 + a] = hi[a]; }
    __syncthreads();
    if (t < 6) {
        float v = red[0][t];
        for (int w = 1; w < kSmallThreads / 32; ++w) v = t < 3 ? fminf(v, red[w][t]) : fmaxf(v, red[w][t]);
        box[t] = v;
    }
    __syncthreads();
    int m = 1;
    while (m < n) m <<= 1;
    for (int k = t; k < m; k += kSmallThreads) {
        uint32_t key = 0xFFFFFFFFu;   // padding sorts last
        if (k < n) {
            uint32_t code = 1u << (3 * kBits);
            if (!(dead_last && removed(s, first + k))) {
                const float v[3] = {d2f_toward0(s.x[first + k]), d2f_toward0(s.y[first + k]),
                                    d2f_toward0(s.z[first + k])};
                code = cell_code(v, box, box + 3, kBits, hilbert);
            }
            key = code << 13 | (uint32_t)k;
        }
        keys[k] = key;
    }
    __syncthreads();
    // bitonic sort, ascending, of the m keys (all distinct)
    for (int size = 2; size <= m; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int i = t; i < m / 2; i += kSmallThreads) {
                const int a = 2 * i - (i & (stride - 1)), b = a + stride;
                const uint32_t ka = keys[a], kb = keys[b];
                if ((ka > kb) == ((a & size) == 0)) { keys[a] = kb; keys[b] = ka; }
            }
            __syncthreads();
        }
    for (int p = t; p < n; p += kSmallThreads) {
        const int k = (int)(keys[p] & 0x1FFFu);
        if (perm) perm[p] = k;
        if (inv) inv[k] = p;
    }
}

// Code of each body's cell (bits per axis; removed bodies get 1 << 3 bits when
// dead_last).  count given: rank[k] = the body's rank in its cell by an atomic increment;
// else rank[k] = k (the values of the stable sort).
__global__ void order_keys_kernel(ddx_state s, int first, int n, bool dead_last, int bits, bool hilbert,
                                  const int* __restrict__ box,
                                  uint32_t* __restrict__ key, uint32_t* __restrict__ rank,
                                  uint32_t* __restrict__ count) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    uint32_t bin = 1u << (3 * bits);
    if (!(dead_last && removed(s, first + k))) {
        const float v[3] = {d2f_toward0(s.x[first + k]), d2f_toward0(s.y[first + k]), d2f_toward0(s.z[first + k])};
        const float lo[3] = {float_of(box[0]), float_of(box[1]), float_of(box[2])};
        const float hi[3] = {float_of(box[3]), float_of(box[4]), float_of(box[5])};
        bin = cell_code(v, lo, hi, bits, hilbert);
    }
    key[k] = bin;
    rank[k] = count ? atomicAdd(&count[bin], 1u) : (uint32_t)k;
}

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

__global__ void radix_scatter_kernel(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin,
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

// Words of radix_sort_stable's scratch for n keys.
size_t radix_temp_words(int n) {
    const int nb = (n + kSortTile - 1) / kSortTile;
    const int nh = 256 * (nb > 0 ? nb : 1);
    return 2 * (size_t)nh + scan_temp_words(nh) + 2 * (size_t)n + 16;
}

// Stable ascending sort of (keys, vals) by the low key_bits bits of the keys; the result is
// in (keys, vals) or in the scratch, returned through *ko / *vo.
cudaError_t radix_sort_stable(uint32_t* keys, uint32_t* vals, int n, int key_bits, uint32_t* temp,
                              uint32_t** ko, uint32_t** vo, cudaStream_t st) {
    const int nb = (n + kSortTile - 1) / kSortTile;
    const int nh = 256 * nb;
    uint32_t* hist = temp;
    uint32_t* offs = hist + nh;
    uint32_t* stmp = offs + nh;
    uint32_t* k2 = stmp + scan_temp_words(nh);
    uint32_t* v2 = k2 + n;
    uint32_t *ka = keys, *va = vals, *kb = k2, *vb = v2;
    for (int shift = 0; shift < key_bits; shift += 8) {
        hist_kernel<<<nb, kThreads, 0, st>>>(ka, n, shift, hist, nb);
        const cudaError_t e = exclusive_scan(hist, offs, nh, stmp, nullptr, st);
        if (e != cudaSuccess) return e;
        radix_scatter_kernel<<<nb, kThreads, 0, st>>>(ka, va, kb, vb, n, shift, offs, nb);
        uint32_t* tk = ka; ka = kb; kb = tk;
        uint32_t* tv = va; va = vb; vb = tv;
    }
    *ko = ka;
    *vo = va;
    return cudaGetLastError();
}

__global__ void order_from_sorted_kernel(int n, const uint32_t* __restrict__ sorted, int* __restrict__ perm,
                                         int* __restrict__ inv) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const uint32_t k = sorted[p];
    if (perm) perm[p] = (int)k;
    if (inv) inv[k] = p;
}

__global__ void order_scatter_kernel(int n, const uint32_t* __restrict__ key, const uint32_t* __restrict__ rank,
                                     const uint32_t* __restrict__ start, int* __restrict__ perm,
                                     int* __restrict__ inv) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t pos = start[key[k]] + rank[k];
    if (perm) perm[pos] = k;
    if (inv) inv[k] = (int)pos;
}

}  // namespace

cudaError_t order_alloc(OrderScratch& o, int cap, bool stable) {
    OrderScratch n{};
    n.cap = cap;
    n.stable = stable;
    const size_t bins = kOrderBins + 1;
    const size_t tw = stable ? radix_temp_words(cap) : scan_temp_words((int)bins);
    if (cudaMalloc(&n.key, 4ull * cap) || cudaMalloc(&n.rank, 4ull * cap) || cudaMalloc(&n.perm, 4ull * cap) ||
        cudaMalloc(&n.count, 4 * bins) || cudaMalloc(&n.start, 4 * bins) || cudaMalloc(&n.temp, 4 * tw) ||
        cudaMalloc(&n.box, 6 * sizeof(int))) {
        order_free(n);
        return cudaErrorMemoryAllocation;
    }
    order_free(o);
    o = n;
    return cudaSuccess;
}

void order_free(OrderScratch& o) {
    cudaFree(o.key); cudaFree(o.rank); cudaFree(o.perm); cudaFree(o.count); cudaFree(o.start);
    cudaFree(o.temp); cudaFree(o.box);
    o = OrderScratch{};
}

cudaError_t order_bodies(const ddx_state& s, int first, int n, bool dead_last, const OrderScratch& o, int* perm,
                         int* inv, bool hilbert, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (n > o.cap) return cudaErrorInvalidValue;
    if (o.stable && n <= kSmallOrder) {
        order_small_kernel<<<1, kSmallThreads, 0, st>>>(s, first, n, dead_last, hilbert, perm, inv);
        return cudaGetLastError();
    }
    const int blk = (n + kThreads - 1) / kThreads;
    order_init_kernel<<<(kOrderBins + 1 + kThreads - 1) / kThreads, kThreads, 0, st>>>(o.count, o.box);
    order_box_kernel<<<blk, kThreads, 0, st>>>(s, first, n, dead_last, o.box);
    if (o.stable) {
        constexpr int kBits = kOrderBits - 1;   // 32^3 cells: two 8-bit digit passes
        order_keys_kernel<<<blk, kThreads, 0, st>>>(s, first, n, dead_last, kBits, hilbert, o.box, o.key, o.rank,
                                                    nullptr);
        uint32_t *ko = nullptr, *vo = nullptr;
        cudaError_t e = radix_sort_stable(o.key, o.rank, n, 3 * kBits + 1, o.temp, &ko, &vo, st);
        if (e != cudaSuccess) return e;
        order_from_sorted_kernel<<<blk, kThreads, 0, st>>>(n, vo, perm, inv);
        return cudaGetLastError();
    }
    order_keys_kernel<<<blk, kThreads, 0, st>>>(s, first, n, dead_last, kOrderBits, hilbert, o.box, o.key, o.rank,
                                                o.count);
    cudaError_t e = exclusive_scan(o.count, o.start, (int)kOrderBins + 1, o.temp, nullptr, st);
    if (e != cudaSuccess) return e;
    order_scatter_kernel<<<blk, kThreads, 0, st>>>(n, o.key, o.rank, o.start, perm, inv);
    return cudaGetLastError();
}

}  // namespace ddx
