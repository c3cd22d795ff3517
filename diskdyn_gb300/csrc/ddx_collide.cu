// Spatial-hash collision candidates (no counterpart in the reference, which has no
// collision detection).  Pair criterion: two live tracers i < j of [i0, i1) collide when
// (xj-xi)^2 + (yj-yi)^2 + (zj-zi)^2 < h^2, every operation rounded on its own (no FMA
// contraction), so the result is identical to a CPU brute force with the same expression.
//
//  1. keys   : cell = floor(x / cs) per axis with cs = 2h (1 + 1e-9), clamped to
//              +-(2^20 - 2) (clamping only merges far cells); the 63-bit cell id is hashed
//              (the 64-bit finaliser of MurmurHash3) into T = 2^k >= 2n buckets;
//  2. sort   : stable radix sort of (bucket, local index) (ddx_sort.cu);
//  3. ranges : first/last sorted position of every bucket;
//  4. count  : every tracer visits the buckets of the 8 cells of its octant: per axis its
//              own cell and the neighbour on the side of the cell's half it lies in (a
//              partner closer than h cannot be further, because the cell is 2h wide); on a
//              clamped axis both neighbours.  It keeps the entries whose cell id is that
//              cell (hash collisions are filtered), j > i, and applies the distance test,
//              counting the partners and keeping the first kSlots of them;
//  5. scan   : exclusive scan of the counts gives each tracer its output slot;
//  6. write  : each tracer writes its kept partners (or walks again, if it has more than
//              kSlots) as (i, j) and sorts its segment by j, so the list is ordered by (i, j).
#include "ddx_internal.cuh"
#include "ddx_sort.cuh"

namespace ddx {
namespace {

constexpr long long kCellLim = (1LL << 20) - 2;
constexpr unsigned long long kNoCell = ~0ull;

__host__ __device__ __forceinline__ unsigned long long pack_cell(long long cx, long long cy, long long cz) {
    const unsigned long long o = 1ull << 20;
    return ((unsigned long long)(cx + o) << 42) | ((unsigned long long)(cy + o) << 21) |
           (unsigned long long)(cz + o);
}
__device__ __forceinline__ void unpack_cell(unsigned long long id, long long& cx, long long& cy, long long& cz) {
    const long long o = 1LL << 20;
    cx = (long long)((id >> 42) & 0x1FFFFF) - o;
    cy = (long long)((id >> 21) & 0x1FFFFF) - o;
    cz = (long long)(id & 0x1FFFFF) - o;
}
__device__ __forceinline__ uint32_t bucket_of(unsigned long long k, uint32_t mask) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return (uint32_t)k & mask;
}
__device__ __forceinline__ long long cell_coord(double x, double inv) {
    double c = floor(x * inv);
    c = fmin(fmax(c, (double)-kCellLim), (double)kCellLim);
    return (long long)c;
}
// Neighbour offsets [lo, hi] along one axis: the cell itself and the neighbour on the side
// of the half the tracer lies in; both neighbours on a clamped axis.  With cells 2h (1 +
// 1e-9) wide, the rounding of x / cs (below 1e-9 of a cell for |cell| < 2^20) cannot put a
// partner within h outside these cells.
__device__ __forceinline__ void octant(double x, double inv, long long c, int& lo, int& hi) {
    if (c <= -kCellLim || c >= kCellLim) {
        lo = -1;
        hi = 1;
        return;
    }
    const double f = x * inv - (double)c;
    lo = f < 0.5 ? -1 : 0;
    hi = f < 0.5 ? 0 : 1;
}

__global__ void keys_kernel(ddx_state s, int i0, int n, double inv, uint32_t mask, uint32_t sentinel,
                            uint32_t* keys, uint32_t* vals, unsigned long long* cellid) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int idx = i0 + p;
    vals[p] = (uint32_t)p;
    if (s.N[idx] == 0.0) {
        keys[p] = sentinel;
        cellid[p] = kNoCell;
        return;
    }
    const unsigned long long id =
        pack_cell(cell_coord(s.x[idx], inv), cell_coord(s.y[idx], inv), cell_coord(s.z[idx], inv));
    cellid[p] = id;
    keys[p] = bucket_of(id, mask);
}

__global__ void ranges_kernel(const uint32_t* __restrict__ keys, int n, uint32_t sentinel,
                              uint32_t* __restrict__ start, uint32_t* __restrict__ end) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const uint32_t k = keys[q];
    if (k == sentinel) return;
    if (q == 0 || keys[q - 1] != k) start[k] = (uint32_t)q;
    if (q == n - 1 || keys[q + 1] != k) end[k] = (uint32_t)q + 1;
}

constexpr uint32_t kSlots = 4;   // partners kept per tracer by the count pass

template <bool WRITE>
__global__ void pairs_kernel(ddx_state s, int i0, int n, double h2, double inv, uint32_t mask, uint32_t sentinel,
                             const uint32_t* __restrict__ keys, const uint32_t* __restrict__ vals,
                             const unsigned long long* __restrict__ cellid, const uint32_t* __restrict__ start,
                             const uint32_t* __restrict__ end, uint32_t* __restrict__ count,
                             int* __restrict__ slots, const uint32_t* __restrict__ offs, int2* __restrict__ pairs,
                             long long cap) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;   // sorted order: neighbours share buckets
    if (q >= n) return;
    const uint32_t p = vals[q];
    if (keys[q] == sentinel) {
        if (!WRITE) count[p] = 0;
        return;
    }
    const int i = i0 + (int)p;
    const long long base = WRITE ? (long long)offs[p] : 0;
    if (WRITE && count[p] <= kSlots) {
        // the count pass kept this tracer's partners: no second walk
        const uint32_t cnt = count[p];
        for (uint32_t k = 0; k < cnt && base + k < cap; ++k) pairs[base + k] = make_int2(i, slots[(size_t)p * kSlots + k]);
        const long long last = base + cnt < cap ? base + cnt : cap;
        for (long long a = base + 1; a < last; ++a) {
            const int2 v = pairs[a];
            long long b = a - 1;
            while (b >= base && pairs[b].y > v.y) { pairs[b + 1] = pairs[b]; --b; }
            pairs[b + 1] = v;
        }
        return;
    }
    const double xi = s.x[i], yi = s.y[i], zi = s.z[i];
    long long cx, cy, cz;
    unpack_cell(cellid[p], cx, cy, cz);
    int lx, hx, ly, hy, lz, hz;
    octant(xi, inv, cx, lx, hx);
    octant(yi, inv, cy, ly, hy);
    octant(zi, inv, cz, lz, hz);
    uint32_t c = 0;
    for (int dx = lx; dx <= hx; ++dx)
        for (int dy = ly; dy <= hy; ++dy)
            for (int dz = lz; dz <= hz; ++dz) {
                const unsigned long long nid = pack_cell(cx + dx, cy + dy, cz + dz);
                const uint32_t b = bucket_of(nid, mask);
                const uint32_t r1 = end[b];
                for (uint32_t r = start[b]; r < r1; ++r) {
                    const uint32_t pj = vals[r];
                    if (pj <= p || cellid[pj] != nid) continue;
                    const int j = i0 + (int)pj;
                    const double ex = __dsub_rn(s.x[j], xi);
                    const double ey = __dsub_rn(s.y[j], yi);
                    const double ez = __dsub_rn(s.z[j], zi);
                    const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez));
                    if (d2 < h2) {
                        if (WRITE && base + c < cap) pairs[base + c] = make_int2(i, j);
                        if (!WRITE && c < kSlots) slots[(size_t)p * kSlots + c] = j;
                        ++c;
                    }
                }
            }
    if (!WRITE) {
        count[p] = c;
        return;
    }
    // order this tracer's partners by j (segments are short)
    const long long last = base + c < cap ? base + c : cap;
    for (long long a = base + 1; a < last; ++a) {
        const int2 v = pairs[a];
        long long b = a - 1;
        while (b >= base && pairs[b].y > v.y) { pairs[b + 1] = pairs[b]; --b; }
        pairs[b + 1] = v;
    }
}

}  // namespace

struct CollideScratch {
    uint32_t *keys = nullptr, *vals = nullptr, *start = nullptr, *end = nullptr, *count = nullptr,
             *offs = nullptr, *temp = nullptr, *total = nullptr;
    int* slots = nullptr;
    unsigned long long* cellid = nullptr;
    int n_cap = 0;
    uint32_t t_cap = 0;
};

void collide_free(CollideScratch*& c) {
    if (!c) return;
    cudaFree(c->keys); cudaFree(c->vals); cudaFree(c->start); cudaFree(c->end); cudaFree(c->count);
    cudaFree(c->offs); cudaFree(c->temp); cudaFree(c->total); cudaFree(c->cellid); cudaFree(c->slots);
    delete c;
    c = nullptr;
}

int collide_run(CollideScratch*& cs, const ddx_state& s, int i0, int i1, double h, int2* pairs,
                long long cap, long long* n_pairs, cudaStream_t st) {
    const int n = i1 - i0;
    *n_pairs = 0;
    if (n <= 1) return DDX_OK;
    uint32_t T = 1024;
    while (T < 2u * (uint32_t)n) T <<= 1;
    int tbits = 0;
    while ((1u << tbits) < T) ++tbits;
    if (!cs) cs = new CollideScratch();
    if (cs->n_cap < n || cs->t_cap < T) {
        const int ncap = n > cs->n_cap ? n : cs->n_cap;
        const uint32_t tcap = T > cs->t_cap ? T : cs->t_cap;
        CollideScratch* nc = new CollideScratch();
        const size_t tw = sort_temp_words(ncap) + scan_temp_words(ncap);
        if (cudaMalloc(&nc->keys, 4ull * ncap) || cudaMalloc(&nc->vals, 4ull * ncap) ||
            cudaMalloc(&nc->count, 4ull * ncap) || cudaMalloc(&nc->offs, 4ull * ncap) ||
            cudaMalloc(&nc->cellid, 8ull * ncap) || cudaMalloc(&nc->slots, 4ull * kSlots * ncap) ||
            cudaMalloc(&nc->start, 4ull * tcap) ||
            cudaMalloc(&nc->end, 4ull * tcap) || cudaMalloc(&nc->temp, 4ull * tw) ||
            cudaMalloc(&nc->total, 16)) {
            collide_free(nc);
            cudaGetLastError();
            return DDX_ERR_NOMEM;
        }
        nc->n_cap = ncap;
        nc->t_cap = tcap;
        collide_free(cs);
        cs = nc;
    }
    const uint32_t mask = T - 1, sentinel = T;
    const double cell = 2.0 * h * (1.0 + 1e-9);
    const double inv = 1.0 / cell;
    const double h2 = h * h;
    const int thr = 256, blk = (n + thr - 1) / thr;
    keys_kernel<<<blk, thr, 0, st>>>(s, i0, n, inv, mask, sentinel, cs->keys, cs->vals, cs->cellid);
    if (radix_sort_pairs(cs->keys, cs->vals, n, tbits + 1, cs->temp, st) != cudaSuccess) return DDX_ERR_CUDA;
    cudaMemsetAsync(cs->start, 0, 4ull * T, st);
    cudaMemsetAsync(cs->end, 0, 4ull * T, st);
    ranges_kernel<<<blk, thr, 0, st>>>(cs->keys, n, sentinel, cs->start, cs->end);
    pairs_kernel<false><<<blk, thr, 0, st>>>(s, i0, n, h2, inv, mask, sentinel, cs->keys, cs->vals, cs->cellid,
                                             cs->start, cs->end, cs->count, cs->slots, nullptr, nullptr, 0);
    uint32_t* scan_temp = cs->temp + sort_temp_words(cs->n_cap);
    if (exclusive_scan(cs->count, cs->offs, n, scan_temp, cs->total, st) != cudaSuccess) return DDX_ERR_CUDA;
    if (pairs && cap > 0)
        pairs_kernel<true><<<blk, thr, 0, st>>>(s, i0, n, h2, inv, mask, sentinel, cs->keys, cs->vals, cs->cellid,
                                                cs->start, cs->end, cs->count, cs->slots, cs->offs, pairs, cap);
    if (cudaGetLastError() != cudaSuccess) return DDX_ERR_CUDA;
    uint32_t tot = 0;
    if (cudaMemcpyAsync(&tot, cs->total, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess) return DDX_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return DDX_ERR_CUDA;
    *n_pairs = tot;
    return DDX_OK;
}

}  // namespace ddx
