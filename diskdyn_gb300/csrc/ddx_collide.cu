// Spatial-hash collision candidates (no counterpart in the reference, which has no
// collision detection).  Pair criterion: two live tracers i < j of [i0, i1) collide when
// (xj-xi)^2 + (yj-yi)^2 + (zj-zi)^2 < h^2, every operation rounded on its own (no FMA
// contraction), so the result is identical to a CPU brute force with the same expression.
//
//  1. keys    : cell = floor(x / cs) per axis with cs = 2h (1 + 1e-9) (decided in FP32
//               where that is certain, in FP64 near a cell edge), clamped to
//               +-(2^19 - 2) (clamping only merges far cells), and the half of the cell the
//               tracer lies in; the cell is hashed (the 32-bit finaliser of MurmurHash3 over
//               a linear form lin of the three 20-bit coordinates) into T = 2^k >= 2n buckets,
//               and an atomic increment of the bucket's size gives the tracer its rank in it;
//  2. starts  : an exclusive scan of the T bucket sizes gives every bucket its first slot;
//               the bucket table holds 16-byte entries {start, size, lin of the first two
//               tracers' cells} (equal cells have equal lin), so one load answers most
//               lookups;
//  3. scatter : every live tracer writes {x, y, z, cell id and halves} and its index to slot
//               start + rank; the tracers of rank 0 and 1 also their cells' lin to the
//               bucket's entry.  Steps 1-3 are a radix sort on the whole bucket id in one
//               pass (a counting sort): the bucket sizes are its histogram, the scan its
//               offsets;
//  4. count   : every tracer, in bucket order, visits the buckets of the 8 cells of its
//               octant: per axis its own cell and the neighbour on the side of the cell's
//               half it lies in (a partner closer than h cannot be further, because the cell
//               is 2h wide); on a clamped axis both neighbours.  It keeps the entries whose
//               cell id is that cell (hash collisions are filtered), j > i, and applies the
//               distance test, counting the partners and keeping the first kSlots of them.
//               Most neighbour cells are empty, and their bucket is then empty or holds one
//               or two tracers of other cells: the 8 bucket entries, loaded together, settle
//               those without touching the tracers (a lin that differs means another cell),
//               and only the rest are walked, shared out over the warp's lanes (a queue of
//               (tracer, cell) items per warp).  A test in FP32 with a proven margin rejects
//               the far candidates first; the FP64 test decides the rest (FP64 runs at 1/64
//               of the FP32 rate here, and a warp pays for it whenever any of its lanes
//               tests);
//  5. scan    : exclusive scan of the counts gives each tracer its output slot;
//  6. write   : each tracer writes its partners (the kept ones, or by walking again if it
//               has more than kSlots) ordered by j, so the list is ordered by (i, j).
// The order of the tracers inside a bucket depends on the atomics, but nothing written does:
// every tracer's partners are sorted by j, and a segment cut by the buffer's end keeps the
// smallest j, so the output is the first cap pairs of the ordered list.
#include "ddx_internal.cuh"
#include "ddx_scan.cuh"

namespace ddx {
namespace {

// Cell ids: offset coordinates u = c + 2^19 in 20-bit fields (x at bit 40, y at 20, z at 0);
// bits 60-62 hold the halves the tracer lies in (z, y, x), which are not part of the cell.
constexpr long long kCellLim = (1LL << 19) - 2;
constexpr uint32_t kOff = 1u << 19;
constexpr unsigned long long kIdMask = (1ull << 60) - 1;

// A tracer in bucket order: its position (copied bit for bit) and its cell id with halves,
// one 32-byte sector.
struct alignas(32) CellRec {
    double x, y, z;
    unsigned long long cell;
};

__device__ __forceinline__ unsigned long long pack_u(uint32_t ux, uint32_t uy, uint32_t uz) {
    return ((unsigned long long)ux << 40) | ((unsigned long long)uy << 20) | (unsigned long long)uz;
}
// Bucket of a cell: fmix32 of lin = ux * kHx + uy * kHy + uz * kHz (mod 2^32).  Cells whose
// forms coincide share a bucket, which the cell-id test separates.  lin is linear, so a
// neighbour's form is the cell's plus the offsets' (neighbour_lin).
constexpr uint32_t kHx = 0x9E3779B1u, kHy = 0x85EBCA77u, kHz = 0xC2B2AE3Du;
__device__ __forceinline__ uint32_t cell_lin(uint32_t ux, uint32_t uy, uint32_t uz) {
    return ux * kHx + uy * kHy + uz * kHz;
}
__device__ __forceinline__ uint32_t neighbour_lin(uint32_t lin, int dx, int dy, int dz) {
    return lin + (uint32_t)dx * kHx + (uint32_t)dy * kHy + (uint32_t)dz * kHz;
}
__device__ __forceinline__ uint32_t bucket_of(uint32_t h, uint32_t mask) {
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h & mask;
}
// Packed id of the neighbour (dx, dy, dz) of a cell: the fields are in [2, 2^20 - 2], so
// adding +-1 to each never carries into the next.
__device__ __forceinline__ unsigned long long neighbour_id(unsigned long long id, int dx, int dy, int dz) {
    return id + (unsigned long long)((long long)dx << 40) + (unsigned long long)((long long)dy << 20) +
           (unsigned long long)(long long)dz;
}
// Cell along one axis and the half the tracer lies in.  k = floor(x * 2/cs) is the half-cell
// index: x * (2/cs) is exactly twice the rounded x / cs (a power-of-two scale), so k >> 1 is
// floor(x / cs) and the low bit of k is the upper half.  The walk takes the cell itself and
// the neighbour on that side, or both neighbours on a clamped axis.  With cells 2h (1 + 1e-9)
// wide, the rounding of x / cs (below 1e-9 of a cell for |cell| < 2^19) cannot put a partner
// within h outside these cells.  The conversion saturates for huge or infinite x (clamped)
// and gives 0 for NaN, whose distance tests fail.
__device__ __forceinline__ float f32_trunc(double x);
__device__ __forceinline__ long long half_cell(double x, double inv2, float inv2f);
__device__ __forceinline__ uint32_t axis_cell(double x, double inv2, float inv2f, uint32_t& upper) {
    const long long k = half_cell(x, inv2, inv2f);
    long long c = k >> 1;
    upper = (uint32_t)(k & 1);
    if (c < -kCellLim) c = -kCellLim;
    if (c > kCellLim) c = kCellLim;
    return (uint32_t)(c + kOff);
}
// Neighbour offsets [lo, hi] along an axis from the cell's field u and the half bit.
__device__ __forceinline__ void axis_walk(uint32_t u, uint32_t upper, int& lo, int& hi) {
    if (u <= kOff - kCellLim || u >= kOff + kCellLim) {
        lo = -1;
        hi = 1;
    } else {
        lo = upper ? 0 : -1;
        hi = upper ? 1 : 0;
    }
}
// x rounded toward zero to float with integer operations only (no FP64 instruction): ±0
// below the float normals, ±inf above the float range or for inf and NaN.  The error is
// below 2^-23 |x| in the normal range.
__device__ __forceinline__ float f32_trunc(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
    const int e = (int)((b >> 52) & 0x7FF) - 1023;
    if (e < -126) return __uint_as_float(sign);
    if (e > 127) return __uint_as_float(sign | 0x7F800000u);
    return __uint_as_float(sign | ((uint32_t)(e + 127) << 23) | ((uint32_t)(b >> 29) & 0x7FFFFFu));
}

// floor(x * inv2) with the product rounded to FP64, as __double2ll_rd(x * inv2) gives it, from
// FP32 arithmetic where that is certain.  pf = trunc32(x) * RN32(inv2), rounded, is within
// (2^-23 + 2^-24 + 2^-24 + 2^-53)|x inv2| < 2^-21.9 |pf| of the FP64 product, so when the
// interval pf +- m, m = 2^-21 |pf| + 2^-100 (the absolute term covers float underflow and the
// sign of a tiny product), rounded (each end moves by at most half an ulp of pf, 2^-24 |pf|),
// lies inside one integer step, its floor is the FP64 product's.  Near an integer, beyond
// +-2^21 (where the cell clamps anyway), and for inf, NaN or an infinite inv2f the FP64 form
// decides.  On the dusty ring (about 1,300 half-cells from the star) about one axis in 800 is
// near an integer, so the FP64 pipe, 1/64 of the FP32 rate on this part, is almost idle.
__device__ __forceinline__ long long half_cell(double x, double inv2, float inv2f) {
    const float pf = __fmul_rn(f32_trunc(x), inv2f);
    const float m = __fmaf_rn(fabsf(pf), 0x1p-21f, 0x1p-100f);
    const int lo = __float2int_rd(__fsub_rn(pf, m)), hi = __float2int_rd(__fadd_rn(pf, m));
    if (lo == hi && fabsf(pf) < 0x1p21f) return lo;
    return __double2ll_rd(x * inv2);
}

__global__ void keys_kernel(ddx_state s, int i0, int n, double inv2, float inv2f, uint32_t mask, uint32_t sentinel,
                            uint32_t* __restrict__ bsize, uint32_t* __restrict__ bucket, uint32_t* __restrict__ rank,
                            unsigned long long* __restrict__ cellid, uint32_t* __restrict__ count) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int idx = i0 + p;
    // N == 0 (either sign) tested on the bits
    if ((((unsigned long long)__double_as_longlong(s.N[idx])) << 1) == 0ull) {
        bucket[p] = sentinel;
        count[p] = 0;
        return;
    }
    uint32_t hx, hy, hz;
    const uint32_t ux = axis_cell(s.x[idx], inv2, inv2f, hx);
    const uint32_t uy = axis_cell(s.y[idx], inv2, inv2f, hy);
    const uint32_t uz = axis_cell(s.z[idx], inv2, inv2f, hz);
    const uint32_t b = bucket_of(cell_lin(ux, uy, uz), mask);
    cellid[p] = pack_u(ux, uy, uz) | ((unsigned long long)(hx << 2 | hy << 1 | hz) << 60);
    bucket[p] = b;
    rank[p] = atomicAdd(&bsize[b], 1u);
}

__global__ void scatter_kernel(ddx_state s, int i0, int n, uint32_t sentinel, const uint32_t* __restrict__ bucket,
                               const uint32_t* __restrict__ rank, const unsigned long long* __restrict__ cellid,
                               uint4* table, CellRec* __restrict__ rec, uint32_t* __restrict__ vals) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const uint32_t b = bucket[p];
    if (b == sentinel) return;
    const uint32_t rk = rank[p];
    const uint32_t q = table[b].x + rk;   // plain load: other fields of the entry are written here
    const int idx = i0 + p;
    CellRec r;
    r.x = s.x[idx];
    r.y = s.y[idx];
    r.z = s.z[idx];
    r.cell = cellid[p];
    rec[q] = r;
    vals[q] = (uint32_t)p;
    if (rk < 2) {
        const unsigned long long id = r.cell & kIdMask;
        const uint32_t lin = cell_lin((uint32_t)(id >> 40) & 0xFFFFFu, (uint32_t)(id >> 20) & 0xFFFFFu,
                                      (uint32_t)id & 0xFFFFFu);
        if (rk == 0) table[b].z = lin;
        else table[b].w = lin;
    }
}

constexpr uint32_t kSlots = 4;   // partners kept per tracer by the count pass

// Inserts (i, j) into the ascending segment seg[0, filled) that holds at most k entries: while
// it has room the segment grows; when full, j replaces the largest entry if it is smaller.
__device__ __forceinline__ void keep_smallest(int2* seg, uint32_t& filled, uint32_t k, int i, int j) {
    long long b;
    if (filled < k) {
        b = filled++;
    } else {
        if (seg[k - 1].y <= j) return;
        b = (long long)k - 1;
    }
    while (b > 0 && seg[b - 1].y > j) {
        seg[b] = seg[b - 1];
        --b;
    }
    seg[b] = make_int2(i, j);
}

// The write pass: every tracer with partners writes them, ordered by j, to its segment of
// the list (offs: the scan of the counts), cut at cap.  The partners kept by the count pass
// are copied; a tracer with more than kSlots walks its octant again.  hf: h as a float,
// rounded up.
__global__ void write_kernel(const CellRec* __restrict__ rec, const uint32_t* __restrict__ vals,
                             const uint4* __restrict__ table, const uint32_t* __restrict__ n_live, int i0,
                             double h2, float hf, uint32_t mask, const uint32_t* __restrict__ count,
                             const int* __restrict__ slots, const uint32_t* __restrict__ offs,
                             int2* __restrict__ pairs, long long cap) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;   // bucket order
    if (q >= *n_live) return;
    const uint32_t p = vals[q];
    const int i = i0 + (int)p;
    const uint32_t cnt = count[p];
    const long long base = offs[p];
    if (cnt == 0 || base >= cap) return;
    const uint32_t k = (long long)cnt < cap - base ? cnt : (uint32_t)(cap - base);
    int2* seg = pairs + base;
    uint32_t filled = 0;
    if (cnt <= kSlots) {
        // the count pass kept all of this tracer's partners: no second walk
        for (uint32_t u = 0; u < cnt; ++u) keep_smallest(seg, filled, k, i, slots[(size_t)p * kSlots + u]);
        return;
    }
    const CellRec me = rec[q];
    const double xi = me.x, yi = me.y, zi = me.z;
    const unsigned long long id0 = me.cell & kIdMask;
    const uint32_t ux = (uint32_t)(id0 >> 40) & 0xFFFFFu, uy = (uint32_t)(id0 >> 20) & 0xFFFFFu,
                   uz = (uint32_t)id0 & 0xFFFFFu;
    int lx, hx, ly, hy, lz, hz;
    axis_walk(ux, (uint32_t)(me.cell >> 62) & 1u, lx, hx);
    axis_walk(uy, (uint32_t)(me.cell >> 61) & 1u, ly, hy);
    axis_walk(uz, (uint32_t)(me.cell >> 60) & 1u, lz, hz);
    const uint32_t lin0 = cell_lin(ux, uy, uz);
    // FP32 rejection: float copies (truncated) of both positions differ from the exact ones
    // by at most 2^-23 of their size, and a partner within h is no larger than M + h (M the
    // largest own coordinate), so the float separation is within 2^-20 (M + h) of the exact
    // one and its square below thr = (h + 2^-18 (M + h))^2 (1 + 2^-16) for every pair the
    // FP64 test accepts.  Used where no float overflows or underflows (M + h < 1e15,
    // h > 1e-12); elsewhere every candidate takes the FP64 test.
    const float fxi = f32_trunc(xi), fyi = f32_trunc(yi), fzi = f32_trunc(zi);
    const float M = fmaxf(fabsf(fxi), fmaxf(fabsf(fyi), fabsf(fzi)));
    const bool filter = M + hf < 1e15f && hf > 1e-12f;   // false for NaN
    const float reach = hf + (M + hf) * 0x1p-18f;
    const float thr = reach * reach * (1.0f + 0x1p-16f);
    // entries of bucket bk that lie in cell nid: j > i within h
    auto walk = [&](unsigned long long nid, uint4 bk) {
        for (uint32_t r = bk.x; r < bk.x + bk.y; ++r) {
            if (r == q) continue;
            const CellRec o = rec[r];
            if ((o.cell & kIdMask) != nid) continue;
            if (filter) {
                const float fx = f32_trunc(o.x) - fxi, fy = f32_trunc(o.y) - fyi, fz = f32_trunc(o.z) - fzi;
                if (fmaf(fx, fx, fmaf(fy, fy, fz * fz)) > thr) continue;
            }
            const uint32_t pj = vals[r];
            if (pj <= p) continue;
            const double ex = __dsub_rn(o.x, xi);
            const double ey = __dsub_rn(o.y, yi);
            const double ez = __dsub_rn(o.z, zi);
            const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez));
            if (d2 < h2) keep_smallest(seg, filled, k, i, i0 + (int)pj);
        }
    };
    if (hx - lx == 1 && hy - ly == 1 && hz - lz == 1) {
        // the usual octant of 8 cells, cell t at (lx + t/4, ly + t/2 % 2, lz + t % 2): walk only
        // the buckets with three or more tracers, or with one of the first two (other than this
        // tracer) in that cell
        const unsigned long long idl = neighbour_id(id0, lx, ly, lz);
        const uint32_t linl = neighbour_lin(lin0, lx, ly, lz);
        const int own = (lx ? 4 : 0) | (ly ? 2 : 0) | (lz ? 1 : 0);   // t of the tracer's cell
        uint32_t need = 0;
#pragma unroll
        for (int t = 0; t < 8; ++t) {
            const uint32_t nlin = neighbour_lin(linl, t >> 2, (t >> 1) & 1, t & 1);
            const uint4 e = table[bucket_of(nlin, mask)];
            const bool self0 = t == own && e.x == q, self1 = t == own && e.x + 1 == q;
            const bool hit = (e.y >= 1 && e.z == nlin && !self0) || (e.y >= 2 && e.w == nlin && !self1) || e.y >= 3;
            if (hit) need |= 1u << t;
        }
        while (need) {
            const int t = __ffs(need) - 1;
            need &= need - 1;
            const int dx = t >> 2, dy = (t >> 1) & 1, dz = t & 1;
            walk(neighbour_id(idl, dx, dy, dz), table[bucket_of(neighbour_lin(linl, dx, dy, dz), mask)]);
        }
    } else {
        for (int dx = lx; dx <= hx; ++dx)
            for (int dy = ly; dy <= hy; ++dy)
                for (int dz = lz; dz <= hz; ++dz)
                    walk(neighbour_id(id0, dx, dy, dz), table[bucket_of(neighbour_lin(lin0, dx, dy, dz), mask)]);
    }
}

// The count pass with the walks shared out over the warp.  Each tracer settles its octant's 8
// bucket entries as in write_kernel; the buckets left to walk go into a per-warp queue of
// (lane, cell) items, and the warp then walks 32 items at a time, each lane on one item with
// the owner's position and cell taken by shuffles, so the walks of one tracer no longer hold
// the other 31 lanes (about 0.45 walks per tracer on the dusty ring, up to eight on one lane).
// Partners are counted per owner in shared memory, and the first kSlots found are kept in the
// order the items run (the write pass sorts them).  A tracer on a clamped axis (more than 8
// cells) walks on its own lane.
constexpr int kCountThreads = 256;

__device__ __forceinline__ uint32_t warp_incl_sum(uint32_t v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    return v;
}

__global__ void __launch_bounds__(kCountThreads, 4) count_kernel(const CellRec* __restrict__ rec,
                                                              const uint32_t* __restrict__ vals,
                                                              const uint4* __restrict__ table,
                                                              const uint32_t* __restrict__ n_live, int i0, double h2,
                                                              float hf, uint32_t mask, uint32_t* __restrict__ count,
                                                              int* __restrict__ slots) {
    __shared__ uint8_t queue[kCountThreads / 32][256];
    __shared__ uint32_t found[kCountThreads];
    const uint32_t FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t q0 = blockIdx.x * blockDim.x + warp * 32;   // the warp's first slot
    const uint32_t q = q0 + lane;
    const uint32_t nl = *n_live;
    if (q0 >= nl) return;   // the whole warp: nothing to do
    const bool live = q < nl;
    uint32_t p = 0, linl = 0, need = 0, own_cnt = 0;
    unsigned long long idl = 0;
    double xi = 0.0, yi = 0.0, zi = 0.0;
    float fxi = 0.f, fyi = 0.f, fzi = 0.f, thr = 0.f;
    found[threadIdx.x] = 0;
    if (live) {
        p = vals[q];
        const CellRec me = rec[q];
        xi = me.x;
        yi = me.y;
        zi = me.z;
        const unsigned long long id0 = me.cell & kIdMask;
        const uint32_t ux = (uint32_t)(id0 >> 40) & 0xFFFFFu, uy = (uint32_t)(id0 >> 20) & 0xFFFFFu,
                       uz = (uint32_t)id0 & 0xFFFFFu;
        int lx, hx, ly, hy, lz, hz;
        axis_walk(ux, (uint32_t)(me.cell >> 62) & 1u, lx, hx);
        axis_walk(uy, (uint32_t)(me.cell >> 61) & 1u, ly, hy);
        axis_walk(uz, (uint32_t)(me.cell >> 60) & 1u, lz, hz);
        const uint32_t lin0 = cell_lin(ux, uy, uz);
        // FP32 rejection threshold as in write_kernel; +inf where the filter does not apply,
        // so that every candidate takes the FP64 test there
        fxi = f32_trunc(xi);
        fyi = f32_trunc(yi);
        fzi = f32_trunc(zi);
        const float M = fmaxf(fabsf(fxi), fmaxf(fabsf(fyi), fabsf(fzi)));
        const float reach = hf + (M + hf) * 0x1p-18f;
        thr = (M + hf < 1e15f && hf > 1e-12f) ? reach * reach * (1.0f + 0x1p-16f) : INFINITY;
        if (hx - lx == 1 && hy - ly == 1 && hz - lz == 1) {
            idl = neighbour_id(id0, lx, ly, lz);
            linl = neighbour_lin(lin0, lx, ly, lz);
            const int own = (lx ? 4 : 0) | (ly ? 2 : 0) | (lz ? 1 : 0);
#pragma unroll
            for (int t = 0; t < 8; ++t) {
                const uint32_t nlin = neighbour_lin(linl, t >> 2, (t >> 1) & 1, t & 1);
                const uint4 e = table[bucket_of(nlin, mask)];
                const bool self0 = t == own && e.x == q, self1 = t == own && e.x + 1 == q;
                const bool hit =
                    (e.y >= 1 && e.z == nlin && !self0) || (e.y >= 2 && e.w == nlin && !self1) || e.y >= 3;
                if (hit) need |= 1u << t;
            }
        } else {
            // a clamped axis: up to 27 cells, walked here
            for (int dx = lx; dx <= hx; ++dx)
                for (int dy = ly; dy <= hy; ++dy)
                    for (int dz = lz; dz <= hz; ++dz) {
                        const unsigned long long nid = neighbour_id(id0, dx, dy, dz);
                        const uint4 bk = table[bucket_of(neighbour_lin(lin0, dx, dy, dz), mask)];
                        for (uint32_t r = bk.x; r < bk.x + bk.y; ++r) {
                            if (r == q) continue;
                            const CellRec o = rec[r];
                            if ((o.cell & kIdMask) != nid) continue;
                            const float ex = f32_trunc(o.x) - fxi, ey = f32_trunc(o.y) - fyi,
                                        ez = f32_trunc(o.z) - fzi;
                            if (fmaf(ex, ex, fmaf(ey, ey, ez * ez)) > thr) continue;
                            const uint32_t pj = vals[r];
                            if (pj <= p) continue;
                            const double dx_ = __dsub_rn(o.x, xi), dy_ = __dsub_rn(o.y, yi), dz_ = __dsub_rn(o.z, zi);
                            const double d2 =
                                __dadd_rn(__dadd_rn(__dmul_rn(dx_, dx_), __dmul_rn(dy_, dy_)), __dmul_rn(dz_, dz_));
                            if (d2 < h2) {
                                if (own_cnt < kSlots) slots[(size_t)p * kSlots + own_cnt] = i0 + (int)pj;
                                ++own_cnt;
                            }
                        }
                    }
        }
    }
    // the warp's queue of (lane, cell) items
    const uint32_t nit = __popc(need);
    const uint32_t inc = warp_incl_sum(nit);
    const uint32_t total = __shfl_sync(FULL, inc, 31);
    {
        uint32_t pos = inc - nit, m = need;
        while (m) {
            const int t = __ffs(m) - 1;
            m &= m - 1;
            queue[warp][pos++] = (uint8_t)(lane << 3 | t);
        }
    }
    __syncwarp();
    for (uint32_t base = 0; base < total; base += 32) {
        const uint32_t g = base + lane;
        const uint32_t item = g < total ? queue[warp][g] : (uint32_t)(lane << 3);
        const int o = (int)(item >> 3), t = (int)(item & 7);
        const double oxi = __shfl_sync(FULL, xi, o), oyi = __shfl_sync(FULL, yi, o), ozi = __shfl_sync(FULL, zi, o);
        const float ofx = __shfl_sync(FULL, fxi, o), ofy = __shfl_sync(FULL, fyi, o), ofz = __shfl_sync(FULL, fzi, o);
        const float othr = __shfl_sync(FULL, thr, o);
        const uint32_t op = __shfl_sync(FULL, p, o), olinl = __shfl_sync(FULL, linl, o);
        const unsigned long long oidl = __shfl_sync(FULL, idl, o);
        if (g >= total) continue;
        const int dx = t >> 2, dy = (t >> 1) & 1, dz = t & 1;
        const unsigned long long nid = neighbour_id(oidl, dx, dy, dz);
        const uint4 bk = table[bucket_of(neighbour_lin(olinl, dx, dy, dz), mask)];
        const uint32_t oq = q0 + (uint32_t)o;
        for (uint32_t r = bk.x; r < bk.x + bk.y; ++r) {
            if (r == oq) continue;
            const CellRec c = rec[r];
            if ((c.cell & kIdMask) != nid) continue;
            const float ex = f32_trunc(c.x) - ofx, ey = f32_trunc(c.y) - ofy, ez = f32_trunc(c.z) - ofz;
            if (fmaf(ex, ex, fmaf(ey, ey, ez * ez)) > othr) continue;
            const uint32_t pj = vals[r];
            if (pj <= op) continue;
            const double dx_ = __dsub_rn(c.x, oxi), dy_ = __dsub_rn(c.y, oyi), dz_ = __dsub_rn(c.z, ozi);
            const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx_, dx_), __dmul_rn(dy_, dy_)), __dmul_rn(dz_, dz_));
            if (d2 < h2) {
                const uint32_t k = atomicAdd(&found[warp * 32 + o], 1u);
                if (k < kSlots) slots[(size_t)op * kSlots + k] = i0 + (int)pj;
            }
        }
    }
    __syncwarp();
    if (live) {
        // partners of a clamped-axis tracer were counted on its own lane (own_cnt), and it has
        // no queue items, so the two counts never share slots
        count[p] = found[threadIdx.x] + own_cnt;
    }
}

}  // namespace

struct CollideScratch {
    uint32_t *bucket = nullptr, *rank = nullptr, *count = nullptr, *offs = nullptr, *temp = nullptr,
             *total = nullptr;
    uint32_t *vals = nullptr, *bsize = nullptr;
    uint4* table = nullptr;
    int* slots = nullptr;
    unsigned long long* cellid = nullptr;
    CellRec* rec = nullptr;
    int n_cap = 0;
    uint32_t t_cap = 0;
};

void collide_free(CollideScratch*& c) {
    if (!c) return;
    cudaFree(c->table); cudaFree(c->bucket); cudaFree(c->rank); cudaFree(c->count); cudaFree(c->offs);
    cudaFree(c->temp); cudaFree(c->total); cudaFree(c->slots); cudaFree(c->cellid); cudaFree(c->vals); cudaFree(c->bsize);
    cudaFree(c->rec);
    delete c;
    c = nullptr;
}

int collide_run(CollideScratch*& cs, const ddx_state& s, int i0, int i1, double h, int2* pairs,
                long long cap, long long* n_pairs, cudaStream_t st) {
    const int n = i1 - i0;
    *n_pairs = 0;
    if (n <= 1) return DDX_OK;
    uint32_t T = 1024;   // buckets: at least 2n, at most 2^30 (one tracer per bucket at the limit)
    while (T < 2u * (uint32_t)n && T < (1u << 30)) T <<= 1;
    if (!cs) cs = new CollideScratch();
    if (cs->n_cap < n || cs->t_cap < T) {
        const int ncap = n > cs->n_cap ? n : cs->n_cap;
        const uint32_t tcap = T > cs->t_cap ? T : cs->t_cap;
        CollideScratch* nc = new CollideScratch();
        const size_t tw = scan_temp_words((int)tcap > ncap ? (int)tcap : ncap);
        if (cudaMalloc(&nc->table, 16ull * tcap) || cudaMalloc(&nc->bsize, 4ull * tcap) ||
            cudaMalloc(&nc->bucket, 4ull * ncap) ||
            cudaMalloc(&nc->rank, 4ull * ncap) || cudaMalloc(&nc->count, 4ull * ncap) ||
            cudaMalloc(&nc->offs, 4ull * ncap) || cudaMalloc(&nc->cellid, 8ull * ncap) ||
            cudaMalloc(&nc->vals, 4ull * ncap) ||
            cudaMalloc(&nc->rec, sizeof(CellRec) * (size_t)ncap) ||
            cudaMalloc(&nc->slots, 4ull * kSlots * ncap) || cudaMalloc(&nc->temp, 4ull * tw) ||
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
    const double inv2 = 2.0 * (1.0 / cell);
    const double h2 = h * h;
    float hf = (float)h;   // rounded up to a float
    if ((double)hf < h) hf = nextafterf(hf, INFINITY);
    const int thr = 256, blk = (n + thr - 1) / thr;
    uint32_t* n_live = cs->total;
    uint32_t* n_found = cs->total + 1;
    cudaMemsetAsync(cs->bsize, 0, 4ull * T, st);
    keys_kernel<<<blk, thr, 0, st>>>(s, i0, n, inv2, (float)inv2, mask, sentinel, cs->bsize, cs->bucket, cs->rank, cs->cellid,
                                     cs->count);
    // entries {start, size, lin of the first two cells (written by the scatter)}
    if (exclusive_scan_table(cs->bsize, cs->table, (int)T, cs->temp, n_live, st) != cudaSuccess) return DDX_ERR_CUDA;
    scatter_kernel<<<blk, thr, 0, st>>>(s, i0, n, sentinel, cs->bucket, cs->rank, cs->cellid, cs->table, cs->rec,
                                        cs->vals);
    count_kernel<<<(n + kCountThreads - 1) / kCountThreads, kCountThreads, 0, st>>>(
        cs->rec, cs->vals, cs->table, n_live, i0, h2, hf, mask, cs->count, cs->slots);
    if (exclusive_scan(cs->count, cs->offs, n, cs->temp, n_found, st) != cudaSuccess) return DDX_ERR_CUDA;
    if (pairs && cap > 0)
        write_kernel<<<blk, thr, 0, st>>>(cs->rec, cs->vals, cs->table, n_live, i0, h2, hf, mask, cs->count,
                                                cs->slots, cs->offs, pairs, cap);
    if (cudaGetLastError() != cudaSuccess) return DDX_ERR_CUDA;
    uint32_t tot = 0;
    if (cudaMemcpyAsync(&tot, n_found, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess) return DDX_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return DDX_ERR_CUDA;
    *n_pairs = tot;
    return DDX_OK;
}

}  // namespace ddx
