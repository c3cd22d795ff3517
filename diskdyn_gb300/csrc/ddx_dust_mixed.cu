// Mixed-precision RK4 of the dust tracers on sm_103a (src/gpu_functions.cu:627-943).
//
// FP64: tracer state, stage positions and velocities, the star term (reduced gravity,
// PR + stellar-wind drag, Lorentz force), the gravity of the planets (bodies
// 1..n_exact-1) and the RK4 combination.  FP32: the gravity of the planetesimals, on
// hi/lo split positions so the separation keeps FP32 relative precision at any distance
// from the star, with plain sums over spans of 16 pair records (32 sources, one sum per
// lane of the f32x2 pair) and one FP32 Kahan sum of each span's two lanes across spans.
//
// Far spans.  The low parts matter only for sources near the tracer: for a source at
// distance r >= X/4 (X the largest |coordinate| of the two), the high parts alone give the
// separation within e = (2 sqrt(3) 2^-22 + 2^-24) r = 8.9e-7 r, and the source's pull
// within 4e (direction and r^-3), a few times the 5.6e-7 that rsqrt.approx and FP32
// rounding leave in every pull; over 1,000 steps of the dusty ring the position errors
// against FP64 did not move (from X/2 to X/4 neither).  So a tracer takes a span with the
// high-part separation (3 of the 9 separation operations) when the span's box (high parts
// of its 32 sources) lies at least X/4 from the tracer's own point, X over the box and the
// point.  The choice depends
// on the tracer and the sources alone, so a tracer's result does not depend on the others
// or on their order.  The tracers are visited in cell order and the sources sit in their
// pair records in cell order (ddx_order.cu), so the lanes of a warp lie close together and
// nearly always make the same choice for a span; per stage the block settles most spans for
// all its tracers at once from its own box (tests whose outcome implies each tracer's), and
// the lanes test only the rest.  This runs from kOrderMinSources planetesimals on; with
// fewer, every span takes the full separation in index order.
//
// Blackwell mapping:
//  - perturbers arrive as 64-byte pair records (two bodies per record, one quantity of
//    both bodies per 8-byte slot), and every FP32 operation of the pair force runs as one
//    f32x2 instruction (add/sub/mul/fma.rn.f32x2) on both bodies, halving the issue
//    slots of the FP32 work; what bounds the kernel now is the latency of the rsqrt.approx
//    and shared-memory results, hence four blocks per SM;
//  - the pair records of all four stages stream through two shared-memory tiles filled
//    by TMA bulk copies (cp.async.bulk ... mbarrier::complete_tx), so tile k+1 lands while
//    tile k is consumed; every thread of the block reads the same record (broadcast);
//  - each mbarrier wait is bounded by the global timer; a block that gives up sets the
//    context's status word, waits (bounded) for its own copies, leaves its tracers
//    untouched and exits.
//
// Near sources.  FP32 leaves about 5.6e-7 of relative error in every pull, which a close
// encounter amplifies: over 1,000 steps of the dusty ring the worst grains ended 1e-8 from
// their FP64 positions while the median stayed at 3e-11.  So a source nearer to the tracer
// than near_eta times the tracer's largest |coordinate| takes the FP64 pair force from the
// FP64 stage positions instead (the FP64 step's arithmetic).  The loop over a span of 32
// sources keeps the largest FP32 reciprocal distance (one three-input max per pair
// record); a span whose largest exceeds 1 / (near_eta own) is summed again without its
// near sources, which are added in FP64.  Far spans hold no source nearer than the near
// radius (near_eta is at most a quarter, and far spans start a quarter of the largest
// coordinate away).
//
// Compensated variant (DDX_PREC_COMPENSATED).  The near radius does not bound the largest
// errors: in this chaotic system a grain amplifies the FP32 rounding of every planetesimal
// pull within tens of AU by three to four orders of magnitude over 1,000 steps.  So spans
// nearer to the tracer than comp_eta times its largest |coordinate| are evaluated in
// float-float arithmetic: each quantity is an unevaluated sum hi + lo of two FP32 numbers,
// carried through error-free transformations (TwoSum; products split by FMA) and one
// Newton step of the reciprocal square root on the float-float square distance, with the
// masses in two parts as well.  That keeps about 44 bits of each pull, against 22 or so in
// FP32, for about ten times the FP32 operations of a pair; farther spans take the FP32
// forms.  The hi + lo positions themselves hold 48 bits, so sources within the near radius
// still take the exact FP64 pull inside those spans.  The per-span choice is made like the
// far-span choice (block box first, then per tracer), so a tracer's result again depends
// only on its own state and the massive set.
#include "ddx_internal.cuh"
#include "ddx_f32x2.cuh"

namespace ddx {
namespace {

constexpr int kThreads = 256;
constexpr int kTilePairs = 256;                 // pair records per tile (16 KiB)

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t; asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t)); return t;
}
__device__ __forceinline__ void mbar_init(uint32_t mb, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(mb), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t mb, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(mb), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, unsigned bytes, uint32_t mb) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(dst), "l"(src), "r"(bytes), "r"(mb) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t mb, unsigned parity) {
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n}" : "=r"(ok) : "r"(mb), "r"(parity) : "memory");
    return ok != 0;
}
// Wait for phase `parity` of the mbarrier to complete, for at most limit_ns.
__device__ __forceinline__ bool mbar_wait(uint32_t mb, unsigned parity, unsigned long long limit_ns) {
    if (mbar_try(mb, parity)) return true;
    const unsigned long long t0 = global_ns();
    while (!mbar_try(mb, parity))
        if (global_ns() - t0 > limit_ns) return false;
    return true;
}

// ---- float-float pulls (compensated variant) -------------------------------------------
__device__ __forceinline__ f2 neg2(f2 a) { return a ^ 0x8000000080000000ull; }
// s + e == a + b exactly (Knuth's TwoSum, no ordering needed)
__device__ __forceinline__ void two_sum2(f2 a, f2 b, f2& s, f2& e) {
    s = add2(a, b);
    const f2 v = sub2(s, a);
    e = add2(sub2(a, sub2(s, v)), sub2(b, v));
}
// One coordinate of source - tracer as an unnormalised pair h + l: h = fp32(a - A), l = the
// rounding error of that difference (TwoSum) plus the difference of the low parts.
__device__ __forceinline__ void sep_ff(f2 a, f2 la, f2 A, f2 LA, f2& h, f2& l) {
    h = sub2(a, A);
    const f2 v = sub2(h, a);
    l = add2(sub2(la, LA), sub2(sub2(a, sub2(h, v)), add2(A, v)));
}
// (h + l)^2 = p + e: p = fp32(h^2), e = (h^2 - p) + 2 h l + l^2
__device__ __forceinline__ void sq_ff(f2 h, f2 l, f2& p, f2& e) {
    p = mul2(h, h);
    e = fma2(h, h, neg2(p));
    e = fma2(add2(h, h), l, e);
    e = fma2(l, l, e);
}
// (S, L) += (fh + fl)(dh + dl): the product's rounding error and cross terms into L, the
// sum's rounding error (TwoSum) into L.
__device__ __forceinline__ void acc_ff(f2 fh, f2 fl, f2 dh, f2 dl, f2& S, f2& L) {
    const f2 ph = mul2(fh, dh);
    f2 pl = fma2(fh, dh, neg2(ph));
    pl = fma2(fh, dl, pl);
    pl = fma2(fl, dh, pl);
    f2 t, e;
    two_sum2(S, ph, t, e);
    S = t;
    L = add2(L, add2(e, pl));
}
// Pulls of the two sources of pair record r on one tracer (hi/lo parts XH..ZL) in
// float-float, added to the span sums (SH, SL) per axis.  ml: the low parts of the two
// masses.  y0, y1: the two FP32 reciprocal distances (rsqrt.approx of the high part of the
// square distance), which decide the near sources.  SKIP: a source whose reciprocal distance
// exceeds inv_near adds nothing (the caller takes its pull in FP64).  A coincident source
// (zero distance) makes the sums non-finite, which removes the tracer as in the other
// variants.
template <bool SKIP>
__device__ __forceinline__ void pair_ff(const BodyPair* r, f2 ml, f2 XH, f2 XL, f2 YH, f2 YL, f2 ZH, f2 ZL,
                                        f2 SH[3], f2 SL[3], float inv_near, float& y0, float& y1) {
    const ulonglong2 q0 = *reinterpret_cast<const ulonglong2*>(r->hx);  // hx, hy
    const ulonglong2 q1 = *reinterpret_cast<const ulonglong2*>(r->hz);  // hz, m
    const ulonglong2 q2 = *reinterpret_cast<const ulonglong2*>(r->lx);  // lx, ly
    const f2 lz = *reinterpret_cast<const f2*>(r->lz);
    f2 dxh, dxl, dyh, dyl, dzh, dzl;
    sep_ff(q0.x, q2.x, XH, XL, dxh, dxl);
    sep_ff(q0.y, q2.y, YH, YL, dyh, dyl);
    sep_ff(q1.x, lz, ZH, ZL, dzh, dzl);
    f2 px, ex, py, ey, pz, ez;
    sq_ff(dxh, dxl, px, ex);
    sq_ff(dyh, dyl, py, ey);
    sq_ff(dzh, dzl, pz, ez);
    f2 a1, t1, a2, t2;
    two_sum2(px, py, a1, t1);
    two_sum2(a1, pz, a2, t2);
    const f2 lo = add2(add2(add2(ex, ey), add2(ez, t1)), t2);
    const f2 RRh = add2(a2, lo);                       // |a2| >> |lo|: Fast2Sum
    const f2 RRl = sub2(lo, sub2(RRh, a2));
    // 1/sqrt(RR) = y + yl: y from rsqrt.approx, yl = y (1 - RR y^2) / 2 (one Newton step),
    // with y^2 = u + eu and RRh u = v + ev exact
    float r0, r1;
    f2_split(RRh, r0, r1);
    y0 = rsqrt_approx(r0);
    y1 = rsqrt_approx(r1);
    const f2 y = f2_join(y0, y1);
    const f2 u = mul2(y, y), eu = fma2(y, y, neg2(u));
    const f2 v = mul2(RRh, u), ev = fma2(RRh, u, neg2(v));
    constexpr f2 kOne2 = 0x3F8000003F800000ull, kHalf2 = 0x3F0000003F000000ull;
    f2 rr = sub2(sub2(kOne2, v), ev);
    rr = fma2(neg2(RRh), eu, rr);
    rr = fma2(neg2(RRl), u, rr);
    const f2 yl = mul2(mul2(y, kHalf2), rr);
    // ri^3 = h3 + l3 from ri^2 = u + (eu + 2 y yl); then f = m ri^3 = fh + fl
    const f2 c2l = fma2(add2(y, y), yl, eu);
    const f2 h3 = mul2(u, y);
    f2 l3 = fma2(u, y, neg2(h3));
    l3 = fma2(u, yl, l3);
    l3 = fma2(c2l, y, l3);
    f2 fh = mul2(q1.y, h3);
    f2 fl = fma2(q1.y, h3, neg2(fh));
    fl = fma2(q1.y, l3, fl);
    fl = fma2(ml, h3, fl);
    if (SKIP) {   // zero pull (exactly) for the near sources
        const unsigned long long keep = (y0 > inv_near ? 0ull : 0xFFFFFFFFull) | (y1 > inv_near ? 0ull : 0xFFFFFFFF00000000ull);
        fh &= keep;
        fl &= keep;
    }
    acc_ff(fh, fl, dxh, dxl, SH[0], SL[0]);
    acc_ff(fh, fl, dyh, dyl, SH[1], SL[1]);
    acc_ff(fh, fl, dzh, dzl, SH[2], SL[2]);
}

// Box of every span's sources (high parts, padding slots left out) at every stage, written
// into the pad slots of the span's first four pair records, so it reaches shared memory with
// the tile: record 0 {min x, max x}, record 1 {min y, max y}, record 2 {min z, max z},
// record 3 {max |coordinate|, 0}; the maximum is NaN when a coordinate is NaN (such a span
// never counts as far).
// One warp per (stage, span): lane u reads source slot u of the span's 32.
__global__ void span_box_kernel(BodyPair* __restrict__ PP, int pcap, int n_src, int nspans) {
    const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;   // stage * nspans + span
    const int u = threadIdx.x & 31;
    if (k >= 4 * nspans) return;                                   // whole warps leave together
    const int stage = k / nspans, span = k - stage * nspans;
    BodyPair* const R = PP + (size_t)stage * pcap + (size_t)span * kPairSpan;
    const int q = span * 2 * kPairSpan + u;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    bool nan = false;
    if (q < n_src) {
        const BodyPair& r = R[u >> 1];
        const float v[3] = {r.hx[u & 1], r.hy[u & 1], r.hz[u & 1]};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            nan = nan || !(v[a] == v[a]);
            lo[a] = v[a];
            hi[a] = v[a];
        }
        if (nan) lo[0] = lo[1] = lo[2] = INFINITY, hi[0] = hi[1] = hi[2] = -INFINITY;
    }
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
        }
    nan = __any_sync(0xffffffffu, nan);
    if (u < 3) {
        R[u].pad[0] = lo[u];
        R[u].pad[1] = hi[u];
    } else if (u == 3) {
        float xm = 0.f;
#pragma unroll
        for (int a = 0; a < 3; ++a) xm = fmaxf(xm, fmaxf(fabsf(lo[a]), fabsf(hi[a])));
        R[3].pad[0] = nan ? __int_as_float(0x7FC00000) : xm;
        R[3].pad[1] = 0.f;
    }
}

// The test of one tracer (high parts xh, yh, zh; own = its largest |coordinate|) against one
// span box (bx, by, bz: min and max per axis; xm: its largest |coordinate|, NaN when a
// coordinate is NaN): far when the box lies at least X = kFar max(xm, own) away.  Rounded
// operations only (no contraction), so the block tests below imply its outcome.
constexpr float kFar = 0.25f;  // far from X/4 on (a power of two: the scaling is exact)

__device__ __forceinline__ bool lane_far(float2 bx, float2 by, float2 bz, float xm, float xh, float yh, float zh,
                                         float own) {
    const float gx = fmaxf(0.f, fmaxf(__fsub_rn(bx.x, xh), __fsub_rn(xh, bx.y)));
    const float gy = fmaxf(0.f, fmaxf(__fsub_rn(by.x, yh), __fsub_rn(yh, by.y)));
    const float gz = fmaxf(0.f, fmaxf(__fsub_rn(bz.x, zh), __fsub_rn(zh, bz.y)));
    const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(gx, gx), __fmul_rn(gy, gy)), __fmul_rn(gz, gz));
    const float X = kFar * fmaxf(xm, own);
    return xm == xm && d2 >= __fmul_rn(X, X);
}

// The same tests for a whole block of tracers from its box b (min and max of the high parts
// per axis, and the largest own): far for every tracer when the nearest point of b is far
// with X = kFar max(xm, largest own); near for every tracer when even the farthest point of
// b is nearer than kFar xm.  Each rounded step is monotone, so these imply lane_far's
// outcome for any tracer inside b.
__device__ __forceinline__ void block_far(float2 bx, float2 by, float2 bz, float xm, const float* b, bool& all_far,
                                          bool& all_near, float& dn, float& df) {
    const float nx = fmaxf(0.f, fmaxf(__fsub_rn(bx.x, b[1]), __fsub_rn(b[0], bx.y)));
    const float ny = fmaxf(0.f, fmaxf(__fsub_rn(by.x, b[3]), __fsub_rn(b[2], by.y)));
    const float nz = fmaxf(0.f, fmaxf(__fsub_rn(bz.x, b[5]), __fsub_rn(b[4], bz.y)));
    const float fx = fmaxf(0.f, fmaxf(__fsub_rn(bx.x, b[0]), __fsub_rn(b[1], bx.y)));
    const float fy = fmaxf(0.f, fmaxf(__fsub_rn(by.x, b[2]), __fsub_rn(b[3], by.y)));
    const float fz = fmaxf(0.f, fmaxf(__fsub_rn(bz.x, b[4]), __fsub_rn(b[5], bz.y)));
    dn = __fadd_rn(__fadd_rn(__fmul_rn(nx, nx), __fmul_rn(ny, ny)), __fmul_rn(nz, nz));
    df = __fadd_rn(__fadd_rn(__fmul_rn(fx, fx), __fmul_rn(fy, fy)), __fmul_rn(fz, fz));
    const float X = kFar * fmaxf(xm, b[6]), Xn = kFar * xm;
    all_far = xm == xm && dn >= __fmul_rn(X, X);
    all_near = !(xm == xm) || df < __fmul_rn(Xn, Xn);
}

// Squared distance from a tracer's point to a span box (rounded operations only, like
// lane_far, so the block tests imply its outcome).
__device__ __forceinline__ float lane_dist2(float2 bx, float2 by, float2 bz, float xh, float yh, float zh) {
    const float gx = fmaxf(0.f, fmaxf(__fsub_rn(bx.x, xh), __fsub_rn(xh, bx.y)));
    const float gy = fmaxf(0.f, fmaxf(__fsub_rn(by.x, yh), __fsub_rn(yh, by.y)));
    const float gz = fmaxf(0.f, fmaxf(__fsub_rn(bz.x, zh), __fsub_rn(zh, bz.y)));
    return __fadd_rn(__fadd_rn(__fmul_rn(gx, gx), __fmul_rn(gy, gy)), __fmul_rn(gz, gz));
}

__device__ __forceinline__ void span_box(const BodyPair* R, float2& bx, float2& by, float2& bz, float& xm) {
    bx = *reinterpret_cast<const float2*>(R[0].pad);
    by = *reinterpret_cast<const float2*>(R[1].pad);
    bz = *reinterpret_cast<const float2*>(R[2].pad);
    xm = R[3].pad[0];
}

// The tracer's FP64 stage coordinate from its three FP32 parts hi + lo + rest (hi = fp32(v),
// lo = fp32(v - hi), rest = fp32(v - hi - lo)): hi + lo is exact in FP64 and within 2^-48 |v|
// of v, rest brings the sum within 2^-72 |v|, below half an FP64 ulp, so the rounded sum is v.
__device__ __forceinline__ double join3(f2 H, f2 L, float rest) {
    float h, l, u;
    f2_split(H, h, u);
    f2_split(L, l, u);
    return ((double)h + (double)l) + (double)rest;
}
__device__ __forceinline__ float rest3(double v, float hi, float lo) {
    return __double2float_rn((v - (double)hi) - (double)lo);
}

// One span of kPairSpan pair records (slots q0 .. q0 + 2 kPairSpan - 1) summed again for a
// tracer with a near source among them: the FP32 partial sum of the sources at or beyond the
// near radius (the same operations as the main loop, so each of their pulls is the same),
// and the FP64 pull of each near source from its FP64 stage position (P: the stage's
// records of bodies n_exact.., src: source of each slot, null when slot q holds source q),
// added to k.  A zero FP64 separation gives an infinite pull, which removes the tracer as in
// the FP64 step.
__device__ __forceinline__ void near_span(const BodyPair* R, int q0, f2 XH, f2 XL, f2 YH, f2 YL, f2 ZH, f2 ZL,
                                          float xr, float yr, float zr, float inv_near, const Body* __restrict__ P,
                                          const int* __restrict__ src, f2& px, f2& py, f2& pz, double& kx,
                                          double& ky, double& kz) {
    const double xt = join3(XH, XL, xr), yt = join3(YH, YL, yr), zt = join3(ZH, ZL, zr);
    px = 0; py = 0; pz = 0;
    for (int u = 0; u < kPairSpan; ++u) {
        const BodyPair* r = R + u;
        const ulonglong2 q0v = *reinterpret_cast<const ulonglong2*>(r->hx);
        const ulonglong2 q1v = *reinterpret_cast<const ulonglong2*>(r->hz);
        const ulonglong2 q2v = *reinterpret_cast<const ulonglong2*>(r->lx);
        const f2 lz = *reinterpret_cast<const f2*>(r->lz);
        const f2 dX = add2(sub2(q0v.x, XH), sub2(q2v.x, XL));
        const f2 dY = add2(sub2(q0v.y, YH), sub2(q2v.y, YL));
        const f2 dZ = add2(sub2(q1v.x, ZH), sub2(lz, ZL));
        const f2 RR = fma2(dX, dX, fma2(dY, dY, mul2(dZ, dZ)));
        float r0, r1;
        f2_split(RR, r0, r1);
        const float i0 = rsqrt_approx(r0), i1 = rsqrt_approx(r1);
        const bool n0 = i0 > inv_near, n1 = i1 > inv_near;
        const f2 ri = f2_join(n0 ? 0.f : i0, n1 ? 0.f : i1);
        const f2 f = mul2(mul2(q1v.y, ri), mul2(ri, ri));
        px = fma2(f, dX, px); py = fma2(f, dY, py); pz = fma2(f, dZ, pz);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if (!(h ? n1 : n0)) continue;
            const int q = q0 + 2 * u + h;
            const Body p = P[src ? src[q] : q];
            const double ex = p.x - xt, ey = p.y - yt, ez = p.z - zt;
            const double rr = ex * ex + ey * ey + ez * ez;
            const double ri64 = rsqrt(rr);
            const double f64 = p.m * (ri64 * ri64 * ri64);
            kx = fma(f64, ex, kx); ky = fma(f64, ey, ky); kz = fma(f64, ez, kz);
        }
    }
}

// One float-float span summed again for a tracer with a near source among its pair records:
// the float-float sums of the other sources into (SH, SL), and the FP64 pull of each near
// source (reciprocal FP32 distance above inv_near) from its FP64 stage record, added to k
// (as near_span does for the FP32 forms).
__device__ __forceinline__ void near_span_ff(const BodyPair* R, const f2* ML, int q0, f2 XH, f2 XL, f2 YH, f2 YL,
                                             f2 ZH, f2 ZL, float xr, float yr, float zr, float inv_near,
                                             const Body* __restrict__ P, const int* __restrict__ src, f2 SH[3],
                                             f2 SL[3], double& kx, double& ky, double& kz) {
    const double xt = join3(XH, XL, xr), yt = join3(YH, YL, yr), zt = join3(ZH, ZL, zr);
    for (int c = 0; c < 3; ++c) SH[c] = SL[c] = 0;
    for (int u = 0; u < kPairSpan; ++u) {
        float y0, y1;
        pair_ff<true>(R + u, __ldg(ML + u), XH, XL, YH, YL, ZH, ZL, SH, SL, inv_near, y0, y1);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if (!((h ? y1 : y0) > inv_near)) continue;
            const int q = q0 + 2 * u + h;
            const Body p = P[src ? src[q] : q];
            const double ex = p.x - xt, ey = p.y - yt, ez = p.z - zt;
            const double rr = ex * ex + ey * ey + ez * ez;
            const double ri64 = rsqrt(rr);
            const double f64 = p.m * (ri64 * ri64 * ri64);
            kx = fma(f64, ex, kx); ky = fma(f64, ey, ky); kz = fma(f64, ez, kz);
        }
    }
}

// Kahan sums across the FP32 spans.  The compensated variant keeps both lanes (its
// float-float spans go to the FP64 acceleration instead, ff_total).  The FP32 forms add
// the span's two lanes (one rounding, against the 16 of each lane's plain sum) and carry one
// FP32 sum per axis: six registers fewer in the loop, which the dusty-ring dust kernel took
// from 8.18 to 8.00 ms.
template <bool F2> struct SpanAcc;
template <> struct SpanAcc<true> {
    f2 S = 0, C = 0;
    __device__ __forceinline__ void add(f2 v) { kahan2(S, C, v); }
    __device__ __forceinline__ double total() const { return f2_total(S, C); }
};
template <> struct SpanAcc<false> {
    float S = 0.f, C = 0.f;
    __device__ __forceinline__ void add(f2 v) {
        float a, b;
        f2_split(v, a, b);
        const float y = __fsub_rn(__fadd_rn(a, b), C);
        const float t = __fadd_rn(S, y);
        C = __fsub_rn(__fsub_rn(t, S), y);
        S = t;
    }
    __device__ __forceinline__ double total() const { return (double)S - (double)C; }
};

// A float-float span sum (both lanes' high parts H and low parts L) in FP64: the lanes' high
// parts added exactly (TwoSum), the error and the low parts in FP32, then two FP64 adds.  The
// compensated variant adds its float-float spans to the stage's FP64 acceleration this way
// rather than through the FP32 Kahan sum, whose error grows as the number of spans times
// 2^-48 of the magnitudes summed: on the dusty ring the 99th percentile of the 1,000-step
// errors halved (1.0e-11 to 5.1e-12), for 0.2 ms of the 24.8 ms step.
__device__ __forceinline__ double ff_total(f2 H, f2 L) {
    float a, b, la, lb;
    f2_split(H, a, b);
    f2_split(L, la, lb);
    const float s = __fadd_rn(a, b), v = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, v)), __fsub_rn(b, v));
    return (double)s + (double)__fadd_rn(__fadd_rn(la, lb), e);
}

// Spans with one bit per block test (all far, all near) in shared memory, per stage; beyond
// this many spans every tracer tests every span itself.
constexpr int kFlagSpans = 4096;

// Bits j0 .. j0 + n - 1 (n <= 32 spans of one tile) of the span bit array w, as bits 0 .. n-1.
// The next word is read only when the range runs into it, so only words of existing spans.
__device__ __forceinline__ uint32_t span_bits(const uint32_t* w, int j0, int n) {
    const int q = j0 >> 5, r = j0 & 31;
    unsigned long long v = w[q];
    if (r + n > 32) v |= (unsigned long long)w[q + 1] << 32;
    return (uint32_t)(v >> r) & (n == 32 ? 0xFFFFFFFFu : (1u << n) - 1u);
}

// Four blocks per SM (64 registers, two 16 KiB tiles each): the FP64 values the compiler
// keeps in local memory are touched only between stages, and the kernel is held by the
// latency of the broadcast shared-memory reads and of rsqrt.approx, which more warps hide.
// Measured on the dusty ring (dust kernel): 3 blocks (80 registers, 32 KiB tiles) 8.50 ms,
// 4 blocks 8.34 ms, 5 blocks (48 registers, 20 KiB tiles) 8.41 ms; two blocks without
// spills were slower than three.  With the near-source test in (8.64 ms at 24 KiB tiles),
// smaller tiles leave more of the SM's 256 KiB to L1, where the spilled values live:
// 8.55 ms at 12 KiB, 8.47 ms at 16 KiB, 8.53 ms at 20 KiB.
// COMP: the compensated variant, three blocks per SM (80 registers; its float-float pair
// needs more than 64): 22.75 ms on the dusty ring against 23.0 ms with two blocks of 128.
template <bool COMP>
__global__ void __launch_bounds__(kThreads, COMP ? 3 : 4)
dust_rk4_mixed_kernel(ddx_state s, StepArgs a, MassiveScratch ms, const SizeBin* __restrict__ bins,
                      const int* __restrict__ perm, bool boxes, const int* __restrict__ src) {
    constexpr int NB = COMP ? 8 : 7;              // box values: 3 x (min, max), largest own[, smallest own]
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) unsigned long long mbar[2];
    __shared__ float bred[kThreads / 32][NB];
    __shared__ float bbox[NB];                    // the block's box at the current stage, largest own
    __shared__ uint32_t allfar[kFlagSpans / 32], allnear[kFlagSpans / 32];
    __shared__ uint32_t allcomp[COMP ? kFlagSpans / 32 : 1], nocomp[COMP ? kFlagSpans / 32 : 1];
    BodyPair* const tiles = reinterpret_cast<BodyPair*>(smem);
    const int tid = threadIdx.x;
    const int slot = blockIdx.x * blockDim.x + tid;   // position in the visiting order
    const int i = perm && slot < a.n_dust ? perm[slot] : slot;
    const int ng = a.n_grav;
    const int t = ng + i;

    bool alive = false;
    double x = 0, y = 0, z = 0, vx = 0, vy = 0, vz = 0, m = 1.0;
    float bet = 0.f, betsw = 0.f, qe = 0.f;
    if (i < a.n_dust) {
        alive = (s.N[t] != 0.0);
        if (alive) {
            x = s.x[t]; y = s.y[t]; z = s.z[t];
            vx = s.vx[t]; vy = s.vy[t]; vz = s.vz[t];
            m = s.m[t];
            const int id = s.id[t];
            if (id >= 0 && id < a.n_grid) {
                const SizeBin b = bins[id];
                bet = b.beta; betsw = b.betasw; qe = b.q;
            }
        }
    }

    const int npairs = pair_count(ng - a.n_exact);
    const int ntiles = (npairs + kTilePairs - 1) / kTilePairs;
    const int G = 4 * ntiles;                       // tiles over all four stages
    const uint32_t mb[2] = {smem_u32(&mbar[0]), smem_u32(&mbar[1])};
    if (tid == 0) {
        mbar_init(mb[0], 1);
        mbar_init(mb[1], 1);
        fence_mbar_init();
    }
    __syncthreads();
    // Thread 0 streams tile g of the sequence (stage-major) into buffer g & 1.  The test
    // hook a.lose_tile leaves one tile's copy unissued, so the waits on it run out.
    // in_flight: tiles issued and not yet consumed (thread 0 only; at most two).
    int in_flight[2] = {-1, -1};
    auto issue = [&](int g) {
        if (g == a.lose_tile) return;
        const int stg = g / ntiles, first = (g - stg * ntiles) * kTilePairs;
        const unsigned bytes = (unsigned)(min(kTilePairs, npairs - first) * sizeof(BodyPair));
        mbar_expect_tx(mb[g & 1], bytes);
        bulk_load(smem_u32(tiles + (g & 1) * kTilePairs), ms.PP + (size_t)stg * ms.pcap + first, bytes,
                  mb[g & 1]);
        in_flight[g & 1] = g;
    };
    if (tid == 0 && G > 0) issue(0);

    const double dt = a.dt, dt2 = a.dt / 2.0, dt6 = a.dt / 6.0;
    // RK4 of src/gpu_functions.cu:627-943 with running sums, so that little FP64 state is
    // live across the FP32 loop: stage s evaluates the acceleration at
    //   x_s = x + r_{s-1} c_s,  r_s = v + k_{s-1} c_s   (c = 0, dt/2, dt/2, dt; r_0 = v),
    // and the update is x += dt/6 sum w_s r_s, v += dt/6 sum w_s k_s with w = 1, 2, 2, 1.
    double rpx = vx, rpy = vy, rpz = vz;      // r_{s-1}
    double kpx = 0, kpy = 0, kpz = 0;         // k_{s-1}
    double Ax = 0, Ay = 0, Az = 0;            // sum w_s r_s
    double Bx = 0, By = 0, Bz = 0;            // sum w_s k_s
    int removed = 0, removed_stage = -1;
    int lost = 0;
    int g = 0;

#pragma unroll 1
    for (int st = 0; st < 4; ++st) {
        double xt = x, yt = y, zt = z, rx = vx, ry = vy, rz = vz;
        if (st > 0) {
            const double c = st == 3 ? dt : dt2;
            xt = x + rpx * c; yt = y + rpy * c; zt = z + rpz * c;
            rx = vx + kpx * c; ry = vy + kpy * c; rz = vz + kpz * c;
        }
        const double w = (st == 1 || st == 2) ? 2.0 : 1.0;
        Ax += w * rx; Ay += w * ry; Az += w * rz;
        rpx = rx; rpy = ry; rpz = rz;
        double kx = 0, ky = 0, kz = 0;
        if (alive) {
            const Body ps = ms.P[st * ms.cap + 0];
            if (!star_term(xt - ps.x, yt - ps.y, zt - ps.z, rx, ry, rz, ps.m, bet, betsw, qe, m, a,
                           kx, ky, kz)) {
                alive = false; removed = 1; removed_stage = st;
            }
        }
        // the planets, in FP64
        for (int j = 1; alive && j < a.n_exact; ++j) {
            const Body p = ms.P[st * ms.cap + j];
            const double ex = p.x - xt, ey = p.y - yt, ez = p.z - zt;
            const double RR = ex * ex + ey * ey + ez * ez;
            if (RR == 0.0) { alive = false; removed = 2; removed_stage = st; break; }
            const double ri = rsqrt(RR);
            const double f = p.m * (ri * ri * ri);
            kx = fma(f, ex, kx); ky = fma(f, ey, ky); kz = fma(f, ez, kz);
        }
        float xh, xl, yh, yl, zh, zl;
        split_hilo(xt, xh, xl); split_hilo(yt, yh, yl); split_hilo(zt, zh, zl);
        const float xr = rest3(xt, xh, xl), yr = rest3(yt, yh, yl), zr = rest3(zt, zh, zl);
        const f2 XH = f2_dup(xh), XL = f2_dup(xl), YH = f2_dup(yh), YL = f2_dup(yl);
        const f2 ZH = f2_dup(zh), ZL = f2_dup(zl);
        const float own = fmaxf(fabsf(xh), fmaxf(fabsf(yh), fabsf(zh)));   // largest |coordinate|
        const float inv_near = near_inv(a.near_eta, own);
        const float Dc = a.comp_eta * own;                                 // compensated spans: nearer than this
        const Body* const Pn = ms.P + (size_t)st * ms.cap + a.n_exact;     // FP64 records of the sources
        // per stage: the block's box (live tracers) and, per span, whether the box settles
        // every tracer's choice (bits in shared memory); spans left open are tested per tracer
        const int nspans = npairs / kPairSpan;
        const bool flags = boxes && nspans <= kFlagSpans;
        if (flags) {
            const float v[8] = {xh, xh, yh, yh, zh, zh, own, own};
#pragma unroll
            for (int q = 0; q < NB; ++q) {
                const bool mx = q < 7 && ((q & 1) || q == 6);
                float w = alive ? v[q] : (mx ? -INFINITY : INFINITY);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    const float u = __shfl_xor_sync(0xffffffffu, w, o);
                    w = mx ? fmaxf(w, u) : fminf(w, u);
                }
                if ((tid & 31) == 0) bred[tid >> 5][q] = w;
            }
            __syncthreads();
            if (tid < NB) {
                const bool mx = tid < 7 && ((tid & 1) || tid == 6);
                float w = bred[0][tid];
                for (int k = 1; k < (int)(blockDim.x >> 5); ++k) w = mx ? fmaxf(w, bred[k][tid]) : fminf(w, bred[k][tid]);
                bbox[tid] = tid >= 6 ? fmaxf(w, 0.f) : w;
            }
            __syncthreads();
            float b[NB];
#pragma unroll
            for (int q = 0; q < NB; ++q) b[q] = bbox[q];
            const BodyPair* PPs = ms.PP + (size_t)st * ms.pcap;
            for (int j0 = 0; j0 < nspans; j0 += blockDim.x) {   // uniform trip count: ballots below
                const int j = j0 + tid;
                bool f = false, nr = false, ca = false, cn = false;
                if (j < nspans) {
                    float2 bx, by, bz;
                    float xm, dn, df;
                    span_box(PPs + (size_t)j * kPairSpan, bx, by, bz, xm);
                    block_far(bx, by, bz, xm, b, f, nr, dn, df);
                    if constexpr (COMP) {
                        // every tracer within comp_eta own of the box / none (b[6], b[7]: the
                        // largest and smallest own); monotone like the far tests
                        const float lo = a.comp_eta * b[7], hi = a.comp_eta * b[6];
                        ca = df < __fmul_rn(lo, lo);
                        cn = !(dn < __fmul_rn(hi, hi));
                    }
                }
                const uint32_t wf = __ballot_sync(0xffffffffu, f), wn = __ballot_sync(0xffffffffu, nr);
                if ((tid & 31) == 0 && j < nspans) { allfar[j >> 5] = wf; allnear[j >> 5] = wn; }   // lane 0: j = 32 w
                if constexpr (COMP) {
                    const uint32_t wa = __ballot_sync(0xffffffffu, ca), wc = __ballot_sync(0xffffffffu, cn);
                    if ((tid & 31) == 0 && j < nspans) { allcomp[j >> 5] = wa; nocomp[j >> 5] = wc; }
                }
            }
            __syncthreads();
        }
        SpanAcc<COMP> ax, ay, az;
        for (int tt = 0; tt < ntiles; ++tt, ++g) {
            lost = __syncthreads_or(lost);      // also: every thread is done with tile g-1
            if (lost) break;
            if (tid == 0 && g + 1 < G) issue(g + 1);
            if (!mbar_wait(mb[g & 1], (g >> 1) & 1, a.wait_ns)) { lost = 1; continue; }
            if (tid == 0) in_flight[g & 1] = -1;
            if (!alive) continue;
            const BodyPair* T = tiles + (g & 1) * kTilePairs;
            const int cnt = min(kTilePairs, npairs - tt * kTilePairs);   // a multiple of kPairSpan
            static_assert(kTilePairs / kPairSpan <= 32, "one mask bit per span of a tile");
            uint32_t fm = 0u, cm = 0u;   // far spans, compensated spans (compensated wins)
            const uint32_t all = cnt / kPairSpan == 32 ? 0xFFFFFFFFu : (1u << (cnt / kPairSpan)) - 1u;
            if (COMP) {
                if (!boxes) {
                    cm = all;              // no spatial order: every span compensated
                } else {
                    uint32_t open = all;
                    if (flags) {
                        const int j0 = tt * (kTilePairs / kPairSpan);
                        const uint32_t ac = span_bits(allcomp, j0, cnt / kPairSpan);
                        cm = ac;
                        open = all & ~(ac | span_bits(nocomp, j0, cnt / kPairSpan));
                    }
                    while (open) {
                        const int j = __ffs(open) - 1;
                        open &= open - 1;
                        float2 bx, by, bz;
                        float xm;
                        span_box(T + j * kPairSpan, bx, by, bz, xm);
                        if (lane_dist2(bx, by, bz, xh, yh, zh) < __fmul_rn(Dc, Dc)) cm |= 1u << j;
                    }
                }
            }
            if (boxes) {
                uint32_t open = all & ~cm;
                if (flags) {
                    const int j0 = tt * (kTilePairs / kPairSpan);   // the tile's first span
                    const uint32_t af = span_bits(allfar, j0, cnt / kPairSpan);
                    fm = af & ~cm;
                    open = all & ~cm & ~(af | span_bits(allnear, j0, cnt / kPairSpan));
                }
                while (open) {   // the same mask in every lane: no divergence here
                    const int j = __ffs(open) - 1;
                    open &= open - 1;
                    float2 bx, by, bz;
                    float xm;
                    span_box(T + j * kPairSpan, bx, by, bz, xm);
                    if (lane_far(bx, by, bz, xm, xh, yh, zh, own)) fm |= 1u << j;
                }
            }
            for (int k = 0; k < cnt; k += kPairSpan) {
                f2 px = 0, py = 0, pz = 0;
                if (COMP && ((cm >> (k / kPairSpan)) & 1u)) {
                    // float-float span sums, added to the stage's FP64 acceleration
                    f2 SH[3] = {0, 0, 0}, SL[3] = {0, 0, 0};
                    const f2* ML = reinterpret_cast<const f2*>(ms.PM + (size_t)st * ms.pcap + tt * kTilePairs + k);
                    float mx = 0.f;
#pragma unroll 2
                    for (int u = 0; u < kPairSpan; ++u) {
                        float y0, y1;
                        pair_ff<false>(T + k + u, __ldg(ML + u), XH, XL, YH, YL, ZH, ZL, SH, SL, inv_near, y0, y1);
                        mx = fmax3(mx, y0, y1);
                    }
                    if (mx > inv_near)   // a source within the near radius: its pull in FP64
                        near_span_ff(T + k, ML, 2 * (tt * kTilePairs + k), XH, XL, YH, YL, ZH, ZL, xr, yr, zr,
                                     inv_near, Pn, src, SH, SL, kx, ky, kz);
                    kx += ff_total(SH[0], SL[0]); ky += ff_total(SH[1], SL[1]); kz += ff_total(SH[2], SL[2]);
                    continue;
                }
                if ((fm >> (k / kPairSpan)) & 1u) {
#pragma unroll
                    for (int u = 0; u < kPairSpan; ++u) {
                        const BodyPair* r = T + k + u;
                        const ulonglong2 q0 = *reinterpret_cast<const ulonglong2*>(r->hx);  // hx, hy
                        const ulonglong2 q1 = *reinterpret_cast<const ulonglong2*>(r->hz);  // hz, m
                        const f2 dX = sub2(q0.x, XH), dY = sub2(q0.y, YH), dZ = sub2(q1.x, ZH);
                        const f2 RR = fma2(dX, dX, fma2(dY, dY, mul2(dZ, dZ)));
                        float r0, r1;
                        f2_split(RR, r0, r1);
                        const f2 ri = f2_join(rsqrt_approx(r0), rsqrt_approx(r1));
                        const f2 f = mul2(mul2(q1.y, ri), mul2(ri, ri));
                        px = fma2(f, dX, px); py = fma2(f, dY, py); pz = fma2(f, dZ, pz);
                    }
                } else {
                    float mx = 0.f;   // largest reciprocal distance of the span
#pragma unroll
                    for (int u = 0; u < kPairSpan; ++u) {
                        const BodyPair* r = T + k + u;
                        const ulonglong2 q0 = *reinterpret_cast<const ulonglong2*>(r->hx);  // hx, hy
                        const ulonglong2 q1 = *reinterpret_cast<const ulonglong2*>(r->hz);  // hz, m
                        const ulonglong2 q2 = *reinterpret_cast<const ulonglong2*>(r->lx);  // lx, ly
                        const f2 lz = *reinterpret_cast<const f2*>(r->lz);
                        const f2 dX = add2(sub2(q0.x, XH), sub2(q2.x, XL));
                        const f2 dY = add2(sub2(q0.y, YH), sub2(q2.y, YL));
                        const f2 dZ = add2(sub2(q1.x, ZH), sub2(lz, ZL));
                        const f2 RR = fma2(dX, dX, fma2(dY, dY, mul2(dZ, dZ)));
                        float r0, r1;
                        f2_split(RR, r0, r1);
                        const float i0 = rsqrt_approx(r0), i1 = rsqrt_approx(r1);
                        mx = fmax3(mx, i0, i1);
                        const f2 ri = f2_join(i0, i1);
                        const f2 f = mul2(mul2(q1.y, ri), mul2(ri, ri));
                        px = fma2(f, dX, px); py = fma2(f, dY, py); pz = fma2(f, dZ, pz);
                    }
                    if (mx > inv_near)   // rare: a source of this span lies within the near radius
                        near_span(T + k, 2 * (tt * kTilePairs + k), XH, XL, YH, YL, ZH, ZL, xr, yr, zr, inv_near,
                                  Pn, src, px, py, pz, kx, ky, kz);
                }
                ax.add(px); ay.add(py); az.add(pz);
            }
        }
        if (ntiles > 0) lost = __syncthreads_or(lost);   // block-uniform before branching on it
        if (lost) break;
        if (alive) {
            const double px = ax.total(), py = ay.total(), pz = az.total();
            // An exact coincidence makes RR = 0, the rsqrt infinite and the sum NaN.
            // (the compensated variant has added its float-float spans to k already)
            if (!(isfinite(px) && isfinite(py) && isfinite(pz) &&
                  (!COMP || (isfinite(kx) && isfinite(ky) && isfinite(kz))))) {
                alive = false; removed = 2; removed_stage = st;
            }
            kx += px; ky += py; kz += pz;
        }
        Bx += w * kx; By += w * ky; Bz += w * kz;
        kpx = kx; kpy = ky; kpz = kz;
    }
    lost = __syncthreads_or(lost);
    if (lost) {
        if (tid == 0) {
            atomicOr(ms.status, kStatusTimeout);
            // let this block's copies that are still in flight land before it exits
            for (int b = 0; b < 2; ++b)
                if (in_flight[b] >= 0) mbar_wait(mb[b], (in_flight[b] >> 1) & 1, a.wait_ns);
        }
        return;
    }
    if (i >= a.n_dust) return;
    if (removed) {
        if (removed == 1 && removed_stage == 3 && a.mode == DDX_MODE_REFERENCE) s.N[i] = 0;
        else s.N[t] = 0;
        return;
    }
    if (!alive) return;
    x += dt6 * Ax; y += dt6 * Ay; z += dt6 * Az;
    vx += dt6 * Bx; vy += dt6 * By; vz += dt6 * Bz;
    s.x[t] = x; s.y[t] = y; s.z[t] = z;
    s.vx[t] = vx; s.vy[t] = vy; s.vz[t] = vz;
}

}  // namespace

cudaError_t launch_dust_mixed(const ddx_state& s, const StepArgs& a, const MassiveScratch& ms,
                              const SizeBin* bins, int precision, cudaStream_t st) {
    if (a.n_dust <= 0) return cudaSuccess;
    const bool comp = precision == DDX_PREC_COMPENSATED;
    const size_t smem = 2 * (size_t)kTilePairs * sizeof(BodyPair);
    static bool attr_set[128] = {};   // the attributes are set once per device
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 128) return cudaErrorInvalidDevice;
    if (!attr_set[dev]) {
        cudaError_t e = cudaFuncSetAttribute(dust_rk4_mixed_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(dust_rk4_mixed_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem);
        if (e != cudaSuccess) return e;
        attr_set[dev] = true;
    }
    const int threads = dust_block_threads(a.n_dust);   // 256 unless the grains are few
    const int blocks = (a.n_dust + threads - 1) / threads;
    // the tracers' visiting order and the spans' boxes, when the context keeps their scratch
    const int* perm = nullptr;
    bool boxes = false;
    const int n_src = a.n_grav - a.n_exact;
    if (ms.slot && ms.dust_order.cap >= a.n_dust && spatial_order_on(a)) {
        cudaError_t e =
            order_bodies(s, a.n_grav, a.n_dust, true, ms.dust_order, ms.dust_order.perm, nullptr, !comp, st);
        if (e != cudaSuccess) return e;
        const int nspans = pair_count(n_src) / kPairSpan;
        span_box_kernel<<<(4 * nspans * 32 + 127) / 128, 128, 0, st>>>(ms.PP, ms.pcap, n_src, nspans);
        perm = ms.dust_order.perm;
        boxes = true;
    }
    // the source of each pair slot, for the FP64 pulls of near sources: the sources sit in
    // cell order when the step ordered them (massive_prepare), else slot q holds source q
    const int* src = ms.slot && spatial_order_on(a) ? ms.src : nullptr;
    if (comp) dust_rk4_mixed_kernel<true><<<blocks, threads, smem, st>>>(s, a, ms, bins, perm, boxes, src);
    else dust_rk4_mixed_kernel<false><<<blocks, threads, smem, st>>>(s, a, ms, bins, perm, boxes, src);
    return cudaGetLastError();
}

}  // namespace ddx
