// RK4 step of the DiskDyn system on sm_103a.
//
// Reference behaviour (src/gpu_functions.cu:71-943, launch sequence src/grid.cu:693-752):
//   massive set : k1x = x; k2x = x + v dt/2; k2r = v + k1v dt/2; k3x = x + k2r dt/2;
//                 k3r = v + k2v dt/2; k4x = x + k3r dt; k4r = v + k3v dt;
//                 kNv = sum_j m_j (x_j - x_i)/r^3 at stage N;  x += dt/6 (v + 2k2r + 2k3r + k4r);
//                 v += dt/6 (k1v + 2k2v + 2k3v + k4v).
//   dust        : the same four stages per tracer, with the star term (gravity reduced by
//                 beta + beta_sw, PR + stellar-wind drag, optional Lorentz force) and the
//                 gravity of massive bodies 1..n_grav-1 taken at their stage positions.
//
// Because k2x depends only on x, v and k3x only on k1v, k4x only on k2v, the four massive
// force evaluations need two dependent passes: pass 1 evaluates A1 (at P1) and A2 (at P2),
// pass 2 evaluates A3 (at P3) and A4 (at P4).  The reference issues 4*(num+1)+4 launches
// per step with CAS atomics; here it is prepare + pass1 + pass2 + dust, deterministic, with
// no atomics.
#include "ddx_internal.cuh"
#include "ddx_f32x2.cuh"

namespace ddx {

// ---------------------------------------------------------------------------------------
// Massive set
// ---------------------------------------------------------------------------------------

constexpr float kFarAway = 1.0e18f;  // padding source position, AU (mass 0)

// FP32 source k = i - n_exact (body i >= n_exact) into its slot q of the pair records of a
// stage: half q & 1 of record q / 2.  The slots follow the sources' cell order when one
// was made for this step (ms.slot), else q = k.
__device__ __forceinline__ void store_pair_slot(MassiveScratch& ms, int stage, int k, const float4 h,
                                                const float4 l) {
    const int q = ms.slot ? ms.slot[k] : k;
    if (stage == 0 && ms.slot) ms.src[q] = k;     // the inverse, for the FP64 pulls of near sources
    BodyPair* r = ms.PP + (size_t)stage * ms.pcap + (q >> 1);
    const int u = q & 1;
    r->hx[u] = h.x; r->hy[u] = h.y; r->hz[u] = h.z; r->m[u] = h.w;
    r->lx[u] = l.x; r->ly[u] = l.y; r->lz[u] = l.z; r->pad[u] = 0.f;
    float2& pm = ms.PM[(size_t)stage * ms.pcap + (q >> 1)];
    if (u) pm.y = l.w; else pm.x = l.w;           // the mass's low part
}

// Zero-mass, far-away filler for the slots past the last FP32 source, so the dust kernel
// always processes whole spans of kPairSpan records.
__device__ __forceinline__ void store_pair_padding(MassiveScratch& ms, int n_src) {
    const int np = pair_count(n_src);
    for (int stage = 0; stage < 4; ++stage)
        for (int q = n_src; q < 2 * np; ++q) {
            BodyPair* r = ms.PP + (size_t)stage * ms.pcap + (q >> 1);
            const int k = q & 1;
            r->hx[k] = kFarAway; r->hy[k] = kFarAway; r->hz[k] = kFarAway; r->m[k] = 0.f;
            r->lx[k] = 0.f; r->ly[k] = 0.f; r->lz[k] = 0.f; r->pad[k] = 0.f;
            float2& pm = ms.PM[(size_t)stage * ms.pcap + (q >> 1)];
            if (k) pm.y = 0.f; else pm.x = 0.f;
        }
}

// The scratch as the kernels of a step see it: the pair slots in cell order only when the
// step orders its sources (else slot k holds source k).
static MassiveScratch slotted(const MassiveScratch& ms, const StepArgs& a) {
    MassiveScratch m = ms;
    if (!spatial_order_on(a)) m.slot = nullptr;
    return m;
}

// P1 = x, P2 = x + v dt/2 (src/gpu_functions.cu:90-99, 219-230).
__global__ void massive_prepare_kernel(ddx_state s, StepArgs a, MassiveScratch ms, int prec) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n_grav) return;
    const double x = s.x[i], y = s.y[i], z = s.z[i], m = s.m[i];
    const double vx = s.vx[i], vy = s.vy[i], vz = s.vz[i];
    const double x2 = x + vx * a.dt2, y2 = y + vy * a.dt2, z2 = z + vz * a.dt2;
    ms.P[0 * ms.cap + i] = make_body(x, y, z, m);
    ms.P[1 * ms.cap + i] = make_body(x2, y2, z2, m);
    if (prec != DDX_PREC_FP64) {   // the FP32 records of the mixed and compensated dust kernels
        float4 h, l;
        split_hilo(x, h.x, l.x); split_hilo(y, h.y, l.y); split_hilo(z, h.z, l.z);
        split_hilo(m, h.w, l.w);
        ms.Phi[0 * ms.cap + i] = h; ms.Plo[0 * ms.cap + i] = l;
        if (i >= a.n_exact) store_pair_slot(ms, 0, i - a.n_exact, h, l);
        split_hilo(x2, h.x, l.x); split_hilo(y2, h.y, l.y); split_hilo(z2, h.z, l.z);
        ms.Phi[1 * ms.cap + i] = h; ms.Plo[1 * ms.cap + i] = l;
        if (i >= a.n_exact) store_pair_slot(ms, 1, i - a.n_exact, h, l);
        if (i == 0) store_pair_padding(ms, a.n_grav - a.n_exact);
    }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ void kahan_add(float& S, float& C, float v) {
    const float y = v - C;
    const float t = S + y;
    C = (t - S) - y;
    S = t;
}

// Acceleration of body i from body j (FP64): m_j (x_j - x_i)/r^3; zero for coincident
// bodies, like the reference's f != 0 test (src/gpu_functions.cu:156-172).
__device__ __forceinline__ void pair64(const Body pi, const Body pj, double& ax,
                                       double& ay, double& az) {
    const double dX = pj.x - pi.x, dY = pj.y - pi.y, dZ = pj.z - pi.z;
    const double RR = dX * dX + dY * dY + dZ * dZ;
    if (RR > 0.0) {
        const double ri = rsqrt(RR);
        const double f = pj.m * (ri * ri * ri);
        ax = fma(f, dX, ax); ay = fma(f, dY, ay); az = fma(f, dZ, az);
    }
}

// Same in FP32 on hi/lo split positions: the difference (hi_j - hi_i) + (lo_j - lo_i)
// keeps FP32 relative precision in the separation even when |x| >> |x_j - x_i|.  Returns
// true, adding nothing, when the source lies within the near radius (reciprocal distance
// above inv_near): the caller takes that pull in FP64.
__device__ __forceinline__ bool pair32(const float4 hi, const float4 li, const float4 hj,
                                       const float4 lj, float inv_near, float& fx, float& fy, float& fz) {
    const float dX = (hj.x - hi.x) + (lj.x - li.x);
    const float dY = (hj.y - hi.y) + (lj.y - li.y);
    const float dZ = (hj.z - hi.z) + (lj.z - li.z);
    const float RR = fmaf(dX, dX, fmaf(dY, dY, dZ * dZ));
    if (RR > 0.f) {
        const float ri = rsqrtf(RR);
        if (ri > inv_near) return true;
        const float f = hj.w * (ri * (ri * ri));
        fx = fmaf(f, dX, fx); fy = fmaf(f, dY, fy); fz = fmaf(f, dZ, fz);
    }
    return false;
}

// One warp per target body i, lanes stride over the sources, fixed-order butterfly
// reduction (deterministic).  Evaluates the accelerations at two stages sa, sb at once.
// In the mixed path the star's own acceleration and every pull of the star or a planet
// (sources 0..n_exact-1) stay FP64; the pulls of the planetesimals run in FP32 with a
// per-lane Kahan sum.
template <int PREC>
__device__ __forceinline__ void massive_two_stage_accel(const MassiveScratch& ms, int ng, int n_exact, float near_eta,
                                                         int i, int sa, int sb, double a_out[6]) {
    const int lane = threadIdx.x & 31;
    double ax = 0, ay = 0, az = 0, bx = 0, by = 0, bz = 0;
    const Body pa = ms.P[sa * ms.cap + i];
    const Body pb = ms.P[sb * ms.cap + i];
    if (PREC == DDX_PREC_FP64) {
        for (int j = lane; j < ng; j += 32) {
            if (j == i) continue;
            pair64(pa, ms.P[sa * ms.cap + j], ax, ay, az);
            pair64(pb, ms.P[sb * ms.cap + j], bx, by, bz);
        }
    } else {
        float Sa[3] = {0.f, 0.f, 0.f}, Ca[3] = {0.f, 0.f, 0.f};
        float Sb[3] = {0.f, 0.f, 0.f}, Cb[3] = {0.f, 0.f, 0.f};
        const float4 ha = ms.Phi[sa * ms.cap + i], la = ms.Plo[sa * ms.cap + i];
        const float4 hb = ms.Phi[sb * ms.cap + i], lb = ms.Plo[sb * ms.cap + i];
        const float inv_a = near_inv(near_eta, fmaxf(fabsf(ha.x), fmaxf(fabsf(ha.y), fabsf(ha.z))));
        const float inv_b = near_inv(near_eta, fmaxf(fabsf(hb.x), fmaxf(fabsf(hb.y), fabsf(hb.z))));
        for (int j = lane; j < ng; j += 32) {
            if (j == i) continue;
            if (i == 0 || j < n_exact) {
                pair64(pa, ms.P[sa * ms.cap + j], ax, ay, az);
                pair64(pb, ms.P[sb * ms.cap + j], bx, by, bz);
            } else {
                float fx = 0.f, fy = 0.f, fz = 0.f;
                if (pair32(ha, la, ms.Phi[sa * ms.cap + j], ms.Plo[sa * ms.cap + j], inv_a, fx, fy, fz))
                    pair64(pa, ms.P[sa * ms.cap + j], ax, ay, az);   // within the near radius: FP64
                kahan_add(Sa[0], Ca[0], fx); kahan_add(Sa[1], Ca[1], fy); kahan_add(Sa[2], Ca[2], fz);
                fx = fy = fz = 0.f;
                if (pair32(hb, lb, ms.Phi[sb * ms.cap + j], ms.Plo[sb * ms.cap + j], inv_b, fx, fy, fz))
                    pair64(pb, ms.P[sb * ms.cap + j], bx, by, bz);
                kahan_add(Sb[0], Cb[0], fx); kahan_add(Sb[1], Cb[1], fy); kahan_add(Sb[2], Cb[2], fz);
            }
        }
        ax += (double)Sa[0] - (double)Ca[0]; ay += (double)Sa[1] - (double)Ca[1];
        az += (double)Sa[2] - (double)Ca[2];
        bx += (double)Sb[0] - (double)Cb[0]; by += (double)Sb[1] - (double)Cb[1];
        bz += (double)Sb[2] - (double)Cb[2];
    }
    a_out[0] = warp_sum(ax); a_out[1] = warp_sum(ay); a_out[2] = warp_sum(az);
    a_out[3] = warp_sum(bx); a_out[4] = warp_sum(by); a_out[5] = warp_sum(bz);
}

__device__ __forceinline__ void store_stage_pos(MassiveScratch& ms, int stage, int i, double x,
                                                double y, double z, double m, int prec, int n_exact) {
    ms.P[stage * ms.cap + i] = make_body(x, y, z, m);
    if (prec != DDX_PREC_FP64) {
        float4 h, l;
        split_hilo(x, h.x, l.x); split_hilo(y, h.y, l.y); split_hilo(z, h.z, l.z);
        split_hilo(m, h.w, l.w);
        ms.Phi[stage * ms.cap + i] = h; ms.Plo[stage * ms.cap + i] = l;
        if (i >= n_exact) store_pair_slot(ms, stage, i - n_exact, h, l);
    }
}

// Pass 1: A1 at P1, A2 at P2; then R2, P3, R3, P4 for the target
// (src/gpu_functions.cu:219-230, 350-362, 482-493).
__device__ __forceinline__ void pass1_update(const ddx_state& s, const StepArgs& a, MassiveScratch& ms, int i,
                                             const double acc[6], int prec) {
    const int c = ms.cap;
    double* A = ms.A;
    double* R = ms.R;
    A[(0 * 3 + 0) * c + i] = acc[0]; A[(0 * 3 + 1) * c + i] = acc[1]; A[(0 * 3 + 2) * c + i] = acc[2];
    A[(1 * 3 + 0) * c + i] = acc[3]; A[(1 * 3 + 1) * c + i] = acc[4]; A[(1 * 3 + 2) * c + i] = acc[5];
    const double x = s.x[i], y = s.y[i], z = s.z[i], m = s.m[i];
    const double vx = s.vx[i], vy = s.vy[i], vz = s.vz[i];
    const double k2rx = vx + acc[0] * a.dt2, k2ry = vy + acc[1] * a.dt2, k2rz = vz + acc[2] * a.dt2;
    const double k3x = x + k2rx * a.dt2, k3y = y + k2ry * a.dt2, k3z = z + k2rz * a.dt2;
    const double k3rx = vx + acc[3] * a.dt2, k3ry = vy + acc[4] * a.dt2, k3rz = vz + acc[5] * a.dt2;
    const double k4x = x + k3rx * a.dt, k4y = y + k3ry * a.dt, k4z = z + k3rz * a.dt;
    R[(0 * 3 + 0) * c + i] = k2rx; R[(0 * 3 + 1) * c + i] = k2ry; R[(0 * 3 + 2) * c + i] = k2rz;
    R[(1 * 3 + 0) * c + i] = k3rx; R[(1 * 3 + 1) * c + i] = k3ry; R[(1 * 3 + 2) * c + i] = k3rz;
    store_stage_pos(ms, 2, i, k3x, k3y, k3z, m, prec, a.n_exact);
    store_stage_pos(ms, 3, i, k4x, k4y, k4z, m, prec, a.n_exact);
}

// PREC: the arithmetic of the accelerations; STORE: the precision whose stage records
// pass 1 writes (the compensated step integrates the massive set in FP64 and writes the
// FP32 records its dust kernel reads).
template <int PREC, int STORE = PREC>
__global__ void massive_pass1_kernel(ddx_state s, StepArgs a, MassiveScratch ms) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (i >= a.n_grav) return;  // warp-uniform
    double acc[6];
    massive_two_stage_accel<PREC>(ms, a.n_grav, a.n_exact, a.near_eta, i, 0, 1, acc);
    if ((threadIdx.x & 31) != 0) return;
    pass1_update(s, a, ms, i, acc, STORE);
}

// Pass 2: A3 at P3, A4 at P4; R4; final combination (src/gpu_functions.cu:613-625).
// Reads only stage records of other bodies, so updating x, v of the target is safe.
__device__ __forceinline__ void pass2_update(const ddx_state& s, const StepArgs& a, MassiveScratch& ms, int i,
                                             const double acc[6]) {
    const int c = ms.cap;
    double* A = ms.A;
    const double* R = ms.R;
    A[(2 * 3 + 0) * c + i] = acc[0]; A[(2 * 3 + 1) * c + i] = acc[1]; A[(2 * 3 + 2) * c + i] = acc[2];
    A[(3 * 3 + 0) * c + i] = acc[3]; A[(3 * 3 + 1) * c + i] = acc[4]; A[(3 * 3 + 2) * c + i] = acc[5];
    const double vx = s.vx[i], vy = s.vy[i], vz = s.vz[i];
    const double k4rx = vx + acc[0] * a.dt, k4ry = vy + acc[1] * a.dt, k4rz = vz + acc[2] * a.dt;
    const double dt = a.dt6;
    s.x[i] += dt * (vx + 2.0 * R[(0 * 3 + 0) * c + i] + 2.0 * R[(1 * 3 + 0) * c + i] + k4rx);
    s.y[i] += dt * (vy + 2.0 * R[(0 * 3 + 1) * c + i] + 2.0 * R[(1 * 3 + 1) * c + i] + k4ry);
    s.z[i] += dt * (vz + 2.0 * R[(0 * 3 + 2) * c + i] + 2.0 * R[(1 * 3 + 2) * c + i] + k4rz);
    s.vx[i] += dt * (A[(0 * 3 + 0) * c + i] + 2.0 * A[(1 * 3 + 0) * c + i] + 2.0 * acc[0] + acc[3]);
    s.vy[i] += dt * (A[(0 * 3 + 1) * c + i] + 2.0 * A[(1 * 3 + 1) * c + i] + 2.0 * acc[1] + acc[4]);
    s.vz[i] += dt * (A[(0 * 3 + 2) * c + i] + 2.0 * A[(1 * 3 + 2) * c + i] + 2.0 * acc[2] + acc[5]);
}

template <int PREC>
__global__ void massive_pass2_kernel(ddx_state s, StepArgs a, MassiveScratch ms) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (i >= a.n_grav) return;
    double acc[6];
    massive_two_stage_accel<PREC>(ms, a.n_grav, a.n_exact, a.near_eta, i, 2, 3, acc);
    if ((threadIdx.x & 31) != 0) return;
    pass2_update(s, a, ms, i, acc);
}

// ---------------------------------------------------------------------------------------
// Mixed massive passes over source slices
// ---------------------------------------------------------------------------------------
// A few thousand targets leave most of the GPU idle when one warp serves one target, so
// the FP32 pulls of the planetesimals are split over source slices: block (target group of
// kSliceThreads, slice k) stages the slice's pair records of the pass's two stages in
// shared memory, every thread (one target) reads each record at once (broadcast) and
// works on both sources of a record with one f32x2 instruction, in plain sums over spans
// of kPairSpan records with a Kahan sum across spans (the dust kernel's scheme).  A
// target's own slot gives RR = 0 and is masked.  The star (target 0) takes the
// planetesimals' pulls in FP64, in an extra row of blocks that spread each slice over a
// whole block (a fixed-order tree sum).  massive_gather_kernel then adds the slices (a
// fixed lane order: deterministic), adds the FP64 pulls of bodies 0..n_exact-1 and applies
// the pass's update.
constexpr int kSliceTile = 256;       // pair records per stage staged at once (16 KiB)
constexpr int kMaxSlices = 64;

__device__ __forceinline__ void pair_f2(const BodyPair& r, f2 XH, f2 XL, f2 YH, f2 YL, f2 ZH, f2 ZL, f2& px,
                                        f2& py, f2& pz) {
    const ulonglong2 q0 = *reinterpret_cast<const ulonglong2*>(r.hx);   // hx, hy
    const ulonglong2 q1 = *reinterpret_cast<const ulonglong2*>(r.hz);   // hz, m
    const ulonglong2 q2 = *reinterpret_cast<const ulonglong2*>(r.lx);   // lx, ly
    const f2 lz = *reinterpret_cast<const f2*>(r.lz);
    const f2 dX = add2(sub2(q0.x, XH), sub2(q2.x, XL));
    const f2 dY = add2(sub2(q0.y, YH), sub2(q2.y, YL));
    const f2 dZ = add2(sub2(q1.x, ZH), sub2(lz, ZL));
    const f2 RR = fma2(dX, dX, fma2(dY, dY, mul2(dZ, dZ)));
    float r0, r1;
    f2_split(RR, r0, r1);
    const f2 ri = f2_join(r0 > 0.f ? rsqrt_approx(r0) : 0.f, r1 > 0.f ? rsqrt_approx(r1) : 0.f);
    const f2 f = mul2(mul2(q1.y, ri), mul2(ri, ri));
    px = fma2(f, dX, px); py = fma2(f, dY, py); pz = fma2(f, dZ, pz);
}

// pair_f2 that also raises mx to the larger reciprocal distance of the two sources (0 for
// a coincident source, the target's own slot included, so it never counts as near).
__device__ __forceinline__ void pair_f2_max(const BodyPair& r, f2 XH, f2 XL, f2 YH, f2 YL, f2 ZH, f2 ZL, f2& px,
                                            f2& py, f2& pz, float& mx) {
    const ulonglong2 q0 = *reinterpret_cast<const ulonglong2*>(r.hx);   // hx, hy
    const ulonglong2 q1 = *reinterpret_cast<const ulonglong2*>(r.hz);   // hz, m
    const ulonglong2 q2 = *reinterpret_cast<const ulonglong2*>(r.lx);   // lx, ly
    const f2 lz = *reinterpret_cast<const f2*>(r.lz);
    const f2 dX = add2(sub2(q0.x, XH), sub2(q2.x, XL));
    const f2 dY = add2(sub2(q0.y, YH), sub2(q2.y, YL));
    const f2 dZ = add2(sub2(q1.x, ZH), sub2(lz, ZL));
    const f2 RR = fma2(dX, dX, fma2(dY, dY, mul2(dZ, dZ)));
    float r0, r1;
    f2_split(RR, r0, r1);
    const float i0 = r0 > 0.f ? rsqrt_approx(r0) : 0.f, i1 = r1 > 0.f ? rsqrt_approx(r1) : 0.f;
    mx = fmax3(mx, i0, i1);
    const f2 ri = f2_join(i0, i1);
    const f2 f = mul2(mul2(q1.y, ri), mul2(ri, ri));
    px = fma2(f, dX, px); py = fma2(f, dY, py); pz = fma2(f, dZ, pz);
}

// One span of kPairSpan pair records (slots q0 ..) summed again for a target with a source
// within the near radius (reciprocal FP32 distance above inv_near): the FP32 partial sum of
// the other sources, with the same operations as pair_f2_max, and the FP64 pull of each near
// source from the FP64 stage records (P: bodies n_exact.. of the stage; src: source of each
// slot, null when slot q holds source q) on the target's FP64 stage position pt, added to n.
// The target's own slot is never near (its reciprocal distance is 0).
__device__ __forceinline__ void near_span_massive(const BodyPair* R, int q0, f2 XH, f2 XL, f2 YH, f2 YL, f2 ZH,
                                                  f2 ZL, float inv_near, const Body pt, const Body* __restrict__ P,
                                                  const int* __restrict__ src, f2& px, f2& py, f2& pz,
                                                  double n[3]) {
    px = 0; py = 0; pz = 0;
    for (int u = 0; u < kPairSpan; ++u) {
        const BodyPair& r = R[u];
        const ulonglong2 q0v = *reinterpret_cast<const ulonglong2*>(r.hx);
        const ulonglong2 q1v = *reinterpret_cast<const ulonglong2*>(r.hz);
        const ulonglong2 q2v = *reinterpret_cast<const ulonglong2*>(r.lx);
        const f2 lz = *reinterpret_cast<const f2*>(r.lz);
        const f2 dX = add2(sub2(q0v.x, XH), sub2(q2v.x, XL));
        const f2 dY = add2(sub2(q0v.y, YH), sub2(q2v.y, YL));
        const f2 dZ = add2(sub2(q1v.x, ZH), sub2(lz, ZL));
        const f2 RR = fma2(dX, dX, fma2(dY, dY, mul2(dZ, dZ)));
        float r0, r1;
        f2_split(RR, r0, r1);
        const float i0 = r0 > 0.f ? rsqrt_approx(r0) : 0.f, i1 = r1 > 0.f ? rsqrt_approx(r1) : 0.f;
        const bool n0 = i0 > inv_near, n1 = i1 > inv_near;
        const f2 ri = f2_join(n0 ? 0.f : i0, n1 ? 0.f : i1);
        const f2 f = mul2(mul2(q1v.y, ri), mul2(ri, ri));
        px = fma2(f, dX, px); py = fma2(f, dY, py); pz = fma2(f, dZ, pz);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if (!(h ? n1 : n0)) continue;
            const int q = q0 + 2 * u + h;
            pair64(pt, P[src ? src[q] : q], n[0], n[1], n[2]);
        }
    }
}

// Deterministic block sum of v (fixed tree order); the result in thread 0.
__device__ __forceinline__ double block_sum(double v, double* red) {
    red[threadIdx.x] = v;
    __syncthreads();
    for (int o = kSliceThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    const double r = red[0];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kSliceThreads)
massive_slice_kernel(StepArgs a, MassiveScratch ms, int sa, int per, int np, double* __restrict__ part) {
    __shared__ __align__(16) BodyPair tile[2][kSliceTile];
    const int k = blockIdx.y;
    const int sb = sa + 1;
    const int n_src = a.n_grav - a.n_exact;
    const int npairs = pair_count(n_src);
    const int r0 = k * per, r1 = min(r0 + per, npairs);
    const int c = ms.cap;
    if (blockIdx.x == gridDim.x - 1) {
        // the star's row: the whole block takes the slice's planetesimals in FP64
        const Body pa = ms.P[sa * c], pb = ms.P[sb * c];
        double d[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        const int q1 = min(2 * r1, n_src);
        for (int q = 2 * r0 + threadIdx.x; q < q1; q += kSliceThreads) {
            pair64(pa, ms.P[sa * c + a.n_exact + q], d[0], d[1], d[2]);
            pair64(pb, ms.P[sb * c + a.n_exact + q], d[3], d[4], d[5]);
        }
        double* red = reinterpret_cast<double*>(&tile[0][0]);     // 2 KiB of the tile space
        double* o = part + (size_t)k * 6 * np;
        for (int q = 0; q < 6; ++q) {
            const double t = block_sum(d[q], red);
            if (threadIdx.x == 0) o[(size_t)q * np] = t;
        }
        return;
    }
    const int i = blockIdx.x * kSliceThreads + threadIdx.x;
    const bool active = i > 0 && i < a.n_grav;                   // the star has its own row
    float4 ha = make_float4(0.f, 0.f, 0.f, 0.f), la = ha, hb = ha, lb = ha;
    if (active) {
        ha = ms.Phi[sa * c + i]; la = ms.Plo[sa * c + i];
        hb = ms.Phi[sb * c + i]; lb = ms.Plo[sb * c + i];
    }
    const f2 XHa = f2_dup(ha.x), XLa = f2_dup(la.x), YHa = f2_dup(ha.y), YLa = f2_dup(la.y);
    const f2 ZHa = f2_dup(ha.z), ZLa = f2_dup(la.z);
    const f2 XHb = f2_dup(hb.x), XLb = f2_dup(lb.x), YHb = f2_dup(hb.y), YLb = f2_dup(lb.y);
    const f2 ZHb = f2_dup(hb.z), ZLb = f2_dup(lb.z);
    f2 SA[3] = {0, 0, 0}, CA[3] = {0, 0, 0}, SB[3] = {0, 0, 0}, CB[3] = {0, 0, 0};
    // near sources: FP64 pulls, summed apart and added to the slice's total
    const float inv_a = near_inv(a.near_eta, fmaxf(fabsf(ha.x), fmaxf(fabsf(ha.y), fabsf(ha.z))));
    const float inv_b = near_inv(a.near_eta, fmaxf(fabsf(hb.x), fmaxf(fabsf(hb.y), fabsf(hb.z))));
    double NA[3] = {0.0, 0.0, 0.0}, NB[3] = {0.0, 0.0, 0.0};
    for (int t0 = r0; t0 < r1; t0 += kSliceTile) {
        const int cnt = min(kSliceTile, r1 - t0);          // a multiple of kPairSpan
        __syncthreads();                                   // the previous tile is consumed
        const uint4* ga = reinterpret_cast<const uint4*>(ms.PP + (size_t)sa * ms.pcap + t0);
        const uint4* gb = reinterpret_cast<const uint4*>(ms.PP + (size_t)sb * ms.pcap + t0);
        uint4* ta = reinterpret_cast<uint4*>(tile[0]);
        uint4* tb = reinterpret_cast<uint4*>(tile[1]);
        for (int w = threadIdx.x; w < cnt * 4; w += kSliceThreads) {
            ta[w] = ga[w];
            tb[w] = gb[w];
        }
        __syncthreads();
        if (!active) continue;
        for (int u0 = 0; u0 < cnt; u0 += kPairSpan) {
            f2 ax = 0, ay = 0, az = 0, bx = 0, by = 0, bz = 0;
            float mxa = 0.f, mxb = 0.f;
#pragma unroll 4
            for (int u = 0; u < kPairSpan; ++u) {
                pair_f2_max(tile[0][u0 + u], XHa, XLa, YHa, YLa, ZHa, ZLa, ax, ay, az, mxa);
                pair_f2_max(tile[1][u0 + u], XHb, XLb, YHb, YLb, ZHb, ZLb, bx, by, bz, mxb);
            }
            if (mxa > inv_a)   // rare: a source of this span within the near radius at stage sa
                near_span_massive(&tile[0][u0], 2 * (t0 + u0), XHa, XLa, YHa, YLa, ZHa, ZLa, inv_a, ms.P[sa * c + i],
                                  ms.P + (size_t)sa * c + a.n_exact, ms.slot ? ms.src : nullptr, ax, ay, az, NA);
            if (mxb > inv_b)
                near_span_massive(&tile[1][u0], 2 * (t0 + u0), XHb, XLb, YHb, YLb, ZHb, ZLb, inv_b, ms.P[sb * c + i],
                                  ms.P + (size_t)sb * c + a.n_exact, ms.slot ? ms.src : nullptr, bx, by, bz, NB);
            kahan2(SA[0], CA[0], ax); kahan2(SA[1], CA[1], ay); kahan2(SA[2], CA[2], az);
            kahan2(SB[0], CB[0], bx); kahan2(SB[1], CB[1], by); kahan2(SB[2], CB[2], bz);
        }
    }
    if (!active) return;
    double* o = part + (size_t)k * 6 * np + i;
    o[0] = f2_total(SA[0], CA[0]) + NA[0]; o[np] = f2_total(SA[1], CA[1]) + NA[1];
    o[2 * np] = f2_total(SA[2], CA[2]) + NA[2];
    o[3 * np] = f2_total(SB[0], CB[0]) + NB[0]; o[4 * np] = f2_total(SB[1], CB[1]) + NB[1];
    o[5 * np] = f2_total(SB[2], CB[2]) + NB[2];
}

// 32 targets per block of 8 warps.  Each warp adds the slices of 4 targets (the lanes take
// slices lane, lane + 32, ..., a fixed butterfly adds the lanes: the same order on every
// run); then warp 0 finishes the 32 targets, one per lane, so the FP64 update runs on full
// warps.
constexpr int kGatherTargets = 32;
constexpr int kGatherThreads = 256;

template <int PASS>
__global__ void __launch_bounds__(kGatherThreads)
massive_gather_kernel(ddx_state s, StepArgs a, MassiveScratch ms, int slices, int np,
                      const double* __restrict__ part) {
    __shared__ double sums[kGatherTargets][6];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i0 = blockIdx.x * kGatherTargets;
    constexpr int per_warp = kGatherTargets / (kGatherThreads / 32);
    for (int t = warp * per_warp; t < (warp + 1) * per_warp; ++t) {
        const int it = i0 + t;
        double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        if (it < a.n_grav)
            for (int k = lane; k < slices; k += 32)
#pragma unroll
                for (int q = 0; q < 6; ++q) acc[q] += part[((size_t)k * 6 + q) * np + it];
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const double v = warp_sum(acc[q]);
            if (lane == 0) sums[t][q] = v;
        }
    }
    __syncthreads();
    if (warp != 0) return;
    const int i = i0 + lane;
    if (i >= a.n_grav) return;
    const int c = ms.cap;
    const int sa = PASS == 1 ? 0 : 2, sb = sa + 1;
    double acc[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) acc[q] = sums[lane][q];
    const Body pa = ms.P[sa * c + i], pb = ms.P[sb * c + i];
    for (int j = 0; j < a.n_exact && j < a.n_grav; ++j) {
        if (j == i) continue;
        pair64(pa, ms.P[sa * c + j], acc[0], acc[1], acc[2]);
        pair64(pb, ms.P[sb * c + j], acc[3], acc[4], acc[5]);
    }
    if (PASS == 1) pass1_update(s, a, ms, i, acc, DDX_PREC_MIXED);
    else pass2_update(s, a, ms, i, acc);
}

// ---------------------------------------------------------------------------------------
// Dust tracers
// ---------------------------------------------------------------------------------------

// Variants of the dust kernel.
enum DustVariant {
    kDustFP64Exact = 0,  // reference arithmetic expression for expression: m/RR/sqrt(RR)
    kDustFP64 = 1,       // FP64 with rsqrt
};

constexpr int kDustThreads = 256;
constexpr int kDustTile = 1024;    // sources per shared-memory tile (32 KiB)

// FP64 gravity of massive bodies 1..n_grav-1 at stage `st` on every tracer of the block.
// Sources are staged through shared memory tile by tile; every thread of the block takes
// part in the loads and barriers whether or not its tracer is still alive.
// Returns false (for the calling thread) on an exact coincidence with a body.
template <int VAR>
__device__ __forceinline__ bool dust_perturb(const MassiveScratch& ms, int ng, int st, bool alive,
                                             double xt, double yt, double zt, double& kx,
                                             double& ky, double& kz, unsigned char* smem) {
    const int nsrc = ng - 1;
    bool ok = true;
    {
        Body* sP = reinterpret_cast<Body*>(smem);
        for (int base = 0; base < nsrc; base += kDustTile) {
            const int cnt = min(kDustTile, nsrc - base);
            __syncthreads();
            for (int k = threadIdx.x; k < cnt; k += blockDim.x)
                sP[k] = ms.P[st * ms.cap + 1 + base + k];
            __syncthreads();
            if (alive && ok) {
                if (VAR == kDustFP64Exact) {
                    // src/gpu_functions.cu:722-735, in order, with its early exit.
                    for (int k = 0; k < cnt; ++k) {
                        const Body p = sP[k];
                        const double dx = xt - p.x, dy = yt - p.y, dz = zt - p.z;
                        const double RR = dx * dx + dy * dy + dz * dz;
                        if (RR == 0) { ok = false; break; }
                        const double f = p.m / RR / sqrt(RR);
                        kx += -f * dx; ky += -f * dy; kz += -f * dz;
                    }
                } else {
#pragma unroll 4
                    for (int k = 0; k < cnt; ++k) {
                        const Body p = sP[k];
                        const double dx = xt - p.x, dy = yt - p.y, dz = zt - p.z;
                        const double RR = dx * dx + dy * dy + dz * dz;
                        const double ri = rsqrt(RR);
                        const double f = p.m * (ri * ri * ri);
                        kx = fma(-f, dx, kx); ky = fma(-f, dy, ky); kz = fma(-f, dz, kz);
                    }
                }
            }
        }
        if (VAR == kDustFP64 && alive && !(isfinite(kx) && isfinite(ky) && isfinite(kz))) ok = false;
    }
    return ok;
}

// Full RK4 of one dust tracer per thread (src/gpu_functions.cu:627-943).
template <int VAR>
__global__ void __launch_bounds__(kDustThreads)
dust_rk4_kernel(ddx_state s, StepArgs a, MassiveScratch ms, const SizeBin* __restrict__ bins) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
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
    const double dt = a.dt, dt2 = a.dt / 2.0, dt6 = a.dt / 6.0;
    double k1vx = 0, k1vy = 0, k1vz = 0, k2vx = 0, k2vy = 0, k2vz = 0;
    double k3vx = 0, k3vy = 0, k3vz = 0, k4vx = 0, k4vy = 0, k4vz = 0;
    double k2rx = 0, k2ry = 0, k2rz = 0, k3rx = 0, k3ry = 0, k3rz = 0;
    double k4rx = 0, k4ry = 0, k4rz = 0;
    int removed = 0;  // 1: sublimated (stage kept in removed_stage), 2: coincidence
    int removed_stage = -1;

#pragma unroll 1
    for (int st = 0; st < 4; ++st) {
        double xt, yt, zt, rx, ry, rz;
        if (st == 0)      { xt = x; yt = y; zt = z; rx = vx; ry = vy; rz = vz; }
        else if (st == 1) {
            k2rx = vx + k1vx * dt2; k2ry = vy + k1vy * dt2; k2rz = vz + k1vz * dt2;
            xt = x + vx * dt2; yt = y + vy * dt2; zt = z + vz * dt2;
            rx = k2rx; ry = k2ry; rz = k2rz;
        } else if (st == 2) {
            k3rx = vx + k2vx * dt2; k3ry = vy + k2vy * dt2; k3rz = vz + k2vz * dt2;
            xt = x + k2rx * dt2; yt = y + k2ry * dt2; zt = z + k2rz * dt2;
            rx = k3rx; ry = k3ry; rz = k3rz;
        } else {
            k4rx = vx + k3vx * dt; k4ry = vy + k3vy * dt; k4rz = vz + k3vz * dt;
            xt = x + k3rx * dt; yt = y + k3ry * dt; zt = z + k3rz * dt;
            rx = k4rx; ry = k4ry; rz = k4rz;
        }
        double kx = 0, ky = 0, kz = 0;
        if (alive) {
            const Body ps = ms.P[st * ms.cap + 0];
            if (!star_term(xt - ps.x, yt - ps.y, zt - ps.z, rx, ry, rz, ps.m, bet, betsw, qe, m,
                           a, kx, ky, kz)) {
                alive = false; removed = 1; removed_stage = st;
            }
        }
        if (!dust_perturb<VAR>(ms, ng, st, alive, xt, yt, zt, kx, ky, kz, smem)) {
            alive = false; removed = 2; removed_stage = st;
        }
        if (st == 0)      { k1vx = kx; k1vy = ky; k1vz = kz; }
        else if (st == 1) { k2vx = kx; k2vy = ky; k2vz = kz; }
        else if (st == 2) { k3vx = kx; k3vy = ky; k3vz = kz; }
        else              { k4vx = kx; k4vy = ky; k4vz = kz; }
    }
    if (i >= a.n_dust) return;
    if (removed) {
        // src/gpu_functions.cu:878 zeroes N[i] (i is the dust-relative index) on a stage-4
        // sublimation and leaves the grain alive; DDX_MODE_REFERENCE reproduces it.
        if (removed == 1 && removed_stage == 3 && a.mode == DDX_MODE_REFERENCE) s.N[i] = 0;
        else s.N[t] = 0;
        return;
    }
    if (!alive) return;
    x += dt6 * (vx + 2.0 * (k2rx + k3rx) + k4rx);
    y += dt6 * (vy + 2.0 * (k2ry + k3ry) + k4ry);
    z += dt6 * (vz + 2.0 * (k2rz + k3rz) + k4rz);
    vx += dt6 * (k1vx + 2.0 * (k2vx + k3vx) + k4vx);
    vy += dt6 * (k1vy + 2.0 * (k2vy + k3vy) + k4vy);
    vz += dt6 * (k1vz + 2.0 * (k2vz + k3vz) + k4vz);
    s.x[t] = x; s.y[t] = y; s.z[t] = z;
    s.vx[t] = vx; s.vy[t] = vy; s.vz[t] = vz;
}

// ---------------------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------------------

cudaError_t launch_massive_prepare(const ddx_state& s, const StepArgs& a, MassiveScratch& ms,
                                   int precision, cudaStream_t st) {
    // the FP32 sources' pair slots in cell order, from their positions at the start of the step
    if (precision != DDX_PREC_FP64 && ms.slot && spatial_order_on(a)) {
        const cudaError_t e =
            order_bodies(s, a.n_exact, a.n_grav - a.n_exact, false, ms.src_order, nullptr, ms.slot,
                         precision == DDX_PREC_MIXED, st);
        if (e != cudaSuccess) return e;
    }
    const int threads = 128;
    const int blocks = (a.n_grav + threads - 1) / threads;
    massive_prepare_kernel<<<blocks, threads, 0, st>>>(s, a, slotted(ms, a), precision);
    return cudaGetLastError();
}

namespace {
int sm_count() {
    static int cached[128] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 128) return 152;
    if (!cached[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) n = 152;
        cached[dev] = n;
    }
    return cached[dev];
}

// The sliced mixed pass: slice sums, then their gather with the pass's update.
// Slice sums are stored [slice][component][np] with np = n_grav rounded up to a block.
int slice_stride(int n_grav) { return (n_grav + kSliceThreads - 1) / kSliceThreads * kSliceThreads; }

bool sliced_fits(const StepArgs& a, const MassiveScratch& ms) {
    return ms.part && ms.part_words >= (long long)massive_slices(a.n_grav, a.n_exact) * 6 * slice_stride(a.n_grav);
}

template <int PASS>
cudaError_t launch_sliced(const ddx_state& s, const StepArgs& a, MassiveScratch& ms, cudaStream_t st) {
    const int spans = pair_count(a.n_grav - a.n_exact) / kPairSpan;
    const int S = spans > 0 ? massive_slices(a.n_grav, a.n_exact) : 0;    // no planetesimals: no slices
    const int np = slice_stride(a.n_grav);
    if (S > 0) {
        const int per = (spans + S - 1) / S * kPairSpan;
        const dim3 grid((a.n_grav + kSliceThreads - 1) / kSliceThreads + 1, S);   // + the star's row
        massive_slice_kernel<<<grid, kSliceThreads, 0, st>>>(a, slotted(ms, a), PASS == 1 ? 0 : 2, per, np, ms.part);
    }
    massive_gather_kernel<PASS><<<(a.n_grav + kGatherTargets - 1) / kGatherTargets, kGatherThreads, 0, st>>>(
        s, a, slotted(ms, a), S, np, ms.part);
    return cudaGetLastError();
}
}  // namespace

int massive_slices(int n_grav, int n_exact) {
    const int groups = (n_grav + kSliceThreads - 1) / kSliceThreads;
    const int spans = pair_count(n_grav - n_exact) / kPairSpan;
    int S = (kSliceBlocksPerSM * sm_count() + groups - 1) / groups;
    if (S > kMaxSlices) S = kMaxSlices;
    if (S > spans) S = spans;
    return S < 1 ? 1 : S;
}

// The bound grows with the groups, so the bound at the capacity covers every smaller system.
long long massive_part_words(int cap) { return massive_part_words_for(cap, sm_count()); }

cudaError_t launch_massive_pass1(const ddx_state& s, const StepArgs& a, MassiveScratch& ms,
                                 int precision, cudaStream_t st) {
    if (precision == DDX_PREC_MIXED && sliced_fits(a, ms)) return launch_sliced<1>(s, a, ms, st);
    const int threads = 128;  // 4 targets per block
    const int blocks = (a.n_grav * 32 + threads - 1) / threads;
    if (precision == DDX_PREC_COMPENSATED)   // the massive set in FP64
        massive_pass1_kernel<DDX_PREC_FP64, DDX_PREC_MIXED><<<blocks, threads, 0, st>>>(s, a, slotted(ms, a));
    else if (precision == DDX_PREC_MIXED)
        massive_pass1_kernel<DDX_PREC_MIXED><<<blocks, threads, 0, st>>>(s, a, slotted(ms, a));
    else massive_pass1_kernel<DDX_PREC_FP64><<<blocks, threads, 0, st>>>(s, a, ms);
    return cudaGetLastError();
}

cudaError_t launch_massive_pass2(const ddx_state& s, const StepArgs& a, MassiveScratch& ms,
                                 int precision, cudaStream_t st) {
    if (precision == DDX_PREC_MIXED && sliced_fits(a, ms)) return launch_sliced<2>(s, a, ms, st);
    const int threads = 128;
    const int blocks = (a.n_grav * 32 + threads - 1) / threads;
    if (precision == DDX_PREC_COMPENSATED)
        massive_pass2_kernel<DDX_PREC_FP64><<<blocks, threads, 0, st>>>(s, a, ms);
    else if (precision == DDX_PREC_MIXED)
        massive_pass2_kernel<DDX_PREC_MIXED><<<blocks, threads, 0, st>>>(s, a, slotted(ms, a));
    else massive_pass2_kernel<DDX_PREC_FP64><<<blocks, threads, 0, st>>>(s, a, ms);
    return cudaGetLastError();
}

int dust_block_threads(int n_dust) {
    static int sm_count[128] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 128) return kDustThreads;
    if (sm_count[dev] == 0) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 1;
        sm_count[dev] = n;
    }
    int threads = kDustThreads;
    while (threads > 64 && (n_dust + threads - 1) / threads < 2 * sm_count[dev]) threads /= 2;
    return threads;
}

cudaError_t launch_dust(const ddx_state& s, const StepArgs& a, const MassiveScratch& ms,
                        const SizeBin* bins, int precision, cudaStream_t st) {
    if (a.n_dust <= 0) return cudaSuccess;
    const int threads = dust_block_threads(a.n_dust);
    const int blocks = (a.n_dust + threads - 1) / threads;
    const size_t smem = (size_t)kDustTile * 32;
    if (precision == DDX_PREC_MIXED || precision == DDX_PREC_COMPENSATED) {
        return launch_dust_mixed(s, a, ms, bins, precision, st);
    } else if (a.mode == DDX_MODE_REFERENCE) {
        dust_rk4_kernel<kDustFP64Exact><<<blocks, threads, smem, st>>>(s, a, ms, bins);
    } else {
        dust_rk4_kernel<kDustFP64><<<blocks, threads, smem, st>>>(s, a, ms, bins);
    }
    return cudaGetLastError();
}

}  // namespace ddx
