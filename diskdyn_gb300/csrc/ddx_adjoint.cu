// Discrete adjoint of the RK4 trajectory and of a differentiable image, in FP64.
// No counterpart in the reference.
//
// Model (the forward these kernels differentiate exactly):
//  - massive set (star at 0): the reference's RK4 with all-pairs gravity
//    (src/gpu_functions.cu:71-625), integrated first for every step, keeping the stage
//    positions P_s(n) of every step: up to 32 bodies by one single-warp kernel for all
//    steps, larger sets (the planetesimals of a dusty ring) by three launches per step, a
//    warp per body;
//  - dust tracers: the reference's RK4 (src/gpu_functions.cu:627-943) under the star term
//    (gravity reduced by beta + beta_sw, PR + stellar-wind drag, the Lorentz force) and the
//    gravity of every massive body at its stage positions.  Tracers are independent
//    given P_s(n), so each thread integrates its tracer over all steps in one launch;
//  - image: the flux of src/gpu_functions.cu:1049-1078 deposited with bilinear weights
//    on the four pixel centres around the projected position, so the image, and the L2
//    loss on it, are continuous and piecewise differentiable in every position (the
//    reference's nearest-pixel binning has a zero gradient almost everywhere).
//
// Backward (checkpoint-and-recompute every K steps):
//  1. image adjoint: dL/dimage -> adjoint of the final tracer positions;
//  2. per segment, last first: recompute the K steps from the checkpoint (the forward
//     already kept the last segment), storing each step's state, stage accelerations
//     a1..a3 and the stages' reciprocal distances (31 doubles per tracer per step for three
//     bodies); reverse sweep of the four RK4 stages per tracer with analytic
//     vector-Jacobian products of the star term and the body gravity; the adjoints of the
//     bodies' stage positions and masses are reduced per block in a fixed order (a
//     transposed shared-memory tile per warp, then the warps, then block partials summed
//     in block order), so the gradient is deterministic; a single-warp kernel then runs
//     the reverse sweep of the massive set.  With more than 32 bodies the sweep runs one
//     launch per step: the block sums of the bodies' adjoints cover that step (a 32 x 32
//     transpose per warp, then the warps in order), are reduced in block order, and the
//     massive set's reverse runs stage by stage, a warp per body.
// FP64 runs at ~1/75 of the FP32 rate here, so the kernels are bound by their count of
// FP64 operations: the forward takes one division and one square root for the star and
// one rsqrt per body per stage, and the reverse reuses them from the record.
// Tracers removed during the forward (N = 0) or without optical data emit nothing, so
// their adjoint is zero and they are skipped.
#include "ddx_internal.cuh"
#include "ddx_flux.cuh"

namespace ddx {
namespace {

// Massive sets up to this size run the one-warp kernels (every step in one launch); larger
// ones the launch-per-pass kernels of the "large massive sets" section.
constexpr int kMaxGrav = 32;
constexpr int kThreads = 128;
constexpr int kWarps = kThreads / 32;
constexpr int kSegComp = 15;   // per tracer per step: x, y, z, vx, vy, vz, a1, a2, a3
constexpr int kMaxStoredIr = 3; // bodies whose 1/|e| the recompute keeps (n_grav <= 4)

struct AdjArgs {
    int ng, nd;
    int nir;                // bodies 1..nir have their 1/|e| kept per stage
    int ncomp;              // doubles per tracer per step in the recompute record
    double dt;
    StepArgs sa;            // star-term constants (FLQ = 0)
    const Body* Ps;         // [n_steps][4][ng]
    const SizeBin* bins;
    const int* id;          // [nd]
    const double* mass;     // [nd] tracer masses (the Lorentz force divides by them)
};


// Per-tracer constants of the star term: a = -Fg d - Fb1 (Fb2 d + r) with
// Fg = g0/R^3, Fb1 = c1/R^2, Fb2 = (d.r)/R^2 (src/gpu_functions.cu:691-704).
// Lorentz force (FLQ = 1, src/gpu_functions.cu:706-713): Fl = cL iR3 (ry - Wz dx, -(rx + Wz dy), 0)
// with cL = q Bstar Rstar^3 / m of the tracer (0 without the force).
struct StarConst {
    double g0, c1, inv_m0, cL;
};
__device__ __forceinline__ StarConst star_const(const AdjArgs& A, double m0, float bet, float betsw, float qe,
                                                double m) {
    StarConst k;
    k.g0 = (1.0 - bet - betsw) * m0;
    k.c1 = (A.sa.SWQ == 1) ? m0 * (bet / kLightAU + betsw / A.sa.vswAU) : bet * m0 / kLightAU;
    k.inv_m0 = 1.0 / m0;
    // a tracer without mass feels no Lorentz force here (the reference would divide by zero)
    k.cL = A.sa.FLQ == 1 && m > 0.0 ? (double)qe * A.sa.Bstar * A.sa.Rstar * A.sa.Rstar * A.sa.Rstar / m : 0.0;
    return k;
}

// Acceleration of a tracer at (x, r) for the stage whose body records are P[0..ng), with one
// square root and one division for the star and one rsqrt per body.  Returns false on
// sublimation (R <= Rmin) or an exact coincidence with a body.  rc (optional, stride rs):
// receives 1/R^2 and 1/R of the star and 1/|e| of bodies 1..nir, which the reverse sweep
// reuses instead of dividing and taking roots again (FP64 division and square root are
// ~9 dependent FP64 operations each, on a pipe 75x slower than FP32).
__device__ __forceinline__ bool tracer_accel(const AdjArgs& A, const StarConst& K, const Body* P, double x,
                                             double y, double z, double rx, double ry, double rz,
                                             double& ax, double& ay, double& az, double* rc, size_t rs) {
    const double dx = x - P[0].x, dy = y - P[0].y, dz = z - P[0].z;
    const double RR = dx * dx + dy * dy + dz * dz;
    if (RR <= A.sa.Rmin * A.sa.Rmin) return false;
    const double iRR = 1.0 / RR;
    const double iR = sqrt(iRR);
    const double iR3 = iR * iRR;
    if (rc) { rc[0] = iRR; rc[rs] = iR; }
    const double Fg = K.g0 * iR3, Fb1 = K.c1 * iRR, Fb2 = (dx * rx + dy * ry + dz * rz) * iRR;
    ax = -Fg * dx - Fb1 * (Fb2 * dx + rx);
    ay = -Fg * dy - Fb1 * (Fb2 * dy + ry);
    az = -Fg * dz - Fb1 * (Fb2 * dz + rz);
    if (K.cL != 0.0) {
        ax += K.cL * iR3 * (ry - A.sa.Wz * dx);
        ay -= K.cL * iR3 * (rx + A.sa.Wz * dy);
    }
    for (int j = 1; j < A.ng; ++j) {
        const double ex = P[j].x - x, ey = P[j].y - y, ez = P[j].z - z;
        const double R2 = ex * ex + ey * ey + ez * ez;
        if (R2 == 0.0) return false;
        const double ir = rsqrt(R2);
        if (rc && j <= A.nir) rc[(1 + j) * rs] = ir;
        const double f = P[j].m * (ir * ir * ir);
        ax += f * ex; ay += f * ey; az += f * ez;
    }
    return true;
}

// ---------------------------------------------------------------------------------------
// Massive set: forward trajectory and reverse sweep (one warp, one body per lane)
// ---------------------------------------------------------------------------------------

__device__ __forceinline__ void massive_acc(const double (*sp)[4], int ng, int j, double& ax, double& ay,
                                            double& az) {
    ax = ay = az = 0.0;
    for (int k = 0; k < ng; ++k) {
        if (k == j) continue;
        const double dx = sp[k][0] - sp[j][0], dy = sp[k][1] - sp[j][1], dz = sp[k][2] - sp[j][2];
        const double RR = dx * dx + dy * dy + dz * dz;
        if (RR > 0.0) {
            const double f = sp[k][3] / (RR * sqrt(RR));
            ax += f * dx; ay += f * dy; az += f * dz;
        }
    }
}

__global__ void massive_traj_kernel(int ng, int n_steps, double dt, double* xv, Body* Ps) {
    __shared__ double sp[kMaxGrav][4];
    const int j = threadIdx.x;
    const bool on = j < ng;
    double x = 0, y = 0, z = 0, vx = 0, vy = 0, vz = 0, m = 0;
    if (on) {
        x = xv[0 * ng + j]; y = xv[1 * ng + j]; z = xv[2 * ng + j];
        vx = xv[3 * ng + j]; vy = xv[4 * ng + j]; vz = xv[5 * ng + j]; m = xv[6 * ng + j];
    }
    const double h2 = dt * 0.5, d6 = dt / 6.0;
    for (int n = 0; n < n_steps; ++n) {
        double px[4], py[4], pz[4], ax[4], ay[4], az[4];
        double r2x = 0, r2y = 0, r2z = 0, r3x = 0, r3y = 0, r3z = 0, r4x = 0, r4y = 0, r4z = 0;
        for (int s = 0; s < 4; ++s) {
            if (s == 0) { px[0] = x; py[0] = y; pz[0] = z; }
            else if (s == 1) {
                r2x = vx + ax[0] * h2; r2y = vy + ay[0] * h2; r2z = vz + az[0] * h2;
                px[1] = x + vx * h2; py[1] = y + vy * h2; pz[1] = z + vz * h2;
            } else if (s == 2) {
                r3x = vx + ax[1] * h2; r3y = vy + ay[1] * h2; r3z = vz + az[1] * h2;
                px[2] = x + r2x * h2; py[2] = y + r2y * h2; pz[2] = z + r2z * h2;
            } else {
                r4x = vx + ax[2] * dt; r4y = vy + ay[2] * dt; r4z = vz + az[2] * dt;
                px[3] = x + r3x * dt; py[3] = y + r3y * dt; pz[3] = z + r3z * dt;
            }
            __syncwarp();
            if (on) { sp[j][0] = px[s]; sp[j][1] = py[s]; sp[j][2] = pz[s]; sp[j][3] = m; }
            __syncwarp();
            if (on) {
                massive_acc(sp, ng, j, ax[s], ay[s], az[s]);
                Ps[((size_t)n * 4 + s) * ng + j] = make_body(px[s], py[s], pz[s], m);
            }
        }
        x += d6 * (vx + 2.0 * r2x + 2.0 * r3x + r4x);
        y += d6 * (vy + 2.0 * r2y + 2.0 * r3y + r4y);
        z += d6 * (vz + 2.0 * r2z + 2.0 * r3z + r4z);
        vx += d6 * (ax[0] + 2.0 * ax[1] + 2.0 * ax[2] + ax[3]);
        vy += d6 * (ay[0] + 2.0 * ay[1] + 2.0 * ay[2] + ay[3]);
        vz += d6 * (az[0] + 2.0 * az[1] + 2.0 * az[2] + az[3]);
    }
    if (on) {
        xv[0 * ng + j] = x; xv[1 * ng + j] = y; xv[2 * ng + j] = z;
        xv[3 * ng + j] = vx; xv[4 * ng + j] = vy; xv[5 * ng + j] = vz;
    }
}

// Vector-Jacobian product of the all-pairs accelerations at one stage for body j:
// out_j = sum_k J_jk (m_j g_k - m_k g_j), J(d) v = v/r^3 - 3 (d.v) d/r^5, and the mass
// adjoint sum_k g_k.(P_j - P_k)/r^3.
__device__ __forceinline__ void massive_vjp(const double (*sp)[4], const double (*sg)[3], int ng, int j,
                                            double& ox, double& oy, double& oz, double& om) {
    ox = oy = oz = om = 0.0;
    const double mj = sp[j][3];
    for (int k = 0; k < ng; ++k) {
        if (k == j) continue;
        const double dx = sp[j][0] - sp[k][0], dy = sp[j][1] - sp[k][1], dz = sp[j][2] - sp[k][2];
        const double RR = dx * dx + dy * dy + dz * dz;
        if (!(RR > 0.0)) continue;
        const double ri3 = 1.0 / (RR * sqrt(RR)), ri5 = ri3 / RR;
        const double vx = mj * sg[k][0] - sp[k][3] * sg[j][0];
        const double vy = mj * sg[k][1] - sp[k][3] * sg[j][1];
        const double vz = mj * sg[k][2] - sp[k][3] * sg[j][2];
        const double dv = dx * vx + dy * vy + dz * vz;
        ox += vx * ri3 - 3.0 * dv * dx * ri5;
        oy += vy * ri3 - 3.0 * dv * dy * ri5;
        oz += vz * ri3 - 3.0 * dv * dz * ri5;
        om += (sg[k][0] * dx + sg[k][1] * dy + sg[k][2] * dz) * ri3;
    }
}

__global__ void massive_reverse_kernel(int ng, double dt, const Body* Ps, const double* mu, int n0, int n1,
                                       double* lam, double* lam_m) {
    __shared__ double sp[kMaxGrav][4];
    __shared__ double sg[kMaxGrav][3];
    const int j = threadIdx.x;
    const bool on = j < ng;
    double lx[3] = {0, 0, 0}, lv[3] = {0, 0, 0}, lm = 0.0;
    if (on) {
        for (int c = 0; c < 3; ++c) { lx[c] = lam[c * ng + j]; lv[c] = lam[(3 + c) * ng + j]; }
        lm = lam_m[j];
    }
    const double h2 = dt * 0.5, d6 = dt / 6.0;
    for (int n = n1 - 1; n >= n0; --n) {
        const int k = n - n0;
        double Lx[3], Lv[3], Lr2[3], Lr3[3], Lr4[3], La[4][3], LP[3] = {0, 0, 0};
        for (int c = 0; c < 3; ++c) {
            Lx[c] = lx[c];
            Lv[c] = lv[c] + d6 * lx[c];
            Lr2[c] = Lr3[c] = 2.0 * d6 * lx[c];
            Lr4[c] = d6 * lx[c];
            La[0][c] = d6 * lv[c];
            La[1][c] = La[2][c] = 2.0 * d6 * lv[c];
            La[3][c] = d6 * lv[c];
        }
        for (int s = 3; s >= 0; --s) {
            __syncwarp();
            if (on) {
                const Body b = Ps[((size_t)n * 4 + s) * ng + j];
                sp[j][0] = b.x; sp[j][1] = b.y; sp[j][2] = b.z; sp[j][3] = b.m;
                for (int c = 0; c < 3; ++c) sg[j][c] = La[s][c];
            }
            __syncwarp();
            double ox = 0, oy = 0, oz = 0, om = 0;
            if (on) {
                massive_vjp(sp, sg, ng, j, ox, oy, oz, om);
                const double* m4 = mu + (((size_t)k * 4 + s) * ng + j) * 4;
                LP[0] = ox + m4[0]; LP[1] = oy + m4[1]; LP[2] = oz + m4[2];
                lm += om + m4[3];
            }
            for (int c = 0; c < 3; ++c) {
                Lx[c] += LP[c];
                if (s == 3) { Lr3[c] += dt * LP[c]; Lv[c] += Lr4[c]; La[2][c] += dt * Lr4[c]; }
                else if (s == 2) { Lr2[c] += h2 * LP[c]; Lv[c] += Lr3[c]; La[1][c] += h2 * Lr3[c]; }
                else if (s == 1) { Lv[c] += h2 * LP[c]; Lv[c] += Lr2[c]; La[0][c] += h2 * Lr2[c]; }
            }
        }
        for (int c = 0; c < 3; ++c) { lx[c] = Lx[c]; lv[c] = Lv[c]; }
    }
    if (on) {
        for (int c = 0; c < 3; ++c) { lam[c * ng + j] = lx[c]; lam[(3 + c) * ng + j] = lv[c]; }
        lam_m[j] = lm;
    }
}

// ---------------------------------------------------------------------------------------
// Dust: forward (with checkpoints or with per-step storage) and reverse sweep
// ---------------------------------------------------------------------------------------

// Integrates every tracer over steps [n0, n1).  ck (optional): the state at every step
// that is a multiple of K (checkpoint c at ck + c*6*nd), including n1 when it is one.
// seg (optional): for every step n >= seg_n0, record n - seg_n0 holds the state, the stage
// accelerations a1..a3 and each stage's reciprocal distances (A.ncomp doubles per tracer).
__global__ void __launch_bounds__(kThreads)
dust_forward_kernel(AdjArgs A, double* y, double* N, int n0, int n1, int K, double* ck, double* seg,
                    int seg_n0) {
    const int i = blockIdx.x * kThreads + threadIdx.x;
    if (i >= A.nd) return;
    const size_t nd = A.nd;
    double x = y[0 * nd + i], yy = y[1 * nd + i], z = y[2 * nd + i];
    double vx = y[3 * nd + i], vy = y[4 * nd + i], vz = y[5 * nd + i];
    bool alive = N[i] != 0.0;
    float bet = 0.f, betsw = 0.f, qe = 0.f;
    const int id = A.id[i];
    if (id >= 0 && id < A.sa.n_grid) { bet = A.bins[id].beta; betsw = A.bins[id].betasw; qe = A.bins[id].q; }
    const StarConst K0 = star_const(A, A.Ps[0].m, bet, betsw, qe, A.mass[i]);
    const double dt = A.dt, h2 = dt / 2.0, d6 = dt / 6.0;
    for (int n = n0; n < n1; ++n) {
        if (ck && n % K == 0) {
            double* c = ck + (size_t)(n / K) * 6 * nd;
            c[0 * nd + i] = x; c[1 * nd + i] = yy; c[2 * nd + i] = z;
            c[3 * nd + i] = vx; c[4 * nd + i] = vy; c[5 * nd + i] = vz;
        }
        double a1x = 0, a1y = 0, a1z = 0, a2x = 0, a2y = 0, a2z = 0, a3x = 0, a3y = 0, a3z = 0;
        if (alive) {
            const Body* P = A.Ps + (size_t)n * 4 * A.ng;
            double* S = (seg && n >= seg_n0) ? seg + (size_t)(n - seg_n0) * A.ncomp * nd + i : nullptr;
            const size_t rstage = (size_t)(2 + A.nir) * nd;   // record stride between stages
            double* rc = S ? S + kSegComp * nd : nullptr;
            double a4x = 0, a4y = 0, a4z = 0;
            bool ok = tracer_accel(A, K0, P, x, yy, z, vx, vy, vz, a1x, a1y, a1z, rc, nd);
            const double r2x = vx + a1x * h2, r2y = vy + a1y * h2, r2z = vz + a1z * h2;
            ok = ok && tracer_accel(A, K0, P + A.ng, x + vx * h2, yy + vy * h2, z + vz * h2, r2x, r2y, r2z,
                                    a2x, a2y, a2z, S ? rc + rstage : nullptr, nd);
            const double r3x = vx + a2x * h2, r3y = vy + a2y * h2, r3z = vz + a2z * h2;
            ok = ok && tracer_accel(A, K0, P + 2 * A.ng, x + r2x * h2, yy + r2y * h2, z + r2z * h2, r3x, r3y,
                                    r3z, a3x, a3y, a3z, S ? rc + 2 * rstage : nullptr, nd);
            const double r4x = vx + a3x * dt, r4y = vy + a3y * dt, r4z = vz + a3z * dt;
            ok = ok && tracer_accel(A, K0, P + 3 * A.ng, x + r3x * dt, yy + r3y * dt, z + r3z * dt, r4x, r4y,
                                    r4z, a4x, a4y, a4z, S ? rc + 3 * rstage : nullptr, nd);
            if (S) {
                const double v[kSegComp] = {x, yy, z, vx, vy, vz, a1x, a1y, a1z, a2x, a2y, a2z, a3x, a3y, a3z};
                for (int c = 0; c < kSegComp; ++c) S[c * nd] = v[c];
            }
            if (!ok) {
                alive = false;   // removed: keeps its last state, emits nothing
            } else {
                x += d6 * (vx + 2.0 * (r2x + r3x) + r4x);
                yy += d6 * (vy + 2.0 * (r2y + r3y) + r4y);
                z += d6 * (vz + 2.0 * (r2z + r3z) + r4z);
                vx += d6 * (a1x + 2.0 * (a2x + a3x) + a4x);
                vy += d6 * (a1y + 2.0 * (a2y + a3y) + a4y);
                vz += d6 * (a1z + 2.0 * (a2z + a3z) + a4z);
            }
        }
    }
    if (ck && n1 % K == 0) {
        double* c = ck + (size_t)(n1 / K) * 6 * nd;
        c[0 * nd + i] = x; c[1 * nd + i] = yy; c[2 * nd + i] = z;
        c[3 * nd + i] = vx; c[4 * nd + i] = vy; c[5 * nd + i] = vz;
    }
    y[0 * nd + i] = x; y[1 * nd + i] = yy; y[2 * nd + i] = z;
    y[3 * nd + i] = vx; y[4 * nd + i] = vy; y[5 * nd + i] = vz;
    if (!alive) N[i] = 0.0;
}

// Warp-wide sums of the per-tracer adjoints of the bodies' stage positions and masses.
// Each source adds 4 rows (x, y, z, m) to a 32 x 32 shared-memory tile, one column per
// lane; row r holds lane k's value at column (k + r) mod 32, so row-wise reads by the 32
// lanes fall in different banks.  A full tile (8 sources) or the end of a step flushes it:
// p = 32 / rows lanes (a power of two) share a row, each adds 32/p columns in lane order
// and a fixed shuffle tree joins the p partials.  Sums land in wp in the order the sources
// were put, a fixed order, so the result is deterministic.  A whole step of three bodies
// (48 rows) costs 49 FP64 additions per lane, against 240 for a shuffle tree per value.
struct RowTile {
    double (*tb)[32];
    double* wp;
    int rows, base, lane;

    __device__ __forceinline__ void flush() {
        if (rows == 0) return;
        __syncwarp();
        int p = 1;
        while (2 * p * rows <= 32) p *= 2;
        const int w = 32 / p, row = lane / p, part = lane % p;
        double t = 0.0;
        if (row < rows)
            for (int k = 0; k < w; ++k) t += tb[row][(part * w + k + row) & 31];
        for (int o = p / 2; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (row < rows && part == 0) wp[base + row] = t;
        base += rows;
        rows = 0;
        __syncwarp();
    }
    __device__ __forceinline__ void put4(const double* v) {
        if (rows == 32) flush();
        for (int c = 0; c < 4; ++c) tb[rows + c][(lane + rows + c) & 31] = v[c];
        rows += 4;
    }
};

// VJP of the tracer acceleration at one stage with adjoint g: adds to (Lx, Lr) and puts,
// per source j, the tracer's adjoints of that source's stage position and mass into T.
// rc (stride rs): the stage's reciprocal distances kept by the recompute.  Called by
// every lane of the warp.
template <class Tile>
__device__ __forceinline__ void tracer_vjp(const AdjArgs& A, const StarConst& K, const Body* P, bool on,
                                           const double* pos, const double* r, const double* g, double* Lx,
                                           double* Lr, const double* rc, size_t rs, Tile& T) {
    {   // star (source 0)
        double s4[4] = {0, 0, 0, 0};
        if (on) {
            const double dx = pos[0] - P[0].x, dy = pos[1] - P[0].y, dz = pos[2] - P[0].z;
            const double iRR = rc[0];
            const double iR3 = rc[rs] * iRR, iR5 = iR3 * iRR;
            const double Fg = K.g0 * iR3, Fb1 = K.c1 * iRR;
            const double dr = dx * r[0] + dy * r[1] + dz * r[2];
            const double Fb2 = dr * iRR;
            const double gd = g[0] * dx + g[1] * dy + g[2] * dz;
            const double gr = g[0] * r[0] + g[1] * r[1] + g[2] * r[2];
            const double gD = Fb2 * gd + gr;
            // a = -Fg d - Fb1 (Fb2 d + r): g^T da/dd = cg g + cd d + cr r ; g^T da/dr = cr d - Fb1 g
            const double cg = -Fg - Fb1 * Fb2;
            double cd = 3.0 * K.g0 * gd * iR5 + 2.0 * (K.c1 * gD + Fb1 * gd * dr) * (iRR * iRR);
            const double cr = -Fb1 * gd * iRR;
            const double d[3] = {dx, dy, dz};
            // Lorentz: g . dFl/dd = cL (-Wz iR3 (gx, gy, 0) - 3 iR5 Q d), Q = gx (ry - Wz dx) - gy (rx + Wz dy);
            // g . dFl/dr = cL iR3 (-gy, gx, 0)
            double lg[3] = {0.0, 0.0, 0.0}, lr[3] = {0.0, 0.0, 0.0};
            if (K.cL != 0.0) {
                const double Wz = A.sa.Wz;
                const double Q = g[0] * (r[1] - Wz * dx) - g[1] * (r[0] + Wz * dy);
                cd -= 3.0 * K.cL * iR5 * Q;
                lg[0] = -K.cL * Wz * iR3 * g[0];
                lg[1] = -K.cL * Wz * iR3 * g[1];
                lr[0] = -K.cL * iR3 * g[1];
                lr[1] = K.cL * iR3 * g[0];
            }
            for (int c = 0; c < 3; ++c) {
                const double ld = cg * g[c] + cd * d[c] + cr * r[c] + lg[c];
                Lx[c] += ld;
                Lr[c] += cr * d[c] - Fb1 * g[c] + lr[c];
                s4[c] = -ld;
            }
            s4[3] = (-Fg * gd - Fb1 * gD) * K.inv_m0;
        }
        T.put4(s4);
    }
    for (int j = 1; j < A.ng; ++j) {
        double v4[4] = {0, 0, 0, 0};
        if (on) {
            const double dx = P[j].x - pos[0], dy = P[j].y - pos[1], dz = P[j].z - pos[2];
            const double ir = (j <= A.nir) ? rc[(1 + j) * rs] : rsqrt(dx * dx + dy * dy + dz * dz);
            const double ir2 = ir * ir;
            const double ri3 = ir2 * ir, ri5 = ri3 * ir2;
            const double gd = g[0] * dx + g[1] * dy + g[2] * dz;
            const double m = P[j].m;
            const double t3 = 3.0 * gd * ri5;
            v4[0] = m * (g[0] * ri3 - t3 * dx);
            v4[1] = m * (g[1] * ri3 - t3 * dy);
            v4[2] = m * (g[2] * ri3 - t3 * dz);
            v4[3] = gd * ri3;
            Lx[0] -= v4[0]; Lx[1] -= v4[1]; Lx[2] -= v4[2];
        }
        T.put4(v4);
    }
}

// Reverse sweep over steps [n0, n1) (descending) from the recompute records.  lam [6][nd]
// holds the adjoint of the state after step n1-1 on entry and of the state before step n0
// on exit.  part[block][k][stage][j][4]: this block's sum of the adjoints of the bodies'
// stage positions and masses.
__global__ void __launch_bounds__(kThreads)
dust_reverse_kernel(AdjArgs A, const double* __restrict__ seg, int n0, int n1, double* __restrict__ lam,
                    const unsigned char* __restrict__ active, double* __restrict__ part) {
    __shared__ double wpart[kWarps][16 * kMaxGrav];   // per warp: [3 - stage][j][4], one step
    __shared__ double tbuf[kWarps][32][32];
    const int i = blockIdx.x * kThreads + threadIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const size_t nd = A.nd;
    const bool on = i < A.nd && active[i];
    double lx[3] = {0, 0, 0}, lv[3] = {0, 0, 0};
    float bet = 0.f, betsw = 0.f, qe = 0.f;
    double mi = 1.0;
    if (on) {
        for (int c = 0; c < 3; ++c) { lx[c] = lam[c * nd + i]; lv[c] = lam[(3 + c) * nd + i]; }
        const int id = A.id[i];
        if (id >= 0 && id < A.sa.n_grid) { bet = A.bins[id].beta; betsw = A.bins[id].betasw; qe = A.bins[id].q; }
        mi = A.mass[i];
    }
    const StarConst K0 = star_const(A, A.Ps[0].m, bet, betsw, qe, mi);
    RowTile T{tbuf[warp], wpart[warp], 0, 0, lane};
    const int Kseg = n1 - n0;
    const double dt = A.dt, h2 = dt / 2.0, d6 = dt / 6.0;
    const size_t rstage = (size_t)(2 + A.nir) * nd;
    for (int n = n1 - 1; n >= n0; --n) {
        const int k = n - n0;
        const double* S = seg + (size_t)k * A.ncomp * nd + (on ? i : 0);
        const double* rc = S + kSegComp * nd;
        double st[kSegComp];
        for (int c = 0; c < kSegComp; ++c) st[c] = on ? S[c * nd] : 0.0;
        const double* x = st;
        const double* v = st + 3;
        const double* a1 = st + 6;
        const double* a2 = st + 9;
        const double* a3 = st + 12;
        double x2[3], r2[3], x3[3], r3[3], x4[3], r4[3];
        for (int c = 0; c < 3; ++c) {
            x2[c] = x[c] + v[c] * h2; r2[c] = v[c] + a1[c] * h2;
            x3[c] = x[c] + r2[c] * h2; r3[c] = v[c] + a2[c] * h2;
            x4[c] = x[c] + r3[c] * dt; r4[c] = v[c] + a3[c] * dt;
        }
        double Lx[3], Lv[3], Lr2[3], Lr3[3], Lr4[3], La1[3], La2[3], La3[3], La4[3];
        for (int c = 0; c < 3; ++c) {
            Lx[c] = lx[c];
            Lv[c] = lv[c] + d6 * lx[c];
            Lr2[c] = Lr3[c] = 2.0 * d6 * lx[c];
            Lr4[c] = d6 * lx[c];
            La1[c] = d6 * lv[c];
            La2[c] = La3[c] = 2.0 * d6 * lv[c];
            La4[c] = d6 * lv[c];
        }
        const Body* P = A.Ps + (size_t)n * 4 * A.ng;
        double Ls[3], Lq[3];
        // stage 4: a4 = a(x4, r4); x4 = x + r3 dt; r4 = v + a3 dt
        Ls[0] = Ls[1] = Ls[2] = 0.0; Lq[0] = Lq[1] = Lq[2] = 0.0;
        tracer_vjp(A, K0, P + 3 * A.ng, on, x4, r4, La4, Ls, Lq, rc + 3 * rstage, nd, T);
        for (int c = 0; c < 3; ++c) {
            Lr4[c] += Lq[c];
            Lx[c] += Ls[c]; Lr3[c] += dt * Ls[c];
            Lv[c] += Lr4[c]; La3[c] += dt * Lr4[c];
        }
        // stage 3: a3 = a(x3, r3); x3 = x + r2 h2; r3 = v + a2 h2
        Ls[0] = Ls[1] = Ls[2] = 0.0; Lq[0] = Lq[1] = Lq[2] = 0.0;
        tracer_vjp(A, K0, P + 2 * A.ng, on, x3, r3, La3, Ls, Lq, rc + 2 * rstage, nd, T);
        for (int c = 0; c < 3; ++c) {
            Lr3[c] += Lq[c];
            Lx[c] += Ls[c]; Lr2[c] += h2 * Ls[c];
            Lv[c] += Lr3[c]; La2[c] += h2 * Lr3[c];
        }
        // stage 2: a2 = a(x2, r2); x2 = x + v h2; r2 = v + a1 h2
        Ls[0] = Ls[1] = Ls[2] = 0.0; Lq[0] = Lq[1] = Lq[2] = 0.0;
        tracer_vjp(A, K0, P + A.ng, on, x2, r2, La2, Ls, Lq, rc + rstage, nd, T);
        for (int c = 0; c < 3; ++c) {
            Lr2[c] += Lq[c];
            Lx[c] += Ls[c]; Lv[c] += h2 * Ls[c];
            Lv[c] += Lr2[c]; La1[c] += h2 * Lr2[c];
        }
        // stage 1: a1 = a(x, v)
        Ls[0] = Ls[1] = Ls[2] = 0.0; Lq[0] = Lq[1] = Lq[2] = 0.0;
        tracer_vjp(A, K0, P, on, x, v, La1, Ls, Lq, rc, nd, T);
        for (int c = 0; c < 3; ++c) {
            Lx[c] += Ls[c]; Lv[c] += Lq[c];
            lx[c] = Lx[c]; lv[c] = Lv[c];
        }
        T.flush();
        T.base = 0;
        __syncthreads();
        for (int e = threadIdx.x; e < 4 * A.ng * 4; e += kThreads) {
            const int s = 3 - e / (A.ng * 4), j = (e / 4) % A.ng, c = e % 4;
            double t = 0.0;
            for (int w = 0; w < kWarps; ++w) t += wpart[w][e];
            part[((((size_t)blockIdx.x * Kseg + k) * 4 + s) * A.ng + j) * 4 + c] = t;
        }
        __syncthreads();
    }
    if (on)
        for (int c = 0; c < 3; ++c) { lam[c * nd + i] = lx[c]; lam[(3 + c) * nd + i] = lv[c]; }
}

// ---------------------------------------------------------------------------------------
// Large massive sets (n_grav > kMaxGrav): the massive set runs one launch per pass (forward)
// and per stage (reverse), a warp per body; the tracers' adjoints of the bodies' stage
// positions and masses are summed per block for every step and reduced in block order.
// ---------------------------------------------------------------------------------------

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Acceleration of body j from every other body at one stage (records P[0..ng)), the
// m / (RR sqrt(RR)) form of massive_acc, lanes strided over the sources with a fixed
// butterfly sum.  All 32 lanes call it.
__device__ __forceinline__ void massive_acc_warp(const Body* __restrict__ P, int ng, int j, double& ax, double& ay,
                                                 double& az) {
    const int lane = threadIdx.x & 31;
    const Body pj = P[j];
    ax = ay = az = 0.0;
    for (int k = lane; k < ng; k += 32) {
        if (k == j) continue;
        const Body pk = P[k];
        const double dx = pk.x - pj.x, dy = pk.y - pj.y, dz = pk.z - pj.z;
        const double RR = dx * dx + dy * dy + dz * dz;
        if (RR > 0.0) {
            const double f = pk.m / (RR * sqrt(RR));
            ax += f * dx; ay += f * dy; az += f * dz;
        }
    }
    ax = warp_sum_d(ax); ay = warp_sum_d(ay); az = warp_sum_d(az);
}

// Step n of the massive forward, first launch: P1 = x, P2 = x + v dt/2 (a thread per body).
__global__ void massive_fwd_init_kernel(int ng, double dt, const double* __restrict__ xv, Body* __restrict__ P) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= ng) return;
    const double h2 = dt * 0.5;
    const double x = xv[j], y = xv[ng + j], z = xv[2 * ng + j], m = xv[6 * ng + j];
    P[j] = make_body(x, y, z, m);
    P[ng + j] = make_body(x + xv[3 * ng + j] * h2, y + xv[4 * ng + j] * h2, z + xv[5 * ng + j] * h2, m);
}

// Second launch: A1 at P1 and A2 at P2 (a warp per body), then P3 = x + (v + A1 dt/2) dt/2
// and P4 = x + (v + A2 dt/2) dt; A1, A2 kept in macc[6][ng].
__global__ void massive_fwd_pass1_kernel(int ng, double dt, const double* __restrict__ xv, Body* __restrict__ P,
                                         double* __restrict__ macc) {
    const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (j >= ng) return;   // warp-uniform
    double a[6];
    massive_acc_warp(P, ng, j, a[0], a[1], a[2]);
    massive_acc_warp(P + ng, ng, j, a[3], a[4], a[5]);
    if ((threadIdx.x & 31) != 0) return;
    const double h2 = dt * 0.5;
    double x[3], v[3];
    for (int c = 0; c < 3; ++c) { x[c] = xv[c * ng + j]; v[c] = xv[(3 + c) * ng + j]; }
    for (int c = 0; c < 6; ++c) macc[c * ng + j] = a[c];
    const double m = xv[6 * ng + j];
    double p3[3], p4[3];
    for (int c = 0; c < 3; ++c) {
        p3[c] = x[c] + (v[c] + a[c] * h2) * h2;
        p4[c] = x[c] + (v[c] + a[3 + c] * h2) * dt;
    }
    P[2 * ng + j] = make_body(p3[0], p3[1], p3[2], m);
    P[3 * ng + j] = make_body(p4[0], p4[1], p4[2], m);
}

// Third launch: A3 at P3 and A4 at P4, then the RK4 combination of the body's state.
__global__ void massive_fwd_pass2_kernel(int ng, double dt, double* __restrict__ xv, const Body* __restrict__ P,
                                         const double* __restrict__ macc) {
    const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (j >= ng) return;
    double a3[3], a4[3];
    massive_acc_warp(P + 2 * ng, ng, j, a3[0], a3[1], a3[2]);
    massive_acc_warp(P + 3 * ng, ng, j, a4[0], a4[1], a4[2]);
    if ((threadIdx.x & 31) != 0) return;
    const double h2 = dt * 0.5, d6 = dt / 6.0;
    for (int c = 0; c < 3; ++c) {
        const double x = xv[c * ng + j], v = xv[(3 + c) * ng + j];
        const double a1 = macc[c * ng + j], a2 = macc[(3 + c) * ng + j];
        const double r2 = v + a1 * h2, r3 = v + a2 * h2, r4 = v + a3[c] * dt;
        xv[c * ng + j] = x + d6 * (v + 2.0 * r2 + 2.0 * r3 + r4);
        xv[(3 + c) * ng + j] = v + d6 * (a1 + 2.0 * a2 + 2.0 * a3[c] + a4[c]);
    }
}

// Body adjoints of one step, lamS[27][ng]: rows 0-2 Lx, 3-5 Lv, 6-8 Lr2, 9-11 Lr3, 12-14 Lr4,
// 15 + 3 s + c the adjoint of stage s's acceleration.  Seeded from the adjoint of the state
// after the step, lam[6][ng] (a thread per body).
__global__ void massive_rev_init_kernel(int ng, double dt, const double* __restrict__ lam, double* __restrict__ lamS) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= ng) return;
    const double d6 = dt / 6.0;
    for (int c = 0; c < 3; ++c) {
        const double lx = lam[c * ng + j], lv = lam[(3 + c) * ng + j];
        lamS[c * ng + j] = lx;
        lamS[(3 + c) * ng + j] = lv + d6 * lx;
        lamS[(6 + c) * ng + j] = 2.0 * d6 * lx;
        lamS[(9 + c) * ng + j] = 2.0 * d6 * lx;
        lamS[(12 + c) * ng + j] = d6 * lx;
        lamS[(15 + c) * ng + j] = d6 * lv;
        lamS[(18 + c) * ng + j] = 2.0 * d6 * lv;
        lamS[(21 + c) * ng + j] = 2.0 * d6 * lv;
        lamS[(24 + c) * ng + j] = d6 * lv;
    }
}

// Reverse stage s (3..0) of one step for body j (a warp per body): the all-pairs VJP of the
// stage's accelerations (massive_vjp) with the tracers' adjoints mu[s][j][4] added, then
// the stage's share of the RK4 reverse; after stage 0, lam holds the adjoint of the state
// before the step.  lam_m accumulates the mass adjoint.
__global__ void massive_rev_stage_kernel(int ng, double dt, const Body* __restrict__ P, const double* __restrict__ mu,
                                         int s, double* __restrict__ lamS, double* __restrict__ lam,
                                         double* __restrict__ lam_m) {
    const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (j >= ng) return;
    const int lane = threadIdx.x & 31;
    const double* G = lamS + (size_t)(15 + 3 * s) * ng;     // adjoints of this stage's accelerations
    const Body pj = P[j];
    const double gj[3] = {G[j], G[ng + j], G[2 * ng + j]};
    double ox = 0, oy = 0, oz = 0, om = 0;
    for (int k = lane; k < ng; k += 32) {
        if (k == j) continue;
        const Body pk = P[k];
        const double dx = pj.x - pk.x, dy = pj.y - pk.y, dz = pj.z - pk.z;
        const double RR = dx * dx + dy * dy + dz * dz;
        if (!(RR > 0.0)) continue;
        const double ri3 = 1.0 / (RR * sqrt(RR)), ri5 = ri3 / RR;
        const double gk[3] = {G[k], G[ng + k], G[2 * ng + k]};
        const double vx = pj.m * gk[0] - pk.m * gj[0];
        const double vy = pj.m * gk[1] - pk.m * gj[1];
        const double vz = pj.m * gk[2] - pk.m * gj[2];
        const double dv = dx * vx + dy * vy + dz * vz;
        ox += vx * ri3 - 3.0 * dv * dx * ri5;
        oy += vy * ri3 - 3.0 * dv * dy * ri5;
        oz += vz * ri3 - 3.0 * dv * dz * ri5;
        om += (gk[0] * dx + gk[1] * dy + gk[2] * dz) * ri3;
    }
    ox = warp_sum_d(ox); oy = warp_sum_d(oy); oz = warp_sum_d(oz); om = warp_sum_d(om);
    if (lane != 0) return;
    const double* m4 = mu + ((size_t)s * ng + j) * 4;
    const double LP[3] = {ox + m4[0], oy + m4[1], oz + m4[2]};
    lam_m[j] += om + m4[3];
    const double h2 = dt * 0.5;
    auto at = [&](int row, int c) -> double& { return lamS[(size_t)(row + c) * ng + j]; };
    for (int c = 0; c < 3; ++c) {
        at(0, c) += LP[c];
        if (s == 3) { at(9, c) += dt * LP[c]; at(3, c) += at(12, c); at(15 + 6, c) += dt * at(12, c); }
        else if (s == 2) { at(6, c) += h2 * LP[c]; at(3, c) += at(9, c); at(15 + 3, c) += h2 * at(9, c); }
        else if (s == 1) { at(3, c) += h2 * LP[c]; at(3, c) += at(6, c); at(15, c) += h2 * at(6, c); }
        else { lam[c * ng + j] = at(0, c); lam[(3 + c) * ng + j] = at(3, c); }
    }
}

// Block sums of the tracers' adjoints of the bodies' stage positions and masses: per warp the
// RowTile transpose (8 sources of 4 values per round), then the warps' sums added in warp
// order by the first 32 threads and written to out[4 * source + c].  Every thread of the
// block calls put4 for every source.
struct BlockRows {
    double (*tb)[32];
    double (*ws)[32];
    double* out;
    int rows, j0, lane, warp;

    __device__ __forceinline__ void flush() {
        if (rows == 0) return;
        __syncwarp();
        int p = 1;
        while (2 * p * rows <= 32) p *= 2;
        const int w = 32 / p, row = lane / p, part = lane % p;
        double t = 0.0;
        if (row < rows)
            for (int k = 0; k < w; ++k) t += tb[row][(part * w + k + row) & 31];
        for (int o = p / 2; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (row < rows && part == 0) ws[warp][row] = t;
        __syncthreads();
        if ((int)threadIdx.x < rows) {
            double u = 0.0;
            for (int v = 0; v < kWarps; ++v) u += ws[v][threadIdx.x];
            out[(size_t)j0 * 4 + threadIdx.x] = u;
        }
        __syncthreads();
        j0 += rows / 4;
        rows = 0;
    }
    __device__ __forceinline__ void put4(const double* v) {
        if (rows == 32) flush();
        for (int c = 0; c < 4; ++c) tb[rows + c][(lane + rows + c) & 31] = v[c];
        rows += 4;
    }
};

// Reverse sweep of one step n (record k of the segment) for every tracer, with the bodies'
// adjoints of its four stages summed per block into part[block][s][j][4].  lam [6][nd]: the
// tracers' adjoints after the step on entry, before it on exit.
__global__ void __launch_bounds__(kThreads)
dust_reverse_step_kernel(AdjArgs A, const double* __restrict__ seg, int k, int n, double* __restrict__ lam,
                         const unsigned char* __restrict__ active, double* __restrict__ part) {
    __shared__ double tbuf[kWarps][32][32];
    __shared__ double ws[kWarps][32];
    const int i = blockIdx.x * kThreads + threadIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const size_t nd = A.nd;
    const bool on = i < A.nd && active[i];
    double lx[3] = {0, 0, 0}, lv[3] = {0, 0, 0};
    float bet = 0.f, betsw = 0.f, qe = 0.f;
    double mi = 1.0;
    if (on) {
        for (int c = 0; c < 3; ++c) { lx[c] = lam[c * nd + i]; lv[c] = lam[(3 + c) * nd + i]; }
        const int id = A.id[i];
        if (id >= 0 && id < A.sa.n_grid) { bet = A.bins[id].beta; betsw = A.bins[id].betasw; qe = A.bins[id].q; }
        mi = A.mass[i];
    }
    const StarConst K0 = star_const(A, A.Ps[0].m, bet, betsw, qe, mi);
    const double dt = A.dt, h2 = dt / 2.0, d6 = dt / 6.0;
    const size_t rstage = (size_t)(2 + A.nir) * nd;
    const double* S = seg + (size_t)k * A.ncomp * nd + (on ? i : 0);
    const double* rc = S + kSegComp * nd;
    double st[kSegComp];
    for (int c = 0; c < kSegComp; ++c) st[c] = on ? S[c * nd] : 0.0;
    const double* x = st;
    const double* v = st + 3;
    const double* a1 = st + 6;
    const double* a2 = st + 9;
    const double* a3 = st + 12;
    double x2[3], r2[3], x3[3], r3[3], x4[3], r4[3];
    for (int c = 0; c < 3; ++c) {
        x2[c] = x[c] + v[c] * h2; r2[c] = v[c] + a1[c] * h2;
        x3[c] = x[c] + r2[c] * h2; r3[c] = v[c] + a2[c] * h2;
        x4[c] = x[c] + r3[c] * dt; r4[c] = v[c] + a3[c] * dt;
    }
    double Lx[3], Lv[3], Lr2[3], Lr3[3], Lr4[3], La1[3], La2[3], La3[3], La4[3];
    for (int c = 0; c < 3; ++c) {
        Lx[c] = lx[c];
        Lv[c] = lv[c] + d6 * lx[c];
        Lr2[c] = Lr3[c] = 2.0 * d6 * lx[c];
        Lr4[c] = d6 * lx[c];
        La1[c] = d6 * lv[c];
        La2[c] = La3[c] = 2.0 * d6 * lv[c];
        La4[c] = d6 * lv[c];
    }
    const Body* P = A.Ps + (size_t)n * 4 * A.ng;
    double* pb = part + (size_t)blockIdx.x * 4 * A.ng * 4;
    double Ls[3], Lq[3];
    {   // stage 4
        BlockRows T{tbuf[warp], ws, pb + (size_t)3 * A.ng * 4, 0, 0, lane, warp};
        Ls[0] = Ls[1] = Ls[2] = 0.0; Lq[0] = Lq[1] = Lq[2] = 0.0;
        tracer_vjp(A, K0, P + 3 * A.ng, on, x4, r4, La4, Ls, Lq, rc + 3 * rstage, nd, T);
        T.flush();
        for (int c = 0; c < 3; ++c) {
            Lr4[c] += Lq[c];
            Lx[c] += Ls[c]; Lr3[c] += dt * Ls[c];
            Lv[c] += Lr4[c]; La3[c] += dt * Lr4[c];
        }
    }
    {   // stage 3
        BlockRows T{tbuf[warp], ws, pb + (size_t)2 * A.ng * 4, 0, 0, lane, warp};
        Ls[0] = Ls[1] = Ls[2] = 0.0; Lq[0] = Lq[1] = Lq[2] = 0.0;
        tracer_vjp(A, K0, P + 2 * A.ng, on, x3, r3, La3, Ls, Lq, rc + 2 * rstage, nd, T);
        T.flush();
        for (int c = 0; c < 3; ++c) {
            Lr3[c] += Lq[c];
            Lx[c] += Ls[c]; Lr2[c] += h2 * Ls[c];
            Lv[c] += Lr3[c]; La2[c] += h2 * Lr3[c];
        }
    }
    {   // stage 2
        BlockRows T{tbuf[warp], ws, pb + (size_t)1 * A.ng * 4, 0, 0, lane, warp};
        Ls[0] = Ls[1] = Ls[2] = 0.0; Lq[0] = Lq[1] = Lq[2] = 0.0;
        tracer_vjp(A, K0, P + A.ng, on, x2, r2, La2, Ls, Lq, rc + rstage, nd, T);
        T.flush();
        for (int c = 0; c < 3; ++c) {
            Lr2[c] += Lq[c];
            Lx[c] += Ls[c]; Lv[c] += h2 * Ls[c];
            Lv[c] += Lr2[c]; La1[c] += h2 * Lr2[c];
        }
    }
    {   // stage 1
        BlockRows T{tbuf[warp], ws, pb, 0, 0, lane, warp};
        Ls[0] = Ls[1] = Ls[2] = 0.0; Lq[0] = Lq[1] = Lq[2] = 0.0;
        tracer_vjp(A, K0, P, on, x, v, La1, Ls, Lq, rc, nd, T);
        T.flush();
        for (int c = 0; c < 3; ++c) {
            Lx[c] += Ls[c]; Lv[c] += Lq[c];
        }
    }
    if (on)
        for (int c = 0; c < 3; ++c) { lam[c * nd + i] = Lx[c]; lam[(3 + c) * nd + i] = Lv[c]; }
}

// mu[k][s][j][c] = sum over blocks of part[b][k][s][j][c], in block order.
__global__ void reduce_parts_kernel(const double* __restrict__ part, int nblk, int per_block, double* __restrict__ mu) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= per_block) return;
    double t = 0.0;
    for (int b = 0; b < nblk; ++b) t += part[(size_t)b * per_block + e];
    mu[e] = t;
}

// ---------------------------------------------------------------------------------------
// Differentiable image: bilinear deposition of the flux, and its adjoint
// ---------------------------------------------------------------------------------------

struct TracerFlux {
    double R, cossc, dcos[3];   // gradient of cossc with respect to (x, y, z)
    bool clamped;
    double u, w, du[3], dw[3];  // continuous pixel coordinates (pixel centres at integers)
    double T, dTdR;
};

__device__ __forceinline__ void tracer_geometry(double x, double y, double z, int id, const ViewConst& v,
                                                const OpticsDev& o, TracerFlux& g) {
    const double R = sqrt(x * x + y * y + z * z);
    g.R = R;
    const double x1 = x * v.cr - y * v.sr, y1 = x * v.sr + y * v.cr;
    // scattering-angle cosine (src/gpu_functions.cu:1017-1023) and its gradient
    const double qx = -x1, qy = v.ly0 - y1, qz = v.lz0 - z;
    const double L = sqrt(qx * qx + qy * qy + qz * qz);
    const double num = x1 * x1 + y1 * y1 + z * z - y1 * v.ly0 - z * v.lz0;
    double c = num / (R * L);
    g.clamped = false;
    if (!(c >= -1)) { c = -1.0; g.clamped = true; }   // NaN too: the table index stays in range
    if (c >= 1.0 - 2.0 / v.ntheta) { c = 1.0 - 2.0 / v.ntheta; g.clamped = true; }
    g.cossc = c;
    const double p[3] = {x1, y1, z}, l0[3] = {0.0, v.ly0, v.lz0}, q[3] = {qx, qy, qz};
    double dp[3];
    for (int k = 0; k < 3; ++k)
        dp[k] = g.clamped ? 0.0 : (2.0 * p[k] - l0[k]) / (R * L) - c * (p[k] / (R * R) - q[k] / (L * L));
    g.dcos[0] = dp[0] * v.cr + dp[1] * v.sr;
    g.dcos[1] = -dp[0] * v.sr + dp[1] * v.cr;
    g.dcos[2] = dp[2];
    // projected coordinates
    const double y2 = y1 * v.ci + z * v.si;
    const double X = x1 * v.cp - y2 * v.sp, Y = x1 * v.sp + y2 * v.cp;
    g.u = X / v.psca + 0.5 * v.xsize - 0.5;
    g.w = Y / v.psca + 0.5 * v.ysize - 0.5;
    const double dXdx1 = v.cp, dXdy1 = -v.sp * v.ci, dXdz = -v.sp * v.si;
    const double dYdx1 = v.sp, dYdy1 = v.cp * v.ci, dYdz = v.cp * v.si;
    g.du[0] = (dXdx1 * v.cr + dXdy1 * v.sr) / v.psca;
    g.du[1] = (-dXdx1 * v.sr + dXdy1 * v.cr) / v.psca;
    g.du[2] = dXdz / v.psca;
    g.dw[0] = (dYdx1 * v.cr + dYdy1 * v.sr) / v.psca;
    g.dw[1] = (-dYdx1 * v.sr + dYdy1 * v.cr) / v.psca;
    g.dw[2] = dYdz / v.psca;
    // temperature (log-log in R on the nR grid) and its slope
    const double* Td = o.Td + (size_t)id * kNR;
    if (!(R > o.Rmin)) { g.T = Td[0]; g.dTdR = 0.0; }   // R <= Rmin, or NaN: no table index from it
    else if (R >= o.Rmax) { g.T = Td[kNR - 1]; g.dTdR = 0.0; }
    else {
        const double* lT = o.lTd + (size_t)id * kNR;
        const double lr = log(R / o.Rmin);
        int k = (int)(lr / o.fR) + 1;
        if (k > kNR - 1) k = kNR - 1;
        if (k < 1) k = 1;
        const double frac = (lr - (k - 1) * o.fR) / o.fR;
        g.T = exp(lT[k - 1] + (lT[k] - lT[k - 1]) * frac);
        g.dTdR = g.T * (lT[k] - lT[k - 1]) / (o.fR * R);
    }
}

// Flux at table wavelength wj with its derivatives in R and cossc.
__device__ __forceinline__ void flux_grad(double n, int id, int wj, const TracerFlux& g, const OpticsDev& o,
                                          const ViewConst& v, double& F, double& dFdR, double& dFdc) {
    const double wvl = o.w[wj];
    const double xq = kHplank * kCspeed / (wvl * kKboltz * g.T);
    double I = 0.0, dIdT = 0.0;
    if (xq < 700.0) {
        const double ex = exp(xq);
        I = (2 * kHplank * kCspeed * kCspeed) / (o.w5[wj] * (ex - 1.0)) * kPI;
        dIdT = I * xq * ex / (ex - 1.0) / g.T;
    }
    const int nth = v.ntheta;
    int cm = floor(0.5 * (g.cossc + 1.0) * (nth - 1));
    const double cosm = (double)cm * 2.0 / (nth - 1) - 1.0, cosp = (double)(cm + 1) * 2.0 / (nth - 1) - 1.0;
    const double wt = (g.cossc - cosm) / (cosp - cosm);
    const int nw = o.n_wav;
    const double lm = o.lQp[(size_t)nw * (o.n_theta * id + cm) + wj];
    const double lp = o.lQp[(size_t)nw * (o.n_theta * id + cm + 1) + wj];
    const double P = exp(lm + (lp - lm) * wt);
    const double dPdc = P * (lp - lm) / (cosp - cosm);
    const double s = o.size[id];
    const double Ks = o.in[wj] * kPI * s * s * o.Qsca[(size_t)nw * id + wj] / (g.R * g.R) / kAU / kAU;
    const double Fscat = Ks * P;
    const double Kt = s * s * o.Qabs[(size_t)nw * id + wj] / v.dist / v.dist;
    const double scale = n * 1e26 * wvl * wvl / kCspeed;
    F = scale * (I * Kt + Fscat);
    dFdR = scale * (dIdT * g.dTdR * Kt - 2.0 * Fscat / g.R);
    dFdc = scale * Ks * dPdc;
}

// Whether the bilinear footprint of a tracer (the four pixel centres around (u, w)) can touch
// the frame: u in (-1, xsize) and w in (-1, ysize).  Outside it every weight on a frame
// pixel is zero, and the pixel indices of a tracer far away (a grain thrown out to 1e15 AU
// by a strong Lorentz force) would overflow int.  False for NaN.
__device__ __forceinline__ bool in_reach(const TracerFlux& g, const ViewConst& v) {
    return g.u > -1.0 && g.u < (double)v.xsize && g.w > -1.0 && g.w < (double)v.ysize;
}

__global__ void image_splat_kernel(const double* __restrict__ y, const double* __restrict__ N,
                                   const int* __restrict__ idv, int nd, const ViewConst* __restrict__ vcp,
                                   OpticsDev o, ImageList il, double* __restrict__ img) {
    __shared__ ViewConst v;
    if (threadIdx.x == 0) v = *vcp;
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nd) return;
    const int id = idv[i];
    const double n = N[i];
    if (id < 0 || id >= o.n_grid || n == 0.0) return;
    TracerFlux g;
    tracer_geometry(y[i], y[(size_t)nd + i], y[2 * (size_t)nd + i], id, v, o, g);
    if (!(g.R > o.Rmin) || !in_reach(g, v)) return;
    const int i0 = (int)floor(g.u), j0 = (int)floor(g.w);
    const double fu = g.u - i0, fw = g.w - j0;
    const size_t npix = (size_t)v.xsize * v.ysize;
    for (int k = 0; k < il.n; ++k) {
        double F, dFdR, dFdc;
        flux_grad(n, id, il.wj[k], g, o, v, F, dFdR, dFdc);
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b) {
                const int px = i0 + a, py = j0 + b;
                if (px < 0 || px >= v.xsize || py < 0 || py >= v.ysize) continue;
                const double wgt = (a ? fu : 1.0 - fu) * (b ? fw : 1.0 - fw);
                atomicAdd(&img[k * npix + (size_t)v.ysize * px + py], F * wgt);
            }
    }
}

__global__ void image_splat_adjoint_kernel(const double* __restrict__ y, const double* __restrict__ N,
                                           const int* __restrict__ idv, int nd, const ViewConst* __restrict__ vcp,
                                           OpticsDev o, ImageList il, const double* __restrict__ G,
                                           double* __restrict__ lam, unsigned char* __restrict__ active) {
    __shared__ ViewConst v;
    if (threadIdx.x == 0) v = *vcp;
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nd) return;
    for (int c = 0; c < 6; ++c) lam[c * (size_t)nd + i] = 0.0;
    active[i] = 0;
    const int id = idv[i];
    const double n = N[i];
    if (id < 0 || id >= o.n_grid || n == 0.0) return;
    TracerFlux g;
    tracer_geometry(y[i], y[(size_t)nd + i], y[2 * (size_t)nd + i], id, v, o, g);
    if (!(g.R > o.Rmin) || !in_reach(g, v)) return;
    active[i] = 1;
    const double pos[3] = {y[i], y[(size_t)nd + i], y[2 * (size_t)nd + i]};
    const int i0 = (int)floor(g.u), j0 = (int)floor(g.w);
    const double fu = g.u - i0, fw = g.w - j0;
    const size_t npix = (size_t)v.xsize * v.ysize;
    double L[3] = {0, 0, 0};
    for (int k = 0; k < il.n; ++k) {
        double F, dFdR, dFdc;
        flux_grad(n, id, il.wj[k], g, o, v, F, dFdR, dFdc);
        double Gw = 0.0, Gu = 0.0, Gv = 0.0;   // sum G*w, sum G*dw/du, sum G*dw/dv
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b) {
                const int px = i0 + a, py = j0 + b;
                if (px < 0 || px >= v.xsize || py < 0 || py >= v.ysize) continue;
                const double gp = G[k * npix + (size_t)v.ysize * px + py];
                const double wu = a ? fu : 1.0 - fu, wv = b ? fw : 1.0 - fw;
                Gw += gp * wu * wv;
                Gu += gp * (a ? 1.0 : -1.0) * wv;
                Gv += gp * wu * (b ? 1.0 : -1.0);
            }
        for (int c = 0; c < 3; ++c) {
            const double dF = dFdR * pos[c] / g.R + dFdc * g.dcos[c];
            L[c] += Gw * dF + F * (Gu * g.du[c] + Gv * g.dw[c]);
        }
    }
    for (int c = 0; c < 3; ++c) lam[c * (size_t)nd + i] = L[c];
}

// Splits the SoA ddx_state into the adjoint's layouts.
__global__ void gather_state_kernel(ddx_state s, int ng, int nd, double* xv_m, double* y, double* N, int* idv,
                                    double* md) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ng) {
        xv_m[0 * ng + i] = s.x[i]; xv_m[1 * ng + i] = s.y[i]; xv_m[2 * ng + i] = s.z[i];
        xv_m[3 * ng + i] = s.vx[i]; xv_m[4 * ng + i] = s.vy[i]; xv_m[5 * ng + i] = s.vz[i];
        xv_m[6 * ng + i] = s.m[i];
    }
    if (i < nd) {
        const int t = ng + i;
        y[0 * (size_t)nd + i] = s.x[t]; y[1 * (size_t)nd + i] = s.y[t]; y[2 * (size_t)nd + i] = s.z[t];
        y[3 * (size_t)nd + i] = s.vx[t]; y[4 * (size_t)nd + i] = s.vy[t]; y[5 * (size_t)nd + i] = s.vz[t];
        N[i] = s.N[t];
        idv[i] = s.id[t];
        md[i] = s.m[t];
    }
}

// grad [6][ng + nd] <- massive adjoint [6][ng] and tracer adjoint [6][nd].
__global__ void scatter_grad_kernel(int ng, int nd, const double* lam_m, const double* lam, double* grad) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const size_t na = (size_t)ng + nd;
    if (i < ng)
        for (int c = 0; c < 6; ++c) grad[c * na + i] = lam_m[c * ng + i];
    if (i < nd)
        for (int c = 0; c < 6; ++c) grad[c * na + ng + i] = lam[c * (size_t)nd + i];
}

}  // namespace

// ---------------------------------------------------------------------------------------
// Host orchestration
// ---------------------------------------------------------------------------------------

struct AdjointScratch {
    int ng = 0, nd = 0, n_steps = 0, K = 0, nck = 0, nblk = 0;
    double dt = 0;
    StepArgs sa{};
    ddx_view view{};
    ImageList il{};
    bool ready = false;
    // buffers
    double *xv_m = nullptr, *y0 = nullptr, *y = nullptr, *N0 = nullptr, *N = nullptr, *ck = nullptr,
           *seg = nullptr, *lam = nullptr, *part = nullptr, *mu = nullptr, *lam_m = nullptr, *lam_mass = nullptr;
    int* idv = nullptr;
    double* md = nullptr;                 // [nd] tracer masses
    double *macc = nullptr, *lamS = nullptr;   // large massive sets: [6][ng] forward A1, A2; [27][ng] body adjoints
    unsigned char* active = nullptr;
    Body* Ps = nullptr;
    ViewConst* vc = nullptr;
    size_t bytes = 0;
};

void adjoint_free(AdjointScratch*& a) {
    if (!a) return;
    cudaFree(a->xv_m); cudaFree(a->y0); cudaFree(a->y); cudaFree(a->N0); cudaFree(a->N); cudaFree(a->ck);
    cudaFree(a->seg); cudaFree(a->lam); cudaFree(a->part); cudaFree(a->mu); cudaFree(a->lam_m);
    cudaFree(a->lam_mass); cudaFree(a->idv); cudaFree(a->active); cudaFree(a->Ps); cudaFree(a->vc);
    cudaFree(a->md); cudaFree(a->macc); cudaFree(a->lamS);
    delete a;
    a = nullptr;
}

// Recompute record per tracer per step: state + a1..a3, then per stage 1/R^2 and 1/R of
// the star and 1/|e| of bodies 1..nir (all bodies when n_grav <= 4).
static int record_nir(int ng) { return ng - 1 <= kMaxStoredIr ? ng - 1 : 0; }
static int record_comps(int ng) { return kSegComp + 4 * (2 + record_nir(ng)); }

static AdjArgs adj_args(const AdjointScratch& a, const SizeBin* bins) {
    AdjArgs A;
    A.ng = a.ng;
    A.nd = a.nd;
    A.nir = record_nir(a.ng);
    A.ncomp = record_comps(a.ng);
    A.dt = a.dt;
    A.sa = a.sa;
    A.Ps = a.Ps;
    A.bins = bins;
    A.id = a.idv;
    A.mass = a.md;
    return A;
}

int adjoint_forward(AdjointScratch*& a, const ddx_state& s, int ng, int nd, double dt, int n_steps, int K,
                    const StepArgs& sa, const ddx_view& view, const ImageList& il, const SizeBin* bins,
                    const OpticsDev& o, double* image, cudaStream_t st) {
    adjoint_free(a);
    a = new AdjointScratch();
    a->ng = ng; a->nd = nd; a->dt = dt; a->n_steps = n_steps; a->K = K; a->sa = sa; a->view = view; a->il = il;
    a->nck = n_steps / K + 1;
    a->nblk = (nd + kThreads - 1) / kThreads;
    const size_t nd6 = 6ull * nd;
    // a large massive set keeps one step's block sums, a small one a whole segment's
    const bool large = ng > kMaxGrav;
    const size_t part_words = large ? (size_t)a->nblk * 4 * ng * 4 : (size_t)a->nblk * K * 4 * ng * 4;
    const size_t mu_words = large ? (size_t)4 * ng * 4 : (size_t)K * 4 * ng * 4;
    bool fail = cudaMalloc(&a->xv_m, sizeof(double) * 7 * ng) || cudaMalloc(&a->y0, sizeof(double) * nd6) ||
                cudaMalloc(&a->y, sizeof(double) * nd6) || cudaMalloc(&a->N0, sizeof(double) * nd) ||
                cudaMalloc(&a->N, sizeof(double) * nd) || cudaMalloc(&a->ck, sizeof(double) * nd6 * a->nck) ||
                cudaMalloc(&a->seg, sizeof(double) * (size_t)record_comps(ng) * nd * K) ||
                cudaMalloc(&a->lam, sizeof(double) * nd6) ||
                cudaMalloc(&a->part, sizeof(double) * (part_words > 0 ? part_words : 1)) ||
                cudaMalloc(&a->mu, sizeof(double) * mu_words) ||
                cudaMalloc(&a->md, sizeof(double) * (nd > 0 ? nd : 1)) ||
                (large && (cudaMalloc(&a->macc, sizeof(double) * 6 * ng) ||
                           cudaMalloc(&a->lamS, sizeof(double) * 27 * ng))) ||
                cudaMalloc(&a->lam_m, sizeof(double) * 6 * ng) || cudaMalloc(&a->lam_mass, sizeof(double) * ng) ||
                cudaMalloc(&a->idv, sizeof(int) * nd) || cudaMalloc(&a->active, nd) ||
                cudaMalloc(&a->Ps, sizeof(Body) * (size_t)n_steps * 4 * ng) || cudaMalloc(&a->vc, sizeof(ViewConst));
    if (fail) {
        adjoint_free(a);
        cudaGetLastError();
        return DDX_ERR_NOMEM;
    }
    const int thr = 256;
    const int blk = ((nd > ng ? nd : ng) + thr - 1) / thr;
    gather_state_kernel<<<blk, thr, 0, st>>>(s, ng, nd, a->xv_m, a->y0, a->N0, a->idv, a->md);
    if (!large) {
        massive_traj_kernel<<<1, 32, 0, st>>>(ng, n_steps, dt, a->xv_m, a->Ps);
    } else {
        // three launches per step (a warp per body), the stage records of every step kept
        const int tb = 256, wb = (ng * 32 + tb - 1) / tb;
        for (int n = 0; n < n_steps; ++n) {
            Body* P = a->Ps + (size_t)n * 4 * ng;
            massive_fwd_init_kernel<<<(ng + tb - 1) / tb, tb, 0, st>>>(ng, dt, a->xv_m, P);
            massive_fwd_pass1_kernel<<<wb, tb, 0, st>>>(ng, dt, a->xv_m, P, a->macc);
            massive_fwd_pass2_kernel<<<wb, tb, 0, st>>>(ng, dt, a->xv_m, P, a->macc);
        }
    }
    cudaMemcpyAsync(a->y, a->y0, sizeof(double) * nd6, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(a->N, a->N0, sizeof(double) * nd, cudaMemcpyDeviceToDevice, st);
    const AdjArgs A = adj_args(*a, bins);
    // the forward also keeps the records of the last segment, which the backward then
    // does not recompute
    const int last0 = ((n_steps + K - 1) / K - 1) * K;
    if (nd > 0)
        dust_forward_kernel<<<a->nblk, kThreads, 0, st>>>(A, a->y, a->N, 0, n_steps, K, a->ck, a->seg, last0);
    if (launch_view_setup(a->vc, view, o.n_theta, st) != cudaSuccess) return DDX_ERR_CUDA;
    const size_t npix = (size_t)view.xsize * view.ysize;
    cudaMemsetAsync(image, 0, sizeof(double) * npix * il.n, st);
    if (nd > 0)
        image_splat_kernel<<<(nd + 255) / 256, 256, 0, st>>>(a->y, a->N, a->idv, nd, a->vc, o, il, image);
    if (cudaGetLastError() != cudaSuccess) return DDX_ERR_CUDA;
    a->ready = true;
    return DDX_OK;
}

int adjoint_backward(AdjointScratch* a, const double* G, double* grad_state, double* grad_mass,
                     const SizeBin* bins, const OpticsDev& o, cudaStream_t st) {
    if (!a || !a->ready) return DDX_ERR_STATE;
    const int ng = a->ng, nd = a->nd, K = a->K;
    const AdjArgs A = adj_args(*a, bins);
    cudaMemsetAsync(a->lam_m, 0, sizeof(double) * 6 * ng, st);
    cudaMemsetAsync(a->lam_mass, 0, sizeof(double) * ng, st);
    if (nd > 0)
        image_splat_adjoint_kernel<<<(nd + 255) / 256, 256, 0, st>>>(a->y, a->N, a->idv, nd, a->vc, o, a->il, G,
                                                                    a->lam, a->active);
    const int nseg = (a->n_steps + K - 1) / K;
    for (int sgi = nseg - 1; sgi >= 0; --sgi) {
        const int n0 = sgi * K, n1 = (n0 + K < a->n_steps) ? n0 + K : a->n_steps;
        const int Kseg = n1 - n0;
        if (nd > 0) {
            // recompute the segment from its checkpoint (the last one's records are still
            // there from the forward); the N flags are not needed since only tracers alive at
            // the end carry an adjoint, and those were alive throughout
            if (sgi != nseg - 1) {
                cudaMemcpyAsync(a->y, a->ck + (size_t)(n0 / K) * 6 * nd, sizeof(double) * 6 * nd,
                                cudaMemcpyDeviceToDevice, st);
                cudaMemcpyAsync(a->N, a->N0, sizeof(double) * nd, cudaMemcpyDeviceToDevice, st);
                dust_forward_kernel<<<a->nblk, kThreads, 0, st>>>(A, a->y, a->N, n0, n1, K, nullptr, a->seg, n0);
            }
            if (ng <= kMaxGrav) {
                dust_reverse_kernel<<<a->nblk, kThreads, 0, st>>>(A, a->seg, n0, n1, a->lam, a->active, a->part);
                const int per = Kseg * 4 * ng * 4;
                reduce_parts_kernel<<<(per + 255) / 256, 256, 0, st>>>(a->part, a->nblk, per, a->mu);
            }
        } else {
            cudaMemsetAsync(a->mu, 0, sizeof(double) * (size_t)(ng <= kMaxGrav ? Kseg : 1) * 4 * ng * 4, st);
        }
        if (ng <= kMaxGrav) {
            massive_reverse_kernel<<<1, 32, 0, st>>>(ng, a->dt, a->Ps, a->mu, n0, n1, a->lam_m, a->lam_mass);
            continue;
        }
        // large massive set: per step, the tracers' reverse with block sums of the bodies'
        // adjoints, their reduction, then the massive set's reverse stage by stage
        const int tb = 256, wb = (ng * 32 + tb - 1) / tb;
        const int per = 4 * ng * 4;
        for (int n = n1 - 1; n >= n0; --n) {
            if (nd > 0) {
                dust_reverse_step_kernel<<<a->nblk, kThreads, 0, st>>>(A, a->seg, n - n0, n, a->lam, a->active,
                                                                       a->part);
                reduce_parts_kernel<<<(per + 255) / 256, 256, 0, st>>>(a->part, a->nblk, per, a->mu);
            }
            massive_rev_init_kernel<<<(ng + tb - 1) / tb, tb, 0, st>>>(ng, a->dt, a->lam_m, a->lamS);
            for (int sg = 3; sg >= 0; --sg)
                massive_rev_stage_kernel<<<wb, tb, 0, st>>>(ng, a->dt, a->Ps + ((size_t)n * 4 + sg) * ng, a->mu, sg,
                                                            a->lamS, a->lam_m, a->lam_mass);
        }
    }
    const int thr = 256, blk = ((nd > ng ? nd : ng) + thr - 1) / thr;
    scatter_grad_kernel<<<blk, thr, 0, st>>>(ng, nd, a->lam_m, a->lam, grad_state);
    cudaMemcpyAsync(grad_mass, a->lam_mass, sizeof(double) * ng, cudaMemcpyDeviceToDevice, st);
    // restore the final state for a later image/backward (the recompute overwrote y and N)
    if (cudaGetLastError() != cudaSuccess) return DDX_ERR_CUDA;
    a->ready = false;
    return DDX_OK;
}

}  // namespace ddx
