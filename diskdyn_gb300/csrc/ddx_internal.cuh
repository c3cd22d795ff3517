// Internal declarations shared by the sm_103a kernels of the DiskDyn dynamical and
// imaging path.  Physical constants carry the reference's values (src/ddyn.cuh:17-38)
// because every flux and drag term is compared against the reference bit-for-bit or to
// a few ulps; changing one would move every result.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "../../include/diskdyn_gb300.h"

namespace ddx {

constexpr double kAU      = 1.49598e11;            // m
constexpr double kLightAU = 63239.6717367;         // speed of light, AU/yr
constexpr double kCspeed  = 299792458.0;           // m/s
constexpr double kKboltz  = 1.3806503E-23;
constexpr double kHplank  = 6.626068E-34;
constexpr double kPI      = 3.14159265358979323846;
constexpr int    kNR      = DDX_NR;

// Per-size-bin dynamical constants, one 16-byte record per bin so a tracer fetches its
// bin with one load (the reference keeps three __constant__ float arrays, which
// serialise when the lanes of a warp hold different bins).
struct __align__(16) SizeBin {
    float beta, betasw, q, pad;
};

// Scalars of one RK4 step, passed by value to the kernels.
struct StepArgs {
    int    n_grav, n_dust;
    double dt, dt2, dt6;    // dt, dt/2, dt/6 formed exactly as the reference forms them
    int    SWQ, FLQ;
    double Wz, Bstar, Rstar, vswAU, Rmin;
    int    mode;            // DDX_MODE_*
};

// One massive body at one RK4 stage: position and mass.  32-byte aligned so a record
// moves with one 256-bit access.
struct __align__(32) Body {
    double x, y, z, m;
};
__host__ __device__ __forceinline__ Body make_body(double x, double y, double z, double m) {
    Body b; b.x = x; b.y = y; b.z = z; b.m = m; return b;
}

// Stage scratch for the massive set.  Positions of the four RK4 stages are kept as
// {x, y, z, m} records so the dust kernel stages them through shared memory with
// 16-byte vector copies.  The mixed path also keeps an FP32 hi/lo split of each
// stage position: x = hi + lo with hi = fp32(x), lo = fp32(x - hi).
struct MassiveScratch {
    Body    *P;      // [4][cap] stage positions P1..P4 with the mass
    float4  *Phi;    // [4][cap] fp32 hi part, m in .w
    float4  *Plo;    // [4][cap] fp32 lo part
    double  *A;      // [4][3][cap] stage accelerations A1..A4
    double  *R;      // [3][3][cap] stage velocities R2..R4
    int      cap;
};

__device__ __forceinline__ void split_hilo(double v, float& hi, float& lo) {
    hi = __double2float_rn(v);
    lo = __double2float_rn(v - (double)hi);
}

}  // namespace ddx

// Launchers implemented in the .cu files (host side, stream-ordered).
namespace ddx {
cudaError_t launch_massive_prepare(const ddx_state& s, const StepArgs& a, MassiveScratch& ms,
                                   int precision, cudaStream_t st);
cudaError_t launch_massive_pass1(const ddx_state& s, const StepArgs& a, MassiveScratch& ms,
                                 int precision, cudaStream_t st);
cudaError_t launch_massive_pass2(const ddx_state& s, const StepArgs& a, MassiveScratch& ms,
                                 int precision, cudaStream_t st);
cudaError_t launch_dust(const ddx_state& s, const StepArgs& a, const MassiveScratch& ms,
                        const SizeBin* bins, int precision, cudaStream_t st);
}  // namespace ddx
