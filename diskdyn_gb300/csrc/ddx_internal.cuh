// Internal declarations shared by the sm_103a kernels of the DiskDyn dynamical and
// imaging path.  Physical constants carry the reference's values (src/ddyn.cuh:17-38)
// because every flux and drag term is compared against the reference bit-for-bit or to
// a few ulps; changing one would move every result.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <vector>
#include "../../include/diskdyn_gb300.h"
#include "../../include/diskdyn_gb300_io.h"

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
    int    n_grid;          // size bins; a tracer whose id is outside [0, n_grid) has no bin
    int    n_exact;         // bodies 0..n_exact-1 (star, planets) act in FP64 in the mixed path
    double dt, dt2, dt6;    // dt, dt/2, dt/6 formed exactly as the reference forms them
    int    SWQ, FLQ;
    double Wz, Bstar, Rstar, vswAU, Rmin;
    int    mode;            // DDX_MODE_*
    int    lose_tile;       // test hook: tile whose copy is never issued (-1: none)
    unsigned long long wait_ns;   // bound on any one device-side wait
    float  near_eta;        // mixed path: an FP32 source nearer to a body than near_eta times the
                            // body's largest |coordinate| takes the FP64 pair force instead (0: none)
    float  comp_eta;        // compensated path: spans nearer to a tracer than comp_eta times its
                            // largest |coordinate| take the float-float pull
};

// Default near radius of the mixed path, relative to the body's largest |coordinate|, and
// of the compensated path, whose float-float pulls leave the 48-bit positions' rounding
// (about 2^-48 of a coordinate) as the largest error of a close pull: exact FP64 pulls out
// to 1.6e-2 of the coordinate bring the worst 1,000-step grain of the dusty ring from 8.6e-10
// to 5.0e-10 of its FP64 position for 5 % more time.
constexpr float kDefaultNearEta = 4.0e-3f;
constexpr float kDefaultCompNearEta = 1.6e-2f;
__host__ __device__ inline float default_near_eta(int precision) {
    return precision == DDX_PREC_COMPENSATED ? kDefaultCompNearEta : kDefaultNearEta;
}
// Default radius of the float-float spans of DDX_PREC_COMPENSATED, relative to the tracer's
// largest |coordinate|.
constexpr float kDefaultCompEta = 0.5f;
// Largest accepted near radius: far spans (dust kernel) start a quarter of the largest
// coordinate away, so a far span holds no source nearer than the near radius.
constexpr float kMaxNearEta = 0.25f;

// 1 / (near_eta * own): a source is near when its FP32 reciprocal distance exceeds this
// (infinite when either factor is 0, so nothing is near).
__device__ __forceinline__ float near_inv(float near_eta, float own) {
    const float r = near_eta * own;
    return r > 0.f ? __frcp_rn(r) : INFINITY;
}
// Largest of three floats (one sm_100+ instruction); a NaN input is ignored unless all are.
__device__ __forceinline__ float fmax3(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

constexpr unsigned long long kDefaultWaitNs = 2000000000ull;   // 2 s

// One massive body at one RK4 stage: position and mass.  32-byte aligned so a record
// moves with one 256-bit access.
struct __align__(32) Body {
    double x, y, z, m;
};
__host__ __device__ __forceinline__ Body make_body(double x, double y, double z, double m) {
    Body b; b.x = x; b.y = y; b.z = z; b.m = m; return b;
}

// Two perturbing bodies (sources 1+2k and 2+2k of one RK4 stage) in the layout the mixed
// dust kernel consumes: every 8-byte slot holds the same quantity of both bodies, so one
// f32x2 instruction works on the pair.  hi/lo is the FP32 split x = hi + lo with
// hi = fp32(x), lo = fp32(x - hi).  64 bytes, moved into shared memory by TMA bulk copies.
// pad: free for the force loops; the mixed dust launch writes the box of each span of
// kPairSpan records into the pads of its first four records.
struct __align__(16) BodyPair {
    float hx[2], hy[2], hz[2], m[2];
    float lx[2], ly[2], lz[2], pad[2];
};

constexpr int kPairSpan = 16;    // pair records per plain-FP32 partial sum (32 sources)

// Pair records per stage for n_src FP32 sources (bodies n_exact..n_grav-1) in pairs,
// padded with zero-mass records to a multiple of kPairSpan.
__host__ __device__ constexpr int pair_count(int n_src) {
    const int np = (n_src + 1) / 2;
    return (np + kPairSpan - 1) / kPairSpan * kPairSpan;
}

// Scratch of one cell ordering (ddx_order.cu) of up to cap bodies.
struct OrderScratch {
    uint32_t *key, *rank;      // [cap] cell of each body, its rank in the cell
    uint32_t *count, *start;   // [kOrderBins + 1] bodies per cell, first position of each cell
    uint32_t *temp;            // scan scratch
    int      *box;             // [6] bounding box, min then max per axis (ordered-int floats)
    int      *perm;            // [cap] the order: perm[position] = body
    int       cap;
    bool      stable;          // stable radix sort (timing-independent order) instead of atomics
};
constexpr int kOrderBits = 6;                                   // cell index bits per axis
constexpr uint32_t kOrderBins = 1u << (3 * kOrderBits);         // cells; one more for removed bodies
cudaError_t order_alloc(OrderScratch& o, int cap, bool stable);
void order_free(OrderScratch& o);
// Orders bodies [first, first + n) of s by the code of their cell on a grid over their
// bounding box (64^3 cells; 32^3 and equal codes in index order when o is stable): the
// Hilbert index on cubic cells when hilbert, else the Morton code on cells stretched to the
// box per axis.  perm[position] = body - first and, when inv is given, inv[body - first] =
// position.  With dead_last, bodies with N == 0 come last.  Stream-ordered.
cudaError_t order_bodies(const ddx_state& s, int first, int n, bool dead_last, const OrderScratch& o, int* perm,
                         int* inv, bool hilbert, cudaStream_t st);

// The mixed step orders its tracers and FP32 sources in space (far spans, ddx_order.cu)
// from this many sources on.  With fewer, the dust kernel is short and the orders and span
// boxes (about 60 us a step) cost more than the far spans save: with 256 planetesimals and
// 262,144 grains a step took 0.15 ms longer.
constexpr int kOrderMinSources = 1024;
__host__ __device__ inline bool spatial_order_on(const StepArgs& a) {
    return a.n_grav - a.n_exact >= kOrderMinSources;
}

// Stage scratch for the massive set.  Positions of the four RK4 stages are kept as
// {x, y, z, m} records for the FP64 dust kernels.  The mixed path also keeps an FP32
// hi/lo split of each stage position, per body (Phi/Plo, for the massive passes) and in
// pair records (PP, for the dust kernel).
struct MassiveScratch {
    Body     *P;      // [4][cap] stage positions P1..P4 with the mass
    float4   *Phi;    // [4][cap] fp32 hi part, m in .w
    float4   *Plo;    // [4][cap] fp32 lo part
    BodyPair *PP;     // [4][pcap] pair records of sources 1..n_grav-1
    float2   *PM;     // [4][pcap] low parts of the two masses of each pair record (m - fp32(m))
    double   *A;      // [4][3][cap] stage accelerations A1..A4
    double   *R;      // [3][3][cap] stage velocities R2..R4
    int      *status; // device status word: DDX_STATUS_* bits set by kernels
    int       cap;
    int       pcap;   // pair records per stage, >= pair_count(cap)
    double   *part;   // [slices][6][n_grav rounded to 256] per-slice sums of the mixed passes
                      // (null: one warp per target instead)
    long long part_words;
    // Spatial order of the mixed dust kernel (all null: index order, every span near).
    int      *slot;      // [cap] pair slot of FP32 source k (body n_exact + k), in cell order
    int      *src;       // [cap] its inverse: FP32 source of pair slot q (written with slot)
    OrderScratch src_order;    // ordering of the FP32 sources (cap bodies)
    OrderScratch dust_order;   // ordering of the tracers of one dust launch
};

// Makes `device` current for the scope of an entry point and makes the caller's current
// device current again on every return path, so a host that drives several GPUs from one
// thread keeps its own choice of device.
class DeviceGuard {
  public:
    explicit DeviceGuard(int device) {
        if (cudaGetDevice(&prev_) != cudaSuccess) prev_ = -1;
        ok_ = cudaSetDevice(device) == cudaSuccess;
    }
    ~DeviceGuard() {
        if (prev_ >= 0) cudaSetDevice(prev_);
    }
    bool ok() const { return ok_; }
    DeviceGuard(const DeviceGuard&) = delete;
    DeviceGuard& operator=(const DeviceGuard&) = delete;

  private:
    int prev_ = -1;
    bool ok_ = false;
};

// Mixed massive passes over source slices (ddx_step.cu): targets per block, and the blocks
// per SM the slices aim at.  The slice sums of a system of up to cap bodies on a GPU with
// sms SMs take massive_part_words_for(cap, sms) doubles: S slices * np targets with
// S <= kSliceBlocksPerSM * sms / groups + 1, so S * np <= (kSliceBlocksPerSM * sms + groups) * 256.
constexpr int kSliceThreads = 256;
constexpr int kSliceBlocksPerSM = 4;
constexpr long long massive_part_words_for(int cap, int sms) {
    return 6LL * kSliceThreads * ((long long)kSliceBlocksPerSM * sms + (cap + kSliceThreads - 1) / kSliceThreads);
}

// Precisions the step entry points take.
inline bool step_precision_ok(int p) {
    return p == DDX_PREC_FP64 || p == DDX_PREC_MIXED || p == DDX_PREC_COMPENSATED;
}

// Bits of the device status word.
constexpr int kStatusTimeout = 1;   // a bounded mbarrier wait gave up

// FP64 -> FP32 toward zero with integer operations only (FP64 instructions, conversions
// included, issue at 1/64 of the FP32 rate on sm_103a): +-0 below the FP32 normals, +-inf
// beyond the FP32 range and for inf or NaN; the error is below 2^-23 |v|.
__device__ __forceinline__ float d2f_toward0(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const int e = (int)((b >> 52) & 0x7FF) - 1023;
    const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
    if (e < -126) return __uint_as_float(sign);
    if (e > 127) return __uint_as_float(sign | 0x7F800000u);
    return __uint_as_float(sign | ((uint32_t)(e + 127) << 23) | ((uint32_t)(b >> 29) & 0x7FFFFFu));
}

__device__ __forceinline__ void split_hilo(double v, float& hi, float& lo) {
    hi = __double2float_rn(v);
    lo = __double2float_rn(v - (double)hi);
}

// Star term of one stage (src/gpu_functions.cu:680-718): gravity reduced by beta+beta_sw,
// PR + stellar-wind drag, optional Lorentz force.  Returns false when the tracer is
// inside the sublimation radius.  Written operation for operation like the reference so
// that the FP64 results agree bit for bit on the same GPU.
__device__ __forceinline__ bool star_term(double dx, double dy, double dz, double rx, double ry,
                                          double rz, double m0, float bet, float betsw, float qe,
                                          double m, const StepArgs& a, double& kx, double& ky,
                                          double& kz) {
    const double RR = dx * dx + dy * dy + dz * dz;
    const double RR3 = RR * sqrt(RR);
    if (RR <= a.Rmin * a.Rmin) return false;
    const double Fg = (1.0 - bet - betsw) * m0 / RR3;
    double Fbase1;
    if (a.SWQ == 1) Fbase1 = m0 / RR * (bet / kLightAU + betsw / a.vswAU);
    else            Fbase1 = bet * m0 / kLightAU / RR;
    const double Fbase2 = (dx * rx + dy * ry + dz * rz) / RR;
    const double Fdrx = Fbase1 * (Fbase2 * dx + rx);
    const double Fdry = Fbase1 * (Fbase2 * dy + ry);
    const double Fdrz = Fbase1 * (Fbase2 * dz + rz);
    double Flx, Fly;
    if (a.FLQ == 1) {
        const double Bz = a.Bstar * a.Rstar * a.Rstar * a.Rstar / RR3;
        Flx = qe * (ry - a.Wz * dx) * Bz / m;
        Fly = -qe * (rx + a.Wz * dy) * Bz / m;
    } else {
        Flx = 0; Fly = 0;
    }
    kx = -Fg * dx - Fdrx + Flx;
    ky = -Fg * dy - Fdry + Fly;
    kz = -Fg * dz - Fdrz;
    return true;
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
// Source slices of the mixed massive passes for n_grav bodies (about four blocks per SM),
// and the doubles of MassiveScratch::part that cover every system of up to cap bodies on
// this device (massive_part_words_for with its SM count).
int massive_slices(int n_grav, int n_exact);
long long massive_part_words(int cap);
cudaError_t launch_dust_mixed(const ddx_state& s, const StepArgs& a, const MassiveScratch& ms,
                              const SizeBin* bins, int precision, cudaStream_t st);

struct CollideScratch;   // ddx_collide.cu
int collide_run(CollideScratch*& cs, const ddx_state& s, int i0, int i1, double h, int2* pairs,
                long long cap, long long* n_pairs, cudaStream_t st);
void collide_free(CollideScratch*& cs);

// ddx_detstep.cu: the massive bodies that can set the time step, with their squared
// distance to the star (formed without contraction) and mass; synchronizes the stream.
constexpr int kDetCandidates = 256;
struct DetStepScratch {
    double* rr = nullptr;
    unsigned long long* kmin = nullptr;
    int* count = nullptr;
    int* cand = nullptr;
    int cap_bodies = 0;
};
int det_step_scan(DetStepScratch*& d, const ddx_state& s, int n_grav, cudaStream_t st,
                  std::vector<double>& rr, std::vector<double>& mi, double& m0);
void det_step_free(DetStepScratch*& d);

// Threads per block of the one-tracer-per-thread dust kernels: 256, halved (down to 64)
// while the grid would cover fewer than two blocks per SM.  FP64 runs at 1/73 of the FP32
// rate, so a few thousand grains on 256-thread blocks leave most SMs idle for tens of
// microseconds; smaller blocks spread them over the whole GPU.
int dust_block_threads(int n_dust);

// ddx_optics_prep.cu: the dust-temperature table (host arrays in and out; synchronizes).
int dust_temp_run(int n_grid, int n_wav, const double* w, const double* in, const double* Qabs, double dist,
                  double* Rmin_AU, double* Rmax_AU, double* Td, cudaStream_t st);
// ddx_optics_prep.cu: the size grid and its optical, beta and beta_sw tables (host arrays
// in and out, arguments checked by the caller; synchronizes).
int dust_grid_run(int n_wav, const double* w, const double* in, const ddx_optical_table& file,
                  const ddx_grid_setup& g, ddx_optical_table& grid, float* q, float* beta, float* betasw,
                  double* Lum, double* betaswconst, cudaStream_t st);
// ddx_api.cu: context facts for the run driver (ddx_run.cu).
int ctx_device(const ddx_ctx* c);
int ctx_optics_n_wav(const ddx_ctx* c);   // 0 when the optics are not set
// ddx_setup.cu: the initial system drawn on the GPU (arguments other than the state
// checked by the caller; synchronizes).
int setup_device_run(const ddx_param* p, double dmin, double dmax, const float* beta, unsigned long long seed,
                     const ddx_state& s, long long cap, ddx_dat_run* run, cudaStream_t st);
}  // namespace ddx
