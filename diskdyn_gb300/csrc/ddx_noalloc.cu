// ddx_step_noalloc: the RK4 step without any device allocation.
//
// Some callers cannot call cudaMalloc.  A host that runs inside a framework which owns
// all device memory through its own pool allocator may be forbidden to allocate behind
// the pool's back, and a long-running integration loop may have to keep a fixed device
// footprint that is declared up front.  The regular entry points grow the context's
// scratch with cudaMalloc on demand, so they cannot serve those callers.  This entry
// point needs no context: its scratch (the massive-set stage buffers and the packed
// size-bin table) is one file-scope __device__ array of a fixed size, which every GPU
// that loads the library holds until the process exits.  The caller passes all inputs
// and outputs as device pointers, as for ddx_step.
//
// The kernels are the same as ddx_step's; only the place of the scratch differs.
#include <mutex>
#include "ddx_internal.cuh"

namespace {

using namespace ddx;

constexpr int kCap = DDX_NOALLOC_MAX_GRAV;

// Byte offsets of the scratch regions, each 256-byte aligned.
constexpr size_t align256(size_t n) { return (n + 255) / 256 * 256; }
constexpr size_t kOffP = 0;
constexpr size_t kOffPhi = kOffP + align256(sizeof(Body) * 4 * kCap);
constexpr size_t kOffPlo = kOffPhi + align256(sizeof(float4) * 4 * kCap);
constexpr int kPcap = pair_count(kCap) + kPairSpan;
constexpr size_t kOffPP = kOffPlo + align256(sizeof(float4) * 4 * kCap);
constexpr size_t kOffPM = kOffPP + align256(sizeof(BodyPair) * 4 * kPcap);
constexpr size_t kOffA = kOffPM + align256(sizeof(float2) * 4 * kPcap);
constexpr size_t kOffR = kOffA + align256(sizeof(double) * 12 * kCap);
constexpr size_t kOffBins = kOffR + align256(sizeof(double) * 9 * kCap);
constexpr size_t kOffStatus = kOffBins + align256(sizeof(SizeBin) * DDX_MAX_SIZE_BINS);
// Slice sums of the mixed massive passes for GPUs of up to kMaxSMs SMs (GB300 has 152).  On a
// GPU with more, the passes find the region too small (sliced_fits) and take the
// one-warp-per-target form instead: the same sums, slower.
constexpr int kMaxSMs = 160;
constexpr long long kPartWords = massive_part_words_for(kCap, kMaxSMs);
constexpr size_t kOffPart = kOffStatus + 256;
constexpr size_t kBytes = kOffPart + align256(sizeof(double) * kPartWords);

static __device__ __align__(256) unsigned char g_step_scratch[kBytes];

// Device address of g_step_scratch per device, resolved once per device with that device
// current.  In host code the symbol itself is only a host-side stand-in.
std::mutex g_mu;
void* g_addr[128] = {};
// Failure-detection test hook: per device, the tile whose copy the next mixed call leaves
// unissued (-1: none) and the bound on its waits.
int g_lose_tile[128];
unsigned long long g_lose_wait[128];
bool g_hooks_init = false;

void hooks_init() {
    if (g_hooks_init) return;
    for (int d = 0; d < 128; ++d) g_lose_tile[d] = -1, g_lose_wait[d] = 0;
    g_hooks_init = true;
}

int scratch_address(int device, unsigned char** out) {
    if (device < 0 || device >= 128) return DDX_ERR_ARG;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[device]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_step_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return DDX_ERR_CUDA;
        }
        // the status word starts cleared (one word, set once per device, before any step)
        if (cudaMemset(static_cast<unsigned char*>(p) + kOffStatus, 0, sizeof(int)) != cudaSuccess ||
            cudaDeviceSynchronize() != cudaSuccess)
            return DDX_ERR_CUDA;
        g_addr[device] = p;
    }
    *out = static_cast<unsigned char*>(g_addr[device]);
    return DDX_OK;
}

__global__ void pack_bins_kernel(SizeBin* bins, int n, const float* beta, const float* betasw,
                                 const float* q) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) bins[k] = SizeBin{beta[k], betasw[k], q[k], 0.f};
}

// Star-only reference behaviour: stage positions stay at the set-up zeros.
__global__ void star_only_kernel(ddx_state s, MassiveScratch ms) {
    if (threadIdx.x < 4) {
        const double m = s.m[0];
        ms.P[threadIdx.x * ms.cap] = make_body(0.0, 0.0, 0.0, m);
        ms.Phi[threadIdx.x * ms.cap] = make_float4(0.f, 0.f, 0.f, (float)m);
        ms.Plo[threadIdx.x * ms.cap] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

}  // namespace

extern "C" int ddx_step_noalloc(int device, const ddx_state* s, int n_grav, int n_dust, double dt,
                                const ddx_phys* p, int n_grid, const float* beta,
                                const float* betasw, const float* q, int precision, int mode,
                                void* stream) {
    if (!s || !s->x || !s->y || !s->z || !s->vx || !s->vy || !s->vz || !s->m || !s->N || !s->id || !p)
        return DDX_ERR_ARG;
    if (n_grav < 1 || n_dust < 0 || n_grid < 1 || !beta || !betasw || !q) return DDX_ERR_ARG;
    if (!step_precision_ok(precision)) return DDX_ERR_ARG;
    if (mode != DDX_MODE_FIXED && mode != DDX_MODE_REFERENCE) return DDX_ERR_ARG;
    if (p->n_planets < 0 || p->n_planets > n_grav) return DDX_ERR_ARG;
    if (n_grav > DDX_NOALLOC_MAX_GRAV || n_grid > DDX_MAX_SIZE_BINS) return DDX_ERR_RANGE;
    if (device < 0 || device >= 128) return DDX_ERR_ARG;
    DeviceGuard dg(device);
    if (!dg.ok()) return DDX_ERR_CUDA;
    unsigned char* base = nullptr;
    int r = scratch_address(device, &base);
    if (r) return r;

    MassiveScratch ms{};   // no spatial order here: slot and the order scratch stay null
    ms.P = reinterpret_cast<Body*>(base + kOffP);
    ms.Phi = reinterpret_cast<float4*>(base + kOffPhi);
    ms.Plo = reinterpret_cast<float4*>(base + kOffPlo);
    ms.A = reinterpret_cast<double*>(base + kOffA);
    ms.R = reinterpret_cast<double*>(base + kOffR);
    ms.PP = reinterpret_cast<BodyPair*>(base + kOffPP);
    ms.PM = reinterpret_cast<float2*>(base + kOffPM);
    ms.status = reinterpret_cast<int*>(base + kOffStatus);
    ms.cap = kCap;
    ms.pcap = kPcap;
    ms.part = reinterpret_cast<double*>(base + kOffPart);
    ms.part_words = kPartWords;   // the passes check it against the device's SM count
    SizeBin* bins = reinterpret_cast<SizeBin*>(base + kOffBins);

    StepArgs a;
    a.n_grav = n_grav;
    a.n_exact = p->n_planets > 1 ? p->n_planets : 1;
    a.n_dust = n_dust;
    a.dt = dt;
    a.dt2 = dt * 0.5;
    a.dt6 = dt / 6.0;
    a.SWQ = p->SWQ;
    a.FLQ = p->FLQ;
    a.Wz = p->Wz;
    a.Bstar = p->Bstar;
    a.Rstar = p->Rstar;
    a.vswAU = p->vsw_AUyr;
    a.Rmin = p->Rmin;
    a.mode = mode;
    a.lose_tile = -1;
    a.wait_ns = kDefaultWaitNs;
    if (precision != DDX_PREC_FP64) {
        std::lock_guard<std::mutex> lk(g_mu);
        hooks_init();
        if (g_lose_tile[device] >= 0) {
            a.lose_tile = g_lose_tile[device];
            a.wait_ns = g_lose_wait[device];
            g_lose_tile[device] = -1;
        }
    }
    a.near_eta = default_near_eta(precision);
    a.comp_eta = kDefaultCompEta;
    a.n_grid = n_grid;

    // Every scratch word a step reads is written earlier in the same step (the packed bins,
    // then the stage records of bodies 0..n_grav-1), so nothing has to be cleared between
    // calls.  The status word alone carries over: kernels only set its bits, and
    // ddx_noalloc_sync_status reads and clears it (the array starts zeroed).
    cudaStream_t st = (cudaStream_t)stream;
    pack_bins_kernel<<<(n_grid + 255) / 256, 256, 0, st>>>(bins, n_grid, beta, betasw, q);
    if (cudaGetLastError() != cudaSuccess) return DDX_ERR_CUDA;
    const ddx_state& sv = *s;
    if (n_grav == 1 && mode == DDX_MODE_REFERENCE) {
        star_only_kernel<<<1, 32, 0, st>>>(sv, ms);
        if (cudaGetLastError() != cudaSuccess) return DDX_ERR_CUDA;
        return launch_dust(sv, a, ms, bins, precision, st) == cudaSuccess ? DDX_OK : DDX_ERR_CUDA;
    }
    if (launch_massive_prepare(sv, a, ms, precision, st) != cudaSuccess) return DDX_ERR_CUDA;
    if (launch_massive_pass1(sv, a, ms, precision, st) != cudaSuccess) return DDX_ERR_CUDA;
    if (launch_massive_pass2(sv, a, ms, precision, st) != cudaSuccess) return DDX_ERR_CUDA;
    return launch_dust(sv, a, ms, bins, precision, st) == cudaSuccess ? DDX_OK : DDX_ERR_CUDA;
}

extern "C" int ddx_noalloc_sync_status(int device, void* stream) {
    if (device < 0 || device >= 128) return DDX_ERR_ARG;
    DeviceGuard dg(device);
    if (!dg.ok()) return DDX_ERR_CUDA;
    unsigned char* base = nullptr;
    int r = scratch_address(device, &base);
    if (r) return r;
    cudaStream_t st = (cudaStream_t)stream;
    int* status = reinterpret_cast<int*>(base + kOffStatus);
    int h = 0;
    if (cudaStreamSynchronize(st) != cudaSuccess) return DDX_ERR_CUDA;
    // a plain copy into a host int and a memset of the one word: no allocation
    if (cudaMemcpy(&h, status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return DDX_ERR_CUDA;
    if (h != 0 && cudaMemset(status, 0, sizeof(int)) != cudaSuccess) return DDX_ERR_CUDA;
    return (h & kStatusTimeout) ? DDX_ERR_TIMEOUT : DDX_OK;
}

extern "C" int ddx_debug_noalloc_lose_tile_copy(int device, int tile, unsigned long long wait_ns) {
    if (device < 0 || device >= 128 || tile < 0 || wait_ns == 0) return DDX_ERR_ARG;
    std::lock_guard<std::mutex> lk(g_mu);
    hooks_init();
    g_lose_tile[device] = tile;
    g_lose_wait[device] = wait_ns;
    return DDX_OK;
}
