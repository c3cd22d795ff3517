// C ABI of the DiskDyn GB300 path: context, tables and the stream-ordered launch
// sequences behind ddx_step / ddx_evolve / ddx_image / ddx_sed.
#include <cstdlib>
#include <cstring>
#include <vector>
#include "ddx_internal.cuh"
#include "ddx_flux.cuh"
#include "../../include/diskdyn_gb300_run.h"

using namespace ddx;

struct ddx_ctx {
    int device = 0;
    // size-bin table
    int n_grid = 0;
    SizeBin* bins = nullptr;
    double* size_d = nullptr;
    // massive-set scratch
    MassiveScratch ms{};
    // optics
    bool optics_set = false;
    OpticsDev od{};
    OpticsDev* od_dev = nullptr;
    double *w = nullptr, *in = nullptr, *Qabs = nullptr, *Qsca = nullptr, *Qp = nullptr,
           *Td = nullptr, *lQp = nullptr, *lTd = nullptr, *w5 = nullptr;
    float2* lQp32p = nullptr;                   // FP32 log tables (mixed photometry)
    float* lTd32 = nullptr;
    PhotoConst photo{};                         // per-call FP32 coefficients, max(n_wav, kMaxImages) slots
    ViewConst* vc = nullptr;
    double* sed_partial = nullptr;
    int sed_partial_cap = 0;
    unsigned long long* counters = nullptr;   // [0]: tracers that took the exact pixel path
    int* status = nullptr;                      // kStatus* bits set by kernels (device)
    float near_eta = -1.f;                      // FP64 pulls within near_eta * |coordinate| (< 0: defaults)
    float comp_eta = kDefaultCompEta;           // compensated path: float-float spans within comp_eta * |coordinate|
    int inject_lose_tile = -1;                  // one-shot test hook for the next mixed dust launch
    unsigned long long inject_wait_ns = 0;
    CollideScratch* collide = nullptr;          // spatial-hash buffers, grown on demand
    AdjointScratch* adjoint = nullptr;          // trajectory checkpoints of the last adjoint forward
    DetStepScratch* detstep = nullptr;          // body scan of ddx_det_step
    float* img32 = nullptr;                     // FP32 interleaved sums of the mixed images
    size_t img32_words = 0;
    // ddx_step_host: copy streams (host to device, device to host) and their events
    cudaStream_t s_in = nullptr, s_out = nullptr;
    cudaEvent_t ev_in = nullptr, ev_comp = nullptr, ev_out = nullptr;
};

namespace {
void take_injection(ddx_ctx* c, StepArgs& a) {
    if (c->inject_lose_tile >= 0) {
        a.lose_tile = c->inject_lose_tile;
        a.wait_ns = c->inject_wait_ns;
        c->inject_lose_tile = -1;
    }
}
}  // namespace

namespace {

int cuda_status(cudaError_t e) { return e == cudaSuccess ? DDX_OK : DDX_ERR_CUDA; }

template <typename T>
cudaError_t dalloc(T** p, size_t n) {
    *p = nullptr;
    if (n == 0) n = 1;
    return cudaMalloc((void**)p, sizeof(T) * n);
}

void free_massive(MassiveScratch& ms) {
    cudaFree(ms.P); cudaFree(ms.Phi); cudaFree(ms.Plo); cudaFree(ms.PP); cudaFree(ms.PM); cudaFree(ms.A);
    cudaFree(ms.R);
    cudaFree(ms.part); cudaFree(ms.slot); cudaFree(ms.src);
    order_free(ms.src_order);
    order_free(ms.dust_order);
    ms = MassiveScratch{};   // the status word belongs to the context, not to the scratch
}

int alloc_massive(ddx_ctx* c, int n_grav);

// The massive set's scratch for n_grav bodies and, for the mixed path, the scratch of the
// spatial order of the sources and of n_dust tracers (grown on demand).
int ensure_massive(ddx_ctx* c, int n_grav, int n_dust, int precision) {
    if (!(c->ms.cap >= n_grav && c->ms.P)) {
        const int r = alloc_massive(c, n_grav);
        if (r) return r;
    }
    if (precision != DDX_PREC_FP64 && c->ms.dust_order.cap < n_dust) {
        if (order_alloc(c->ms.dust_order, n_dust, false) != cudaSuccess) {
            cudaGetLastError();
            return DDX_ERR_NOMEM;
        }
    }
    return DDX_OK;
}

int alloc_massive(ddx_ctx* c, int n_grav) {
    free_massive(c->ms);
    int cap = 64;
    while (cap < n_grav) cap *= 2;
    MassiveScratch ms{};
    ms.cap = cap;
    ms.pcap = pair_count(cap) + kPairSpan;
    ms.status = c->status;
    ms.part_words = massive_part_words(cap);
    if (dalloc(&ms.P, (size_t)4 * cap) != cudaSuccess || dalloc(&ms.Phi, (size_t)4 * cap) != cudaSuccess ||
        dalloc(&ms.Plo, (size_t)4 * cap) != cudaSuccess || dalloc(&ms.PP, (size_t)4 * ms.pcap) != cudaSuccess ||
        dalloc(&ms.PM, (size_t)4 * ms.pcap) != cudaSuccess ||
        dalloc(&ms.A, (size_t)12 * cap) != cudaSuccess || dalloc(&ms.R, (size_t)9 * cap) != cudaSuccess ||
        dalloc(&ms.part, (size_t)ms.part_words) != cudaSuccess || dalloc(&ms.slot, (size_t)cap) != cudaSuccess ||
        dalloc(&ms.src, (size_t)cap) != cudaSuccess ||
        order_alloc(ms.src_order, cap, true) != cudaSuccess) {
        ms.status = nullptr;
        free_massive(ms);
        cudaGetLastError();
        return DDX_ERR_NOMEM;
    }
    c->ms = ms;
    return DDX_OK;
}

bool state_ok(const ddx_state* s) {
    return s && s->x && s->y && s->z && s->vx && s->vy && s->vz && s->m && s->N && s->id;
}

int make_step_args(const ddx_ctx* c, const ddx_phys* p, int n_grav, int n_dust, double dt, int mode, StepArgs& a,
                   int precision = DDX_PREC_MIXED) {
    if (!p || n_grav < 1 || n_dust < 0) return DDX_ERR_ARG;
    a.near_eta = c->near_eta >= 0.f ? c->near_eta : default_near_eta(precision);
    a.comp_eta = c->comp_eta;
    a.n_grid = c->n_grid;
    if (mode != DDX_MODE_FIXED && mode != DDX_MODE_REFERENCE) return DDX_ERR_ARG;
    if (p->n_planets < 0 || p->n_planets > n_grav) return DDX_ERR_ARG;
    a.n_grav = n_grav;
    a.n_exact = p->n_planets > 1 ? p->n_planets : 1;
    a.n_dust = n_dust;
    a.dt = dt;
    a.dt2 = dt * 0.5;          // src/grid.cu:711,716 pass dt*0.5
    a.dt6 = dt / 6.0;          // src/grid.cu:750 passes dt/6.0
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
    return DDX_OK;
}

// Star-only systems: the reference never runs the massive stages when n_grav <= 1
// (src/grid.cu:698, 747), so its stage arrays keep the zeros written at set-up and the
// star never moves.  DDX_MODE_REFERENCE reproduces that; DDX_MODE_FIXED advances the star
// ballistically through the regular passes.
__global__ void star_only_reference_kernel(ddx_state s, MassiveScratch ms) {
    if (threadIdx.x < 4) {
        const double m = s.m[0];
        ms.P[threadIdx.x * ms.cap] = make_body(0.0, 0.0, 0.0, m);
        ms.Phi[threadIdx.x * ms.cap] = make_float4(0.f, 0.f, 0.f, (float)m);
        ms.Plo[threadIdx.x * ms.cap] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

// The massive set's whole step: stage positions P1..P4 for the dust and the RK4
// combination of the massive bodies (the dust reads only the stage positions).
int enqueue_massive(ddx_ctx* c, const ddx_state& s, const StepArgs& a, int precision, cudaStream_t st) {
    if (a.n_grav == 1 && a.mode == DDX_MODE_REFERENCE) {
        star_only_reference_kernel<<<1, 32, 0, st>>>(s, c->ms);
        return cuda_status(cudaGetLastError());
    }
    if (launch_massive_prepare(s, a, c->ms, precision, st) != cudaSuccess) return DDX_ERR_CUDA;
    if (launch_massive_pass1(s, a, c->ms, precision, st) != cudaSuccess) return DDX_ERR_CUDA;
    if (launch_massive_pass2(s, a, c->ms, precision, st) != cudaSuccess) return DDX_ERR_CUDA;
    return DDX_OK;
}

int enqueue_step(ddx_ctx* c, const ddx_state& s, StepArgs a, int precision, cudaStream_t st) {
    take_injection(c, a);
    const int r = enqueue_massive(c, s, a, precision, st);
    if (r) return r;
    return cuda_status(launch_dust(s, a, c->ms, c->bins, precision, st));
}

// Dust chunks of ddx_step_host: one wave of the mixed kernel (3 resident blocks of 256 on
// every SM) first and last, the rest in one launch between them.  The first chunk's copy in
// and the last chunk's copy out are all that is not overlapped; every extra launch costs
// the spread of its blocks' finishing times, so there are no more than three.
std::vector<int> dust_chunks(int n_dust) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) sms = 152;
    const int wave = sms * 3 * 256;
    if (n_dust < 4 * wave) return {n_dust};
    return {wave, n_dust - 2 * wave, wave};
}

ddx_state shifted(const ddx_state& s, long long o) {
    return ddx_state{s.x + o, s.y + o, s.z + o, s.vx + o, s.vy + o, s.vz + o, s.m + o, s.N + o, s.id + o};
}

// Copies of bodies [o, o + n) between a host state and the device state.
bool h2d_range(const ddx_state& d, const ddx_host_state& h, long long o, long long n, cudaStream_t st) {
    if (n <= 0) return true;
    double* const dd[8] = {d.x, d.y, d.z, d.vx, d.vy, d.vz, d.m, d.N};
    const double* const hh[8] = {h.x, h.y, h.z, h.vx, h.vy, h.vz, h.m, h.N};
    for (int f = 0; f < 8; ++f)
        if (cudaMemcpyAsync(dd[f] + o, hh[f] + o, sizeof(double) * n, cudaMemcpyHostToDevice, st) != cudaSuccess)
            return false;
    return cudaMemcpyAsync(d.id + o, h.id + o, sizeof(int) * n, cudaMemcpyHostToDevice, st) == cudaSuccess;
}
bool d2h_range(const ddx_host_state& h, const ddx_state& d, long long o, long long n, cudaStream_t st) {
    if (n <= 0) return true;
    double* const hh[7] = {h.x, h.y, h.z, h.vx, h.vy, h.vz, h.N};
    const double* const dd[7] = {d.x, d.y, d.z, d.vx, d.vy, d.vz, d.N};
    for (int f = 0; f < 7; ++f)
        if (cudaMemcpyAsync(hh[f] + o, dd[f] + o, sizeof(double) * n, cudaMemcpyDeviceToHost, st) != cudaSuccess)
            return false;
    return true;
}

bool host_state_ok(const ddx_host_state* h, long long n) {
    return h && h->x && h->y && h->z && h->vx && h->vy && h->vz && h->N && h->m && h->id && h->cap >= n;
}

int ensure_pipeline(ddx_ctx* c) {
    if (c->s_in) return DDX_OK;
    if (cudaStreamCreateWithFlags(&c->s_in, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->s_out, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_in, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_comp, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_out, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        return DDX_ERR_CUDA;
    }
    return DDX_OK;
}

void free_optics(ddx_ctx* c) {
    cudaFree(c->w); cudaFree(c->in); cudaFree(c->Qabs); cudaFree(c->Qsca); cudaFree(c->Qp);
    cudaFree(c->Td); cudaFree(c->lQp); cudaFree(c->lTd); cudaFree(c->w5);
    cudaFree(c->lQp32p); cudaFree(c->lTd32);
    cudaFree(c->photo.A); cudaFree(c->photo.C2); cudaFree(c->photo.esh);
    c->w = c->in = c->Qabs = c->Qsca = c->Qp = c->Td = c->lQp = c->lTd = c->w5 = nullptr;
    c->lQp32p = nullptr;
    c->lTd32 = nullptr;
    c->photo = PhotoConst{};
    c->optics_set = false;
}

}  // namespace

extern "C" {

int ddx_abi_version(void) { return DDX_ABI_VERSION; }

const char* ddx_status_string(int status) {
    switch (status) {
        case DDX_OK: return "ok";
        case DDX_ERR_ARG: return "invalid argument";
        case DDX_ERR_CUDA: return "CUDA runtime error";
        case DDX_ERR_NOMEM: return "device allocation failed";
        case DDX_ERR_STATE: return "required table not set";
        case DDX_ERR_RANGE: return "size beyond limit";
        case DDX_ERR_TIMEOUT: return "device-side wait timed out";
        case DDX_ERR_NONFINITE: return "non-finite value";
        case DDX_ERR_IO: return "file input/output failed";
        default: return "unknown status";
    }
}

int ddx_create(ddx_ctx** out, int device) {
    if (!out) return DDX_ERR_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return DDX_ERR_CUDA;
    }
    DeviceGuard dg(device);
    if (!dg.ok()) return DDX_ERR_CUDA;
    ddx_ctx* c = new ddx_ctx();
    c->device = device;
    if (dalloc(&c->vc, 1) != cudaSuccess || dalloc(&c->od_dev, 1) != cudaSuccess ||
        dalloc(&c->counters, 4) != cudaSuccess || dalloc(&c->status, 1) != cudaSuccess) {
        cudaFree(c->vc); cudaFree(c->od_dev); cudaFree(c->counters); cudaFree(c->status);
        delete c;
        return DDX_ERR_NOMEM;
    }
    cudaMemset(c->counters, 0, 4 * sizeof(unsigned long long));
    cudaMemset(c->status, 0, sizeof(int));
    *out = c;
    return DDX_OK;
}

int ddx_destroy(ddx_ctx* c) {
    if (!c) return DDX_ERR_ARG;
    DeviceGuard dg(c->device);
    free_massive(c->ms);
    free_optics(c);
    cudaFree(c->bins); cudaFree(c->size_d); cudaFree(c->vc); cudaFree(c->od_dev);
    cudaFree(c->sed_partial); cudaFree(c->counters); cudaFree(c->status); cudaFree(c->img32);
    collide_free(c->collide);
    adjoint_free(c->adjoint);
    det_step_free(c->detstep);
    if (c->s_in) cudaStreamDestroy(c->s_in);
    if (c->s_out) cudaStreamDestroy(c->s_out);
    if (c->ev_in) cudaEventDestroy(c->ev_in);
    if (c->ev_comp) cudaEventDestroy(c->ev_comp);
    if (c->ev_out) cudaEventDestroy(c->ev_out);
    delete c;
    return DDX_OK;
}

int ddx_set_size_table(ddx_ctx* c, int n_grid, const double* size, const float* beta,
                       const float* betasw, const float* q) {
    if (!c || n_grid < 0 || (n_grid > 0 && (!size || !beta || !betasw || !q))) return DDX_ERR_ARG;
    if (n_grid > DDX_MAX_SIZE_BINS) return DDX_ERR_RANGE;
    DeviceGuard dg(c->device);
    std::vector<SizeBin> h(n_grid > 0 ? n_grid : 1);
    for (int k = 0; k < n_grid; ++k) h[k] = SizeBin{beta[k], betasw[k], q[k], 0.f};
    cudaFree(c->bins); cudaFree(c->size_d);
    c->bins = nullptr; c->size_d = nullptr;
    if (dalloc(&c->bins, h.size()) != cudaSuccess || dalloc(&c->size_d, h.size()) != cudaSuccess)
        return DDX_ERR_NOMEM;
    if (cudaMemcpy(c->bins, h.data(), sizeof(SizeBin) * h.size(), cudaMemcpyHostToDevice) != cudaSuccess)
        return DDX_ERR_CUDA;
    if (n_grid > 0 && cudaMemcpy(c->size_d, size, sizeof(double) * n_grid, cudaMemcpyHostToDevice) != cudaSuccess)
        return DDX_ERR_CUDA;
    c->n_grid = n_grid;
    if (c->optics_set) c->od.size = c->size_d;
    return DDX_OK;
}

int ddx_set_optics(ddx_ctx* c, int n_grid, int n_wav, int n_theta, const double* w,
                   const double* in, const double* Qabs, const double* Qsca,
                   const double* Qpfunc, const double* Td, double Rmin, double Rmax) {
    if (!c || n_grid < 1 || n_wav < 1 || n_theta < 2 || !w || !in || !Qabs || !Qsca || !Qpfunc || !Td)
        return DDX_ERR_ARG;
    if (n_grid > DDX_MAX_SIZE_BINS) return DDX_ERR_RANGE;
    if (!(Rmin > 0.0) || !(Rmax > Rmin)) return DDX_ERR_ARG;
    if (c->n_grid != n_grid) return DDX_ERR_STATE;   // the size table gives the grain sizes
    DeviceGuard dg(c->device);
    free_optics(c);
    const size_t nq = (size_t)n_grid * n_theta * n_wav, nw = (size_t)n_grid * n_wav,
                 nt = (size_t)n_grid * DDX_NR;
    const size_t nslot = (size_t)(n_wav > kMaxImages ? n_wav : kMaxImages);
    if (dalloc(&c->w, n_wav) || dalloc(&c->in, n_wav) || dalloc(&c->Qabs, nw) || dalloc(&c->Qsca, nw) ||
        dalloc(&c->Qp, nq) || dalloc(&c->Td, nt) || dalloc(&c->lQp, nq) || dalloc(&c->lTd, nt) ||
        dalloc(&c->w5, n_wav) || dalloc(&c->lQp32p, (size_t)n_grid * (n_theta - 1) * n_wav) ||
        dalloc(&c->lTd32, nt) || dalloc(&c->photo.A, n_grid * nslot) ||
        dalloc(&c->photo.C2, nslot) || dalloc(&c->photo.esh, nslot)) {
        free_optics(c);
        cudaGetLastError();
        return DDX_ERR_NOMEM;
    }
    cudaError_t e = cudaSuccess;
    e = e ? e : cudaMemcpy(c->w, w, sizeof(double) * n_wav, cudaMemcpyHostToDevice);
    e = e ? e : cudaMemcpy(c->in, in, sizeof(double) * n_wav, cudaMemcpyHostToDevice);
    e = e ? e : cudaMemcpy(c->Qabs, Qabs, sizeof(double) * nw, cudaMemcpyHostToDevice);
    e = e ? e : cudaMemcpy(c->Qsca, Qsca, sizeof(double) * nw, cudaMemcpyHostToDevice);
    e = e ? e : cudaMemcpy(c->Qp, Qpfunc, sizeof(double) * nq, cudaMemcpyHostToDevice);
    e = e ? e : cudaMemcpy(c->Td, Td, sizeof(double) * nt, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { free_optics(c); return DDX_ERR_CUDA; }
    OpticsDev& o = c->od;
    o.w = c->w; o.in = c->in; o.Qabs = c->Qabs; o.Qsca = c->Qsca; o.Qp = c->Qp; o.Td = c->Td;
    o.size = c->size_d; o.lQp = c->lQp; o.lTd = c->lTd; o.w5 = c->w5;
    o.lQp32p = c->lQp32p; o.lTd32 = c->lTd32;
    o.Rmin = Rmin; o.Rmax = Rmax; o.fR = 0.0;
    o.n_grid = n_grid; o.n_wav = n_wav; o.n_theta = n_theta;
    if (cudaMemcpy(c->od_dev, &o, sizeof(OpticsDev), cudaMemcpyHostToDevice) != cudaSuccess) return DDX_ERR_CUDA;
    if (launch_optics_prepare(o, c->od_dev, 0) != cudaSuccess) return DDX_ERR_CUDA;
    if (cudaMemcpy(&o, c->od_dev, sizeof(OpticsDev), cudaMemcpyDeviceToHost) != cudaSuccess) return DDX_ERR_CUDA;
    c->optics_set = true;
    return DDX_OK;
}

int ddx_step(ddx_ctx* c, const ddx_state* s, int n_grav, int n_dust, double dt,
             const ddx_phys* phys, int precision, int mode, void* stream) {
    return ddx_evolve(c, s, n_grav, n_dust, dt, 1, phys, precision, mode, stream);
}

int ddx_step_host(ddx_ctx* c, const ddx_host_state* in, ddx_host_state* out, const ddx_state* s, int n_grav,
                  int n_dust, double dt, const ddx_phys* phys, int precision, int mode, void* stream) {
    if (!c || !state_ok(s) || n_grav < 1 || n_dust < 0) return DDX_ERR_ARG;
    if (!step_precision_ok(precision)) return DDX_ERR_ARG;
    const long long n_all = (long long)n_grav + n_dust;
    if (!host_state_ok(in, n_all) || !host_state_ok(out, n_all)) return DDX_ERR_ARG;
    if (!c->bins) return DDX_ERR_STATE;
    StepArgs a;
    int r = make_step_args(c, phys, n_grav, n_dust, dt, mode, a, precision);
    if (r) return r;
    DeviceGuard dg(c->device);
    if ((r = ensure_massive(c, n_grav, n_dust, precision)) || (r = ensure_pipeline(c))) return r;
    cudaStream_t st = (cudaStream_t)stream;
    take_injection(c, a);
    // the massive bodies: in, step, out (small)
    if (!h2d_range(*s, *in, 0, n_grav, st)) return DDX_ERR_CUDA;
    if ((r = enqueue_massive(c, *s, a, precision, st))) return r;
    if (!d2h_range(*out, *s, 0, n_grav, st)) return DDX_ERR_CUDA;
    // the dust, chunk by chunk: copy-in stream -> compute stream -> copy-out stream.  The
    // reference mode's stage-4 write lands at the chunk's own index, so it runs unchunked.
    // So does the spatially ordered mixed step (enough planetesimals): a chunk is a range
    // of indices, which covers the whole disk at a fraction of its density, so the chunks'
    // orders give looser boxes and fewer far spans, and every chunk repeats the order and
    // the span boxes.  Measured on the dusty ring, three chunks cost more (10.2 ms a step)
    // than the copies they hide: one chunk has its copy in overlapped with the massive set's
    // work and only the copy out exposed (0.3 ms).
    const bool ordered = precision != DDX_PREC_FP64 && spatial_order_on(a);
    const std::vector<int> chunks =
        a.mode == DDX_MODE_REFERENCE || ordered ? std::vector<int>{n_dust} : dust_chunks(n_dust);
    int o = 0;
    for (const int len : chunks) {
        if (len <= 0) continue;
        if (!h2d_range(*s, *in, n_grav + o, len, c->s_in) || cudaEventRecord(c->ev_in, c->s_in) != cudaSuccess ||
            cudaStreamWaitEvent(st, c->ev_in, 0) != cudaSuccess)
            return DDX_ERR_CUDA;
        StepArgs ac = a;
        ac.n_dust = len;
        if (o > 0) ac.lose_tile = -1;
        if (launch_dust(shifted(*s, o), ac, c->ms, c->bins, precision, st) != cudaSuccess) return DDX_ERR_CUDA;
        if (cudaEventRecord(c->ev_comp, st) != cudaSuccess || cudaStreamWaitEvent(c->s_out, c->ev_comp, 0) != cudaSuccess ||
            !d2h_range(*out, *s, n_grav + o, len, c->s_out))
            return DDX_ERR_CUDA;
        o += len;
    }
    if (cudaEventRecord(c->ev_out, c->s_out) != cudaSuccess || cudaStreamWaitEvent(st, c->ev_out, 0) != cudaSuccess)
        return DDX_ERR_CUDA;
    return cuda_status(cudaStreamSynchronize(st));
}

int ddx_evolve(ddx_ctx* c, const ddx_state* s, int n_grav, int n_dust, double dt, int n_steps,
               const ddx_phys* phys, int precision, int mode, void* stream) {
    if (!c || !state_ok(s) || n_steps < 0) return DDX_ERR_ARG;
    if (!step_precision_ok(precision)) return DDX_ERR_ARG;
    if (!c->bins) return DDX_ERR_STATE;
    StepArgs a;
    int r = make_step_args(c, phys, n_grav, n_dust, dt, mode, a, precision);
    if (r) return r;
    DeviceGuard dg(c->device);
    if ((r = ensure_massive(c, n_grav, n_dust, precision))) return r;
    cudaStream_t st = (cudaStream_t)stream;
    for (int k = 0; k < n_steps; ++k)
        if ((r = enqueue_step(c, *s, a, precision, st))) return r;
    return DDX_OK;
}

namespace {
int prepare_call(ddx_ctx* c, const ddx_state* s, int n_grav, int n_dust, double dt,
                 const ddx_phys* phys, int precision, int mode, StepArgs& a) {
    if (!c || !state_ok(s)) return DDX_ERR_ARG;
    if (!step_precision_ok(precision)) return DDX_ERR_ARG;
    if (!c->bins) return DDX_ERR_STATE;
    int r = make_step_args(c, phys, n_grav, n_dust, dt, mode, a, precision);
    if (r) return r;
    return ensure_massive(c, n_grav, n_dust, precision);   // the caller made c's device current
}
}  // namespace

int ddx_massive_rk4(ddx_ctx* c, const ddx_state* s, int n_grav, int n_dust, double dt,
                    const ddx_phys* phys, int precision, int mode, void* stream) {
    if (!c) return DDX_ERR_ARG;
    DeviceGuard dg(c->device);
    StepArgs a;
    int r = prepare_call(c, s, n_grav, n_dust, dt, phys, precision, mode, a);
    if (r) return r;
    cudaStream_t st = (cudaStream_t)stream;
    if (a.n_grav == 1 && a.mode == DDX_MODE_REFERENCE) {
        star_only_reference_kernel<<<1, 32, 0, st>>>(*s, c->ms);
        return cuda_status(cudaGetLastError());
    }
    if (launch_massive_prepare(*s, a, c->ms, precision, st) != cudaSuccess) return DDX_ERR_CUDA;
    return cuda_status(launch_massive_pass1(*s, a, c->ms, precision, st));
}

int ddx_small_rk4(ddx_ctx* c, const ddx_state* s, int n_grav, int n_dust, double dt,
                  const ddx_phys* phys, int precision, int mode, void* stream) {
    if (!c) return DDX_ERR_ARG;
    DeviceGuard dg(c->device);
    StepArgs a;
    int r = prepare_call(c, s, n_grav, n_dust, dt, phys, precision, mode, a);
    if (r) return r;
    take_injection(c, a);
    return cuda_status(launch_dust(*s, a, c->ms, c->bins, precision, (cudaStream_t)stream));
}

int ddx_collide(ddx_ctx* c, const ddx_state* s, int i0, int i1, double h, int* pairs,
                long long cap, long long* n_pairs, void* stream) {
    if (!c || !state_ok(s) || !n_pairs || i0 < 0 || i1 < i0 || cap < 0 || (cap > 0 && !pairs) || !(h > 0.0))
        return DDX_ERR_ARG;
    if ((long long)i1 - i0 > (1LL << 30)) return DDX_ERR_RANGE;
    DeviceGuard dg(c->device);
    return collide_run(c->collide, *s, i0, i1, h, reinterpret_cast<int2*>(pairs), cap, n_pairs,
                       (cudaStream_t)stream);
}

int ddx_det_step(ddx_ctx* c, const ddx_state* s, int n_grav, int n_step, const double* disk_Rin,
                 int n_disks, const double* blob_a, const double* blob_ecc, const double* blob_sigma,
                 int n_blobs, double* dt, void* stream) {
    if (!c || !s || !s->x || !s->y || !s->z || !s->m || !dt || n_grav < 1 || n_step < 1 || n_disks < 0 ||
        n_blobs < 0 || (n_disks > 0 && !disk_Rin) || (n_blobs > 0 && (!blob_a || !blob_ecc || !blob_sigma)))
        return DDX_ERR_ARG;
    DeviceGuard dg(c->device);
    std::vector<double> rr, mi;
    double m0 = 0.0;
    const int r = det_step_scan(c->detstep, *s, n_grav, (cudaStream_t)stream, rr, mi, m0);
    if (r) return r;
    // src/grid.cu:315-341, term by term (this file is compiled without FP contraction)
    const double PI2 = 6.28318530717958623200;   // src/ddyn.cuh:29
    double dtdynmin = 1e137;
    for (size_t k = 0; k < rr.size(); ++k) {
        const double R = pow(rr[k], 3.0 / 2.0);
        const double dttmp = PI2 * sqrt(R / (m0 + mi[k])) / n_step;
        if (dttmp < dtdynmin) dtdynmin = dttmp;
    }
    for (int i = 0; i < n_disks; ++i) {
        const double dttmp = PI2 * sqrt(disk_Rin[i] / (m0)) / n_step;
        if (dttmp < dtdynmin) dtdynmin = dttmp;
    }
    for (int i = 0; i < n_blobs; ++i) {
        const double dttmp = PI2 * sqrt((blob_a[i] * (1.0 - blob_ecc[i]) - blob_sigma[i]) / (m0)) / n_step;
        if (dttmp < dtdynmin) dtdynmin = dttmp;
    }
    *dt = dtdynmin;
    return DDX_OK;
}

int ddx_dust_temp(ddx_ctx* c, int n_grid, int n_wav, const double* w, const double* in, const double* Qabs,
                  double dist, double* Rmin_AU, double* Rmax_AU, double* Td, void* stream) {
    if (!c || n_grid < 1 || n_wav < 2 || !w || !in || !Qabs || !Rmin_AU || !Rmax_AU || !Td) return DDX_ERR_ARG;
    if (!(dist > 0.0) || !(*Rmax_AU > 0.0)) return DDX_ERR_ARG;
    if (n_grid > DDX_MAX_SIZE_BINS) return DDX_ERR_RANGE;
    DeviceGuard dg(c->device);
    return dust_temp_run(n_grid, n_wav, w, in, Qabs, dist, Rmin_AU, Rmax_AU, Td, (cudaStream_t)stream);
}

int ddx_dust_grid(ddx_ctx* c, int n_wav, const double* w, const double* in, const ddx_optical_table* file,
                  const ddx_grid_setup* g, ddx_optical_table* grid, float* q, float* beta, float* betasw,
                  double* Lum, double* betaswconst, void* stream) {
    if (!c || !w || !in || !file || !g || !grid || !q || !beta || !betasw || !Lum || !betaswconst) return DDX_ERR_ARG;
    if (!file->s || !file->Qabs || !file->Qsca || !file->Qpfunc) return DDX_ERR_ARG;
    if (!grid->s || !grid->Qabs || !grid->Qsca || !grid->Qpfunc) return DDX_ERR_ARG;
    if (n_wav < 2 || file->n_wav != n_wav || grid->n_wav != n_wav) return DDX_ERR_ARG;
    if (file->n_theta < 1 || grid->n_theta != file->n_theta || (g->radQ == 1 && file->n_theta < 2)) return DDX_ERR_ARG;
    if (file->n_size < 2 || g->n_grid < 2 || grid->n_size != g->n_grid) return DDX_ERR_ARG;
    if (!(g->amin > 0.0) || !(g->amax > g->amin) || !(g->rho > 0.0) || !(g->mstar > 0.0)) return DDX_ERR_ARG;
    if (g->n_grid > DDX_MAX_SIZE_BINS) return DDX_ERR_RANGE;
    DeviceGuard dg(c->device);
    return dust_grid_run(n_wav, w, in, *file, *g, *grid, q, beta, betasw, Lum, betaswconst, (cudaStream_t)stream);
}

}  // extern "C"

namespace ddx {
int ctx_device(const ddx_ctx* c) { return c->device; }
int ctx_optics_n_wav(const ddx_ctx* c) { return c->optics_set ? c->od.n_wav : 0; }
}  // namespace ddx

extern "C" {

int ddx_setup_device(ddx_ctx* c, const ddx_param* p, double dmin, double dmax, const float* beta,
                     unsigned long long seed, const ddx_state* s, long long cap, ddx_dat_run* run, void* stream) {
    if (!c || !p || !beta || !run || !state_ok(s)) return DDX_ERR_ARG;
    DeviceGuard dg(c->device);
    return setup_device_run(p, dmin, dmax, beta, seed, *s, cap, run, (cudaStream_t)stream);
}

int ddx_adjoint_forward(ddx_ctx* c, const ddx_state* s, int n_grav, int n_dust, double dt, int n_steps,
                        int ckpt_every, const ddx_phys* phys, const ddx_view* view, const int* wj, int n_img,
                        double* image, void* stream) {
    if (!c || !state_ok(s) || !phys || !view || !wj || !image || n_steps < 1 || ckpt_every < 1) return DDX_ERR_ARG;
    if (n_grav > DDX_ADJ_MAX_GRAV) return DDX_ERR_RANGE;
    if (n_img < 1 || n_img > kMaxImages || view->xsize < 1 || view->ysize < 1 || !(view->fov > 0.0)) return DDX_ERR_ARG;
    if (!c->bins || !c->optics_set) return DDX_ERR_STATE;
    StepArgs a;
    int r = make_step_args(c, phys, n_grav, n_dust, dt, DDX_MODE_FIXED, a);
    if (r) return r;
    ImageList il;
    il.n = n_img;
    for (int k = 0; k < n_img; ++k) {
        if (wj[k] < 0 || wj[k] >= c->od.n_wav) return DDX_ERR_ARG;
        il.wj[k] = wj[k];
    }
    DeviceGuard dg(c->device);
    const int K = ckpt_every < n_steps ? ckpt_every : n_steps;
    return adjoint_forward(c->adjoint, *s, n_grav, n_dust, dt, n_steps, K, a, *view, il, c->bins, c->od, image,
                           (cudaStream_t)stream);
}

int ddx_adjoint_backward(ddx_ctx* c, const double* dL_dimage, double* grad_state, double* grad_mass,
                         void* stream) {
    if (!c || !dL_dimage || !grad_state || !grad_mass) return DDX_ERR_ARG;
    if (!c->adjoint) return DDX_ERR_STATE;
    DeviceGuard dg(c->device);
    return adjoint_backward(c->adjoint, dL_dimage, grad_state, grad_mass, c->bins, c->od, (cudaStream_t)stream);
}

int ddx_set_near_radius(ddx_ctx* c, double eta) {
    if (!c || eta != eta || eta > (double)kMaxNearEta) return DDX_ERR_ARG;
    c->near_eta = eta < 0.0 ? -1.f : (float)eta;   // negative: the defaults of each precision
    return DDX_OK;
}

int ddx_set_compensated_radius(ddx_ctx* c, double eta) {
    if (!c || !(eta >= 0.0)) return DDX_ERR_ARG;   // +inf: every span
    c->comp_eta = (float)eta;
    return DDX_OK;
}

int ddx_debug_lose_tile_copy(ddx_ctx* c, int tile, unsigned long long wait_ns) {
    if (!c || tile < 0 || wait_ns == 0) return DDX_ERR_ARG;
    c->inject_lose_tile = tile;
    c->inject_wait_ns = wait_ns;
    return DDX_OK;
}

int ddx_massive_final(ddx_ctx* c, const ddx_state* s, int n_grav, int n_dust, double dt,
                      const ddx_phys* phys, int precision, int mode, void* stream) {
    if (!c) return DDX_ERR_ARG;
    DeviceGuard dg(c->device);
    StepArgs a;
    int r = prepare_call(c, s, n_grav, n_dust, dt, phys, precision, mode, a);
    if (r) return r;
    if (a.n_grav == 1 && a.mode == DDX_MODE_REFERENCE) return DDX_OK;
    return cuda_status(launch_massive_pass2(*s, a, c->ms, precision, (cudaStream_t)stream));
}

int ddx_image(ddx_ctx* c, const ddx_state* s, int n_grav, int n_dust, const ddx_view* view,
              const int* wj, int n_img, double* Fd, int precision, void* stream) {
    if (!c || !state_ok(s) || !view || !wj || !Fd || n_grav < 0 || n_dust < 0) return DDX_ERR_ARG;
    if (precision != DDX_PREC_FP64 && precision != DDX_PREC_MIXED) return DDX_ERR_ARG;
    if (n_img < 1 || view->xsize < 1 || view->ysize < 1 || !(view->fov > 0.0) || !(view->dist > 0.0))
        return DDX_ERR_ARG;
    if (n_img > kMaxImages) return DDX_ERR_RANGE;
    if (!c->optics_set) return DDX_ERR_STATE;
    ImageList il;
    il.n = n_img;
    for (int k = 0; k < n_img; ++k) {
        if (wj[k] < 0 || wj[k] >= c->od.n_wav) return DDX_ERR_ARG;
        il.wj[k] = wj[k];
    }
    DeviceGuard dg(c->device);
    if (precision == DDX_PREC_MIXED) {
        const size_t need = (size_t)view->xsize * view->ysize * image_k4(n_img);
        if (need > c->img32_words) {
            cudaFree(c->img32);
            c->img32 = nullptr;
            c->img32_words = 0;
            if (dalloc(&c->img32, need) != cudaSuccess) {
                cudaGetLastError();
                return DDX_ERR_NOMEM;
            }
            c->img32_words = need;
        }
        return cuda_status(launch_image_mixed(*s, n_grav, n_dust, *view, c->od, il, c->vc, c->photo, Fd, c->img32,
                                              c->counters, (cudaStream_t)stream));
    }
    return cuda_status(launch_image(*s, n_grav, n_dust, *view, c->od, il, c->vc, Fd, c->counters,
                                    (cudaStream_t)stream));
}

int ddx_sed(ddx_ctx* c, const ddx_state* s, int n_grav, int n_dust, const ddx_view* view,
            double* Fsed, int precision, int mode, void* stream) {
    if (!c || !state_ok(s) || !view || !Fsed || n_grav < 0 || n_dust < 0) return DDX_ERR_ARG;
    if (precision != DDX_PREC_FP64 && precision != DDX_PREC_MIXED) return DDX_ERR_ARG;
    if (mode != DDX_MODE_FIXED && mode != DDX_MODE_REFERENCE) return DDX_ERR_ARG;
    if (!(view->dist > 0.0)) return DDX_ERR_ARG;
    if (!c->optics_set) return DDX_ERR_STATE;
    DeviceGuard dg(c->device);
    const int nb = sed_blocks(n_dust);
    const int need = nb * c->od.n_wav;
    if (need > c->sed_partial_cap) {
        cudaFree(c->sed_partial);
        c->sed_partial = nullptr;
        c->sed_partial_cap = 0;
        if (dalloc(&c->sed_partial, need) != cudaSuccess) return DDX_ERR_NOMEM;
        c->sed_partial_cap = need;
    }
    if (precision == DDX_PREC_MIXED)
        return cuda_status(launch_sed_mixed(*s, n_grav, n_dust, *view, c->od, c->vc, c->photo, c->sed_partial,
                                            mode, Fsed, (cudaStream_t)stream));
    return cuda_status(launch_sed(*s, n_grav, n_dust, *view, c->od, c->vc, c->sed_partial, mode,
                                  Fsed, (cudaStream_t)stream));
}

int ddx_debug_pixels(ddx_ctx* c, const ddx_state* s, int n_grav, int n_dust, const ddx_view* view,
                     int* pix, int* exact) {
    if (!c || !state_ok(s) || !view || !pix || !exact || n_grav < 0 || n_dust < 0) return DDX_ERR_ARG;
    if (view->xsize < 1 || view->ysize < 1 || !(view->fov > 0.0)) return DDX_ERR_ARG;
    DeviceGuard dg(c->device);
    const int n_theta = c->optics_set ? c->od.n_theta : 2;
    return cuda_status(launch_pixels(*s, n_grav, n_dust, *view, n_theta, c->vc, pix, exact, 0));
}

int ddx_sync_status(ddx_ctx* c, void* stream) {
    if (!c) return DDX_ERR_ARG;
    DeviceGuard dg(c->device);
    if (cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess) return DDX_ERR_CUDA;
    int h = 0;
    if (cudaMemcpy(&h, c->status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return DDX_ERR_CUDA;
    if (h != 0 && cudaMemset(c->status, 0, sizeof(int)) != cudaSuccess) return DDX_ERR_CUDA;
    return (h & kStatusTimeout) ? DDX_ERR_TIMEOUT : DDX_OK;
}

// Number of tracers that took the exact (reference-sequence) pixel path since the
// context was created; a diagnostic for the guard band of ddx_image.
unsigned long long ddx_debug_exact_pixel_count(ddx_ctx* c) {
    if (!c) return 0;
    unsigned long long h = 0;
    cudaMemcpy(&h, c->counters, sizeof(h), cudaMemcpyDeviceToHost);
    return h;
}

}  // extern "C"
