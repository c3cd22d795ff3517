// ORACLE -- test infrastructure, not product code.
//
// Host runner for the reference DiskDyn kernels compiled unmodified into a cubin
// (oracle/ref/ref_kernels.cu).  It replays the reference host code's launch sequences --
// Grid::massive_RK4 / small_RK4 / massive_final (src/grid.cu:693-752), null_flux +
// calc_flux (src/grid.cu:12-19, 43-54) and the SED loop (src/grid.cu:21-41, 56-66,
// 396-406) -- with the same grid and block sizes, through the CUDA driver API.  The
// kernels' `coord` argument is a struct of 41 double pointers and one int pointer passed
// by value (src/ddyn.cuh:44-58); RefCoord below has the same member order.
#include <cuda.h>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

namespace {

struct RefCoord {
    double *m, *N;
    double *x, *y, *z, *vx, *vy, *vz;
    double *k1x, *k2x, *k3x, *k4x;
    double *k1y, *k2y, *k3y, *k4y;
    double *k1z, *k2z, *k3z, *k4z;
    double *k2rx, *k2ry, *k2rz;
    double *k3rx, *k3ry, *k3rz;
    double *k4rx, *k4ry, *k4rz;
    double *k1vx, *k1vy, *k1vz;
    double *k2vx, *k2vy, *k2vz;
    double *k3vx, *k3vy, *k3vz;
    double *k4vx, *k4vy, *k4vz;
    int *id;
};
static_assert(sizeof(RefCoord) == 42 * sizeof(void*), "coord layout");

struct Phys {
    int radQ, SWQ, FLQ;
    double Wz, Bstar, Rstar, rho, vsw_AUyr, Rmin;
};
struct View {
    double dist, fov, PA, inc, longitude;
    int xsize, ysize;
};

CUmodule g_mod = nullptr;
CUcontext g_ctx = nullptr;
CUfunction f_null_coord, f_m0, f_m1, f_m2, f_m3, f_m4, f_m5, f_m6, f_m7, f_m8, f_mfinal, f_dust,
    f_null_flux, f_null_part, f_sum, f_flux, f_flux_sed;
char g_err[512];

#define CK(call)                                                             \
    do {                                                                     \
        CUresult r_ = (call);                                                \
        if (r_ != CUDA_SUCCESS) {                                            \
            const char* s_ = nullptr;                                        \
            cuGetErrorString(r_, &s_);                                       \
            snprintf(g_err, sizeof g_err, "%s failed: %s", #call, s_ ? s_ : "?"); \
            return (int)r_;                                                  \
        }                                                                    \
    } while (0)

int launch(CUfunction f, int grid, int block, unsigned smem, void** args) {
    CK(cuLaunchKernel(f, grid, 1, 1, block, 1, 1, smem, 0, args, nullptr));
    return 0;
}

// Device copy of a state: 41 double arrays + id, all n_all long, zero-initialised like
// Grid::null_gpu (src/grid.cu:4-10).
struct DevState {
    RefCoord c{};
    std::vector<CUdeviceptr> bufs;
    int n_all = 0;
    int alloc(int n) {
        n_all = n;
        double** p = &c.m;
        for (int k = 0; k < 41; ++k) {
            CUdeviceptr d;
            CK(cuMemAlloc(&d, sizeof(double) * (size_t)(n > 0 ? n : 1)));
            CK(cuMemsetD8(d, 0, sizeof(double) * (size_t)(n > 0 ? n : 1)));
            bufs.push_back(d);
            p[k] = (double*)d;
        }
        CUdeviceptr d;
        CK(cuMemAlloc(&d, sizeof(int) * (size_t)(n > 0 ? n : 1)));
        bufs.push_back(d);
        c.id = (int*)d;
        return 0;
    }
    ~DevState() {
        for (auto d : bufs) cuMemFree(d);
    }
};

int upload(DevState& ds, int n_all, double* x, double* y, double* z, double* vx, double* vy,
           double* vz, double* m, double* N, int* id) {
    const size_t b = sizeof(double) * n_all;
    CK(cuMemcpyHtoD((CUdeviceptr)ds.c.x, x, b));
    CK(cuMemcpyHtoD((CUdeviceptr)ds.c.y, y, b));
    CK(cuMemcpyHtoD((CUdeviceptr)ds.c.z, z, b));
    CK(cuMemcpyHtoD((CUdeviceptr)ds.c.vx, vx, b));
    CK(cuMemcpyHtoD((CUdeviceptr)ds.c.vy, vy, b));
    CK(cuMemcpyHtoD((CUdeviceptr)ds.c.vz, vz, b));
    CK(cuMemcpyHtoD((CUdeviceptr)ds.c.m, m, b));
    CK(cuMemcpyHtoD((CUdeviceptr)ds.c.N, N, b));
    CK(cuMemcpyHtoD((CUdeviceptr)ds.c.id, id, sizeof(int) * n_all));
    return 0;
}

int set_size_table(int n_grid, const double* size, const float* beta, const float* betasw,
                   const float* q) {
    if (n_grid > 2700) { snprintf(g_err, sizeof g_err, "n_grid > 2700"); return -1; }
    CUdeviceptr d; size_t bytes;
    CK(cuModuleGetGlobal(&d, &bytes, g_mod, "size"));
    CK(cuMemcpyHtoD(d, size, sizeof(double) * n_grid));
    CK(cuModuleGetGlobal(&d, &bytes, g_mod, "beta"));
    CK(cuMemcpyHtoD(d, beta, sizeof(float) * n_grid));
    CK(cuModuleGetGlobal(&d, &bytes, g_mod, "betasw"));
    CK(cuMemcpyHtoD(d, betasw, sizeof(float) * n_grid));
    CK(cuModuleGetGlobal(&d, &bytes, g_mod, "q"));
    CK(cuMemcpyHtoD(d, q, sizeof(float) * n_grid));
    return 0;
}

// Grid::massive_RK4 + small_RK4 + massive_final (src/grid.cu:693-752).
int step_once(RefCoord& c, int n_grav, int n_dust, double dt, const Phys& p) {
    if (n_grav > 1) {
        int TILE = 32, n_thread = 64;
        int block0 = int((n_grav - 1.0) / n_thread + 1.0);
        int num = int((n_grav - 1.0) / TILE + 1);
        unsigned smem = 2 * TILE * 32 + TILE * TILE * 3 * sizeof(double);
        int n_planets = 0;  // unused by the kernels
        void* a0[] = {&n_grav, &c};
        if (launch(f_m0, block0, n_thread, 0, a0)) return -1;
        if (launch(f_m1, block0, n_thread, 0, a0)) return -1;
        CUfunction tiles[4] = {f_m2, f_m4, f_m6, f_m8};
        CUfunction stages[3] = {f_m3, f_m5, f_m7};
        double hs[3] = {dt * 0.5, dt * 0.5, dt};
        for (int s = 0; s < 4; ++s) {
            for (int i = 0; i < num; ++i) {
                int nl = num - i;
                int ii = i;
                void* a[] = {&ii, &n_grav, &TILE, &c, &n_planets};
                if (launch(tiles[s], nl, TILE * TILE, smem, a)) return -1;
            }
            if (s < 3) {
                double h = hs[s];
                void* a[] = {&n_grav, &c, &h};
                if (launch(stages[s], block0, n_thread, 0, a)) return -1;
            }
        }
    }
    if (n_dust > 0) {
        int block = int((n_dust - 1.0) / 128.0 + 1.0);
        int FLQ = p.FLQ, SWQ = p.SWQ;
        double Wz = p.Wz, Bstar = p.Bstar, Rstar = p.Rstar, rho = p.rho, vsw = p.vsw_AUyr, Rmin = p.Rmin;
        void* a[] = {&n_grav, &n_dust, &c, &dt, &FLQ, &Wz, &Bstar, &Rstar, &rho, &SWQ, &vsw, &Rmin};
        if (launch(f_dust, block, 128, 0, a)) return -1;
    }
    if (n_grav > 1) {
        int block0 = int((n_grav - 1.0) / 128.0 + 1.0);
        double d6 = dt / 6.0;
        void* a[] = {&n_grav, &c, &d6};
        if (launch(f_mfinal, block0, 128, 0, a)) return -1;
    }
    return 0;
}

struct DevOptics {
    CUdeviceptr Qabs = 0, Qsca = 0, Qp = 0, Td = 0, w = 0, in = 0;
    int up(int n_grid, int n_wav, int n_theta, const double* w_, const double* in_,
           const double* Qabs_, const double* Qsca_, const double* Qp_, const double* Td_) {
        size_t nw = (size_t)n_grid * n_wav, nq = nw * n_theta, nt = (size_t)n_grid * 100;
        CK(cuMemAlloc(&Qabs, nw * 8)); CK(cuMemcpyHtoD(Qabs, Qabs_, nw * 8));
        CK(cuMemAlloc(&Qsca, nw * 8)); CK(cuMemcpyHtoD(Qsca, Qsca_, nw * 8));
        CK(cuMemAlloc(&Qp, nq * 8)); CK(cuMemcpyHtoD(Qp, Qp_, nq * 8));
        CK(cuMemAlloc(&Td, nt * 8)); CK(cuMemcpyHtoD(Td, Td_, nt * 8));
        CK(cuMemAlloc(&w, n_wav * 8)); CK(cuMemcpyHtoD(w, w_, n_wav * 8));
        CK(cuMemAlloc(&in, n_wav * 8)); CK(cuMemcpyHtoD(in, in_, n_wav * 8));
        return 0;
    }
    ~DevOptics() {
        for (CUdeviceptr d : {Qabs, Qsca, Qp, Td, w, in}) if (d) cuMemFree(d);
    }
};

}  // namespace

extern "C" {

const char* ref_error(void) { return g_err; }

int ref_load(const char* cubin) {
    if (g_mod) return 0;
    CK(cuInit(0));
    CUdevice dev;
    CK(cuDeviceGet(&dev, 0));
    CK(cuDevicePrimaryCtxRetain(&g_ctx, dev));
    CK(cuCtxSetCurrent(g_ctx));
    CK(cuModuleLoad(&g_mod, cubin));
    struct { CUfunction* f; const char* n; } fs[] = {
        {&f_null_coord, "_Z17null_coord_driveri5coord"},
        {&f_m0, "_Z16RK4calc_massive0i5coord"},
        {&f_m1, "_Z16RK4calc_massive1i5coord"},
        {&f_m2, "_Z16RK4calc_massive2iii5coordi"},
        {&f_m3, "_Z16RK4calc_massive3i5coordd"},
        {&f_m4, "_Z16RK4calc_massive4iii5coordi"},
        {&f_m5, "_Z16RK4calc_massive5i5coordd"},
        {&f_m6, "_Z16RK4calc_massive6iii5coordi"},
        {&f_m7, "_Z16RK4calc_massive7i5coordd"},
        {&f_m8, "_Z16RK4calc_massive8iii5coordi"},
        {&f_mfinal, "_Z21RK4calc_massive_finali5coordd"},
        {&f_dust, "_Z12RK4calc_dustii5coorddiddddidd"},
        {&f_null_flux, "_Z16null_flux_driveriPd"},
        {&f_null_part, "_Z21null_flux_part_driveriPd"},
        {&f_sum, "_Z15sum_flux_driveriPd"},
        {&f_flux, "_Z16calc_flux_driverii5coorddddPdS0_S0_S0_S0_S0_S0_iiiidddiid"},
        {&f_flux_sed, "_Z20calc_flux_sed_driverii5coorddddPdS0_S0_S0_S0_S0_S0_iiiiddd"},
    };
    for (auto& e : fs) CK(cuModuleGetFunction(e.f, g_mod, e.n));
    return 0;
}

// Runs n_steps reference steps on a host state (arrays of n_grav + n_dust, updated in
// place).  kpos_out (optional, 12*n_grav doubles, [stage][xyz][body]) receives the stage
// positions k1..k4 of the massive set from the last step.  ms_per_step (optional) gets
// the mean device time per step from CUDA events.
int ref_step(int n_grav, int n_dust, double* x, double* y, double* z, double* vx, double* vy,
             double* vz, double* m, double* N, int* id, int n_grid, const double* size,
             const float* beta, const float* betasw, const float* q, double dt, int n_steps,
             const Phys* p, double* kpos_out, double* ms_per_step) {
    if (!g_mod) { snprintf(g_err, sizeof g_err, "ref_load not called"); return -1; }
    CK(cuCtxSetCurrent(g_ctx));
    if (set_size_table(n_grid, size, beta, betasw, q)) return -1;
    const int n_all = n_grav + n_dust;
    DevState ds;
    if (ds.alloc(n_all)) return -1;
    if (upload(ds, n_all, x, y, z, vx, vy, vz, m, N, id)) return -1;
    CUevent e0, e1;
    CK(cuEventCreate(&e0, 0));
    CK(cuEventCreate(&e1, 0));
    CK(cuCtxSynchronize());
    CK(cuEventRecord(e0, 0));
    for (int k = 0; k < n_steps; ++k)
        if (step_once(ds.c, n_grav, n_dust, dt, *p)) return -1;
    CK(cuEventRecord(e1, 0));
    CK(cuEventSynchronize(e1));
    float ms = 0.f;
    CK(cuEventElapsedTime(&ms, e0, e1));
    cuEventDestroy(e0);
    cuEventDestroy(e1);
    if (ms_per_step) *ms_per_step = n_steps > 0 ? ms / n_steps : 0.0;
    const size_t b = sizeof(double) * n_all;
    CK(cuMemcpyDtoH(x, (CUdeviceptr)ds.c.x, b));
    CK(cuMemcpyDtoH(y, (CUdeviceptr)ds.c.y, b));
    CK(cuMemcpyDtoH(z, (CUdeviceptr)ds.c.z, b));
    CK(cuMemcpyDtoH(vx, (CUdeviceptr)ds.c.vx, b));
    CK(cuMemcpyDtoH(vy, (CUdeviceptr)ds.c.vy, b));
    CK(cuMemcpyDtoH(vz, (CUdeviceptr)ds.c.vz, b));
    CK(cuMemcpyDtoH(N, (CUdeviceptr)ds.c.N, b));
    if (kpos_out) {
        double* src[12] = {ds.c.k1x, ds.c.k1y, ds.c.k1z, ds.c.k2x, ds.c.k2y, ds.c.k2z,
                           ds.c.k3x, ds.c.k3y, ds.c.k3z, ds.c.k4x, ds.c.k4y, ds.c.k4z};
        for (int k = 0; k < 12; ++k)
            CK(cuMemcpyDtoH(kpos_out + (size_t)k * n_grav, (CUdeviceptr)src[k], sizeof(double) * n_grav));
    }
    return 0;
}

// Reference images at wj[0..n_img-1] into Fd[img][xsize*ysize] (host).
int ref_image(int n_grav, int n_dust, double* x, double* y, double* z, double* N, int* id,
              int n_grid, int n_wav, int n_theta, const double* size, const double* w,
              const double* in, const double* Qabs, const double* Qsca, const double* Qp,
              const double* Td, double Rmin, double Rmax, const View* v, const int* wj,
              int n_img, double* Fd) {
    if (!g_mod) { snprintf(g_err, sizeof g_err, "ref_load not called"); return -1; }
    CK(cuCtxSetCurrent(g_ctx));
    std::vector<float> zf(n_grid, 0.f);
    if (set_size_table(n_grid, size, zf.data(), zf.data(), zf.data())) return -1;
    const int n_all = n_grav + n_dust;
    DevState ds;
    if (ds.alloc(n_all)) return -1;
    std::vector<double> zero(n_all, 0.0);
    if (upload(ds, n_all, x, y, z, zero.data(), zero.data(), zero.data(), zero.data(), N, id)) return -1;
    DevOptics o;
    if (o.up(n_grid, n_wav, n_theta, w, in, Qabs, Qsca, Qp, Td)) return -1;
    const int npix = v->xsize * v->ysize;
    CUdeviceptr Fdd;
    CK(cuMemAlloc(&Fdd, sizeof(double) * npix));
    for (int k = 0; k < n_img; ++k) {
        int np = npix;
        double* Fp = (double*)Fdd;
        void* a0[] = {&np, &Fp};
        if (launch(f_null_flux, int((npix - 1.0) / 128.0 + 1.0), 128, 0, a0)) return -1;
        if (n_dust > 0) {
            double dist = v->dist, rot = v->longitude, incl = v->inc, PA = v->PA, fov = v->fov;
            double *Qa = (double*)o.Qabs, *Qs = (double*)o.Qsca, *Qpp = (double*)o.Qp, *Tdd = (double*)o.Td,
                   *wd = (double*)o.w, *ind = (double*)o.in;
            int nw = n_wav, ng = n_grid, nt = n_theta, wjk = wj[k], xs = v->xsize, ys = v->ysize;
            double rmin = Rmin, rmax = Rmax;
            void* a[] = {&n_grav, &n_dust, &ds.c, &dist, &rmin, &rmax, &Qa, &Qs, &Qpp, &Tdd, &Fp, &wd, &ind,
                         &nw, &ng, &nt, &wjk, &rot, &incl, &PA, &xs, &ys, &fov};
            if (launch(f_flux, int((n_dust - 1.0) / 128.0 + 1.0), 128, 0, a)) return -1;
        }
        CK(cuCtxSynchronize());
        CK(cuMemcpyDtoH(Fd + (size_t)k * npix, Fdd, sizeof(double) * npix));
    }
    cuMemFree(Fdd);
    return 0;
}

// Reference SED at every table wavelength into Fsed[n_wav] (host), through the
// per-wavelength loop of src/grid.cu:396-406.
int ref_sed(int n_grav, int n_dust, double* x, double* y, double* z, double* N, int* id,
            int n_grid, int n_wav, int n_theta, const double* size, const double* w,
            const double* in, const double* Qabs, const double* Qsca, const double* Qp,
            const double* Td, double Rmin, double Rmax, const View* v, double* Fsed,
            double* ms_total) {
    if (!g_mod) { snprintf(g_err, sizeof g_err, "ref_load not called"); return -1; }
    CK(cuCtxSetCurrent(g_ctx));
    std::vector<float> zf(n_grid, 0.f);
    if (set_size_table(n_grid, size, zf.data(), zf.data(), zf.data())) return -1;
    const int n_all = n_grav + n_dust;
    DevState ds;
    if (ds.alloc(n_all)) return -1;
    std::vector<double> zero(n_all, 0.0);
    if (upload(ds, n_all, x, y, z, zero.data(), zero.data(), zero.data(), zero.data(), N, id)) return -1;
    DevOptics o;
    if (o.up(n_grid, n_wav, n_theta, w, in, Qabs, Qsca, Qp, Td)) return -1;
    CUdeviceptr Fdust, dtmp;
    size_t bytes;
    CK(cuMemAlloc(&Fdust, sizeof(double) * (n_dust > 0 ? n_dust : 1)));
    CK(cuModuleGetGlobal(&dtmp, &bytes, g_mod, "doubletmp"));
    CUevent e0, e1;
    CK(cuEventCreate(&e0, 0));
    CK(cuEventCreate(&e1, 0));
    CK(cuEventRecord(e0, 0));
    for (int j = 0; j < n_wav; ++j) {
        double zero1 = 0.0;
        CK(cuMemcpyHtoD(dtmp, &zero1, sizeof(double)));
        if (n_dust > 0) {
            double* Fp = (double*)Fdust;
            int nd = n_dust;
            void* a0[] = {&nd, &Fp};
            if (launch(f_null_part, int((n_dust - 1.0) / 128.0 + 1.0), 128, 0, a0)) return -1;
            double dist = v->dist, rot = v->longitude, incl = v->inc, PA = v->PA;
            double *Qa = (double*)o.Qabs, *Qs = (double*)o.Qsca, *Qpp = (double*)o.Qp, *Tdd = (double*)o.Td,
                   *wd = (double*)o.w, *ind = (double*)o.in;
            int nw = n_wav, ng = n_grid, nt = n_theta, jj = j;
            double rmin = Rmin, rmax = Rmax;
            void* a[] = {&n_grav, &n_dust, &ds.c, &dist, &rmin, &rmax, &Qa, &Qs, &Qpp, &Tdd, &Fp, &wd, &ind,
                         &nw, &ng, &nt, &jj, &rot, &incl, &PA};
            if (launch(f_flux_sed, int((n_dust - 1.0) / 64.0 + 1.0), 64, 0, a)) return -1;
            void* a2[] = {&nd, &Fp};
            if (launch(f_sum, int((n_dust - 1.0) / 128.0 + 1.0), 128, 128 * sizeof(double), a2)) return -1;
            double flux = 0.0;
            CK(cuMemcpyDtoH(&flux, dtmp, sizeof(double)));
            Fsed[j] = flux;
        } else {
            Fsed[j] = 0.0;
        }
    }
    CK(cuEventRecord(e1, 0));
    CK(cuEventSynchronize(e1));
    float ms = 0.f;
    CK(cuEventElapsedTime(&ms, e0, e1));
    if (ms_total) *ms_total = ms;
    cuEventDestroy(e0);
    cuEventDestroy(e1);
    cuMemFree(Fdust);
    return 0;
}

}  // extern "C"
