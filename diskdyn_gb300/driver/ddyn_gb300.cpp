// ddyn_gb300: a whole DiskDyn run from a parameter file through the C ABI of libddx.so, in
// the order of the reference's main program (src/ddyn.cu: read_in_param, the optical and
// stellar tables, Grid::setup, calculate_dust_temp, Grid::evolve with its outputs).  It is
// the C++ caller the ABI is meant for: every call below is one a patched Grid would make.
//
//   ddyn_gb300 <system.param> --table <mie table> --spec <spectrum> [--out <dir>]
//              [--precision fp64|mixed|compensated] [--mode fixed|reference]
//              [--setup host|device] [--seed N] [--device N] [--t-end T] [--dry-run]
//
// --table replaces the parameter file's composition path, --spec its spectral type (the
// Kurucz library is not part of this package).  --dry-run reads the files and prints the
// system's counts without a GPU.  Outputs take the reference's names under --out:
// <stub>_<t>.dat, <stub>_SED_<t>.dat and <stub>_<wavelength um>_<t>.fits.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "diskdyn_gb300.h"
#include "diskdyn_gb300_io.h"
#include "diskdyn_gb300_run.h"
#include "diskdyn_gb300_setup.h"

namespace {

constexpr double kAUm = 1.49598e11;           // m (src/ddyn.cuh)
constexpr double kYears = 3.1556926e7;        // s, a year (src/ddyn.cuh)
constexpr const char* kVersion = "2.0-gb300";

int fail(const char* what, int status) {
    std::fprintf(stderr, "ddyn_gb300: %s failed (status %d)\n", what, status);
    return status ? status : 1;
}

struct Options {
    std::string param, table, spec, out = ".";
    int precision = DDX_PREC_FP64, mode = DDX_MODE_FIXED, device = 0;
    bool host_setup = true, dry_run = false;
    long long seed = -2;                      // the reference's ran3 seed
    double t_end = -1.0;
};

bool parse(int argc, char** argv, Options& o) {
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        auto next = [&](std::string& v) {
            if (i + 1 >= argc) return false;
            v = argv[++i];
            return true;
        };
        std::string v;
        if (a == "--table") { if (!next(o.table)) return false; }
        else if (a == "--spec") { if (!next(o.spec)) return false; }
        else if (a == "--out") { if (!next(o.out)) return false; }
        else if (a == "--precision") {
            if (!next(v)) return false;
            if (v == "fp64") o.precision = DDX_PREC_FP64;
            else if (v == "mixed") o.precision = DDX_PREC_MIXED;
            else if (v == "compensated") o.precision = DDX_PREC_COMPENSATED;
            else return false;
        } else if (a == "--mode") {
            if (!next(v)) return false;
            if (v == "fixed") o.mode = DDX_MODE_FIXED;
            else if (v == "reference") o.mode = DDX_MODE_REFERENCE;
            else return false;
        } else if (a == "--setup") {
            if (!next(v)) return false;
            if (v == "host") o.host_setup = true;
            else if (v == "device") o.host_setup = false;
            else return false;
        } else if (a == "--seed") { if (!next(v)) return false; o.seed = std::atoll(v.c_str()); }
        else if (a == "--device") { if (!next(v)) return false; o.device = std::atoi(v.c_str()); }
        else if (a == "--t-end") { if (!next(v)) return false; o.t_end = std::atof(v.c_str()); }
        else if (a == "--dry-run") o.dry_run = true;
        else if (!a.empty() && a[0] != '-' && o.param.empty()) o.param = a;
        else return false;
    }
    return !o.param.empty() && !o.table.empty() && !o.spec.empty();
}

// Device copy of the whole state (ddx_state of device arrays).
struct DeviceState {
    ddx_state s{};
    bool alloc(long long n) {
        double** f[8] = {&s.x, &s.y, &s.z, &s.vx, &s.vy, &s.vz, &s.m, &s.N};
        for (double** p : f)
            if (cudaMalloc(p, sizeof(double) * (size_t)n) != cudaSuccess) return false;
        return cudaMalloc(&s.id, sizeof(int) * (size_t)n) == cudaSuccess;
    }
    ~DeviceState() {
        cudaFree(s.x); cudaFree(s.y); cudaFree(s.z); cudaFree(s.vx); cudaFree(s.vy); cudaFree(s.vz);
        cudaFree(s.m); cudaFree(s.N); cudaFree(s.id);
    }
};

// Host arrays behind a ddx_host_state.
struct HostState {
    std::vector<double> x, y, z, vx, vy, vz, N, m;
    std::vector<int> id;
    ddx_host_state h{};
    void alloc(long long n) {
        for (auto* v : {&x, &y, &z, &vx, &vy, &vz, &N, &m}) v->assign((size_t)n, 0.0);
        id.assign((size_t)n, 0);
        h = ddx_host_state{x.data(), y.data(), z.data(), vx.data(), vy.data(), vz.data(), N.data(), m.data(),
                           id.data(), n};
    }
};

struct Writer {
    std::string base;
    const ddx_param* p;
    ddx_dat_run run;
    const std::vector<double>* w;
    const std::vector<double>* in;
    const std::vector<int>* wj;
    const std::vector<float>* beta;
    int xsize, ysize;
    int status = DDX_OK;
    int files = 0;
};

int on_output(void* user, const ddx_output* o) {
    Writer& W = *static_cast<Writer*>(user);
    char path[4096];
    int r = DDX_OK;
    if (o->kind == DDX_OUT_IMAGES) {
        const size_t npix = (size_t)W.xsize * W.ysize;
        for (size_t j = 0; j < W.wj->size() && r == DDX_OK; ++j) {
            const double wl = (*W.w)[(*W.wj)[j]];
            std::snprintf(path, sizeof path, "%s_%.2f_%.3f.fits", W.base.c_str(), wl * 1e6, o->time);
            r = ddx_fits_write(path, kVersion, W.xsize, W.ysize, o->data + j * npix, wl, W.p->fov, W.p->dist);
            ++W.files;
        }
    } else if (o->kind == DDX_OUT_SED) {
        std::snprintf(path, sizeof path, "%s_SED_%.2f.dat", W.base.c_str(), o->time);
        r = ddx_sed_write(path, kVersion, (int)W.w->size(), W.w->data(), W.in->data(), o->data);
        ++W.files;
    } else {
        ddx_dat_run run = W.run;
        run.time = o->time;
        run.dt = o->model_dt;
        run.tlastd = o->tlastd;
        run.tlastf = o->tlastf;
        run.tlasts = o->tlasts;
        std::snprintf(path, sizeof path, "%s_%.2f.dat", W.base.c_str(), o->time);
        r = ddx_dat_write(path, kVersion, W.p, &run, o->state, W.beta->data());
        ++W.files;
    }
    if (r != DDX_OK) {
        W.status = r;
        std::fprintf(stderr, "ddyn_gb300: writing %s failed (status %d)\n", path, r);
        return 1;   // stop the run
    }
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    Options o;
    if (!parse(argc, argv, o)) {
        std::fprintf(stderr,
                     "usage: ddyn_gb300 <system.param> --table <mie table> --spec <spectrum> [--out <dir>]\n"
                     "       [--precision fp64|mixed|compensated] [--mode fixed|reference] [--setup host|device]\n"
                     "       [--seed N] [--device N] [--t-end T] [--dry-run]\n");
        return 2;
    }
    // the parameter file (read_in_param)
    ddx_param p;
    int r = ddx_param_read(o.param.c_str(), &p);
    if (r) {
        std::fprintf(stderr, "ddyn_gb300: the parameter file was rejected (usage code %d)\n", p.usage_code);
        return fail("ddx_param_read", r);
    }
    if (o.t_end > 0.0) p.t_end = o.t_end;
    // the optical table (add_optical_data) and the stellar spectrum (add_specfile)
    ddx_optical_table file{};
    double dmin = 0.0, dmax = 0.0;
    if ((r = ddx_optical_read(o.table.c_str(), &file, nullptr, &dmin, &dmax))) return fail("ddx_optical_read", r);
    std::vector<double> fs((size_t)file.n_size), fa((size_t)file.n_size * file.n_wav),
        fsc((size_t)file.n_size * file.n_wav), fq((size_t)file.n_size * file.n_theta * file.n_wav),
        w((size_t)file.n_wav);
    file.s = fs.data(); file.Qabs = fa.data(); file.Qsca = fsc.data(); file.Qpfunc = fq.data();
    if ((r = ddx_optical_read(o.table.c_str(), &file, w.data(), &dmin, &dmax))) return fail("ddx_optical_read", r);
    int nspec = 0;
    if ((r = ddx_spec_read(o.spec.c_str(), p.rstar, p.dist, &nspec, nullptr, nullptr, 0))) return fail("ddx_spec_read", r);
    std::vector<double> sw((size_t)nspec), sf((size_t)nspec);
    if ((r = ddx_spec_read(o.spec.c_str(), p.rstar, p.dist, &nspec, sw.data(), sf.data(), nspec)))
        return fail("ddx_spec_read", r);
    const int n_wav = file.n_wav;
    std::vector<double> in((size_t)n_wav);
    std::vector<int> wj((size_t)p.nwavs);
    if ((r = ddx_stellar_grid(n_wav, w.data(), nspec, sw.data(), sf.data(), p.nwavs, p.wavs, in.data(), wj.data())))
        return fail("ddx_stellar_grid", r);
    // the mass grid and the system's counts (detminmax, Grid::setup)
    if ((r = ddx_param_grid(&p, dmin, dmax))) return fail("ddx_param_grid", r);
    ddx_dat_run run{};
    if ((r = ddx_setup_count(&p, dmin, dmax, &run))) return fail("ddx_setup_count", r);
    const int n_grav = p.n_planets + run.n_mass, n_dust = run.n_dust;
    std::printf("system: %d massive (%d star and planets), %d grain tracers, %d size bins, %d wavelengths\n",
                n_grav, p.n_planets, n_dust, p.n_grid, n_wav);
    if (o.dry_run) return 0;

    ddx_ctx* ctx = nullptr;
    if ((r = ddx_create(&ctx, o.device))) return fail("ddx_create", r);
    cudaSetDevice(o.device);
    // the size grid's tables (interpolate_dust_to_grid, calculate_beta)
    const int n_grid = p.n_grid, n_theta = file.n_theta;
    std::vector<double> gs((size_t)n_grid), ga((size_t)n_grid * n_wav), gsc((size_t)n_grid * n_wav),
        gq((size_t)n_grid * n_theta * n_wav);
    ddx_optical_table grid{n_grid, n_wav, n_theta, gs.data(), ga.data(), gsc.data(), gq.data()};
    std::vector<float> q((size_t)n_grid), beta((size_t)n_grid), betasw((size_t)n_grid);
    double Lum = 0.0, bswc = 0.0;
    ddx_grid_setup g{n_grid, p.amin, p.amax, dmax, p.kqe, p.radQ, p.SWQ, p.rho, p.dist, p.planets[0].m, p.mloss, p.vsw};
    if ((r = ddx_dust_grid(ctx, n_wav, w.data(), in.data(), &file, &g, &grid, q.data(), beta.data(), betasw.data(),
                           &Lum, &bswc, nullptr)))
        return fail("ddx_dust_grid", r);
    // the temperature table out to the largest configured radius (calculate_dust_temp)
    double Rmax = 0.0;
    for (int k = 0; k < p.n_disks; ++k) Rmax = std::max(Rmax, p.disks[k].Rout);
    for (int k = 0; k < p.n_blobs; ++k) Rmax = std::max(Rmax, p.blobs[k].a * (1.0 + p.blobs[k].ecc) + p.blobs[k].sigma);
    for (int k = 1; k < p.n_planets; ++k) {
        const ddx_planet& pl = p.planets[k];
        Rmax = std::max(Rmax, std::sqrt(pl.x * pl.x + pl.y * pl.y + pl.z * pl.z));
    }
    double Rmin = 0.0;
    std::vector<double> Td((size_t)n_grid * DDX_NR);
    if ((r = ddx_dust_temp(ctx, n_grid, n_wav, w.data(), in.data(), ga.data(), p.dist, &Rmin, &Rmax, Td.data(),
                           nullptr)))
        return fail("ddx_dust_temp", r);
    run.Rmax = Rmax;
    run.nR = DDX_NR;
    if ((r = ddx_set_size_table(ctx, n_grid, gs.data(), beta.data(), betasw.data(), q.data())) ||
        (r = ddx_set_optics(ctx, n_grid, n_wav, n_theta, w.data(), in.data(), ga.data(), gsc.data(), gq.data(),
                            Td.data(), Rmin, Rmax)))
        return fail("the table upload", r);
    // the bodies (Grid::setup), on the device either way
    const long long n_all = run.n_all;
    DeviceState d;
    if (!d.alloc(n_all)) return fail("cudaMalloc of the state", DDX_ERR_NOMEM);
    if (o.host_setup) {
        HostState h;
        h.alloc(n_all);
        if ((r = ddx_setup_host(&p, dmin, dmax, beta.data(), o.seed, &h.h, &run))) return fail("ddx_setup_host", r);
        const double* hf[8] = {h.x.data(), h.y.data(), h.z.data(), h.vx.data(), h.vy.data(), h.vz.data(), h.m.data(),
                               h.N.data()};
        double* df[8] = {d.s.x, d.s.y, d.s.z, d.s.vx, d.s.vy, d.s.vz, d.s.m, d.s.N};
        for (int f = 0; f < 8; ++f)
            if (cudaMemcpy(df[f], hf[f], sizeof(double) * (size_t)n_all, cudaMemcpyHostToDevice) != cudaSuccess)
                return fail("cudaMemcpy of the state", DDX_ERR_CUDA);
        if (cudaMemcpy(d.s.id, h.id.data(), sizeof(int) * (size_t)n_all, cudaMemcpyHostToDevice) != cudaSuccess)
            return fail("cudaMemcpy of the state", DDX_ERR_CUDA);
    } else if ((r = ddx_setup_device(ctx, &p, dmin, dmax, beta.data(), (unsigned long long)o.seed, &d.s, n_all, &run,
                                     nullptr))) {
        return fail("ddx_setup_device", r);
    }
    run.Rmax = Rmax;
    run.nR = DDX_NR;
    // the step (Grid::det_step)
    std::vector<double> rin, ba, be, bs;
    for (int k = 0; k < p.n_disks; ++k) rin.push_back(p.disks[k].Rin);
    for (int k = 0; k < p.n_blobs; ++k) {
        ba.push_back(p.blobs[k].a);
        be.push_back(p.blobs[k].ecc);
        bs.push_back(p.blobs[k].sigma);
    }
    double dt = 0.0;
    if ((r = ddx_det_step(ctx, &d.s, n_grav, p.n_step, rin.data(), (int)rin.size(), ba.data(), be.data(), bs.data(),
                          (int)ba.size(), &dt, nullptr)))
        return fail("ddx_det_step", r);
    // Grid::evolve with its outputs
    const ddx_phys phys{p.radQ, p.SWQ, p.FLQ, p.Wz, p.Bstar, p.rstar, p.rho, p.vsw * kYears / kAUm, Rmin, p.n_planets};
    const ddx_view view{p.dist, p.fov, p.PA, p.inc, p.longitude, p.xsize, p.ysize};
    ddx_cadence cad{p.t_write, p.t_fits, p.t_sed, p.t_end, 0.0, 0.0, 0.0, 0.0, 0.0, 1};
    Writer W{o.out + "/" + p.name_stub, &p, run, &w, &in, &wj, &beta, p.xsize, p.ysize};
    r = ddx_run(ctx, &d.s, n_grav, n_dust, dt, &phys, o.precision, o.mode, &view, wj.data(), p.nwavs, &cad, on_output,
                &W, nullptr);
    if (W.status) return fail("an output", W.status);
    if (r) return fail("ddx_run", r);
    std::printf("run: dt %.6g yr, t_end %.6g yr reached at %.6g, %d files written\n", dt, p.t_end, cad.time, W.files);
    ddx_destroy(ctx);
    return 0;
}
