// Dust-temperature table on the GPU: Grid::calculate_dust_temp (src/grid.cu:754-834) with
// the Planck function intens (src/functions.cu:390-397).
//
// The reference runs it on the host once per run, n_grid x nT x n_wav Planck evaluations
// (nT = 1,999 temperatures from 2 Tsub down to 3 K in steps of 2 K), sequentially.  Here:
//  1. star_kernel: per size bin, the trapezoid integral of Qabs * in / pi times dist^2,
//     and the sublimation radius 0.5 sqrt(star / gflux(Tsub));
//  2. radius_kernel: one thread per (bin, temperature), Ra = 0.5 sqrt(star / gflux(T)),
//     every sum over wavelengths in the reference's order;
//  3. temp_kernel: one thread per (bin, grid radius): the bracket of R in Ra.  The
//     reference walks Ra sequentially with a pointer that it steps back by one after each
//     radius; because Ra increases with decreasing T and the radii increase, that walk
//     ends at the first index with Ra > R (at most nT - 1), which a binary search finds
//     directly.  Where the reference's walk would step outside its arrays (an index -1, or
//     past nT - 1), the index is clamped, as in the oracle.
//
// And the size grid with its tables: interpolate_dust_to_grid (src/functions.cu:243-300) and
// calculate_beta (:338-388).  The reference's host loops become:
//  - on the host, O(n_grid): the bin radii, q, the size brackets (the reference's walk over
//    the table sizes) and their log ratios, with libm and the reference's rounding;
//  - grid_interp_kernel: one thread per value of the three interpolated tables
//    (n_grid x n_wav x (n_theta + 2) log-log interpolations);
//  - qpr_kernel: one thread per (bin, wavelength), the phase-function trapezoids for the
//    asymmetry parameter g and Qpr = (Qabs + Qsca (1 - g)) in;
//  - qsum_kernel: one thread per bin, the trapezoid of Qpr over wavelength;
//  - on the host: beta, beta_sw, the luminosity and the wind-drag constant.
// Every device sum and product is rounded separately (__dadd_rn, __dmul_rn: no fused
// multiply-adds), in the reference's order, so the tables differ from the reference's only
// by the CUDA math library's log and exp.
#include <vector>
#include "ddx_internal.cuh"

namespace ddx {
namespace {

constexpr double kTsub = 2000.0;   // sublimation temperature, K (src/ddyn.cuh)
constexpr double kMSun = 1.98892e30;
constexpr double kYear = 3.1556926e7;
constexpr double kLsun = 3.827e26;  // the luminosity unit of calculate_beta, W

__device__ __forceinline__ double intens(double temp, double wvl, double w5) {
    return (2 * kHplank * kCspeed * kCspeed) / (w5 * (exp(kHplank * kCspeed / (wvl * kKboltz * temp)) - 1));
}

__device__ __forceinline__ double trapezoid_planck(const double* w, const double* w5, const double* Q, int n_wav,
                                                   double T) {
    double g = 0.0;
    for (int i = 1; i < n_wav; i++)
        g += 0.5 * (w[i] - w[i - 1]) * (Q[i - 1] * intens(T, w[i - 1], w5[i - 1]) + Q[i] * intens(T, w[i], w5[i]));
    return g;
}

__global__ void w5_kernel(const double* w, int n_wav, double* w5) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_wav) w5[i] = pow(w[i], 5);
}

__global__ void star_kernel(const double* w, const double* w5, const double* in, const double* Qabs, int n_grid,
                            int n_wav, double dist, double* star, double* rsub) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_grid) return;
    const double* Q = Qabs + (size_t)k * n_wav;
    double s = 0.0;
    for (int i = 1; i < n_wav; i++)
        s += 0.5 * (w[i] - w[i - 1]) * (Q[i - 1] * in[i - 1] + Q[i] * in[i]) / kPI;
    s *= pow(dist, 2.0);
    star[k] = s;
    rsub[k] = 0.5 * sqrt(s / trapezoid_planck(w, w5, Q, n_wav, kTsub));
}

__global__ void radius_kernel(const double* w, const double* w5, const double* Qabs, const double* star,
                              int n_grid, int n_wav, int nT, double* Ra) {
    const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (e >= (size_t)n_grid * nT) return;
    const int k = (int)(e / nT), j = (int)(e % nT);
    const double T = 2 * kTsub - 2.0 * j;   // the reference's T -= 2.0 from 2 Tsub, exact
    Ra[e] = 0.5 * sqrt(star[k] / trapezoid_planck(w, w5, Qabs + (size_t)k * n_wav, n_wav, T));
}

__global__ void temp_kernel(const double* Ra, int n_grid, int nT, double Rmin, double Rmax, double* Td) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_grid * kNR) return;
    const int k = e / kNR, i = e % kNR;
    const double* R_ = Ra + (size_t)k * nT;
    const double R = Rmin * exp(log(Rmax / Rmin) * ((double)i) / ((double)kNR - 1.0));
    // first index with Ra > R, at most nT - 1
    int lo = 0, hi = nT - 1;
    while (lo < hi) {
        const int mid = (lo + hi) / 2;
        if (R_[mid] <= R) lo = mid + 1;
        else hi = mid;
    }
    const int ip = lo;
    const int im = ip > 0 ? ip - 1 : 0;
    const double Tm = 2 * kTsub - 2.0 * im, Tp = 2 * kTsub - 2.0 * ip;
    Td[e] = exp(log(Tm) + log(Tp / Tm) * log(R / R_[im]) / log(R_[ip] / R_[im]));
}

__global__ void min_kernel(const double* v, int n, double start, double* out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double m = start;
    for (int k = 0; k < n; ++k)
        if (v[k] < m) m = v[k];
    *out = m;
}

// The two table sizes around a bin and the log ratios of its interpolation.
struct Bracket {
    int im, ip;
    double la;   // log(a_i / s_im)
    double ls;   // log(s_ip / s_im)
};

// exp(log(Qm) + la * log(Qp / Qm) / ls), rounded step by step as the reference rounds it
__device__ __forceinline__ double loglog(double Qm, double Qp, double la, double ls) {
    return exp(__dadd_rn(log(Qm), __ddiv_rn(__dmul_rn(la, log(__ddiv_rn(Qp, Qm))), ls)));
}

// One thread per output value.  Row r of a bin i: r = 0 Qabs, r = 1 Qsca, r = 2 + k the
// phase function at angle k; each row n_wav long, so a warp reads and writes consecutive
// wavelengths.
__global__ void grid_interp_kernel(const Bracket* br, const double* Qabs, const double* Qsca, const double* Qpf,
                                   int n_grid, int n_wav, int n_theta, double* oQabs, double* oQsca, double* oQpf) {
    const size_t rows_per_bin = (size_t)n_theta + 2;
    const size_t total = (size_t)n_grid * rows_per_bin * n_wav;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += stride) {
        const size_t row = e / n_wav;
        const size_t j = e - row * n_wav;
        const size_t i = row / rows_per_bin;
        const int r = (int)(row - i * rows_per_bin);
        const Bracket b = br[i];
        if (r < 2) {
            const double* Q = r == 0 ? Qabs : Qsca;
            double* O = r == 0 ? oQabs : oQsca;
            O[i * n_wav + j] = loglog(Q[(size_t)b.im * n_wav + j], Q[(size_t)b.ip * n_wav + j], b.la, b.ls);
        } else {
            const size_t k = (size_t)(r - 2);
            oQpf[(i * n_theta + k) * n_wav + j] = loglog(Qpf[((size_t)b.im * n_theta + k) * n_wav + j],
                                                         Qpf[((size_t)b.ip * n_theta + k) * n_wav + j], b.la, b.ls);
        }
    }
}

// One thread per (bin, wavelength): the trapezoids of the phase function P(cos theta) and
// of cos(theta) P over the n_theta angles (the reference's cos grid k 2/(n_theta-1) - 1),
// g = their ratio, and Qpr = (Qabs + Qsca (1 - g)) in.
__global__ void qpr_kernel(const double* Qa, const double* Qs, const double* Qp, const double* in, int n_grid,
                           int n_wav, int n_theta, double* Qpr) {
    const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (e >= (size_t)n_grid * n_wav) return;
    const size_t i = e / n_wav, j = e - i * n_wav;
    const double* P = Qp + i * n_theta * n_wav + j;
    const double den = n_theta - 1.0;
    double g = 0.0, S = 0.0, costm = -1.0, Pm = P[0];
    for (int k = 1; k < n_theta; k++) {
        const double costp = __dsub_rn(__ddiv_rn(__dmul_rn((double)k, 2.0), den), 1.0);
        const double Pp = P[(size_t)k * n_wav];
        const double d = __dsub_rn(costp, costm);
        S = __dadd_rn(S, __dmul_rn(__dmul_rn(0.5, __dadd_rn(Pm, Pp)), d));
        g = __dadd_rn(g, __dmul_rn(__dmul_rn(0.5, __dadd_rn(__dmul_rn(costm, Pm), __dmul_rn(costp, Pp))), d));
        costm = costp;
        Pm = Pp;
    }
    g = __ddiv_rn(g, S);
    Qpr[e] = __dmul_rn(__dadd_rn(Qa[e], __dmul_rn(Qs[e], __dsub_rn(1.0, g))), in[j]);
}

// One thread per bin: the trapezoid of Qpr over wavelength, in the reference's order.
__global__ void qsum_kernel(const double* Qpr, const double* w, int n_grid, int n_wav, double* Qsum) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_grid) return;
    const double* q = Qpr + (size_t)i * n_wav;
    double s = 0.0;
    for (int j = 0; j < n_wav - 1; j++)
        s = __dadd_rn(s, __dmul_rn(__dmul_rn(0.5, __dsub_rn(w[j + 1], w[j])), __dadd_rn(q[j + 1], q[j])));
    Qsum[i] = s;
}

}  // namespace

int dust_grid_run(int n_wav, const double* w, const double* in, const ddx_optical_table& file,
                  const ddx_grid_setup& g, ddx_optical_table& grid, float* q, float* beta, float* betasw,
                  double* Lum, double* betaswconst, cudaStream_t st) {
    const int ng = g.n_grid, nd = file.n_size, nt = file.n_theta;
    // Bin radii, q and brackets: the reference's walk over the table sizes, which keeps one
    // index for all bins and steps it back by one after each.  Guards only where that walk
    // would leave the table: below s[0] the first interval, beyond the last size the last.
    std::vector<Bracket> br(ng);
    const double f = log(g.amax / g.amin) / ((double)ng - 1.0);
    int ip = 0;
    for (int i = 0; i < ng; i++) {
        double a = g.amin * exp((double)i * f);
        q[i] = (float)(g.kqe * a * 1e9);
        if (i == ng - 1 && (a - g.dmax) > 1e-12) return DDX_ERR_RANGE;   // the reference's exit 54
        if (i == ng - 1 && (a - g.dmax) < 1e-12 && (a - g.dmax) > 0) a = g.dmax;
        while (ip < nd - 1 && file.s[ip] < a) ip++;
        int im = ip - 1;
        if (im < 0) {
            im = 0;
            ip = 1;
        }
        br[i] = Bracket{im, ip, log(a / file.s[im]), log(file.s[ip] / file.s[im])};
        grid.s[i] = a;
        ip--;
    }

    const size_t nQf = (size_t)nd * n_wav, nPf = nQf * nt, nQg = (size_t)ng * n_wav, nPg = nQg * nt;
    // one device arena: brackets, then the doubles
    const size_t n_dbl = 2 * nQf + nPf + 3 * nQg + nPg + 2 * (size_t)n_wav + ng;
    char* arena = nullptr;
    const size_t br_bytes = ((sizeof(Bracket) * ng + 255) / 256) * 256;
    if (cudaMalloc(&arena, br_bytes + sizeof(double) * n_dbl) != cudaSuccess) {
        cudaGetLastError();
        return DDX_ERR_NOMEM;
    }
    Bracket* dbr = reinterpret_cast<Bracket*>(arena);
    double* p = reinterpret_cast<double*>(arena + br_bytes);
    double *fQa = p, *fQs = fQa + nQf, *fQp = fQs + nQf, *gQa = fQp + nPf, *gQs = gQa + nQg, *gQp = gQs + nQg,
           *Qpr = gQp + nPg, *dw = Qpr + nQg, *din = dw + n_wav, *Qsum = din + n_wav;
    std::vector<double> qsum(ng, 0.0);
    int r = DDX_OK;
    bool ok = cudaMemcpyAsync(dbr, br.data(), sizeof(Bracket) * ng, cudaMemcpyHostToDevice, st) == cudaSuccess &&
              cudaMemcpyAsync(fQa, file.Qabs, sizeof(double) * nQf, cudaMemcpyHostToDevice, st) == cudaSuccess &&
              cudaMemcpyAsync(fQs, file.Qsca, sizeof(double) * nQf, cudaMemcpyHostToDevice, st) == cudaSuccess &&
              cudaMemcpyAsync(fQp, file.Qpfunc, sizeof(double) * nPf, cudaMemcpyHostToDevice, st) == cudaSuccess &&
              cudaMemcpyAsync(dw, w, sizeof(double) * n_wav, cudaMemcpyHostToDevice, st) == cudaSuccess &&
              cudaMemcpyAsync(din, in, sizeof(double) * n_wav, cudaMemcpyHostToDevice, st) == cudaSuccess;
    if (ok) {
        const size_t total = nQg * ((size_t)nt + 2);
        const size_t want = (total + 255) / 256;
        const unsigned blocks = (unsigned)(want < 152u * 16u ? want : 152u * 16u);
        grid_interp_kernel<<<blocks, 256, 0, st>>>(dbr, fQa, fQs, fQp, ng, n_wav, nt, gQa, gQs, gQp);
        if (g.radQ == 1) {
            qpr_kernel<<<(unsigned)((nQg + 127) / 128), 128, 0, st>>>(gQa, gQs, gQp, din, ng, n_wav, nt, Qpr);
            qsum_kernel<<<(ng + 127) / 128, 128, 0, st>>>(Qpr, dw, ng, n_wav, Qsum);
            ok = cudaMemcpyAsync(qsum.data(), Qsum, sizeof(double) * ng, cudaMemcpyDeviceToHost, st) == cudaSuccess;
        }
        ok = ok && cudaGetLastError() == cudaSuccess &&
             cudaMemcpyAsync(grid.Qabs, gQa, sizeof(double) * nQg, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
             cudaMemcpyAsync(grid.Qsca, gQs, sizeof(double) * nQg, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
             cudaMemcpyAsync(grid.Qpfunc, gQp, sizeof(double) * nPg, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
             cudaStreamSynchronize(st) == cudaSuccess;
    }
    if (!ok) {
        cudaGetLastError();
        r = DDX_ERR_CUDA;
    }
    cudaFree(arena);
    if (r != DDX_OK) return r;

    // calculate_beta's scalars and per-bin values, its expressions in its order
    *betaswconst = 3.0 * g.mloss * 2 * kMSun * kYear * g.vsw / 32.0 / kPI / g.mstar / g.rho / kAU / kAU / kAU;
    double Star = 0.0;
    for (int j = 0; j < n_wav - 1; j++) Star += 0.5 * (w[j + 1] - w[j]) * (in[j + 1] + in[j]);
    *Lum = Star * 4.0 * kPI * pow(g.dist, 2.0) / kLsun;
    for (int i = 0; i < ng; i++) {
        beta[i] = g.radQ == 1
                      ? (float)(0.57 * qsum[i] / Star * (*Lum / g.mstar * (4.0 * kPI * kPI)) / grid.s[i] / 1e6 / g.rho / 1e-3)
                      : 0.0f;
        betasw[i] = g.SWQ == 1 ? (float)(*betaswconst / grid.s[i]) : 0.0f;
    }
    return DDX_OK;
}

int dust_temp_run(int n_grid, int n_wav, const double* w, const double* in, const double* Qabs, double dist,
                  double* Rmin_AU, double* Rmax_AU, double* Td, cudaStream_t st) {
    const int nT = (int)floor((2 * kTsub - 3) * 0.5) + 1;
    const double Rmax = *Rmax_AU * 2 * kAU;
    double *dw = nullptr, *dw5 = nullptr, *din = nullptr, *dQ = nullptr, *dstar = nullptr, *drsub = nullptr,
           *dRa = nullptr, *dTd = nullptr, *dmin = nullptr;
    const size_t nw = (size_t)n_grid * n_wav;
    int r = DDX_OK;
    if (cudaMalloc(&dw, sizeof(double) * n_wav) || cudaMalloc(&dw5, sizeof(double) * n_wav) ||
        cudaMalloc(&din, sizeof(double) * n_wav) || cudaMalloc(&dQ, sizeof(double) * nw) ||
        cudaMalloc(&dstar, sizeof(double) * n_grid) || cudaMalloc(&drsub, sizeof(double) * n_grid) ||
        cudaMalloc(&dRa, sizeof(double) * (size_t)n_grid * nT) || cudaMalloc(&dTd, sizeof(double) * n_grid * kNR) ||
        cudaMalloc(&dmin, sizeof(double))) {
        cudaGetLastError();
        r = DDX_ERR_NOMEM;
    }
    double Rmin = Rmax;
    if (r == DDX_OK) {
        cudaMemcpyAsync(dw, w, sizeof(double) * n_wav, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(din, in, sizeof(double) * n_wav, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(dQ, Qabs, sizeof(double) * nw, cudaMemcpyHostToDevice, st);
        w5_kernel<<<(n_wav + 255) / 256, 256, 0, st>>>(dw, n_wav, dw5);
        star_kernel<<<(n_grid + 127) / 128, 128, 0, st>>>(dw, dw5, din, dQ, n_grid, n_wav, dist, dstar, drsub);
        min_kernel<<<1, 32, 0, st>>>(drsub, n_grid, Rmax, dmin);
        const size_t nr = (size_t)n_grid * nT;
        radius_kernel<<<(unsigned)((nr + 127) / 128), 128, 0, st>>>(dw, dw5, dQ, dstar, n_grid, n_wav, nT, dRa);
        if (cudaMemcpyAsync(&Rmin, dmin, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            r = DDX_ERR_CUDA;
        } else {
            temp_kernel<<<(n_grid * kNR + 127) / 128, 128, 0, st>>>(dRa, n_grid, nT, Rmin, Rmax, dTd);
            if (cudaMemcpyAsync(Td, dTd, sizeof(double) * n_grid * kNR, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess || cudaGetLastError() != cudaSuccess)
                r = DDX_ERR_CUDA;
        }
    }
    cudaFree(dw); cudaFree(dw5); cudaFree(din); cudaFree(dQ); cudaFree(dstar); cudaFree(drsub);
    cudaFree(dRa); cudaFree(dTd); cudaFree(dmin);
    if (r == DDX_OK) {
        *Rmin_AU = Rmin / kAU;
        *Rmax_AU = Rmax / kAU;
    }
    return r;
}

}  // namespace ddx
