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
#include <vector>
#include "ddx_internal.cuh"

namespace ddx {
namespace {

constexpr double kTsub = 2000.0;   // sublimation temperature, K (src/ddyn.cuh)

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

}  // namespace

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
