// Scattered + thermal images and SEDs of the dust tracers on sm_103a.
//
// Reference: calc_flux_driver (src/gpu_functions.cu:983-1081), calc_flux_sed_driver
// (:1083-1156), sum_flux_driver (:961-981), host loops src/grid.cu:28-66, 396-424.
// The reference runs one pass over the tracers per image wavelength and four launches
// plus two symbol copies per SED wavelength.  Here one pass covers every image
// wavelength, and one pass covers the whole SED with a deterministic two-level sum.
//
// Pixel indices: the reference obtains them through atan2/cos/sin/sqrt chains in FP64.
// The same projection is the rotation x1 = x cos(rot) - y sin(rot), ... which costs a
// handful of FMAs.  Its result differs from the reference's chain by far less than
// 1e-12 pixel (error analysis in guard_width), so whenever the projected coordinate is
// farther than the guard width from a pixel edge the floor is the same.  Tracers inside
// the guard band take the reference's exact expression sequence, so every pixel index is
// identical to the reference kernel's on the same GPU.
#include "ddx_internal.cuh"
#include "ddx_flux.cuh"

namespace ddx {

// Constants of one view, computed on the device with the device math library so that
// every quantity the reference recomputes per thread has the same bits here.
__global__ void view_setup_kernel(ViewConst* vc, ddx_view v, int n_theta) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    ViewConst c;
    c.dist = v.dist;
    c.rot = v.longitude;
    c.incl = v.inc;
    c.PA = v.PA;
    c.fov = v.fov;
    c.xsize = v.xsize;
    c.ysize = v.ysize;
    c.ntheta = n_theta;
    if (v.xsize >= v.ysize) c.psca = v.fov / v.xsize;
    else                    c.psca = v.fov / v.ysize;
    c.cr = cos(v.longitude); c.sr = sin(v.longitude);
    c.ci = cos(v.inc);       c.si = sin(v.inc);
    c.cp = cos(v.PA);        c.sp = sin(v.PA);
    c.ly0 = -v.dist * sin(v.inc);
    c.lz0 = v.dist * cos(v.inc);
    *vc = c;
}

// Reference geometry sequence (src/gpu_functions.cu:1001-1044), kept out of line so the
// common path does not carry its registers.  It reproduces the reference's whole
// expression graph up to the pixel floor -- including R, the scattering-angle cosine and
// the products they share with the pixel chain (x*x of the rotated position, z*z) --
// because the compiler's FMA contraction of a product depends on how many expressions
// use it.  Returns the pixel and the clamped scattering-angle cosine.
__device__ __noinline__ void exact_pixel(double x, double y, double z, const ViewConst& v,
                                         int& xim, int& yim, double& cossc_out) {
    const double rot = v.rot, incl = v.incl, PA = v.PA, dist = v.dist, FOV = v.fov;
    const int xsize = v.xsize, ysize = v.ysize, ntheta = v.ntheta;
    double phi = atan2(y, x);
    double R = sqrt(x * x + y * y + z * z);
    double Rd = sqrt(x * x + y * y);
    x = Rd * cos(phi + rot);
    y = Rd * sin(phi + rot);
    double ly = -dist * sin(incl) - y;
    double lz = dist * cos(incl) - z;
    double cossc = (x * x + (-y) * ly + (-z) * lz) / R / sqrt(x * x + ly * ly + lz * lz);
    if (cossc < -1) cossc = -1.0;
    if (cossc >= 1.0 - 2.0 / ntheta) cossc = 1.0 - 2.0 / ntheta;
    y = sqrt(y * y + z * z) * cos(atan2(z, y) - incl);
    phi = atan2(y, x);
    Rd = sqrt(x * x + y * y);
    x = Rd * cos(phi + PA);
    y = Rd * sin(phi + PA);
    double psca;
    if (xsize >= ysize) psca = FOV / xsize;
    else                psca = FOV / ysize;
    x = x + 0.5 * psca * xsize;
    y = y + 0.5 * psca * ysize;
    xim = floor(x / psca);
    yim = floor(y / psca);
    cossc_out = cossc;
}

// Width of the band around a pixel edge inside which the fast projection is not trusted.
// The reference chain (atan2, cos, sin: <= 2 ulp each; sqrt, +, *: correctly rounded)
// is within ~1e-14 * R of the exact projection, the rotation here within ~1e-15 * R, so
// the two pixel coordinates differ by < 2e-14 * R/psca + a few ulp of the coordinate.
// The band is 50x wider than that.
__device__ __forceinline__ double guard_width(double R, double u, const ViewConst& v) {
    return 1e-12 * (R / v.psca + fabs(u) + 1.0);
}

__device__ __forceinline__ bool near_edge(double u, double g) {
    const double f = u - floor(u);
    return f < g || f > 1.0 - g;
}

// Fast projection of (x, y, z) to the image plane; returns the unfloored pixel coordinates.
__device__ __forceinline__ void fast_pixel_coord(double x, double y, double z, const ViewConst& v,
                                                 double& u, double& w) {
    const double x1 = x * v.cr - y * v.sr;
    const double y1 = x * v.sr + y * v.cr;
    const double y2 = y1 * v.ci + z * v.si;
    double X = x1 * v.cp - y2 * v.sp;
    double Y = x1 * v.sp + y2 * v.cp;
    X = X + 0.5 * v.psca * v.xsize;
    Y = Y + 0.5 * v.psca * v.ysize;
    u = X / v.psca;
    w = Y / v.psca;
}

// Scattering-angle cosine of a tracer at rotated position (x1, y1, z) for an observer at
// distance dist along (0, -sin i, cos i), clamped like the reference
// (src/gpu_functions.cu:1017-1023).
__device__ __forceinline__ double scatter_cos(double x1, double y1, double z, double R,
                                              const ViewConst& v) {
    const double ly = v.ly0 - y1;
    const double lz = v.lz0 - z;
    double cossc = (x1 * x1 + (-y1) * ly + (-z) * lz) / R / sqrt(x1 * x1 + ly * ly + lz * lz);
    if (cossc < -1) cossc = -1.0;
    if (cossc >= 1.0 - 2.0 / v.ntheta) cossc = 1.0 - 2.0 / v.ntheta;
    return cossc;
}

// Dust temperature at radius R for bin id: log-log interpolation on the nR grid
// (src/gpu_functions.cu:1049-1063), using the table of log T built at set-up.
__device__ __forceinline__ double dust_temperature(double R, int id, const OpticsDev& o) {
    const double* Td = o.Td + (size_t)id * kNR;
    if (R <= o.Rmin) return Td[0];
    if (R >= o.Rmax) return Td[kNR - 1];
    const double* lTd = o.lTd + (size_t)id * kNR;
    const double lr = log(R / o.Rmin);
    int Rid = (int)(lr / o.fR) + 1;
    if (Rid > kNR - 1) Rid = kNR - 1;
    const double frac = (lr - (Rid - 1) * o.fR) / o.fR;
    return exp(lTd[Rid - 1] + (lTd[Rid] - lTd[Rid - 1]) * frac);
}

// Flux of one tracer at table wavelength wj, in Jy, before the multiplicity N
// (src/gpu_functions.cu:1064-1078): Planck*pi thermal emission + scattered starlight
// with a log-linear phase-function interpolation in the scattering-angle cosine.
__device__ __forceinline__ double tracer_flux(double n, int id, int wj, double R, double T,
                                              int cosinm, double wt, const OpticsDev& o,
                                              double dist, double w5, double wvl) {
    const double I = (2 * kHplank * kCspeed * kCspeed) /
                     (w5 * (exp(kHplank * kCspeed / (wvl * kKboltz * T)) - 1.0)) * kPI;
    const int nw = o.n_wav;
    const double lm = o.lQp[(size_t)nw * (o.n_theta * id + cosinm) + wj];
    const double lp = o.lQp[(size_t)nw * (o.n_theta * id + cosinm + 1) + wj];
    const double P = exp(lm + (lp - lm) * wt);
    const double s = o.size[id];
    const double Fscat = o.in[wj] * kPI * s * s * o.Qsca[(size_t)nw * id + wj] * P / R / R / kAU / kAU;
    const double Fther = I * s * s * o.Qabs[(size_t)nw * id + wj] / dist / dist;
    return n * (Fther + Fscat) * 1e26 * wvl * wvl / kCspeed;
}

// Phase-function bracket of a scattering-angle cosine (src/gpu_functions.cu:1066-1072).
__device__ __forceinline__ void phase_bracket(double cossc, int ntheta, int& cosinm, double& wt) {
    cosinm = floor(0.5 * (cossc + 1.0) * (ntheta - 1));
    const int cosinp = cosinm + 1;
    const double cosm = (double)(cosinm)*2.0 / (ntheta - 1) - 1.0;
    const double cosp = (double)(cosinp)*2.0 / (ntheta - 1) - 1.0;
    wt = (cossc - cosm) / (cosp - cosm);
}

// One thread per tracer, all image wavelengths in one pass; FP64 scatter-add.
__global__ void __launch_bounds__(256)
image_kernel(ddx_state s, int n_grav, int n_dust, const ViewConst* __restrict__ vcp,
             OpticsDev o, ImageList il, double* __restrict__ Fd, unsigned long long* __restrict__ nexact) {
    __shared__ ViewConst v;
    __shared__ double w5s[kMaxImages], wvls[kMaxImages];
    if (threadIdx.x == 0) v = *vcp;
    if (threadIdx.x < il.n) {
        const double wvl = o.w[il.wj[threadIdx.x]];
        wvls[threadIdx.x] = wvl;
        w5s[threadIdx.x] = pow(wvl, 5);
    }
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_dust) return;
    const int t = n_grav + i;
    const int id = s.id[t];
    if (id < 0) return;
    const double x = s.x[t], y = s.y[t], z = s.z[t];
    const double n = s.N[t];
    const double R = sqrt(x * x + y * y + z * z);

    double u, w;
    fast_pixel_coord(x, y, z, v, u, w);
    int xim, yim;
    double cossc;
    const double g = guard_width(R, fmax(fabs(u), fabs(w)), v);
    const bool exact = near_edge(u, g) || near_edge(w, g);
    if (exact) {
        exact_pixel(x, y, z, v, xim, yim, cossc);
        atomicAdd(nexact, 1ull);
    } else {
        xim = (int)floor(u);
        yim = (int)floor(w);
    }
    if (xim < 0 || xim > v.xsize - 1 || yim < 0 || yim > v.ysize - 1) return;
    if (!(R > o.Rmin)) return;

    if (!exact) {
        const double x1 = x * v.cr - y * v.sr;
        const double y1 = x * v.sr + y * v.cr;
        cossc = scatter_cos(x1, y1, z, R, v);
    }
    int cosinm; double wt;
    phase_bracket(cossc, v.ntheta, cosinm, wt);
    const double T = dust_temperature(R, id, o);
    const size_t npix = (size_t)v.xsize * v.ysize;
    const size_t pix = (size_t)v.ysize * xim + yim;
    for (int k = 0; k < il.n; ++k) {
        const double F = tracer_flux(n, id, il.wj[k], R, T, cosinm, wt, o, v.dist, w5s[k], wvls[k]);
        atomicAdd(&Fd[k * npix + pix], F);
    }
}

// Pixel index of every tracer (ysize*xim + yim, or -1 when it has no optics or falls
// outside the image) and whether the exact reference sequence decided it.
__global__ void pixel_kernel(ddx_state s, int n_grav, int n_dust, const ViewConst* __restrict__ vcp,
                             int* __restrict__ pix, int* __restrict__ exact) {
    __shared__ ViewConst v;
    if (threadIdx.x == 0) v = *vcp;
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_dust) return;
    const int t = n_grav + i;
    pix[i] = -1;
    exact[i] = 0;
    if (s.id[t] < 0) return;
    const double x = s.x[t], y = s.y[t], z = s.z[t];
    const double R = sqrt(x * x + y * y + z * z);
    double u, w;
    fast_pixel_coord(x, y, z, v, u, w);
    int xim, yim;
    const double g = guard_width(R, fmax(fabs(u), fabs(w)), v);
    if (near_edge(u, g) || near_edge(w, g)) {
        double cossc;
        exact_pixel(x, y, z, v, xim, yim, cossc);
        exact[i] = 1;
    } else {
        xim = (int)floor(u);
        yim = (int)floor(w);
    }
    if (xim < 0 || xim > v.xsize - 1 || yim < 0 || yim > v.ysize - 1) return;
    pix[i] = v.ysize * xim + yim;
}

// SED: each block accumulates, per wavelength, the flux of the tracers of its chunks in a
// fixed order; a second kernel sums the block partials in block order.  Deterministic.
constexpr int kSedThreads = 256;

__global__ void __launch_bounds__(kSedThreads)
sed_partial_kernel(ddx_state s, int n_grav, int n_dust, const ViewConst* __restrict__ vcp,
                   OpticsDev o, int mode, double* __restrict__ partial) {
    extern __shared__ double sed_smem[];
    double* acc = sed_smem;                      // [n_wav] block accumulator
    double* red = sed_smem + o.n_wav;            // [kSedThreads/32] warp partials
    __shared__ ViewConst v;
    if (threadIdx.x == 0) v = *vcp;
    for (int j = threadIdx.x; j < o.n_wav; j += blockDim.x) acc[j] = 0.0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int base = blockIdx.x * blockDim.x; base < n_dust; base += gridDim.x * blockDim.x) {
        const int i = base + threadIdx.x;
        bool on = false;
        int id = 0, cosinm = 0;
        double R = 1.0, T = 1.0, wt = 0.0, n = 0.0;
        if (i < n_dust) {
            const int t = n_grav + i;
            id = s.id[t];
            if (id >= 0) {
                const double x = s.x[t], y = s.y[t], z = s.z[t];
                n = s.N[t];
                R = sqrt(x * x + y * y + z * z);
                // The reference rotates by the spherical radius here (src/gpu_functions.cu:1106-1107);
                // the image kernel uses the cylindrical one.
                double x1 = x * v.cr - y * v.sr;
                double y1 = x * v.sr + y * v.cr;
                if (mode == DDX_MODE_REFERENCE) {
                    const double Rd = sqrt(x * x + y * y);
                    if (Rd > 0.0) { x1 *= R / Rd; y1 *= R / Rd; }
                    else { x1 = R * v.cr; y1 = R * v.sr; }
                }
                const double cossc = scatter_cos(x1, y1, z, R, v);
                phase_bracket(cossc, v.ntheta, cosinm, wt);
                T = dust_temperature(R, id, o);
                on = R > o.Rmin;
            }
        }
        for (int j = 0; j < o.n_wav; ++j) {
            double F = 0.0;
            if (on) {
                const double wvl = o.w[j];
                F = tracer_flux(n, id, j, R, T, cosinm, wt, o, v.dist, o.w5[j], wvl);
            }
            F = warp_sum_d(F);
            if (lane == 0) red[warp] = F;
            __syncthreads();
            if (threadIdx.x == 0) {
                double b = 0.0;
                for (int k = 0; k < kSedThreads / 32; ++k) b += red[k];
                acc[j] += b;
            }
            __syncthreads();
        }
    }
    for (int j = threadIdx.x; j < o.n_wav; j += blockDim.x)
        partial[(size_t)blockIdx.x * o.n_wav + j] = acc[j];
}

__global__ void sed_final_kernel(const double* __restrict__ partial, int nblocks, int n_wav,
                                 double* __restrict__ Fsed) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n_wav) return;
    double s = 0.0;
    for (int b = 0; b < nblocks; ++b) s += partial[(size_t)b * n_wav + j];
    Fsed[j] = s;
}

// Device-side table preparation: log of the phase-function and temperature tables, and
// lambda^5, with the device math library (the reference evaluates the same logs and
// pow per thread).
__global__ void optics_prepare_kernel(OpticsDev o) {
    const size_t nq = (size_t)o.n_grid * o.n_theta * o.n_wav;
    const size_t nt = (size_t)o.n_grid * kNR;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < nq; k += (size_t)gridDim.x * blockDim.x)
        o.lQp[k] = log(o.Qp[k]);
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < nt; k += (size_t)gridDim.x * blockDim.x)
        o.lTd[k] = log(o.Td[k]);
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < (size_t)o.n_wav; k += (size_t)gridDim.x * blockDim.x)
        o.w5[k] = pow(o.w[k], 5);
}

__global__ void fR_kernel(OpticsDev* od) {
    if (threadIdx.x == 0 && blockIdx.x == 0) od->fR = log(od->Rmax / od->Rmin) / ((double)kNR - 1.0);
}

// ---------------------------------------------------------------------------------------

cudaError_t launch_optics_prepare(OpticsDev& o, OpticsDev* o_dev, cudaStream_t st) {
    optics_prepare_kernel<<<304, 256, 0, st>>>(o);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    fR_kernel<<<1, 32, 0, st>>>(o_dev);
    return cudaGetLastError();
}

cudaError_t launch_image(const ddx_state& s, int n_grav, int n_dust, const ddx_view& view,
                         const OpticsDev& o, const ImageList& il, ViewConst* vc, double* Fd,
                         unsigned long long* nexact, cudaStream_t st) {
    view_setup_kernel<<<1, 32, 0, st>>>(vc, view, o.n_theta);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const size_t npix = (size_t)view.xsize * view.ysize;
    e = cudaMemsetAsync(Fd, 0, sizeof(double) * npix * il.n, st);
    if (e != cudaSuccess) return e;
    if (n_dust <= 0) return cudaSuccess;
    const int threads = 256;
    const int blocks = (n_dust + threads - 1) / threads;
    image_kernel<<<blocks, threads, 0, st>>>(s, n_grav, n_dust, vc, o, il, Fd, nexact);
    return cudaGetLastError();
}

cudaError_t launch_view_setup(ViewConst* vc, const ddx_view& view, int n_theta, cudaStream_t st) {
    view_setup_kernel<<<1, 32, 0, st>>>(vc, view, n_theta);
    return cudaGetLastError();
}

cudaError_t launch_pixels(const ddx_state& s, int n_grav, int n_dust, const ddx_view& view,
                          int n_theta, ViewConst* vc, int* pix, int* exact, cudaStream_t st) {
    view_setup_kernel<<<1, 32, 0, st>>>(vc, view, n_theta);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || n_dust <= 0) return e;
    pixel_kernel<<<(n_dust + 255) / 256, 256, 0, st>>>(s, n_grav, n_dust, vc, pix, exact);
    return cudaGetLastError();
}

int sed_blocks(int n_dust) {
    int b = (n_dust + kSedThreads - 1) / kSedThreads;
    return b < 1 ? 1 : (b > 1216 ? 1216 : b);
}

cudaError_t launch_sed(const ddx_state& s, int n_grav, int n_dust, const ddx_view& view,
                       const OpticsDev& o, ViewConst* vc, double* partial, int mode,
                       double* Fsed, cudaStream_t st) {
    view_setup_kernel<<<1, 32, 0, st>>>(vc, view, o.n_theta);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const int nb = sed_blocks(n_dust);
    const size_t smem = sizeof(double) * (o.n_wav + kSedThreads / 32);
    sed_partial_kernel<<<nb, kSedThreads, smem, st>>>(s, n_grav, n_dust, vc, o, mode, partial);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    sed_final_kernel<<<(o.n_wav + 127) / 128, 128, 0, st>>>(partial, nb, o.n_wav, Fsed);
    return cudaGetLastError();
}

}  // namespace ddx
