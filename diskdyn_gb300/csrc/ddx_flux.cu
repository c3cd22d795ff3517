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

// Whether a tracer is certainly off the frame: its fast pixel coordinates lie more than the
// guard band g plus 2 pixels outside it (the reference sequence then lies outside too), or
// beyond 2^30 pixels (where the reference's own int conversion of the floor overflows), or
// are NaN.  Such a tracer adds nothing, and no int conversion of its coordinates is made.
__device__ __forceinline__ bool far_off_frame(double u, double w, double g, const ViewConst& v) {
    const double m = g + 2.0;
    return !(u > -m && u < v.xsize + m && w > -m && w < v.ysize + m && fabs(u) < 0x1p30 && fabs(w) < 0x1p30);
}

// Scattering-angle cosine of a tracer at rotated position (x1, y1, z) for an observer at
// distance dist along (0, -sin i, cos i), clamped like the reference
// (src/gpu_functions.cu:1017-1023).
__device__ __forceinline__ double scatter_cos(double x1, double y1, double z, double R,
                                              const ViewConst& v) {
    const double ly = v.ly0 - y1;
    const double lz = v.lz0 - z;
    double cossc = (x1 * x1 + (-y1) * ly + (-z) * lz) / R / sqrt(x1 * x1 + ly * ly + lz * lz);
    if (!(cossc >= -1)) cossc = -1.0;            // also a NaN cosine: a table index from it stays in range
    if (cossc >= 1.0 - 2.0 / v.ntheta) cossc = 1.0 - 2.0 / v.ntheta;
    return cossc;
}

// Dust temperature at radius R for bin id: log-log interpolation on the nR grid
// (src/gpu_functions.cu:1049-1063), using the table of log T built at set-up.
__device__ __forceinline__ double dust_temperature(double R, int id, const OpticsDev& o) {
    const double* Td = o.Td + (size_t)id * kNR;
    if (!(R > o.Rmin)) return Td[0];             // R <= Rmin, or NaN: no table index from it
    if (R >= o.Rmax) return Td[kNR - 1];
    const double* lTd = o.lTd + (size_t)id * kNR;
    const double lr = log(R / o.Rmin);
    int Rid = (int)(lr / o.fR) + 1;
    if (Rid > kNR - 1) Rid = kNR - 1;
    if (Rid < 1) Rid = 1;
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
    if (id < 0 || id >= o.n_grid) return;
    const double x = s.x[t], y = s.y[t], z = s.z[t];
    const double n = s.N[t];
    const double R = sqrt(x * x + y * y + z * z);

    double u, w;
    fast_pixel_coord(x, y, z, v, u, w);
    int xim, yim;
    double cossc;
    const double g = guard_width(R, fmax(fabs(u), fabs(w)), v);
    if (far_off_frame(u, w, g, v)) return;
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
    if (far_off_frame(u, w, g, v)) return;
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
            if (id >= 0 && id < o.n_grid) {
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
    const size_t nq2 = (size_t)o.n_grid * (o.n_theta - 1) * o.n_wav;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < nq2; k += (size_t)gridDim.x * blockDim.x) {
        const size_t j = k % o.n_wav, r = k / o.n_wav;
        const size_t cm = r % (o.n_theta - 1), g = r / (o.n_theta - 1);
        const size_t q = (g * o.n_theta + cm) * o.n_wav + j;
        o.lQp32p[k] = make_float2((float)log2(o.Qp[q]), (float)log2(o.Qp[q + o.n_wav]));
    }
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < nt; k += (size_t)gridDim.x * blockDim.x) {
        o.lTd[k] = log(o.Td[k]);
        o.lTd32[k] = (float)o.lTd[k];
    }
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

// ---------------------------------------------------------------------------------------
// Mixed precision: FP32 photometry, pixel indices still bit-identical to the reference
// ---------------------------------------------------------------------------------------
//
// FP64 runs at 1/73 of the FP32 rate here, and the FP64 kernels above spend it on
// transcendental functions per tracer and wavelength.  The mixed kernels do the whole
// per-tracer chain in FP32 and keep FP64 only where a result must be exact:
//  - pixel index: the FP32 projection is trusted when it lies farther than
//    64 eps32 (R/psca + |u| + 1) pixel from an edge (a bound on its rounding error, 3x
//    the worst case of the operation chain); otherwise the FP64 fast projection and, in
//    its own band, the reference's exact sequence decide, as in image_kernel;
//  - R > Rmin: decided in FP64 when R is within 1e-5 of Rmin;
//  - the per-pixel sums: FP64 atomics.  The FP32 flux is converted to FP64 exactly, by
//    moving its bits (scaling by 2^-esh on the way), so the SM's FP64 pipe is not used.
// The FP64 -> FP32 conversions of the state truncate by moving bits too (1 ulp).

namespace {

constexpr float kEps32 = 5.9604645e-8f;   // 2^-24

// FP32 constants of a view, formed on the host (FP32 roundings of the exact values; the
// guard band above allows for them) and passed by value, so no block spends FP64
// divisions on them.
struct View32 {
    float cr, sr, ci, si, cp, sp;
    float inv_psca, hx, hy;               // 1/psca, 0.5 psca xsize, 0.5 psca ysize
    double inv_psca64;                    // 1/psca in FP64 (the guard-band path)
    float inv_d;                          // 1/dist
    float htheta, cmax;                   // (ntheta-1)/2, 1 - 2/ntheta
    float Rmin, Rmax, fR, inv_fR;
    int xsize, ysize, ntheta;
};

View32 make_view32(const ddx_view& v, const OpticsDev& o) {
    View32 w;
    const double psca = v.xsize >= v.ysize ? v.fov / v.xsize : v.fov / v.ysize;
    w.cr = (float)cos(v.longitude); w.sr = (float)sin(v.longitude);
    w.ci = (float)cos(v.inc); w.si = (float)sin(v.inc);
    w.cp = (float)cos(v.PA); w.sp = (float)sin(v.PA);
    w.inv_psca = (float)(1.0 / psca);
    w.inv_psca64 = 1.0 / psca;
    w.hx = (float)(0.5 * psca * v.xsize);
    w.hy = (float)(0.5 * psca * v.ysize);
    w.inv_d = (float)(1.0 / v.dist);
    w.htheta = 0.5f * (float)(o.n_theta - 1);
    w.cmax = (float)(1.0 - 2.0 / o.n_theta);
    w.Rmin = (float)o.Rmin; w.Rmax = (float)o.Rmax;
    w.fR = (float)o.fR; w.inv_fR = (float)(1.0 / o.fR);
    w.xsize = v.xsize; w.ysize = v.ysize; w.ntheta = o.n_theta;
    return w;
}

// FP64 -> FP32 by truncating the significand (error < 1 ulp of the float); values below
// the FP32 normal range become zero, values above it infinite, and NaN stays NaN (so that a
// NaN tracer fails every range test downstream).
__device__ __forceinline__ float d2f_trunc(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const int e = (int)((b >> 52) & 0x7ff) - 1023;
    const unsigned int sign = (unsigned int)(b >> 32) & 0x80000000u;
    if (e < -126) return __uint_as_float(sign);
    if (e > 127) return __uint_as_float((b << 12) != 0ull && e == 1024 ? 0x7fc00000u : (sign | 0x7f800000u));
    return __uint_as_float(sign | ((unsigned int)(e + 127) << 23) | (unsigned int)((b >> 29) & 0x7fffffu));
}

// f * 2^sh as FP64, exactly, for normal f (zero and subnormal f give 0).
__device__ __forceinline__ double f2d_scaled(float f, int sh) {
    const unsigned int b = __float_as_uint(f);
    const unsigned int e = (b >> 23) & 0xffu;
    if (e == 0) return 0.0;
    const unsigned long long d = ((unsigned long long)(b & 0x80000000u) << 32) |
                                 ((unsigned long long)(e - 127 + 1023 + sh) << 52) |
                                 ((unsigned long long)(b & 0x7fffffu) << 29);
    return __longlong_as_double((long long)d);
}

__device__ __forceinline__ bool near_edge32(float u, float g) {
    const float f = u - floorf(u);
    return f < g || f > 1.0f - g;
}

// The FP64 decisions of the mixed image, out of line so that none of their FP64 work is
// hoisted into the common FP32 path.  R32: the tracer's FP32 radius from truncated
// coordinates (at most 2^-22 below the FP64 one), so R32 (1 + 1e-6) bounds the radius from
// above for the guard band without an FP64 square root.  The coordinates are scaled by the
// reciprocal pixel size instead of divided (one more rounding, 3e-16 of the coordinate, far
// inside the 1e-12 band), which keeps this path at about 25 FP64 operations (about 55 with
// the square root and the three divisions).
__device__ __forceinline__ void fast_pixel_coord_mul(double x, double y, double z, const ViewConst& v,
                                                     double inv_psca, double& u, double& w) {
    const double x1 = x * v.cr - y * v.sr;
    const double y1 = x * v.sr + y * v.cr;
    const double y2 = y1 * v.ci + z * v.si;
    u = (x1 * v.cp - y2 * v.sp + 0.5 * v.psca * v.xsize) * inv_psca;
    w = (x1 * v.sp + y2 * v.cp + 0.5 * v.psca * v.ysize) * inv_psca;
}
__device__ __noinline__ void pixel_fp64(double x, double y, double z, float R32, double inv_psca, const ViewConst& v,
                                        int& xim, int& yim, unsigned long long* counters) {
    atomicAdd(&counters[1], 1ull);
    const double Rd = (double)R32 * (1.0 + 1e-6);
    double ud, wd;
    fast_pixel_coord_mul(x, y, z, v, inv_psca, ud, wd);
    // guard_width with R/psca as R * inv_psca: a bound either way (no FP64 division)
    const double gd = 1e-12 * (Rd * inv_psca + fmax(fabs(ud), fabs(wd)) + 1.0);
    if (far_off_frame(ud, wd, gd, v)) {
        xim = yim = -1;
        return;
    }
    if (near_edge(ud, gd) || near_edge(wd, gd)) {
        double cs;
        exact_pixel(x, y, z, v, xim, yim, cs);
        atomicAdd(&counters[0], 1ull);
    } else {
        xim = (int)floor(ud);
        yim = (int)floor(wd);
    }
}

__device__ __noinline__ bool outside_rmin_fp64(double x, double y, double z, double Rmin) {
    return sqrt(x * x + y * y + z * z) > Rmin;
}

__device__ __forceinline__ float ex2_approx(float a) {
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
    return r;
}
__device__ __forceinline__ float rcp_approx(float a) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
    return r;
}

// Scattering-angle cosine of src/gpu_functions.cu:1017-1023 rewritten for FP32 range:
// with A = x1^2 + y1^2 + z^2, q = y1 sin(i) - z cos(i) and d the distance,
// (A + d q) / (R sqrt(A + 2 d q + d^2)) = (A/d + q) / (R sqrt(A/d^2 + 2 q/d + 1));
// clamped like the reference.  A = R^2, or R^2 + z^2 where the reference rotates by the
// spherical radius.
__device__ __forceinline__ float scatter_cos32(float y1, float z, float R, float A, const View32& v) {
    const float q = y1 * v.si - z * v.ci;
    const float ad = A * v.inv_d;
    float c = (ad + q) / (R * sqrtf(fmaf(ad, v.inv_d, fmaf(2.0f * q, v.inv_d, 1.0f))));
    if (!(c >= -1.0f)) c = -1.0f;   // NaN too (a tracer beyond the float range): the table index stays in range
    if (c >= v.cmax) c = v.cmax;
    return c;
}

// Everything about a tracer that does not depend on the wavelength, in FP32.
struct Tracer32 {
    float n, invR2, wt, rT;
    int id, cm;
};

// Accuracy: the Planck factor 1/(exp(x) - 1), x = hc/(lambda k T), turns a relative
// error d in T into about x d in the flux, and x reaches tens on the Wien side.  So T (once
// per tracer) and exp(x) use the accurate logf/expf; the phase function, whose error is
// not amplified, takes one ex2.approx on a table of base-2 logs.
__device__ __forceinline__ void tracer32_photometry(float R, float cossc, int id, float n, const View32& v,
                                                    const OpticsDev& o, Tracer32& t) {
    int cm = (int)floorf((cossc + 1.0f) * v.htheta);
    cm = cm < 0 ? 0 : (cm > v.ntheta - 2 ? v.ntheta - 2 : cm);
    t.cm = cm;
    t.wt = (cossc - ((float)cm / v.htheta - 1.0f)) * v.htheta;
    const float* lT = o.lTd32 + (size_t)id * kNR;
    float lTv;
    if (R >= v.Rmax) {
        lTv = lT[kNR - 1];
    } else {
        const float lr = logf(R / v.Rmin);
        int Rid = (int)(lr * v.inv_fR) + 1;
        Rid = Rid < 1 ? 1 : (Rid > kNR - 1 ? kNR - 1 : Rid);
        const float frac = (lr - (float)(Rid - 1) * v.fR) * v.inv_fR;
        lTv = lT[Rid - 1] + (lT[Rid] - lT[Rid - 1]) * frac;
    }
    t.rT = expf(-lTv);                    // 1/T
    t.invR2 = 1.0f / (R * R);
    t.n = n;
    t.id = id;
}

// Scaled flux of tracer t at one wavelength: l = (log2 P(cm), log2 P(cm+1)) from the
// tracer's row of base-2 log phase-function pairs (bin, cos bracket cm), a = (At, As) of its
// bin at the wavelength, C2j = h c / (lambda k).
__device__ __forceinline__ float flux32_row(const Tracer32& t, float2 l, float2 a, float C2j) {
    const float x = C2j * t.rT;
    const float e = expf(x);
    // exp(x) - 1 loses digits for small x: Taylor series there (error < x^8/8! < 1e-7 rel)
    const float ser = x * (1.0f + x * (0.5f + x * (1.0f / 6 + x * (1.0f / 24 + x * (1.0f / 120 + x * (1.0f / 720 + x * (1.0f / 5040)))))));
    const float em1 = x < 0.5f ? ser : e - 1.0f;
    const float pl = rcp_approx(em1);     // 0 once the exponential overflows
    const float P = ex2_approx(l.x + (l.y - l.x) * t.wt);
    return t.n * fmaf(a.x, pl, a.y * P * t.invR2);
}

// The same at wavelength slot j (table wavelength J) from the rows: lq2[J] and A[j], one
// 8-byte load each.
__device__ __forceinline__ float flux32(const Tracer32& t, const float2* lq2, const float2* A, int j, int J,
                                        float C2j) {
    return flux32_row(t, lq2[J], A[j], C2j);
}

}  // namespace

// At, As, C2, esh for the wavelength slots of one call: one block per slot.
__global__ void photo_prepare_kernel(OpticsDev o, const ViewConst* __restrict__ vcp, ImageList il, int use_list,
                                     PhotoConst pc) {
    __shared__ double smax[256];
    const int j = blockIdx.x;
    const int J = use_list ? il.wj[j] : j;
    const double dist = vcp->dist;
    const double wvl = o.w[J];
    const double common = 1e26 * wvl * wvl / kCspeed;
    const double ct = (2 * kHplank * kCspeed * kCspeed) / o.w5[J] * kPI / dist / dist * common;
    const double cs = o.in[J] * kPI / kAU / kAU * common;
    double m = 0.0;
    for (int k = threadIdx.x; k < o.n_grid; k += blockDim.x) {
        const double s2 = o.size[k] * o.size[k];
        const double at = ct * s2 * o.Qabs[(size_t)o.n_wav * k + J];
        const double as = cs * s2 * o.Qsca[(size_t)o.n_wav * k + J];
        m = fmax(m, fmax(fabs(at), fabs(as)));
    }
    smax[threadIdx.x] = m;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) smax[threadIdx.x] = fmax(smax[threadIdx.x], smax[threadIdx.x + h]);
        __syncthreads();
    }
    int e = 0;
    if (smax[0] > 0.0 && isfinite(smax[0])) { frexp(smax[0], &e); e = 1 - e; }
    const double scale = ldexp(1.0, e);
    for (int k = threadIdx.x; k < o.n_grid; k += blockDim.x) {
        const double s2 = o.size[k] * o.size[k];
        pc.A[(size_t)k * pc.n_lam + j] = make_float2((float)(ct * s2 * o.Qabs[(size_t)o.n_wav * k + J] * scale),
                                                     (float)(cs * s2 * o.Qsca[(size_t)o.n_wav * k + J] * scale));
    }
    if (threadIdx.x == 0) {
        pc.C2[j] = (float)(kHplank * kCspeed / (wvl * kKboltz));
        pc.esh[j] = e;
    }
}

// Images, mixed precision: one thread per tracer, every image wavelength in one pass.  The
// sums go to an FP32 buffer interleaved by wavelength, Fi[pixel][K4] (K4 = n_img rounded up
// to 4), in the wavelengths' scaled domain (2^esh), as 16-byte vector atomics: one request
// adds four wavelengths of a tracer, a quarter of the requests of one FP64 atomic per
// wavelength, and FP32 atomics do not issue through the FP64 pipe.
// Warp aggregation: adjacent lanes whose tracers land on the same pixel form a run; a
// segmented tree sum (five shuffle steps) gives each run's first lane the run's fluxes, and
// that lane issues one atomic for all of them.  A warp without such runs skips the shuffles.
// The gain grows with the tracers per pixel that sit next to each other in the state (all
// of them when the tracers are stored in pixel order).
// image_convert_kernel then writes the FP64 x-major images.
__global__ void __launch_bounds__(256)
image_mixed_kernel(ddx_state s, int n_grav, int n_dust, const ViewConst* __restrict__ vcp, View32 v32, OpticsDev o,
                   ImageList il, PhotoConst pc, float* __restrict__ Fi, int K4,
                   unsigned long long* __restrict__ counters) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    bool valid = false;
    size_t pix = 0;
    Tracer32 tr;
    if (i < n_dust) {
        const int t = n_grav + i;
        const int id = s.id[t];
        if (id >= 0 && id < o.n_grid) {
            const double x = s.x[t], y = s.y[t], z = s.z[t];
            const float xf = d2f_trunc(x), yf = d2f_trunc(y), zf = d2f_trunc(z);
            const float R = sqrtf(fmaf(xf, xf, fmaf(yf, yf, zf * zf)));
            const float x1 = xf * v32.cr - yf * v32.sr;
            const float y1 = xf * v32.sr + yf * v32.cr;
            const float y2 = y1 * v32.ci + zf * v32.si;
            const float u = (x1 * v32.cp - y2 * v32.sp + v32.hx) * v32.inv_psca;
            const float w = (x1 * v32.sp + y2 * v32.cp + v32.hy) * v32.inv_psca;
            const float g = 64.0f * kEps32 * (R * v32.inv_psca + fmaxf(fabsf(u), fabsf(w)) + 1.0f);
            // more than g + 2 pixels off the frame (or NaN): off the frame in FP64 and in the
            // reference's sequence too, and no int conversion of the coordinates is made
            const float mg = g + 2.0f;
            const bool reach = u > -mg && u < (float)v32.xsize + mg && w > -mg && w < (float)v32.ysize + mg;
            int xim = -1, yim = -1;
            if (!reach) {
            } else if (near_edge32(u, g) || near_edge32(w, g)) {
                pixel_fp64(x, y, z, R, v32.inv_psca64, *vcp, xim, yim, counters);
            } else {
                xim = (int)floorf(u);
                yim = (int)floorf(w);
            }
            valid = !(xim < 0 || xim > v32.xsize - 1 || yim < 0 || yim > v32.ysize - 1);
            if (valid && !(R > v32.Rmin * (1.0f + 1e-5f)))
                valid = !(R < v32.Rmin * (1.0f - 1e-5f)) && outside_rmin_fp64(x, y, z, o.Rmin);
            if (valid) {
                tracer32_photometry(R, scatter_cos32(y1, zf, R, R * R, v32), id, d2f_trunc(s.N[t]), v32, o, tr);
                pix = (size_t)v32.ysize * xim + yim;
            }
        }
    }
    // Runs of adjacent lanes on one pixel (a lane without a pixel gets a key of its own):
    // the first lane of each run is its head.  A warp whose lanes all differ from their
    // neighbours (tracers in no particular order) learns so from one shuffle and one ballot
    // and goes straight to the atomics.
    const unsigned FULL = 0xffffffffu;
    const unsigned long long key = valid ? (unsigned long long)pix : ~0ull - (unsigned long long)lane;
    const unsigned long long prev = __shfl_up_sync(FULL, key, 1);
    const bool head = lane == 0 || prev != key;
    const unsigned heads = __ballot_sync(FULL, head);
    const bool runs = heads != FULL;
    if (!valid && !runs) return;   // no shuffles in this warp: nothing left for this lane
    // the segmented tree sum's steps: bit k set when lane + 2^k is in this lane's run
    unsigned take = 0u;
    if (runs) {
        const unsigned seg = __popc(heads & (FULL >> (31 - lane)));   // runs begun at or below this lane
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            const unsigned so = __shfl_down_sync(FULL, seg, 1 << k);
            if (lane + (1 << k) < 32 && so == seg) take |= 1u << k;
        }
    }
    const float2* lq2 = valid ? o.lQp32p + ((size_t)tr.id * (o.n_theta - 1) + tr.cm) * o.n_wav : nullptr;
    const float2* A = valid ? pc.A + (size_t)tr.id * pc.n_lam : nullptr;
    float* row = Fi + pix * K4;
    // eight wavelengths at a time, their table loads issued together before the arithmetic
    for (int g = 0; g < il.n; g += 8) {
        float f[8];
        if (valid) {
            float2 lv[8], av[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int k = g + u;
                lv[u] = k < il.n ? lq2[il.wj[k]] : make_float2(0.f, 0.f);
                av[u] = k < il.n ? A[k] : make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int k = g + u;
                f[u] = k < il.n ? flux32_row(tr, lv[u], av[u], pc.C2[k]) : 0.0f;
            }
        } else {
#pragma unroll
            for (int u = 0; u < 8; ++u) f[u] = 0.0f;
        }
        if (runs) {
            // after step k each lane holds the sum of its run over lanes [lane, lane + 2^(k+1));
            // the run being contiguous, its head ends with the whole run
#pragma unroll
            for (int k = 0; k < 5; ++k) {
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    if (g + u >= il.n) break;   // warp-uniform: no shuffles for the padding slots
                    const float v = __shfl_down_sync(FULL, f[u], 1 << k);
                    if ((take >> k) & 1u) f[u] += v;
                }
            }
        }
        if (!valid || !head) continue;
#pragma unroll
        for (int h = 0; h < 8; h += 4)
            if (g + h < il.n && (f[h] != 0.0f || f[h + 1] != 0.0f || f[h + 2] != 0.0f || f[h + 3] != 0.0f))
                atomicAdd(reinterpret_cast<float4*>(row + g + h), make_float4(f[h], f[h + 1], f[h + 2], f[h + 3]));
    }
}

// One thread per pixel: the interleaved FP32 sums to the FP64 x-major images,
// Fd[k][pixel] = Fi[pixel][k] 2^-esh[k] (an exact power-of-two scaling).
__global__ void image_convert_kernel(const float* __restrict__ Fi, int K4, int n_img, size_t npix,
                                     const int* __restrict__ esh, double* __restrict__ Fd) {
    const size_t pix = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (pix >= npix) return;
    const float4* row = reinterpret_cast<const float4*>(Fi + pix * K4);
    for (int g = 0; g < n_img; g += 4) {
        const float4 v = row[g >> 2];
        const float f[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (g + u < n_img) Fd[(size_t)(g + u) * npix + pix] = f2d_scaled(f[u], -esh[g + u]);
    }
}

// SED, mixed precision.  Each warp takes 32 tracers at a time; lane l accumulates the
// wavelengths lam0 + l + 32 c (c < kSedChunks) over all of them, so the table reads of a
// step are contiguous across the lanes and no per-wavelength reduction is needed inside
// the loop.  Per lane: a plain FP32 sum over each group of 32 tracers, added to an FP32
// Kahan sum; then FP64 sums over the warps in a fixed order and over the blocks in
// sed_final_kernel.  Deterministic.
constexpr int kSedChunks = 8;   // wavelengths per pass: 32 * kSedChunks

__global__ void __launch_bounds__(kSedThreads, 3)
sed_mixed_kernel(ddx_state s, int n_grav, int n_dust, View32 v32, OpticsDev o,
                 PhotoConst pc, int mode, int lam0, double* __restrict__ partial) {
    __shared__ double red[kSedThreads / 32][32 * kSedChunks];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int gw = blockIdx.x * (kSedThreads / 32) + warp, nw = gridDim.x * (kSedThreads / 32);
    float S[kSedChunks], Cc[kSedChunks], C2r[kSedChunks];
    const int rem = pc.n_lam - lam0;
    const int nchunks = rem >= 32 * kSedChunks ? kSedChunks : (rem + 31) / 32;
#pragma unroll
    for (int c = 0; c < kSedChunks; ++c) {
        S[c] = 0.f; Cc[c] = 0.f;
        const int j = lam0 + c * 32 + lane;
        C2r[c] = j < pc.n_lam ? pc.C2[j] : 0.f;
    }
    for (int base = gw * 32; base < n_dust; base += nw * 32) {
        const int i = base + lane;
        Tracer32 tr;
        bool on = false;
        tr.n = 0.f; tr.invR2 = 0.f; tr.wt = 0.f; tr.rT = 0.f; tr.id = 0; tr.cm = 0;
        if (i < n_dust) {
            const int t = n_grav + i;
            const int id = s.id[t];
            if (id >= 0 && id < o.n_grid) {
                const double x = s.x[t], y = s.y[t], z = s.z[t];
                const float xf = d2f_trunc(x), yf = d2f_trunc(y), zf = d2f_trunc(z);
                const float R = sqrtf(fmaf(xf, xf, fmaf(yf, yf, zf * zf)));
                float y1 = xf * v32.sr + yf * v32.cr;
                float A = R * R;
                if (mode == DDX_MODE_REFERENCE) {
                    // the reference rotates by the spherical radius (src/gpu_functions.cu:1106-1107)
                    const float Rd = sqrtf(fmaf(xf, xf, yf * yf));
                    y1 = Rd > 0.f ? y1 * (R / Rd) : R * v32.sr;
                    A = fmaf(zf, zf, A);
                }
                on = R > v32.Rmin * (1.0f + 1e-5f) ||
                     (R >= v32.Rmin * (1.0f - 1e-5f) && outside_rmin_fp64(x, y, z, o.Rmin));
                if (on) tracer32_photometry(R, scatter_cos32(y1, zf, R, A, v32), id, d2f_trunc(s.N[t]), v32, o, tr);
            }
        }
        const unsigned live = __ballot_sync(0xffffffffu, on);
        float G[kSedChunks];                                      // this group's plain sums
#pragma unroll
        for (int c = 0; c < kSedChunks; ++c) G[c] = 0.f;
        const int off = lam0 + lane;                              // this lane's first wavelength
        for (unsigned m = live; m; m &= m - 1) {
            const int src = __ffs(m) - 1;
            Tracer32 b;
            b.n = __shfl_sync(0xffffffffu, tr.n, src);
            b.invR2 = __shfl_sync(0xffffffffu, tr.invR2, src);
            b.wt = __shfl_sync(0xffffffffu, tr.wt, src);
            b.rT = __shfl_sync(0xffffffffu, tr.rT, src);
            b.id = __shfl_sync(0xffffffffu, tr.id, src);
            b.cm = __shfl_sync(0xffffffffu, tr.cm, src);
            const float2* lq2 = o.lQp32p + ((size_t)b.id * (o.n_theta - 1) + b.cm) * o.n_wav + off;
            const float2* A = pc.A + (size_t)b.id * pc.n_lam + off;
#pragma unroll
            for (int c = 0; c < kSedChunks; ++c) {
                if (c >= nchunks) break;                          // warp-uniform
                if (off + c * 32 < pc.n_lam) G[c] += flux32(b, lq2, A, c * 32, c * 32, C2r[c]);
            }
        }
#pragma unroll
        for (int c = 0; c < kSedChunks; ++c) {
            const float yk = G[c] - Cc[c];
            const float tk = S[c] + yk;
            Cc[c] = (tk - S[c]) - yk;
            S[c] = tk;
        }
    }
#pragma unroll
    for (int c = 0; c < kSedChunks; ++c) {
        const int j = lam0 + c * 32 + lane;
        red[warp][c * 32 + lane] = j < pc.n_lam ? f2d_scaled(S[c], -pc.esh[j]) - f2d_scaled(Cc[c], -pc.esh[j]) : 0.0;
    }
    __syncthreads();
    for (int jj = threadIdx.x; jj < 32 * kSedChunks; jj += blockDim.x) {
        const int j = lam0 + jj;
        if (j >= pc.n_lam) continue;
        double b = 0.0;
        for (int w = 0; w < kSedThreads / 32; ++w) b += red[w][jj];
        partial[(size_t)blockIdx.x * o.n_wav + j] = b;
    }
}

int sed_mixed_blocks(int n_dust) { return sed_blocks(n_dust); }

cudaError_t launch_photo_prepare(const OpticsDev& o, const ViewConst* vc, const ImageList* il,
                                 PhotoConst pc, cudaStream_t st) {
    ImageList none{};
    photo_prepare_kernel<<<pc.n_lam, 256, 0, st>>>(o, vc, il ? *il : none, il ? 1 : 0, pc);
    return cudaGetLastError();
}

cudaError_t launch_image_mixed(const ddx_state& s, int n_grav, int n_dust, const ddx_view& view,
                               const OpticsDev& o, const ImageList& il, ViewConst* vc, PhotoConst pc,
                               double* Fd, float* Fi, unsigned long long* counters, cudaStream_t st) {
    view_setup_kernel<<<1, 32, 0, st>>>(vc, view, o.n_theta);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    pc.n_lam = il.n;
    if ((e = launch_photo_prepare(o, vc, &il, pc, st)) != cudaSuccess) return e;
    const size_t npix = (size_t)view.xsize * view.ysize;
    const int K4 = image_k4(il.n);
    if ((e = cudaMemsetAsync(Fi, 0, sizeof(float) * npix * K4, st)) != cudaSuccess) return e;
    if (n_dust > 0)
        image_mixed_kernel<<<(n_dust + 255) / 256, 256, 0, st>>>(s, n_grav, n_dust, vc, make_view32(view, o), o, il,
                                                                 pc, Fi, K4, counters);
    image_convert_kernel<<<(unsigned)((npix + 255) / 256), 256, 0, st>>>(Fi, K4, il.n, npix, pc.esh, Fd);
    return cudaGetLastError();
}

cudaError_t launch_sed_mixed(const ddx_state& s, int n_grav, int n_dust, const ddx_view& view,
                             const OpticsDev& o, ViewConst* vc, PhotoConst pc, double* partial, int mode,
                             double* Fsed, cudaStream_t st) {
    view_setup_kernel<<<1, 32, 0, st>>>(vc, view, o.n_theta);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    pc.n_lam = o.n_wav;
    if ((e = launch_photo_prepare(o, vc, nullptr, pc, st)) != cudaSuccess) return e;
    const int nb = sed_mixed_blocks(n_dust);
    const View32 v32 = make_view32(view, o);
    for (int lam0 = 0; lam0 < o.n_wav; lam0 += 32 * kSedChunks) {
        sed_mixed_kernel<<<nb, kSedThreads, 0, st>>>(s, n_grav, n_dust, v32, o, pc, mode, lam0, partial);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    sed_final_kernel<<<(o.n_wav + 127) / 128, 128, 0, st>>>(partial, nb, o.n_wav, Fsed);
    return cudaGetLastError();
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
