// Declarations shared by the flux kernels and the C ABI layer.
#pragma once
#include "ddx_internal.cuh"

namespace ddx {

constexpr int kMaxImages = 64;   // image wavelengths per ddx_image call

// Constants of one observer geometry (device resident, written by view_setup_kernel).
struct ViewConst {
    double dist, rot, incl, PA, psca, fov;
    double cr, sr, ci, si, cp, sp;   // cos/sin of rot, incl, PA
    double ly0, lz0;                 // -dist sin(incl), dist cos(incl)
    int xsize, ysize, ntheta;
};

// Device optical tables (pointers into context-owned buffers).
struct OpticsDev {
    const double *w, *in, *Qabs, *Qsca, *Qp, *Td, *size;
    double *lQp, *lTd, *w5;          // derived on the device
    // mixed photometry: lQp32p[k][cm][j] = (log2 Qp[k][cm][j], log2 Qp[k][cm+1][j]), the
    // bracket of a scattering-angle bin in one 8-byte load; lTd32 = (float) log Td
    float2* lQp32p;                  // [n_grid][n_theta-1][n_wav]
    float* lTd32;                    // [n_grid][100]
    double Rmin, Rmax, fR;           // fR = log(Rmax/Rmin)/(nR-1)
    int n_grid, n_wav, n_theta;
};

struct ImageList {
    int n;
    int wj[kMaxImages];
};

// Per-call FP32 photometry coefficients of the mixed path, for n_lam wavelengths
// (the image list, or every table wavelength for the SED).  The flux of a tracer of bin k
// at wavelength slot j, before its multiplicity N, is
//   (At[k][j] / (exp(C2[j] / T) - 1) + As[k][j] P / R^2) * 2^-esh[j]
// with At, As scaled by 2^esh[j] so that their largest value over the bins lies in [1, 2).
struct PhotoConst {
    float2* A;                       // [n_grid][n_lam] = (At, As)
    float* C2;                       // [n_lam] h c / (lambda k), K
    int* esh;                        // [n_lam]
    int n_lam;
};

cudaError_t launch_photo_prepare(const OpticsDev& o, const ViewConst* vc, const ImageList* il,
                                 PhotoConst pc, cudaStream_t st);
// Mixed images: Fi is an FP32 scratch of npix * image_k4(n_img) floats (256-byte aligned).
inline int image_k4(int n_img) { return (n_img + 3) / 4 * 4; }
cudaError_t launch_image_mixed(const ddx_state& s, int n_grav, int n_dust, const ddx_view& view,
                               const OpticsDev& o, const ImageList& il, ViewConst* vc, PhotoConst pc,
                               double* Fd, float* Fi, unsigned long long* counters, cudaStream_t st);
cudaError_t launch_sed_mixed(const ddx_state& s, int n_grav, int n_dust, const ddx_view& view,
                             const OpticsDev& o, ViewConst* vc, PhotoConst pc, double* partial, int mode,
                             double* Fsed, cudaStream_t st);
int sed_mixed_blocks(int n_dust);

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

cudaError_t launch_optics_prepare(OpticsDev& o, OpticsDev* o_dev, cudaStream_t st);
cudaError_t launch_image(const ddx_state& s, int n_grav, int n_dust, const ddx_view& view,
                         const OpticsDev& o, const ImageList& il, ViewConst* vc, double* Fd,
                         unsigned long long* nexact, cudaStream_t st);
cudaError_t launch_sed(const ddx_state& s, int n_grav, int n_dust, const ddx_view& view,
                       const OpticsDev& o, ViewConst* vc, double* partial, int mode,
                       double* Fsed, cudaStream_t st);
int sed_blocks(int n_dust);
cudaError_t launch_view_setup(ViewConst* vc, const ddx_view& view, int n_theta, cudaStream_t st);

// Discrete adjoint (ddx_adjoint.cu).
struct AdjointScratch;
int adjoint_forward(AdjointScratch*& a, const ddx_state& s, int ng, int nd, double dt, int n_steps, int K,
                    const StepArgs& sa, const ddx_view& view, const ImageList& il, const SizeBin* bins,
                    const OpticsDev& o, double* image, cudaStream_t st);
int adjoint_backward(AdjointScratch* a, const double* G, double* grad_state, double* grad_mass,
                     const SizeBin* bins, const OpticsDev& o, cudaStream_t st);
void adjoint_free(AdjointScratch*& a);
cudaError_t launch_pixels(const ddx_state& s, int n_grav, int n_dust, const ddx_view& view,
                          int n_theta, ViewConst* vc, int* pix, int* exact, cudaStream_t st);

}  // namespace ddx
