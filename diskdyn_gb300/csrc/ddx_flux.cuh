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
    double Rmin, Rmax, fR;           // fR = log(Rmax/Rmin)/(nR-1)
    int n_grid, n_wav, n_theta;
};

struct ImageList {
    int n;
    int wj[kMaxImages];
};

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
