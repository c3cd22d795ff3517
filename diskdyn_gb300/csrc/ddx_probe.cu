// Compute-pipe throughput probe: independent FMA chains on every SM, timed with events.
// The FP32 and FP64 FMA rates it reports are the roofline denominators of the force
// kernels, which are bound by those pipes rather than by HBM or the tensor cores.
#include "ddx_internal.cuh"

namespace {

constexpr int kIters = 2048;

__global__ void fma32_kernel(float* out, float a, float b) {
    float r[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) r[j] = threadIdx.x + j;
    for (int i = 0; i < kIters; ++i) {
#pragma unroll
        for (int j = 0; j < 16; ++j) r[j] = fmaf(r[j], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < 16; ++j) s += r[j];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void fma64_kernel(double* out, double a, double b) {
    double r[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) r[j] = threadIdx.x + j;
    for (int i = 0; i < kIters / 8; ++i) {
#pragma unroll
        for (int j = 0; j < 8; ++j) r[j] = fma(r[j], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < 8; ++j) s += r[j];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" int ddx_probe_fma_peak(int device, double* fp32_tflops, double* fp64_tflops) {
    if (!fp32_tflops || !fp64_tflops) return DDX_ERR_ARG;
    ddx::DeviceGuard dg(device);
    if (!dg.ok()) return DDX_ERR_CUDA;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int threads = 256, blocks = sms * 8;
    const size_t n = (size_t)threads * blocks;
    void* buf = nullptr;
    if (cudaMalloc(&buf, n * sizeof(double)) != cudaSuccess) return DDX_ERR_NOMEM;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best32 = 1e30f, best64 = 1e30f, ms = 0.f;
    for (int rep = 0; rep < 3; ++rep) {
        cudaEventRecord(e0);
        fma32_kernel<<<blocks, threads>>>((float*)buf, 0.999f, 1e-3f);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        best32 = ms < best32 ? ms : best32;
        cudaEventRecord(e0);
        fma64_kernel<<<blocks, threads>>>((double*)buf, 0.999, 1e-3);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        best64 = ms < best64 ? ms : best64;
    }
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    if (err != cudaSuccess) return DDX_ERR_CUDA;
    *fp32_tflops = 2.0 * 16 * kIters * (double)n / (best32 * 1e-3) / 1e12;
    *fp64_tflops = 2.0 * 8 * (kIters / 8) * (double)n / (best64 * 1e-3) / 1e12;
    return DDX_OK;
}
