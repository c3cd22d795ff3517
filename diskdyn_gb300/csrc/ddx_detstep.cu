// Time step of a run (Grid::det_step, src/grid.cu:312-342), with the body scan on the GPU.
//
// The reference copies the whole state to the host and scans the massive bodies there:
//   dt = min over i in 1..n_grav-1 of 2 pi sqrt(pow(|x_i - x_0|^2, 3/2) / (m_0 + m_i)) / n_step
// (and over the disks and blobs of the configuration).  Everything after the squared
// distance is weakly monotone in key_i = pow(RR_i, 1.5) / (m_0 + m_i) for all bodies alike
// (IEEE division, sqrt and multiplication by a positive constant are monotone), so the
// minimum dt comes from the body of least key.  The GPU forms RR_i without contraction
// (the same value the reference's host code gets), an approximate key, its minimum, and
// the few bodies whose approximate key lies within 1e-12 of it; the host then evaluates
// the reference's own expression, with the host libm's pow, on those candidates only.
// The approximate key is within a few ulp of the exact one, so the true minimiser is
// always among the candidates and the result is the reference's to the bit.
#include "ddx_internal.cuh"

namespace ddx {

namespace {

constexpr int kDetThreads = 256;

// Positive doubles order like their bit patterns, so atomicMin on the bits is a min.
__global__ void det_key_kernel(ddx_state s, int n_grav, double* __restrict__ rr, unsigned long long* kmin) {
    __shared__ unsigned long long smin[kDetThreads / 32];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long k = ~0ull;
    if (i >= 1 && i < n_grav) {
        const double dx = __dsub_rn(s.x[i], s.x[0]);
        const double dy = __dsub_rn(s.y[i], s.y[0]);
        const double dz = __dsub_rn(s.z[i], s.z[0]);
        const double RR = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
        rr[i] = RR;
        const double key = RR * sqrt(RR) / (s.m[0] + s.m[i]);
        if (key >= 0.0) k = __double_as_longlong(key);   // NaN keys are never the minimum
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long t = __shfl_xor_sync(0xffffffffu, k, o);
        k = t < k ? t : k;
    }
    if ((threadIdx.x & 31) == 0) smin[threadIdx.x >> 5] = k;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long b = smin[0];
        for (int w = 1; w < kDetThreads / 32; ++w) b = smin[w] < b ? smin[w] : b;
        if (b != ~0ull) atomicMin(kmin, b);
    }
}

// Bodies whose approximate key is within 1e-12 of the minimum, as (index) into cand.
__global__ void det_cand_kernel(ddx_state s, int n_grav, const double* __restrict__ rr,
                                const unsigned long long* kmin, int* count, int* cand, int cap) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 1 || i >= n_grav || *kmin == ~0ull) return;
    const double lim = __longlong_as_double((long long)*kmin) * (1.0 + 1e-12);
    const double RR = rr[i];
    const double key = RR * sqrt(RR) / (s.m[0] + s.m[i]);
    if (key <= lim) {
        const int k = atomicAdd(count, 1);
        if (k < cap) cand[k] = i;
    }
}

}  // namespace

void det_step_free(DetStepScratch*& d) {
    if (!d) return;
    cudaFree(d->rr); cudaFree(d->kmin); cudaFree(d->count); cudaFree(d->cand);
    delete d;
    d = nullptr;
}

int det_step_scan(DetStepScratch*& d, const ddx_state& s, int n_grav, cudaStream_t st,
                  std::vector<double>& rr, std::vector<double>& mi, double& m0) {
    rr.clear();
    mi.clear();
    if (cudaMemcpyAsync(&m0, s.m, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess) return DDX_ERR_CUDA;
    if (n_grav <= 1) return cudaStreamSynchronize(st) == cudaSuccess ? DDX_OK : DDX_ERR_CUDA;
    if (!d || d->cap_bodies < n_grav) {
        det_step_free(d);
        d = new DetStepScratch();
        int cap = 1024;
        while (cap < n_grav) cap *= 2;
        d->cap_bodies = cap;
        if (cudaMalloc(&d->rr, sizeof(double) * cap) || cudaMalloc(&d->kmin, sizeof(unsigned long long)) ||
            cudaMalloc(&d->count, sizeof(int)) || cudaMalloc(&d->cand, sizeof(int) * kDetCandidates)) {
            det_step_free(d);
            cudaGetLastError();
            return DDX_ERR_NOMEM;
        }
    }
    const int blocks = (n_grav + kDetThreads - 1) / kDetThreads;
    cudaMemsetAsync(d->kmin, 0xff, sizeof(unsigned long long), st);
    cudaMemsetAsync(d->count, 0, sizeof(int), st);
    det_key_kernel<<<blocks, kDetThreads, 0, st>>>(s, n_grav, d->rr, d->kmin);
    det_cand_kernel<<<blocks, kDetThreads, 0, st>>>(s, n_grav, d->rr, d->kmin, d->count, d->cand, kDetCandidates);
    if (cudaGetLastError() != cudaSuccess) return DDX_ERR_CUDA;
    int count = 0;
    if (cudaMemcpyAsync(&count, d->count, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return DDX_ERR_CUDA;
    std::vector<int> idx;
    if (count <= kDetCandidates) {
        idx.resize(count);
        if (count && cudaMemcpy(idx.data(), d->cand, sizeof(int) * count, cudaMemcpyDeviceToHost) != cudaSuccess)
            return DDX_ERR_CUDA;
    } else {   // a degenerate system (many bodies at one key): take every body
        idx.resize(n_grav - 1);
        for (int i = 1; i < n_grav; ++i) idx[i - 1] = i;
    }
    // gather RR and m of the candidates
    std::vector<double> all_rr, all_m;
    if (count > kDetCandidates) {
        all_rr.resize(n_grav);
        all_m.resize(n_grav);
        if (cudaMemcpy(all_rr.data(), d->rr, sizeof(double) * n_grav, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(all_m.data(), s.m, sizeof(double) * n_grav, cudaMemcpyDeviceToHost) != cudaSuccess)
            return DDX_ERR_CUDA;
    }
    for (int i : idx) {
        double r, m;
        if (count > kDetCandidates) {
            r = all_rr[i];
            m = all_m[i];
        } else if (cudaMemcpy(&r, d->rr + i, sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess ||
                   cudaMemcpy(&m, s.m + i, sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) {
            return DDX_ERR_CUDA;
        }
        rr.push_back(r);
        mi.push_back(m);
    }
    return DDX_OK;
}

}  // namespace ddx
