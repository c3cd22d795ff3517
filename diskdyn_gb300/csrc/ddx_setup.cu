// Initial system on the GPU: the bodies of Grid::setup (src/grid.cu:79-190) drawn by one
// thread each, straight into the device state.
//
// The host builds the plan (ddx_setup.cpp: the segments of bodies with the same generator
// inputs, the gravitating masses of the getbod chain in double, each mass bin's mass, size
// bin and grains per tracer), so counts, order, bins and grain numbers are those of the
// reference's set-up and the gravitating masses agree with its long double chain to
// rounding.  The orbits follow the reference's draws (genorb_disk, genorb_blob,
// src/functions.cu:157-232) and coe2rv (:6-46) in FP64, but the uniform numbers come from
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3",
// SC'11) with the key = the seed and the counter = (draw, body index, a constant): every
// body has its own stream, independent of the launch shape.
#include <cstdint>
#include <vector>

#include "ddx_host.h"
#include "ddx_internal.cuh"

namespace ddx {
namespace {

constexpr double kPI2 = 6.28318530717958623200;
constexpr int kMaxTries = 1024;                 // rejection draws per body
constexpr uint32_t kStreamTag = 0x53455455u;    // fourth counter word of the set-up streams

struct DiskDev {
    double Rin, Rout, sigmae, gammas, dhdr;
};
struct BlobDev {
    double a, ecc, inc, w, o, nu, sigma, vkepp;
    int collcloud;
};

// Philox4x32 with 10 rounds: per round two 32x32 -> 64-bit products of words 0 and 2 with
// the multipliers, a swap and the key xor; the key is bumped by the Weyl constants
// between rounds.
__device__ __forceinline__ void philox10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        if (r) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const uint32_t lo0 = 0xD2511F53u * c[0], hi0 = __umulhi(0xD2511F53u, c[0]);
        const uint32_t lo1 = 0xCD9E8D57u * c[2], hi1 = __umulhi(0xCD9E8D57u, c[2]);
        const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0;
        c[1] = lo1;
        c[2] = n2;
        c[3] = lo0;
    }
}

// 53 random bits of two words as a double in (0, 1]
__device__ __forceinline__ double unit(uint32_t a, uint32_t b) {
    const uint64_t k = ((uint64_t)(a >> 5) << 26) | (b >> 6);
    return (double)(k + 1) * 0x1.0p-53;
}

struct Stream {
    uint32_t k0, k1, lo, hi, draw;
    __device__ void pair(double& u1, double& u2) {
        uint32_t c[4] = {draw++, lo, hi, kStreamTag};
        philox10(c, k0, k1);
        u1 = unit(c[0], c[1]);
        u2 = unit(c[2], c[3]);
    }
};

__device__ __forceinline__ double gauss(double u1, double u2) { return sqrt(-2.0 * log(u1)) * cos(kPI2 * u2); }

__device__ void coe2rv(double M, double m, double a, double e, double i, double w, double o, double nu, double* s,
                       double beta) {
    const double p = a * (1.0 - e * e);
    const double mu = (M + m) * (1.0 - beta);
    double snu, cnu, so, co, sw, cw, si, ci;
    sincos(nu, &snu, &cnu);
    sincos(o, &so, &co);
    sincos(w, &sw, &cw);
    sincos(i, &si, &ci);
    const double xe = p * cnu / (1.0 + e * cnu), ye = p * snu / (1.0 + e * cnu);
    const double vk = sqrt(mu / p);
    const double vxe = -vk * snu, vye = vk * (e + cnu);
    const double r11 = co * cw - so * sw * ci, r12 = -co * sw - so * cw * ci;
    const double r21 = so * cw + co * sw * ci, r22 = -so * sw + co * cw * ci;
    const double r31 = sw * si, r32 = cw * si;
    s[0] = xe * r11 + ye * r12;
    s[1] = xe * r21 + ye * r22;
    s[2] = xe * r31 + ye * r32;
    s[3] = vxe * r11 + vye * r12;
    s[4] = vxe * r21 + vye * r22;
    s[5] = vxe * r31 + vye * r32;
}

__global__ void setup_kernel(const ddx_host::SetupSegment* seg, int n_seg, const double* mass, const DiskDev* disks,
                             const BlobDev* blobs, double M, long long first, long long n_all, uint32_t k0,
                             uint32_t k1, ddx_state st, int* flag) {
    const long long i = first + blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n_all) return;
    int lo = 0, hi = n_seg - 1;                 // the last segment starting at or before i
    while (lo < hi) {
        const int mid = (lo + hi + 1) / 2;
        if (seg[mid].first <= i) lo = mid;
        else hi = mid - 1;
    }
    const ddx_host::SetupSegment g = seg[lo];
    const long long k = i - g.first;
    const double m = g.massive ? mass[g.mass_off + k] : g.m;
    Stream rs{k0, k1, (uint32_t)i, (uint32_t)((unsigned long long)i >> 32), 0};
    double s[6], u1, u2;
    bool ok = false;
    if (g.kind == 0) {
        const DiskDev d = disks[g.j];
        double e = 0.0;
        for (int t = 0; t < kMaxTries && !ok; t++) {
            rs.pair(u1, u2);
            e = fabs(gauss(u1, u2) * d.sigmae);
            ok = e < 1.0;
        }
        const double amin = d.Rin / (1.0 - e), amax = d.Rout / (1.0 + e), gp = 2.0 + d.gammas;
        double ua, unu, ui1, ui2, uw, uo;
        rs.pair(ua, unu);
        rs.pair(ui1, ui2);
        rs.pair(uw, uo);
        const double a = pow(ua * (pow(amax, gp) - pow(amin, gp)) + pow(amin, gp), 1.0 / gp);
        const double inc = fabs(gauss(ui1, ui2) * d.dhdr);
        coe2rv(M, m, a, e, inc, kPI2 * uw, kPI2 * uo, kPI2 * unu, s, g.beta);
    } else {
        const BlobDev b = blobs[g.j];
        double a = 0.0;
        for (int t = 0; t < kMaxTries && !ok; t++) {
            rs.pair(u1, u2);
            a = b.a + gauss(u1, u2) * b.sigma;
            ok = a > 0.0;
        }
        rs.pair(u1, u2);
        const double nu = b.nu + gauss(u1, u2) * b.sigma / a;
        coe2rv(M, m, a, b.ecc, b.inc, b.w, b.o, nu, s, g.beta);
        if (b.collcloud == 0) {
            rs.pair(u1, u2);
            const double voff = b.vkepp * 0.01 * sqrt(s[3] * s[3] + s[4] * s[4] + s[5] * s[5]);
            const double ct = -1.0 + 2.0 * u1, stt = sqrt(1.0 - ct * ct);
            double sg, cg;
            sincos(kPI2 * u2, &sg, &cg);
            s[3] += voff * stt * cg;
            s[4] += voff * stt * sg;
            s[5] += voff * ct;
        }
    }
    if (!ok) atomicOr(flag, 1);
    st.x[i] = s[0];
    st.y[i] = s[1];
    st.z[i] = s[2];
    st.vx[i] = s[3];
    st.vy[i] = s[4];
    st.vz[i] = s[5];
    st.m[i] = m;
    st.N[i] = g.N;
    st.id[i] = g.id;
}

size_t align256(size_t n) { return (n + 255) / 256 * 256; }

}  // namespace

int setup_device_run(const ddx_param* p, double dmin, double dmax, const float* beta, unsigned long long seed,
                     const ddx_state& s, long long cap, ddx_dat_run* run, cudaStream_t st) {
    ddx_host::SetupPlan plan;
    const int r = ddx_host::plan_setup(*p, dmin, dmax, beta, ddx_host::Masses::fast, plan);
    if (r) return r;
    if (cap < plan.n_all || plan.n_all > 0x7fffffffLL) return DDX_ERR_RANGE;

    // star and planets: copies of the configuration
    const int np = p->n_planets;
    double* dst[8] = {s.x, s.y, s.z, s.vx, s.vy, s.vz, s.N, s.m};
    std::vector<double> cols((size_t)8 * np);
    std::vector<int> ids(np, -1);
    for (int j = 0; j < np; j++) {
        const ddx_planet& b = p->planets[j];
        const double v[8] = {b.x, b.y, b.z, b.vx, b.vy, b.vz, 1.0, b.m};
        for (int f = 0; f < 8; f++) cols[(size_t)f * np + j] = v[f];
    }
    std::vector<DiskDev> dk(p->n_disks > 0 ? p->n_disks : 1);
    for (int j = 0; j < p->n_disks; j++) {
        const ddx_disk& d = p->disks[j];
        dk[j] = DiskDev{d.Rin, d.Rout, d.sigmae, d.gammas, d.dhdr};
    }
    std::vector<BlobDev> bl(p->n_blobs > 0 ? p->n_blobs : 1);
    for (int j = 0; j < p->n_blobs; j++) {
        const ddx_blob& b = p->blobs[j];
        bl[j] = BlobDev{b.a, b.ecc, b.inc, b.w, b.o, b.nu, b.sigma, b.vkepp, b.collcloud};
    }

    // one device arena: flag, segments, masses, disks, blobs
    const size_t nseg = plan.seg.size(), nmass = plan.mass.size();
    const size_t o_seg = align256(sizeof(int));
    const size_t o_mass = o_seg + align256(sizeof(ddx_host::SetupSegment) * (nseg + 1));
    const size_t o_disk = o_mass + align256(sizeof(double) * (nmass + 1));
    const size_t o_blob = o_disk + align256(sizeof(DiskDev) * dk.size());
    const size_t bytes = o_blob + align256(sizeof(BlobDev) * bl.size());
    char* arena = nullptr;
    if (cudaMalloc(&arena, bytes) != cudaSuccess) {
        cudaGetLastError();
        return DDX_ERR_NOMEM;
    }
    int* dflag = reinterpret_cast<int*>(arena);
    auto* dseg = reinterpret_cast<ddx_host::SetupSegment*>(arena + o_seg);
    auto* dmass = reinterpret_cast<double*>(arena + o_mass);
    auto* ddisk = reinterpret_cast<DiskDev*>(arena + o_disk);
    auto* dblob = reinterpret_cast<BlobDev*>(arena + o_blob);

    int flag = 0;
    bool ok = cudaMemsetAsync(dflag, 0, sizeof(int), st) == cudaSuccess;
    for (int f = 0; f < 8 && ok && np > 0; f++)
        ok = cudaMemcpyAsync(dst[f], cols.data() + (size_t)f * np, sizeof(double) * np, cudaMemcpyHostToDevice,
                             st) == cudaSuccess;
    ok = ok && (np == 0 ||
                cudaMemcpyAsync(s.id, ids.data(), sizeof(int) * np, cudaMemcpyHostToDevice, st) == cudaSuccess);
    const long long nb = plan.n_all - np;
    if (ok && nb > 0) {
        ok = cudaMemcpyAsync(dseg, plan.seg.data(), sizeof(ddx_host::SetupSegment) * nseg, cudaMemcpyHostToDevice,
                             st) == cudaSuccess &&
             (nmass == 0 || cudaMemcpyAsync(dmass, plan.mass.data(), sizeof(double) * nmass, cudaMemcpyHostToDevice,
                                            st) == cudaSuccess) &&
             cudaMemcpyAsync(ddisk, dk.data(), sizeof(DiskDev) * dk.size(), cudaMemcpyHostToDevice, st) ==
                 cudaSuccess &&
             cudaMemcpyAsync(dblob, bl.data(), sizeof(BlobDev) * bl.size(), cudaMemcpyHostToDevice, st) == cudaSuccess;
        if (ok) {
            setup_kernel<<<(unsigned)((nb + 255) / 256), 256, 0, st>>>(dseg, (int)nseg, dmass, ddisk, dblob,
                                                                        p->planets[0].m, np, plan.n_all,
                                                                        (uint32_t)seed, (uint32_t)(seed >> 32), s,
                                                                        dflag);
            ok = cudaGetLastError() == cudaSuccess;
        }
    }
    ok = ok && cudaMemcpyAsync(&flag, dflag, sizeof(int), cudaMemcpyDeviceToHost, st) == cudaSuccess &&
         cudaStreamSynchronize(st) == cudaSuccess;
    cudaFree(arena);
    if (!ok) {
        cudaGetLastError();
        return DDX_ERR_CUDA;
    }
    run->n_mass = (int)plan.n_mass;
    run->n_dust = (int)plan.n_dust;
    run->n_all = (int)plan.n_all;
    return flag ? DDX_ERR_RANGE : DDX_OK;
}

}  // namespace ddx
