// A whole run: Grid::evolve (src/grid.cu:344-437) with its output cadence.
//
// The clock, the step-size clipping and the output triggers are the reference's host
// arithmetic, unchanged (ddx_host::Clock, ddx_clock.cpp), so the output times are the
// reference's to the bit.  What changes is the traffic around them:
//  - the steps go to the stream back to back; the host never waits for a step;
//  - an output is computed on the device for all its wavelengths at once (ddx_image,
//    ddx_sed) into a device slot, then copied to a pinned host slot on a copy stream that
//    waits for it, so the next steps overlap the copy; a data dump first snapshots the
//    state with device-to-device copies;
//  - the host hands a finished output to the callback as soon as its copy has landed
//    (polled between launches), in the order the outputs were queued.
// Two slots per output kind let one output be in flight while the callback consumes the
// previous one; the state has one snapshot slot.
#include <deque>
#include <vector>

#include "../../include/diskdyn_gb300_run.h"
#include "ddx_host.h"
#include "ddx_internal.cuh"

namespace {

struct Slot {
    double* dev = nullptr;
    double* host = nullptr;
    bool busy = false;
};

struct Pending {
    int kind, slot;
    double time, model_dt, tlastd, tlastf, tlasts;
    cudaEvent_t done;
};

constexpr int kFields = 8;   // x y z vx vy vz N m, then id

class Runner {
  public:
    Runner(ddx_ctx* c, const ddx_state& s, int n_grav, int n_dust, int precision, int mode, const ddx_view& v,
           const int* wj, int nwavs, ddx_output_fn fn, void* user, cudaStream_t st)
        : c_(c), s_(s), ng_(n_grav), nd_(n_dust), prec_(precision), mode_(mode), v_(v), wj_(wj), nwavs_(nwavs),
          fn_(fn), user_(user), st_(st) {}

    ~Runner() { release(); }

    int init() {
        n_all_ = (size_t)ng_ + nd_;
        n_img_ = (size_t)nwavs_ * v_.xsize * v_.ysize;
        n_sed_ = (size_t)ddx::ctx_optics_n_wav(c_);
        if (cudaStreamCreateWithFlags(&cs_, cudaStreamNonBlocking) != cudaSuccess) return fail();
        for (int k = 0; k < 2; k++) {
            if (n_img_ && (cudaMalloc(&img_[k].dev, sizeof(double) * n_img_) != cudaSuccess ||
                           cudaMallocHost(&img_[k].host, sizeof(double) * n_img_) != cudaSuccess))
                return fail(DDX_ERR_NOMEM);
            if (cudaMalloc(&sed_[k].dev, sizeof(double) * (n_sed_ + 1)) != cudaSuccess ||
                cudaMallocHost(&sed_[k].host, sizeof(double) * (n_sed_ + 1)) != cudaSuccess)
                return fail(DDX_ERR_NOMEM);
        }
        const size_t sbytes = (sizeof(double) * kFields + sizeof(int)) * n_all_;
        if (cudaMalloc(&snap_dev_, sbytes) != cudaSuccess || cudaMallocHost(&snap_host_, sbytes) != cudaSuccess)
            return fail(DDX_ERR_NOMEM);
        return DDX_OK;
    }

    // Queues one output of `kind` with the clock values it records.
    int enqueue(int kind, double time, const ddx_cadence& cad) {
        Pending p{kind, 0, time, cad.model_dt, cad.tlastd, cad.tlastf, cad.tlasts, nullptr};
        int r = DDX_OK;
        if (kind == DDX_OUT_STATE) {
            while (snap_busy_ && r == DDX_OK) r = drain_one();
            if (r) return r;
            double* src[kFields] = {s_.x, s_.y, s_.z, s_.vx, s_.vy, s_.vz, s_.N, s_.m};
            char* d = reinterpret_cast<char*>(snap_dev_);
            for (int f = 0; f < kFields; f++)
                if (cudaMemcpyAsync(d + sizeof(double) * n_all_ * f, src[f], sizeof(double) * n_all_,
                                    cudaMemcpyDeviceToDevice, st_) != cudaSuccess)
                    return fail();
            if (cudaMemcpyAsync(d + sizeof(double) * n_all_ * kFields, s_.id, sizeof(int) * n_all_,
                                cudaMemcpyDeviceToDevice, st_) != cudaSuccess)
                return fail();
            snap_busy_ = true;
            r = copy_back(snap_host_, snap_dev_, (sizeof(double) * kFields + sizeof(int)) * n_all_, p);
        } else {
            Slot* slots = kind == DDX_OUT_IMAGES ? img_ : sed_;
            int k = next_[kind == DDX_OUT_IMAGES ? 0 : 1];
            while (slots[k].busy && r == DDX_OK) r = drain_one();
            if (r) return r;
            if (kind == DDX_OUT_IMAGES)
                r = ddx_image(c_, &s_, ng_, nd_, &v_, wj_, nwavs_, slots[k].dev, prec_, st_);
            else
                r = ddx_sed(c_, &s_, ng_, nd_, &v_, slots[k].dev, prec_, mode_, st_);
            if (r) return r;
            slots[k].busy = true;
            next_[kind == DDX_OUT_IMAGES ? 0 : 1] = 1 - k;
            p.slot = k;
            const size_t n = kind == DDX_OUT_IMAGES ? n_img_ : n_sed_;
            r = copy_back(slots[k].host, slots[k].dev, sizeof(double) * n, p);
        }
        return r;
    }

    // Hands finished outputs to the callback, oldest first; with `block`, waits for one.
    int drain(bool block) {
        int r = DDX_OK;
        while (!q_.empty() && r == DDX_OK) {
            if (!block) {
                const cudaError_t e = cudaEventQuery(q_.front().done);
                if (e == cudaErrorNotReady) break;
                if (e != cudaSuccess) return fail();
            }
            r = drain_one();
        }
        return r;
    }

    bool stopped() const { return stop_; }

  private:
    int copy_back(void* host, const void* dev, size_t bytes, Pending& p) {
        cudaEvent_t ready = nullptr;
        if (cudaEventCreateWithFlags(&ready, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventRecord(ready, st_) != cudaSuccess || cudaStreamWaitEvent(cs_, ready, 0) != cudaSuccess ||
            cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, cs_) != cudaSuccess ||
            cudaEventCreateWithFlags(&p.done, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventRecord(p.done, cs_) != cudaSuccess) {
            if (ready) cudaEventDestroy(ready);
            return fail();
        }
        cudaEventDestroy(ready);   // released once the copy stream has passed it
        q_.push_back(p);
        return DDX_OK;
    }

    int drain_one() {
        if (q_.empty()) return DDX_OK;
        Pending p = q_.front();
        q_.pop_front();
        if (cudaEventSynchronize(p.done) != cudaSuccess) {
            cudaEventDestroy(p.done);
            return fail();
        }
        cudaEventDestroy(p.done);
        ddx_output o{};
        o.kind = p.kind;
        o.time = p.time;
        o.model_dt = p.model_dt;
        o.tlastd = p.tlastd;
        o.tlastf = p.tlastf;
        o.tlasts = p.tlasts;
        ddx_host_state hs{};
        if (p.kind == DDX_OUT_STATE) {
            double* h = snap_host_;
            hs = ddx_host_state{h, h + n_all_, h + 2 * n_all_, h + 3 * n_all_, h + 4 * n_all_, h + 5 * n_all_,
                                h + 6 * n_all_, h + 7 * n_all_, reinterpret_cast<int*>(h + kFields * n_all_),
                                (long long)n_all_};
            o.state = &hs;
        } else {
            Slot& sl = (p.kind == DDX_OUT_IMAGES ? img_ : sed_)[p.slot];
            o.data = sl.host;
            o.n = (long long)(p.kind == DDX_OUT_IMAGES ? n_img_ : n_sed_);
        }
        const int stop = fn_ ? fn_(user_, &o) : 0;
        if (p.kind == DDX_OUT_STATE) snap_busy_ = false;
        else (p.kind == DDX_OUT_IMAGES ? img_ : sed_)[p.slot].busy = false;
        if (stop) stop_ = true;
        return DDX_OK;
    }

    int fail(int code = DDX_ERR_CUDA) {
        cudaGetLastError();
        return code;
    }

    void release() {
        while (!q_.empty()) {
            cudaEventSynchronize(q_.front().done);
            cudaEventDestroy(q_.front().done);
            q_.pop_front();
        }
        for (int k = 0; k < 2; k++) {
            cudaFree(img_[k].dev); cudaFreeHost(img_[k].host);
            cudaFree(sed_[k].dev); cudaFreeHost(sed_[k].host);
        }
        cudaFree(snap_dev_);
        cudaFreeHost(snap_host_);
        if (cs_) cudaStreamDestroy(cs_);
    }

    ddx_ctx* c_;
    ddx_state s_;
    int ng_, nd_, prec_, mode_;
    ddx_view v_;
    const int* wj_;
    int nwavs_;
    ddx_output_fn fn_;
    void* user_;
    cudaStream_t st_, cs_ = nullptr;
    size_t n_all_ = 0, n_img_ = 0, n_sed_ = 0;
    Slot img_[2], sed_[2];
    int next_[2] = {0, 0};
    double* snap_dev_ = nullptr;
    double* snap_host_ = nullptr;
    bool snap_busy_ = false, stop_ = false;
    std::deque<Pending> q_;
};

}  // namespace

extern "C" int ddx_run(ddx_ctx* ctx, const ddx_state* s, int n_grav, int n_dust, double dt, const ddx_phys* phys,
                       int precision, int mode, const ddx_view* view, const int* wj, int nwavs, ddx_cadence* cad,
                       ddx_output_fn fn, void* user, void* stream) {
    if (!ctx || !s || !phys || !view || !cad || n_grav < 1 || n_dust < 0 || nwavs < 0) return DDX_ERR_ARG;
    if (nwavs > 0 && !wj) return DDX_ERR_ARG;
    if (!(dt > 0.0) || !(cad->t_write > 0.0) || !(cad->t_fits > 0.0) || !(cad->t_sed > 0.0)) return DDX_ERR_ARG;
    if (ddx::ctx_optics_n_wav(ctx) == 0) return DDX_ERR_STATE;
    ddx::DeviceGuard dg(ddx::ctx_device(ctx));
    cudaStream_t st = (cudaStream_t)stream;
    Runner run(ctx, *s, n_grav, n_dust, precision, mode, *view, wj, nwavs, fn, user, st);
    int r = run.init();
    ddx_host::Clock clk;
    clk.start(*cad, dt);
    auto out = [&](int kind) { return r ? r : (r = run.enqueue(kind, clk.time, clk.c)); };
    if (r == DDX_OK && cad->initial_outputs) {
        if (nwavs > 0) out(DDX_OUT_IMAGES);
        out(DDX_OUT_SED);
        out(DDX_OUT_STATE);
    }
    while (r == DDX_OK && clk.running() && !run.stopped()) {
        r = ddx_step(ctx, s, n_grav, n_dust, clk.dttmp, phys, precision, mode, stream);
        if (r) break;
        const int due = clk.advance();
        if (due & (1 << DDX_OUT_SED)) out(DDX_OUT_SED);
        if ((due & (1 << DDX_OUT_IMAGES)) && nwavs > 0) out(DDX_OUT_IMAGES);
        if (due & (1 << DDX_OUT_STATE)) out(DDX_OUT_STATE);
        if (r == DDX_OK) r = run.drain(false);
    }
    const int r2 = run.drain(true);
    if (r == DDX_OK) r = r2;
    const int r3 = ddx_sync_status(ctx, stream);
    if (r == DDX_OK) r = r3;
    *cad = clk.c;
    return r;
}
