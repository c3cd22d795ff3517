// Grid::evolve's clock on the host (src/grid.cu:344-437): the step size and the output
// triggers, in the reference's FP64 arithmetic and order, shared by ddx_run and
// ddx_schedule (which lists what a run will do, without a GPU).
#include "../../include/diskdyn_gb300.h"
#include "../../include/diskdyn_gb300_run.h"
#include "ddx_host.h"

namespace ddx_host {

namespace {

// dttmp cut so that the step ends on the next data, image or SED output time or on t_end
// (src/grid.cu:375-378, 431-434)
void clip(double time, const ddx_cadence& c, double& dttmp) {
    if (time + dttmp > c.tlastd + c.t_write) dttmp = c.t_write + c.tlastd - time;
    if (time + dttmp > c.tlastf + c.t_fits) dttmp = c.t_fits + c.tlastf - time;
    if (time + dttmp > c.tlasts + c.t_sed) dttmp = c.t_sed + c.tlasts - time;
    if (time + dttmp > c.t_end) dttmp = c.t_end - time;
}

}  // namespace

void Clock::start(const ddx_cadence& cad, double dt_) {
    c = cad;
    dt = dt_;
    time = cad.time;
    dttmp = dt;
    clip(time, c, dttmp);
}

int Clock::advance() {
    int mask = 0;
    time += dttmp;
    if (time >= c.tlasts + c.t_sed || time >= c.t_end) {
        mask |= 1 << DDX_OUT_SED;
        c.tlasts = time;
        dttmp = dt;
    }
    if (time >= c.tlastf + c.t_fits || time >= c.t_end) {
        mask |= 1 << DDX_OUT_IMAGES;
        c.tlastf = time;
        dttmp = dt;
    }
    if (time >= c.tlastd + c.t_write || time >= c.t_end) {
        mask |= 1 << DDX_OUT_STATE;
        c.tlastd = time;
        dttmp = dt;
    }
    clip(time, c, dttmp);
    c.time = time;
    return mask;
}

}  // namespace ddx_host

extern "C" int ddx_schedule(const ddx_cadence* cad, double dt, long long cap, double* step_dt, int* outputs,
                            long long* n_steps) {
    if (!cad || !n_steps || cap < 0 || (cap > 0 && (!step_dt || !outputs))) return DDX_ERR_ARG;
    if (!(dt > 0.0) || !(cad->t_write > 0.0) || !(cad->t_fits > 0.0) || !(cad->t_sed > 0.0)) return DDX_ERR_ARG;
    ddx_host::Clock clk;
    clk.start(*cad, dt);
    long long n = 0;
    while (clk.running()) {
        const double h = clk.dttmp;
        const int mask = clk.advance();
        if (n < cap) {
            step_dt[n] = h;
            outputs[n] = mask;
        }
        n++;
        if (n > (1LL << 40)) return DDX_ERR_RANGE;
    }
    *n_steps = n;
    return n > cap && cap > 0 ? DDX_ERR_RANGE : DDX_OK;
}
