/* DiskDyn GB300 path -- a whole run: Grid::evolve's loop with its output cadence.
 *
 * ddx_run steps the system from cad->time to cad->t_end with the reference's step-size
 * clipping and output triggers (src/grid.cu:344-437) and hands every output to a host
 * callback.  The steps are launched back to back without a host round trip; each image set
 * and SED is computed on the device for all its wavelengths in one call (the reference makes
 * one launch sequence and one synchronisation per wavelength) and copied to pinned host
 * memory on a second stream while the next steps run; a data dump snapshots the state in
 * device memory and copies the snapshot the same way.
 */
#ifndef DISKDYN_GB300_RUN_H
#define DISKDYN_GB300_RUN_H

#include "diskdyn_gb300_io.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Output intervals and the run clock, yr (cconfig's t_write, t_fits, t_sed, t_end and the
 * Grid members time, tlastd, tlastf, tlasts).  ddx_run updates the clock fields. */
typedef struct {
    double t_write, t_fits, t_sed, t_end;
    double time, tlastd, tlastf, tlasts;
    double model_dt;        /* the dt a data file records: the reference's Grid::dt member,
                               0 for a new run and the file's value after a restart (its
                               evolve loop steps with a local dt and never updates it) */
    int initial_outputs;    /* 1: images, SED and data file before the first step, as the
                               reference does for a run from a parameter file */
} ddx_cadence;

#define DDX_OUT_IMAGES 1    /* data: nwavs images of xsize*ysize pixels, x-major (ddx_image) */
#define DDX_OUT_SED    2    /* data: n_wav fluxes (ddx_sed) */
#define DDX_OUT_STATE  3    /* state: every body (the data file's content) */

/* One output.  The pointers are host memory that stays valid until the callback returns. */
typedef struct {
    int kind;                          /* DDX_OUT_* */
    double time;                       /* run time of the output, yr */
    double model_dt, tlastd, tlastf, tlasts;   /* the data file's run values at this output */
    const double *data;                /* images or SED */
    long long n;                       /* doubles in data */
    const ddx_host_state *state;       /* DDX_OUT_STATE: n_grav + n_dust bodies */
} ddx_output;

/* Called on the host thread of ddx_run, in the reference's output order (per step: SED,
 * images, data file).  A non-zero return stops the run after the outputs already queued. */
typedef int (*ddx_output_fn)(void *user, const ddx_output *out);

/* Grid::evolve from cad->time to cad->t_end: fixed steps of dt (ddx_det_step's value), each
 * shortened so that it ends exactly on the next output time or on t_end; after a step, the
 * SED when time >= tlasts + t_sed, the images of wj[nwavs] when time >= tlastf + t_fits,
 * the state when time >= tlastd + t_write (each also at t_end), with the step size reset to
 * dt after an output, all in the reference's FP64 arithmetic.  Each step is ddx_step with
 * `precision` and `mode`; outputs use the same precision (and mode for the SED).  The size
 * table and optics must be set.  Returns the first non-zero status of a step or output call,
 * DDX_ERR_TIMEOUT if a bounded device wait gave up, or DDX_OK; cad holds the clock reached.
 * Synchronises `stream` before it returns. */
int ddx_run(ddx_ctx *ctx, const ddx_state *s, int n_grav, int n_dust, double dt, const ddx_phys *phys,
            int precision, int mode, const ddx_view *view, const int *wj, int nwavs, ddx_cadence *cad,
            ddx_output_fn fn, void *user, void *stream);

/* One ddx_step of a system held in host memory: in (host, n_grav + n_dust bodies) is copied
 * to the device state s, stepped, and the updated positions, velocities and grain numbers
 * come back into out (m and id are not changed by a step and are not copied back).  The
 * massive bodies go first; the dust's copy in runs on its own stream, overlapping the massive
 * set's work.  The dust then goes through in up to three chunks (one wave of the dust
 * kernel, the bulk, one wave), the copy in of chunk k+1 and the copy out of chunk k-1 on their
 * own streams overlapping chunk k's compute.  The reference mode, the mixed step with 1,024
 * planetesimals or more (whose spatial order works best over all the grains at once), and
 * fewer than four waves of grains run the dust in one chunk.  Overlap needs page-locked host memory.
 * in and out may be the same arrays.  Synchronises `stream`. */
int ddx_step_host(ddx_ctx *ctx, const ddx_host_state *in, ddx_host_state *out, const ddx_state *s, int n_grav,
                  int n_dust, double dt, const ddx_phys *phys, int precision, int mode, void *stream);

/* The steps and outputs ddx_run makes for this cadence and dt, on the host without a GPU:
 * step_dt[k] is step k's size and outputs[k] the outputs due after it, a mask of
 * 1 << DDX_OUT_SED, 1 << DDX_OUT_IMAGES and 1 << DDX_OUT_STATE (the images are skipped by
 * ddx_run when nwavs = 0).  *n_steps = the number of steps; with cap = 0 only the count is
 * returned, and DDX_ERR_RANGE when a non-zero cap is too small. */
int ddx_schedule(const ddx_cadence *cad, double dt, long long cap, double *step_dt, int *outputs,
                 long long *n_steps);

#ifdef __cplusplus
}
#endif

#endif /* DISKDYN_GB300_RUN_H */
