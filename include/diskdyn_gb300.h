/*
 * diskdyn_gb300.h -- C ABI of the GB300 (sm_103a) DiskDyn dynamical and imaging path.
 *
 * The library replaces the per-step kernel launches and the flux kernels that the
 * reference's `class Grid` issues.  Every entry point takes plain device pointers and
 * sizes, is stream-ordered on a caller-supplied CUDA stream (passed as `void*`; NULL is
 * the legacy default stream, which is what the reference uses), and returns an int status
 * (DDX_OK == 0) instead of calling exit().  A context is not re-entrant: calls that share
 * one context must not overlap in host threads.
 *
 * State layout is the reference's: one SoA array per field, n_all = n_grav + n_dust
 * entries, massive bodies first with the star at index 0, then the dust tracers
 * (src/grid.cu:104-189 of the reference).  Units are AU, yr and mass*4*pi^2 in Msun,
 * so an acceleration is m/r^2 (src/ddyn.cuh:17-38, src/read_in.cu:76).
 */
#ifndef DISKDYN_GB300_H
#define DISKDYN_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define DDX_ABI_VERSION 4

/* Status codes.  The reference exits the process instead (src/error.cu:75-91,
 * src/ddyn.cuh:400-408). */
#define DDX_OK              0
#define DDX_ERR_ARG         1   /* null pointer, negative count, unknown enum value */
#define DDX_ERR_CUDA        2   /* a CUDA runtime call or kernel launch failed */
#define DDX_ERR_NOMEM       3   /* device allocation failed */
#define DDX_ERR_STATE       4   /* a table needed by the call was never set */
#define DDX_ERR_RANGE       5   /* a size is beyond a documented limit */
#define DDX_ERR_TIMEOUT     6   /* a bounded device-side wait gave up */
#define DDX_ERR_NONFINITE   7   /* NaN/Inf found where a finite value is required */
#define DDX_ERR_IO          8   /* a file could not be opened, read or written */

/* Arithmetic of the force stage. */
#define DDX_PREC_FP64   0   /* every operation in FP64, like the reference */
#define DDX_PREC_MIXED  1   /* FP64 state, Kepler term and stage combination; FP32
                               body-body perturbations with compensated sums, except
                               for sources within the near radius (ddx_set_near_radius),
                               which take the FP64 pair force */

#define DDX_PREC_COMPENSATED 2 /* FP64 state, Kepler term, stage combination, planets and
                               massive-set gravity; the planetesimals' pull on each tracer
                               in float-float (pairs of FP32 numbers carried through
                               error-free transformations, about 44 bits) for every span of
                               planetesimals nearer than ddx_set_compensated_radius, in FP32
                               beyond, in FP64 within the near radius.  For runs that need
                               errors near FP64's at several times FP64's throughput;
                               ddx_step and its variants only */

/* Behaviour switch for the reference's known defects. */
#define DDX_MODE_FIXED      0   /* defects corrected (default) */
#define DDX_MODE_REFERENCE  1   /* defects reproduced where they are deterministic */

/* Maximum number of size bins; the reference keeps them in __constant__ arrays of
 * this length (src/ddyn.cuh:33 `nsize`, src/ddyn.cu:29-32). */
#define DDX_MAX_SIZE_BINS 2700
/* Radial grid of the dust-temperature table (src/ddyn.cuh:32 `nR`). */
#define DDX_NR 100

/* Device pointers to the particle state.  Replaces the state half of
 * `struct coord` (src/ddyn.cuh:44-58); the 32 RK4 scratch arrays of that struct are
 * not part of the interface, the context owns its own scratch. */
typedef struct {
    double *x, *y, *z;      /* AU */
    double *vx, *vy, *vz;   /* AU/yr */
    double *m;              /* mass * 4 pi^2, Msun */
    double *N;              /* grains per tracer; 0 marks a removed tracer */
    int    *id;             /* size-bin index, -1 = no optical data */
} ddx_state;

/* Physics switches and stellar constants, in the units the reference passes to
 * RK4calc_dust (src/grid.cu:737, src/read_in.cu:591-603). */
typedef struct {
    int    radQ, SWQ, FLQ;  /* radiation pressure / stellar-wind drag / Lorentz force */
    double Wz;              /* stellar rotation rate, 1/yr */
    double Bstar;           /* surface field, Msun/yr^2/A */
    double Rstar;           /* AU */
    double rho;             /* bulk density, kg/m^3 (unused by the force; kept for parity) */
    double vsw_AUyr;        /* stellar-wind speed, AU/yr */
    double Rmin;            /* sublimation radius, AU */
    int    n_planets;       /* star + planets, the leading massive bodies (cconfig.n_planets:
                               the star is planet 0, src/read_in.cu:62-65,94).
                               DDX_PREC_MIXED computes the gravity of bodies
                               0..n_planets-1 in FP64 and only that of the planetesimals
                               n_planets..n_grav-1 in FP32.  0 <= n_planets <= n_grav;
                               0 counts as 1 (the star alone). */
} ddx_phys;

/* Observer geometry, in the units the reference passes to calc_flux_driver
 * (src/grid.cu:51-52, src/read_in.cu:608-624). */
typedef struct {
    double dist;            /* distance, m */
    double fov;             /* field of view, AU */
    double PA, inc, longitude;  /* radians */
    int    xsize, ysize;    /* pixels */
} ddx_view;

typedef struct ddx_ctx ddx_ctx;

/* Create a context on `device`.  Replaces the buffer ownership of Grid::allocgpu
 * (src/init.cu:543-602); scratch grows on demand.  Every entry point makes its device (the
 * context's, or the `device` argument) current while it runs and makes the caller's
 * current device current again before it returns. */
int ddx_create(ddx_ctx **out, int device);
int ddx_destroy(ddx_ctx *ctx);

/* Per-size-bin table: grain size [m], beta, beta_sw, charge q.  Host pointers, n_grid
 * entries, n_grid <= DDX_MAX_SIZE_BINS.  Replaces the __constant__ fill of
 * Grid::sync_dust_to_gpu (src/init.cu:649-660). */
int ddx_set_size_table(ddx_ctx *ctx, int n_grid, const double *size, const float *beta,
                       const float *betasw, const float *q);

/* Optical tables, host pointers, copied to the device.  Layouts as in the reference
 * (src/read_in.cu:450-498, src/grid.cu:793-825):
 *   w[n_wav] (m), in[n_wav] (stellar flux at the observer), Qabs/Qsca[n_grid][n_wav],
 *   Qpfunc[n_grid][n_theta][n_wav], Td[n_grid][DDX_NR] (K) on the log-R grid
 *   [Rmin, Rmax] (AU).  Replaces the table half of Grid::sync_dust_to_gpu
 *   (src/init.cu:642-647). */
int ddx_set_optics(ddx_ctx *ctx, int n_grid, int n_wav, int n_theta, const double *w,
                   const double *in, const double *Qabs, const double *Qsca,
                   const double *Qpfunc, const double *Td, double Rmin, double Rmax);

/* One fixed-dt RK4 step of the whole system: massive all-pairs gravity, then every
 * dust tracer under stellar gravity reduced by beta, PR and stellar-wind drag, the
 * optional Lorentz force and the gravity of every massive body, then the massive
 * combination.  Equivalent to the reference's
 *     massive_RK4(dt); small_RK4(dt); massive_final(dt);   (src/grid.cu:387-389)
 * The size table must be set.  `precision` is DDX_PREC_*, `mode` is DDX_MODE_*.
 * DDX_PREC_MIXED with 1,024 planetesimals or more visits the tracers and reads the FP32
 * planetesimals in a spatial order (Hilbert cells) and takes spans of 32 planetesimals that
 * lie at least a quarter of the largest |coordinate| of the two away from a tracer with the
 * FP32 high parts alone.
 * Each tracer's result depends on its own data and the massive set only (not on the
 * other tracers or their order), and the result is the same from run to run. */
int ddx_step(ddx_ctx *ctx, const ddx_state *s, int n_grav, int n_dust, double dt,
             const ddx_phys *phys, int precision, int mode, void *stream);

/* The same step split at the reference's three call sites, for a caller that keeps
 * them apart (src/grid.cu:387-389):
 *   ddx_massive_rk4   <- Grid::massive_RK4  : stage positions P1..P4 of the massive set
 *                                             (accelerations A1, A2 evaluated);
 *   ddx_small_rk4     <- Grid::small_RK4    : full RK4 of every dust tracer against them;
 *   ddx_massive_final <- Grid::massive_final: A3, A4 and the RK4 combination of the
 *                                             massive set.
 * They must be called in this order, on one stream, with the same state, sizes, dt,
 * physics, precision and mode; the stage positions live in the context in between. */
int ddx_massive_rk4(ddx_ctx *ctx, const ddx_state *s, int n_grav, int n_dust, double dt,
                    const ddx_phys *phys, int precision, int mode, void *stream);
int ddx_small_rk4(ddx_ctx *ctx, const ddx_state *s, int n_grav, int n_dust, double dt,
                  const ddx_phys *phys, int precision, int mode, void *stream);
int ddx_massive_final(ddx_ctx *ctx, const ddx_state *s, int n_grav, int n_dust, double dt,
                      const ddx_phys *phys, int precision, int mode, void *stream);

/* n_steps calls of ddx_step with the same dt, with the launches of all steps enqueued
 * back to back (no host synchronisation in between). */
int ddx_evolve(ddx_ctx *ctx, const ddx_state *s, int n_grav, int n_dust, double dt,
               int n_steps, const ddx_phys *phys, int precision, int mode, void *stream);

/* ddx_step without any device allocation.  No counterpart in the reference.
 *
 * Some callers cannot call cudaMalloc, for example a host inside a framework whose pool
 * allocator owns all device memory, or a loop that must keep a fixed device footprint.
 * This entry point needs no context.  Its scratch is one file-scope __device__ array of
 * fixed size (about 12 MiB), which every GPU that loads the library holds until the
 * process exits.  It takes at most DDX_NOALLOC_MAX_GRAV massive bodies and
 * DDX_MAX_SIZE_BINS size bins and answers DDX_ERR_RANGE beyond that.  beta, betasw and q
 * are device pointers with n_grid entries; everything else is as for ddx_step.  In FP64
 * the results equal ddx_step's to the bit.  In DDX_PREC_MIXED the spatial order needs
 * scratch that grows with n_dust, so this entry point reads the planetesimals in index
 * order and always with the full hi/lo separation: its results agree with ddx_step's to
 * the rounding of the FP32 perturbations.
 *
 * The first call on a device resolves the array's device address (cudaGetSymbolAddress
 * with that device current) and clears its status word (a synchronous one-word memset).
 * Make that first call before any stream capture.  All calls share the one array, so
 * calls that overlap on the GPU (different streams, different host threads) race;
 * serialise them.  Each call writes every scratch word it reads, so no result carries over
 * from the previous call, with one exception: the status word, in which a mixed-precision
 * dust block that gave up a bounded wait (its tracers left unchanged) sets a bit.  That
 * word collects these reports over calls until ddx_noalloc_sync_status reads and clears it.
 * A call returns before its kernels finish, so it cannot report them itself.
 * On a GPU with more than 160 SMs the mixed massive passes take their one-warp-per-target
 * form here (the same sums, slower), because the fixed array holds the slice sums for 160. */
#define DDX_NOALLOC_MAX_GRAV 8192
int ddx_step_noalloc(int device, const ddx_state *s, int n_grav, int n_dust, double dt,
                     const ddx_phys *phys, int n_grid, const float *beta, const float *betasw,
                     const float *q, int precision, int mode, void *stream);

/* Synchronises `stream` on `device` and reports whether a kernel of ddx_step_noalloc on that
 * device gave up a bounded wait since the last call of this function: DDX_ERR_TIMEOUT if so
 * (the tracers of the blocks concerned were left unchanged), DDX_OK otherwise.  Clears the
 * report.  Allocates nothing: one 4-byte copy to a host variable.  No counterpart in the
 * reference, whose kernels have no waits. */
int ddx_noalloc_sync_status(int device, void *stream);

/* Failure-detection test hook of ddx_step_noalloc (no counterpart in the reference): the
 * next mixed-precision call on `device` leaves the TMA copy of source tile `tile` unissued
 * and bounds its waits by wait_ns, as ddx_debug_lose_tile_copy does for a context.  Nothing
 * faults or hangs. */
int ddx_debug_noalloc_lose_tile_copy(int device, int tile, unsigned long long wait_ns);

/* Images at the table wavelengths wj[0..n_img-1]: scattered + thermal flux of every
 * dust tracer with id >= 0, projected through `view` and summed into
 * Fd[img][xsize*ysize] (device pointer), pixel (x, y) at Fd[img*npix + ysize*x + y]
 * (x-major, like the reference).  Fd is overwritten.  Pixel indices are bit-identical
 * to the reference's calc_flux_driver on the same GPU.  Replaces
 *     null_flux(); calc_flux(wj);   per image wavelength (src/grid.cu:411-421). */
int ddx_image(ddx_ctx *ctx, const ddx_state *s, int n_grav, int n_dust,
              const ddx_view *view, const int *wj, int n_img, double *Fd, int precision,
              void *stream);

/* SED: total flux of all dust tracers at every table wavelength, Fsed[n_wav] (device
 * pointer), overwritten.  Replaces the per-wavelength loop
 *     null_flux_part(); calc_flux_sed(j); copy_sed(j);   (src/grid.cu:396-406)
 * mode DDX_MODE_REFERENCE keeps the reference's rotation by the spherical radius
 * (src/gpu_functions.cu:1106-1107); DDX_MODE_FIXED rotates by the cylindrical one. */
int ddx_sed(ddx_ctx *ctx, const ddx_state *s, int n_grav, int n_dust,
            const ddx_view *view, double *Fsed, int precision, int mode, void *stream);

/* Collision candidates through a spatial-hash grid built by a one-pass radix (counting)
 * sort on the hashed cell ids (no counterpart in the reference, which has no collision
 * detection).  Two live tracers (N != 0)
 * i < j of the state range [i0, i1) collide when
 *     (xj-xi)^2 + (yj-yi)^2 + (zj-zi)^2 < h^2     (FP64, every operation rounded alone),
 * which makes the list identical to a brute-force test with that expression.  Writes up
 * to `cap` pairs (i, j) as int pairs[2k], pairs[2k+1] (device pointer), ordered by i then
 * j, and the total number found to *n_pairs (host); when *n_pairs > cap the call can be
 * repeated with a larger buffer.  Synchronises `stream`.  At most 2^30 tracers. */
int ddx_collide(ddx_ctx *ctx, const ddx_state *s, int i0, int i1, double h, int *pairs,
                long long cap, long long *n_pairs, void *stream);

/* Time step of a run; replaces Grid::det_step (src/grid.cu:312-342), called once at the
 * start of Grid::evolve (src/grid.cu:349).  With n_step steps per orbit:
 *   dt = min( 2 pi sqrt(pow(|x_i - x_0|^2, 3/2) / (m_0 + m_i)) / n_step, i = 1..n_grav-1,
 *             2 pi sqrt(disk_Rin[k] / m_0) / n_step,
 *             2 pi sqrt((blob_a[k] (1 - blob_ecc[k]) - blob_sigma[k]) / m_0) / n_step )
 * and 1e137 when there is no term, the reference's expressions and rounding to the bit
 * (the disk and blob terms take sqrt(R / m_0), not R^(3/2), as the reference does).  The
 * body scan runs on the GPU over the device state; the disk and blob arrays are host
 * pointers (configuration data) and *dt is written on the host.  Synchronises `stream`. */
int ddx_det_step(ddx_ctx *ctx, const ddx_state *s, int n_grav, int n_step, const double *disk_Rin,
                 int n_disks, const double *blob_a, const double *blob_ecc, const double *blob_sigma,
                 int n_blobs, double *dt, void *stream);

/* Dust-temperature table; replaces Grid::calculate_dust_temp (src/grid.cu:754-834), which
 * the reference runs on the host before the first step.  In: the optical tables w[n_wav]
 * (m), in[n_wav], Qabs[n_grid][n_wav] and dist (m), host pointers, and *Rmax_AU = the
 * largest configured radius (disks' Rout, blobs' a(1+e)+sigma, planets' distances; the
 * reference's loop at src/grid.cu:759-765).  Out: Td[n_grid][DDX_NR] (host), the grain
 * temperature on the log-radius grid from *Rmin_AU (the smallest sublimation radius at
 * 2000 K) to *Rmax_AU (twice the input, as the reference sets it).  The Planck integrals run
 * on the GPU, one thread per (bin, temperature).  Synchronises `stream`. */
int ddx_dust_temp(ddx_ctx *ctx, int n_grid, int n_wav, const double *w, const double *in,
                  const double *Qabs, double dist, double *Rmin_AU, double *Rmax_AU, double *Td,
                  void *stream);

/* Optical tables of one grain composition on n_size grain radii, host pointers: the
 * reference's cfg->s, Qabs, Qsca and Qpfunc (src/ddyn.cuh), as read from the Mie table
 * file (ddx_optical_read) or resampled onto the mass grid (ddx_dust_grid). */
typedef struct {
    int n_size, n_wav, n_theta;
    double *s;          /* [n_size] grain radius, m, increasing */
    double *Qabs;       /* [n_size][n_wav] */
    double *Qsca;       /* [n_size][n_wav] */
    double *Qpfunc;     /* [n_size][n_theta][n_wav], n_theta angles uniform in cos(theta) */
} ddx_optical_table;

/* Inputs of the mass grid and of the radiation-pressure and wind-drag tables, in the
 * reference's units (cconfig, src/ddyn.cuh). */
typedef struct {
    int n_grid;                 /* size bins (detminmax, src/read_in.cu:339) */
    double amin, amax;          /* smallest and largest grain radius of the grid, m */
    double dmax;                /* largest radius of the optical table file, m */
    double kqe;                 /* q = kqe * a * 1e9 per bin */
    int radQ, SWQ;              /* radiation pressure and stellar-wind drag on (1) or off */
    double rho;                 /* grain density, kg/m^3 */
    double dist;                /* distance, m */
    double mstar;               /* star mass * 4 pi^2 (Msun): cfg->planets[0].m */
    double mloss;               /* stellar mass-loss rate as the parameter file gives it */
    double vsw;                 /* stellar-wind speed, m/s */
} ddx_grid_setup;

/* Size grid and per-bin tables; replaces interpolate_dust_to_grid and calculate_beta
 * (src/functions.cu:243-300, 338-388), called from Grid::setup (src/grid.cu:74-76).
 * In (host): the table file's optics `file` on w[n_wav] (m), the stellar flux in[n_wav] of
 * ddx_stellar_grid and the grid set-up g.  Out (host, caller-allocated): `grid` with
 * n_size = g->n_grid (s = the bin radii a_i = amin exp(i ln(amax/amin)/(n_grid-1)), the
 * tables interpolated log-log between the two file sizes around a_i), q[n_grid],
 * beta[n_grid], betasw[n_grid], *Lum (Lsun) and *betaswconst.  The bin radii, q, betasw, Lum
 * and the size brackets are computed on the host with the reference's expressions and
 * rounding; the table interpolation and the phase-function integrals for beta run on the
 * GPU, with the reference's operation order (no contractions), so they differ from it
 * only by the CUDA math library's log and exp.  A bin at or below s[0] is interpolated on
 * the first file interval and one beyond the last size on the last interval (the reference
 * reads outside its table there).  Returns DDX_ERR_RANGE when the last bin overshoots dmax
 * by more than 1e-12 (the reference's exit code 54) or n_grid > DDX_MAX_SIZE_BINS.
 * Synchronises `stream`. */
int ddx_dust_grid(ddx_ctx *ctx, int n_wav, const double *w, const double *in,
                  const ddx_optical_table *file, const ddx_grid_setup *g, ddx_optical_table *grid,
                  float *q, float *beta, float *betasw, double *Lum, double *betaswconst,
                  void *stream);

/* Discrete adjoint of the trajectory and image (no counterpart in the reference).
 *
 * ddx_adjoint_forward integrates the initial state `s` (read only) for n_steps fixed-dt
 * RK4 steps in FP64 -- the massive set (at most DDX_ADJ_MAX_GRAV bodies: star, planets and
 * gravitating planetesimals, all-pairs) and the dust tracers under the physics of ddx_step
 * (radiation pressure, PR and stellar-wind drag, the Lorentz force when phys->FLQ is 1, with
 * the tracers' masses from s->m, a massless tracer feeling none; the gravity of every massive
 * body) -- keeping the massive set's stage positions of every step and a checkpoint of the
 * tracer state every ckpt_every steps in the context.  It
 * then writes image[n_img][xsize*ysize] (device): the flux of ddx_image deposited with
 * bilinear weights on the four pixel centres around each tracer's projected position
 * (pixel (x, y) centred at psca*(x + 1/2 - xsize/2)), which is continuous in the
 * positions, unlike the nearest-pixel binning of ddx_image.
 *
 * ddx_adjoint_backward takes dL/dimage (device, the layout of image) for any scalar L
 * and writes dL/d(initial state) to grad_state[6][n_grav + n_dust] (rows x, y, z, vx, vy,
 * vz; device) and dL/d(mass*4pi^2) of the massive bodies to grad_mass[n_grav] (device),
 * by checkpoint-and-recompute: every segment is recomputed from its checkpoint and swept
 * backwards through the RK4 stages.  One backward per forward. */
#define DDX_ADJ_MAX_GRAV 131072
int ddx_adjoint_forward(ddx_ctx *ctx, const ddx_state *s, int n_grav, int n_dust, double dt,
                        int n_steps, int ckpt_every, const ddx_phys *phys, const ddx_view *view,
                        const int *wj, int n_img, double *image, void *stream);
int ddx_adjoint_backward(ddx_ctx *ctx, const double *dL_dimage, double *grad_state,
                         double *grad_mass, void *stream);

/* Diagnostics (no reference counterpart).  ddx_debug_pixels writes, for every dust
 * tracer, the pixel index ysize*x + y that ddx_image uses (or -1 for a tracer without
 * optical data or outside the image) to pix[n_dust], and 1/0 to exact[n_dust] when the
 * reference's own expression sequence decided it (tracers within the guard band of a
 * pixel edge).  Both device pointers.  ddx_debug_exact_pixel_count returns how many
 * tracers took that exact path in ddx_image calls on this context. */
int ddx_debug_pixels(ddx_ctx *ctx, const ddx_state *s, int n_grav, int n_dust,
                     const ddx_view *view, int *pix, int *exact);
unsigned long long ddx_debug_exact_pixel_count(ddx_ctx *ctx);

/* Throughput probe (no reference counterpart): chains of independent FMAs on every SM of
 * `device`, timed with CUDA events.  Writes the measured FP32 and FP64 FMA rates in
 * TFLOP/s (2 flops per FMA); used as the compute-pipe roofline denominators. */
int ddx_probe_fma_peak(int device, double *fp32_tflops, double *fp64_tflops);

/* Synchronises `stream` and reports whether a kernel of this context gave up a bounded
 * device-side wait since the last call: DDX_ERR_TIMEOUT if so (the tracers of the
 * blocks concerned were left unchanged), DDX_OK otherwise.  Clears the report.  No
 * counterpart in the reference, whose kernels have no waits. */
int ddx_sync_status(ddx_ctx *ctx, void *stream);

/* Near radius of DDX_PREC_MIXED (no counterpart in the reference, which is FP64 throughout).
 * FP32 leaves about 5.6e-7 of relative error in each planetesimal pull, and a close
 * encounter amplifies it along the trajectory.  So in the mixed step a planetesimal nearer
 * to a body (tracer or massive) than eta times that body's largest |coordinate| at the RK4
 * stage takes the FP64 pair force from the FP64 stage positions, as in DDX_PREC_FP64;
 * every other planetesimal stays FP32.  The test uses the FP32 distance, so the choice is
 * deterministic.  DDX_PREC_COMPENSATED applies the same rule inside its float-float spans.
 * Defaults: 4e-3 for DDX_PREC_MIXED (0.52 AU at 130 AU) and 1.6e-2 for
 * DDX_PREC_COMPENSATED; a value set here applies to both, a negative one restores the
 * defaults; 0 turns the FP64 pulls off; eta <= 0.25 and not NaN, else DDX_ERR_ARG.  Applies
 * to later steps of this context; ddx_step_noalloc always uses the defaults. */
int ddx_set_near_radius(ddx_ctx *ctx, double eta);

/* Radius of the float-float spans of DDX_PREC_COMPENSATED (no counterpart in the
 * reference).  A span of 32 planetesimals whose box lies nearer to a tracer than eta times
 * the tracer's largest |coordinate| at the RK4 stage takes the float-float pull; farther
 * spans take the FP32 forms of DDX_PREC_MIXED.  Default 0.5; +infinity makes every span
 * float-float; eta >= 0, else DDX_ERR_ARG.  ddx_step_noalloc uses the default. */
int ddx_set_compensated_radius(ddx_ctx *ctx, double eta);

/* Failure-detection test hook (no counterpart in the reference).  The next mixed-precision
 * dust launch of this context leaves the TMA copy of source tile `tile` (counted over the
 * four stages) unissued and bounds its waits by wait_ns instead of 2 s, so the blocks
 * give up, report DDX_ERR_TIMEOUT through ddx_sync_status and leave their tracers
 * unchanged.  Nothing faults or hangs; the context stays usable. */
int ddx_debug_lose_tile_copy(ddx_ctx *ctx, int tile, unsigned long long wait_ns);

/* Error string for a status code. */
const char *ddx_status_string(int status);

/* ABI version of the loaded library (DDX_ABI_VERSION). */
int ddx_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* DISKDYN_GB300_H */
