/* DiskDyn GB300 path -- host-side input and output in the reference's formats.
 *
 * These calls run on the host (no GPU, no context).  They read and write the files the
 * reference's driver reads and writes, so a run can start from the same parameter file
 * and produce the same outputs.
 */
#ifndef DISKDYN_GB300_IO_H
#define DISKDYN_GB300_IO_H

#include "diskdyn_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

#define DDX_PARAM_MAX_PLANETS 64   /* star + planets */
#define DDX_PARAM_MAX_DISKS   32
#define DDX_PARAM_MAX_BLOBS   32
#define DDX_PARAM_MAX_WAVS    16   /* the reference tokenises at most 16 values per line */
#define DDX_PARAM_STR         512

/* A massive body of the configuration: AU, AU/yr, mass * 4 pi^2 in Msun (planet_cart,
 * src/ddyn.cuh). */
typedef struct {
    double x, y, z, vx, vy, vz, m;
} ddx_planet;

/* A disk (diskconf, src/ddyn.cuh); units as the reference stores them: Rin, Rout in AU,
 * dhdr = atan(dh/dr), amax/amin/dmax in m, masses and Mtot in kg, eta = (eta_a + 2)/3. */
typedef struct {
    double Rin, Rout, dhdr, sigmae, amax, mmax, amin, mmin, dmax, dmmax, eta, gammas, C, Mtot;
    long long Ngrav, Nsmall;
} ddx_disk;

/* A blob (blobconf, src/ddyn.cuh); angles in radians, sizes in m, masses in kg. */
typedef struct {
    double a, ecc, inc, w, o, nu, sigma, amax, mmax, amin, mmin, dmax, dmmax, eta, C, Mtot, vkepp;
    long long Ngrav, Nsmall;
    int collcloud;                 /* 0: collision products, 1: cloud */
} ddx_blob;

/* The fields of the reference's configdata that its parameter file sets, in its units
 * (src/read_in.cu:508-733): distances in m (dist), AU (rstar), angles in radians,
 * wavelengths in m, wind speed in m/s, bulk density in kg/m^3, kqe per year. */
typedef struct {
    int verb, gpuid, gl;
    double t_gl, t_write, t_fits, t_sed, t_end;
    int n_step;
    char sptype[DDX_PARAM_STR];
    double teff, rstar, Bstar, Wz, mloss, vsw;
    double dist, fov, PA, inc, longitude;
    int xsize, ysize;
    int nwavs;
    double wavs[DDX_PARAM_MAX_WAVS];
    char specfile[DDX_PARAM_STR];
    int radQ, SWQ, FLQ;
    int n_planets;                 /* star + planets, like cconfig.n_planets */
    ddx_planet planets[DDX_PARAM_MAX_PLANETS];
    double rho, kqe;
    char comp[DDX_PARAM_STR];
    int n_disks;
    ddx_disk disks[DDX_PARAM_MAX_DISKS];
    int n_blobs;
    ddx_blob blobs[DDX_PARAM_MAX_BLOBS];
    char name_stub[DDX_PARAM_STR];
    int usage_code;                /* on a rejected file: the reference's exit_with_usage
                                      code (src/error.cu), else 0 */
    /* Set after the parameter file by the optics set-up (the reference's detminmax and
     * optical-table read, src/read_in.cu:268-342, 419-505); written to and read from the
     * data-file header.  Zero after ddx_param_read. */
    double amin, amax, mmin, mmax, f;  /* dust size (m) and mass (kg) range, ln mass-bin step */
    int n_grid, n_wav, n_theta, n_dust;
    long long seed;
} ddx_param;

/* Run-time values of a data file (Grid members, src/ddyn.cuh): time, step and the times of
 * the last outputs (yr), the radius-grid size and the outer radius of the temperature
 * table (AU; bodies beyond it, or inside the star, are written commented out with "## ").
 * n_mass counts the massive bodies after the star and planets. */
typedef struct {
    double time, dt, tlastd, tlastf, tlasts, Rmax;
    int nR;
    int n_mass, n_dust, n_all;
} ddx_dat_run;

/* Host state of every body, massive first, in the GPU state's units (mass * 4 pi^2 in
 * Msun); cap = capacity of each array for ddx_dat_read. */
typedef struct {
    double *x, *y, *z, *vx, *vy, *vz, *N, *m;
    int *id;
    long long cap;
} ddx_host_state;

/* Data file in the reference's layout (Grid::writegrid, src/grid.cu:441-673): the header
 * of configuration and run values, then the star and planets and every other body, one
 * per line: x y z [AU] vx vy vz [AU/yr] N, m [kg], radius [m] and beta of its size bin,
 * id.  beta[n_grid] is the size-bin table (bodies with id < 0 get 0).  The reference names
 * the file <stub>_<time %.2f>.dat; the caller passes the path. */
int ddx_dat_write(const char *path, const char *version, const ddx_param *p, const ddx_dat_run *run,
                  const ddx_host_state *s, const float *beta);

/* Reads a data file the way the reference's restart does (read_in_model,
 * src/read_in.cu:736-1014, and Grid::read_in, src/grid.cu:205-310): the header into *p
 * and *run, the bodies into *s, with the size bin of every body after the planets
 * recomputed as round(ln(m / mmin) / f) (-1 beyond the grid).  With s == NULL or
 * s->cap < run->n_all only the header is read (call again with room for run->n_all).
 * run->nR and run->Rmax are inputs (the file does not hold Rmax; it comes from the
 * temperature table).  Rejects a file written by another version (usage code 55) or with
 * another nR (56). */
int ddx_dat_read(const char *path, const char *version, ddx_param *p, ddx_dat_run *run, ddx_host_state *s);

/* SED file (Grid::write_sed, src/grid.cu:675-691): wavelength [micron], stellar flux and
 * excess flux [Jy] per table wavelength; w in m, in = the stellar flux table, exc = the
 * SED of ddx_sed. */
int ddx_sed_write(const char *path, const char *version, int n_wav, const double *w, const double *in,
                  const double *exc);

/* FITS image (Grid::write_image, src/fits.cu:9-85): a primary 2-D FP64 image of
 * xsize x ysize pixels, image[y][x] = F[ysize*x + y] (F is x-major, as ddx_image writes
 * it), with the keys WAVELENG [micron], FLUX (total, Jy), PIXELSCA [arcsec/px],
 * VERSION, a HISTORY card and DATE.  The reference names the file
 * <stub>_<wavelength %.2f>_<time %.3f>.fits. */
int ddx_fits_write(const char *path, const char *version, int xsize, int ysize, const double *F,
                   double wavelength_m, double fov_AU, double dist_m);

/* Parses a DiskDyn parameter file the way read_in_param does (src/read_in.cu:508-733):
 * the same tokeniser, section order, unit conversions, star at planet 0, planets through
 * coe2rv and the centre-of-mass correction, disks and blobs with their derived masses.
 * Returns 0, or DDX_ERR_ARG (1) with p->usage_code set to the reference's exit code where
 * the reference would exit (-1 for a disk line with fewer than 11 values, which the
 * reference reads past), DDX_ERR_IO (8) if the file cannot be opened (usage code 3), or
 * DDX_ERR_RANGE (5) beyond the fixed table sizes above. */
int ddx_param_read(const char *path, ddx_param *p);

/* Mie table file of a grain composition (add_optical_data, src/read_in.cu:419-505; the
 * layout of the reference's table generator): a first line that is skipped, a header line
 * "# n_wav n_theta n_size amin amax" (radii in micron), then per size a line "#s <radius>"
 * (micron), n_wav lines "<wavelength> <Qabs> <Qsca>" (micron) and the n_theta * n_wav
 * phase-function values ten per line.  Lines are read 254 characters at a time, as the
 * reference reads them.  With t->s == NULL only the header is read: t->n_size, n_wav,
 * n_theta, *dmin and *dmax (m).  Otherwise t's counts must be the file's, and t's arrays
 * and w[n_wav] (m; taken from the first size) are filled.  The values are the reference's
 * to the bit.  Returns DDX_ERR_IO if the file cannot be opened (the reference's exit code
 * 39), DDX_ERR_ARG for counts that differ from the header or for data the reference would
 * write outside its arrays (values before the first size line, more sizes or values than
 * the header announces). */
int ddx_optical_read(const char *path, ddx_optical_table *t, double *w, double *dmin, double *dmax);

/* Stellar spectrum file (add_specfile, src/read_in.cu:377-417): lines "<wavelength> <flux>",
 * '#' lines and lines without two numbers skipped; each flux scaled by
 * (rstar_AU * AU)^2 / dist_m^2 as the reference scales it.  *nspec = the number of points;
 * wvl and F (cap entries each) are filled when they are non-NULL and cap >= *nspec, else
 * only the count is returned.  Returns DDX_ERR_IO if the file cannot be opened (exit code
 * 39). */
int ddx_spec_read(const char *path, double rstar_AU, double dist_m, int *nspec, double *wvl, double *F,
                  int cap);

/* Stellar flux on the table wavelengths and the image wavelength indices
 * (interpolate_stellar_to_grid, src/functions.cu:302-336): in[j] log-log interpolated in
 * the spectrum (spec_w, spec_F, nspec >= 2), 0 below its first wavelength or next to a zero
 * flux, F_last (w_last / w)^4 beyond it; wj[k] = i - 1 for the first i with
 * w[i] >= wavs[k] (at most n_wav - 2), as the reference sets it (so -1 for wavs[k] == w[0]).
 * The reference's walk over the spectrum is kept step for step, so the values are its own
 * to the bit; where it would read past the last spectrum point (a table wavelength equal to
 * it) the walk stops there.  Returns DDX_ERR_RANGE if an image wavelength lies outside
 * [w[0], w[n_wav-1]] (the reference's exit code 43). */
int ddx_stellar_grid(int n_wav, const double *w, int nspec, const double *spec_w, const double *spec_F,
                     int nwavs, const double *wavs, double *in, int *wj);

#ifdef __cplusplus
}
#endif

#endif /* DISKDYN_GB300_IO_H */
