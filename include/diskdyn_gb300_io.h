/* DiskDyn GB300 path -- host-side input and output in the reference's formats.
 *
 * These calls run on the host (no GPU, no context).  They read and write the files the
 * reference's driver reads and writes, so a run can start from the same parameter file
 * and produce the same outputs.
 */
#ifndef DISKDYN_GB300_IO_H
#define DISKDYN_GB300_IO_H

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
} ddx_param;

/* Parses a DiskDyn parameter file the way read_in_param does (src/read_in.cu:508-733):
 * the same tokeniser, section order, unit conversions, star at planet 0, planets through
 * coe2rv and the centre-of-mass correction, disks and blobs with their derived masses.
 * Returns 0, or DDX_ERR_ARG (1) with p->usage_code set to the reference's exit code where
 * the reference would exit (-1 for a disk line with fewer than 11 values, which the
 * reference reads past), DDX_ERR_IO (8) if the file cannot be opened (usage code 3), or
 * DDX_ERR_RANGE (5) beyond the fixed table sizes above. */
int ddx_param_read(const char *path, ddx_param *p);

#ifdef __cplusplus
}
#endif

#endif /* DISKDYN_GB300_IO_H */
