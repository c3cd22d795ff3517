/* DiskDyn GB300 path -- start-of-run set-up: the mass grid of a parameter file and the
 * initial bodies of its star, planets, disks and blobs.
 *
 * The reference builds them on the host in its main program and Grid::setup
 * (src/ddyn.cu:84-101, src/grid.cu:68-190).  ddx_setup_host does the same with the
 * reference's generator and gives its bodies; ddx_setup_device draws the same
 * distributions on the GPU with a counter-based generator, straight into the device
 * state, for systems too large for a serial generator.
 */
#ifndef DISKDYN_GB300_SETUP_H
#define DISKDYN_GB300_SETUP_H

#include "diskdyn_gb300_io.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Grain-size range and number constants, after ddx_param_read and before the optics
 * (detminmax, confCdisks and confCblobs, src/read_in.cu:236-342).  dmin and dmax (m) are the
 * optical table's smallest and largest radii (ddx_optical_read).  Clips every disk's and
 * blob's grain range to them (amin, mmin, dmax, dmmax), sets the global p->amin, amax,
 * mmin, mmax, the number of mass bins n_grid (a mass ratio of 1.1 per bin) and their log
 * spacing f, and each disk's and blob's number constant C = Mtot / the integral of
 * m^(1 - eta) between mmin and mmax.  The reference's values to the bit. */
int ddx_param_grid(ddx_param *p, double dmin, double dmax);

/* Body counts of the initial system (run->n_mass, n_dust, n_all) after ddx_param_grid:
 * star and planets, the Ngrav gravitating bodies of every disk and blob, and per disk and
 * blob round(Nsmall / Ngrid) tracers in each of its Ngrid mass bins. */
int ddx_setup_count(const ddx_param *p, double dmin, double dmax, ddx_dat_run *run);

/* Grid::setup's bodies on the host (src/grid.cu:79-190), in its order: star and planets;
 * the gravitating bodies of each disk and blob, masses from the top of the size
 * distribution down (getbod), orbits drawn by genorb_disk / genorb_blob; then the grains of
 * each disk and blob, round(Nsmall / Ngrid) tracers per mass bin, each carrying N = the
 * bin's grain number / tracers, orbits drawn with the bin's beta (src/functions.cu:157-239).
 * The generator is the reference's ran3 seeded with `seed` (the reference uses -2), drawn in
 * the reference's order, so the bodies are the reference's to the bit on x86-64 (the
 * gravitating masses go through long double there as in the reference; on Arm, long double
 * is wider).  beta[p->n_grid] is ddx_dust_grid's table.  s->cap must hold run->n_all
 * (ddx_setup_count).  Returns DDX_ERR_RANGE if it does not, or if a bin falls beyond
 * n_grid. */
int ddx_setup_host(const ddx_param *p, double dmin, double dmax, const float *beta, long long seed,
                   ddx_host_state *s, ddx_dat_run *run);

/* The same system drawn on the GPU into the device state s (n_all = run->n_all entries,
 * cap >= n_all): the same counts, order, grain masses, size bins and grain numbers as
 * ddx_setup_host, the gravitating masses from the same getbod chain evaluated in double
 * without cancellation (to 1e-16; the reference's chain carries the rounding of each next
 * limit into a difference of two nearly equal powers, about 1e-6 on typical files), and
 * orbits from the
 * same distributions, drawn with Philox4x32-10 (Salmon et al., SC'11) keyed by `seed`, one
 * counter stream per body, so the result does not depend on the launch and is reproducible
 * for a seed, but it is not ran3's sequence.  The rejection draws (eccentricities >= 1,
 * blob radii <= 0) stop after 1,024 tries per body; a body that exhausts them makes the call
 * return DDX_ERR_RANGE.  Synchronises `stream`. */
int ddx_setup_device(ddx_ctx *ctx, const ddx_param *p, double dmin, double dmax, const float *beta,
                     unsigned long long seed, const ddx_state *s, long long cap, ddx_dat_run *run,
                     void *stream);

#ifdef __cplusplus
}
#endif

#endif /* DISKDYN_GB300_SETUP_H */
