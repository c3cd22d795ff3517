/*
 * ORACLE -- test infrastructure, not product code.
 *
 * A plain-C FP64 restatement of the reference DiskDyn hot path, written to check the
 * CUDA kernels of diskdyn_gb300 and to serve as the timed CPU baseline.  Nothing in the
 * product links or calls this file; only the tests, the smoke check and the CPU-baseline
 * leg of bench.py do.
 *
 * Each function states the reference lines it follows (paths within the DiskDyn project).
 * Arithmetic is kept in the reference's order, expression by expression; the only
 * intended differences are the summation order of the massive-set accelerations (the
 * reference adds them with CAS atomics in a hardware-dependent order) and libm instead of
 * the CUDA math library.  Build with -ffp-contract=off so x86 and Arm hosts agree.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define ORA_AU      1.49598e11
#define ORA_LIGHTAU 63239.6717367
#define ORA_CSPEED  299792458.0
#define ORA_KBOLTZ  1.3806503E-23
#define ORA_HPLANK  6.626068E-34
#define ORA_PI      3.14159265358979323846
#define ORA_NR      100
#define ORA_TSUB    2000.0

typedef struct {
    double *x, *y, *z, *vx, *vy, *vz, *m, *N;
    int *id;
} ora_state;

typedef struct {
    int radQ, SWQ, FLQ;
    double Wz, Bstar, Rstar, rho, vsw_AUyr, Rmin;
} ora_phys;

typedef struct {
    double dist, fov, PA, inc, longitude;
    int xsize, ysize;
} ora_view;

/* ------------------------------------------------------------------------------------
 * Massive set: src/grid.cu:693-752 with src/gpu_functions.cu:71-625.
 * Stage accelerations: a_i = sum_{j != i} m_j (x_j - x_i) / (RR sqrt(RR)), pairs with
 * RR == 0 contribute nothing (src/gpu_functions.cu:156-178).  The reference forms
 * kv = dX / f then multiplies by m_j (:164, :190); the same two roundings are used here.
 * ------------------------------------------------------------------------------------ */
static void massive_accel(int ng, const double *kx, const double *ky, const double *kz,
                          const double *m, double *ax, double *ay, double *az) {
    int i;
#pragma omp parallel for schedule(static) if (ng > 256)
    for (i = 0; i < ng; ++i) {
        double KX = 0.0, KY = 0.0, KZ = 0.0;
        for (int j = 0; j < ng; ++j) {
            if (j == i) continue;
            double dX = kx[j] - kx[i];
            double dY = ky[j] - ky[i];
            double dZ = kz[j] - kz[i];
            double RR = dX * dX + dY * dY + dZ * dZ;
            double f = RR * sqrt(RR);
            if (f != 0) {
                KX += (dX / f) * m[j];
                KY += (dY / f) * m[j];
                KZ += (dZ / f) * m[j];
            }
        }
        ax[i] = KX; ay[i] = KY; az[i] = KZ;
    }
}

/* Stage positions of the massive set, 4 x 3 x ng doubles written to kpos as
 * [stage][xyz][i], and the final update of x, v.  With ng <= 1 the reference skips the
 * massive stages entirely (src/grid.cu:698, 747): the stage arrays keep their set-up
 * zeros and the star does not move; ref_single = 1 reproduces that. */
static void massive_rk4(int ng, ora_state s, double dt, double *kpos, int ref_single) {
    size_t n = (size_t)ng;
    if (ng <= 1) {
        if (ref_single) {
            memset(kpos, 0, sizeof(double) * 12 * n);
        } else {
            /* A lone star feels no force: its stage positions are ballistic and the RK4
             * combination moves it by v dt. */
            for (int st = 0; st < 4; ++st) {
                double c = st == 0 ? 0.0 : (st == 3 ? dt : dt * 0.5);
                kpos[(st * 3 + 0) * n] = s.x[0] + s.vx[0] * c;
                kpos[(st * 3 + 1) * n] = s.y[0] + s.vy[0] * c;
                kpos[(st * 3 + 2) * n] = s.z[0] + s.vz[0] * c;
            }
            if (ng == 1) {
                double d6 = dt / 6.0;
                s.x[0] += d6 * (s.vx[0] + 2.0 * s.vx[0] + 2.0 * s.vx[0] + s.vx[0]);
                s.y[0] += d6 * (s.vy[0] + 2.0 * s.vy[0] + 2.0 * s.vy[0] + s.vy[0]);
                s.z[0] += d6 * (s.vz[0] + 2.0 * s.vz[0] + 2.0 * s.vz[0] + s.vz[0]);
            }
        }
        return;
    }
    double *k1x = kpos + 0 * n, *k1y = kpos + 1 * n, *k1z = kpos + 2 * n;
    double *k2x = kpos + 3 * n, *k2y = kpos + 4 * n, *k2z = kpos + 5 * n;
    double *k3x = kpos + 6 * n, *k3y = kpos + 7 * n, *k3z = kpos + 8 * n;
    double *k4x = kpos + 9 * n, *k4y = kpos + 10 * n, *k4z = kpos + 11 * n;
    double *buf = (double *)malloc(sizeof(double) * 21 * n);
    double *k1vx = buf, *k1vy = buf + n, *k1vz = buf + 2 * n;
    double *k2vx = buf + 3 * n, *k2vy = buf + 4 * n, *k2vz = buf + 5 * n;
    double *k3vx = buf + 6 * n, *k3vy = buf + 7 * n, *k3vz = buf + 8 * n;
    double *k4vx = buf + 9 * n, *k4vy = buf + 10 * n, *k4vz = buf + 11 * n;
    double *k2rx = buf + 12 * n, *k2ry = buf + 13 * n, *k2rz = buf + 14 * n;
    double *k3rx = buf + 15 * n, *k3ry = buf + 16 * n, *k3rz = buf + 17 * n;
    double *k4rx = buf + 18 * n, *k4ry = buf + 19 * n, *k4rz = buf + 20 * n;
    double h = dt * 0.5;       /* src/grid.cu:711,716 */
    for (int i = 0; i < ng; ++i) { k1x[i] = s.x[i]; k1y[i] = s.y[i]; k1z[i] = s.z[i]; }
    massive_accel(ng, k1x, k1y, k1z, s.m, k1vx, k1vy, k1vz);
    for (int i = 0; i < ng; ++i) {             /* RK4calc_massive3 */
        k2x[i] = s.x[i] + s.vx[i] * h; k2y[i] = s.y[i] + s.vy[i] * h; k2z[i] = s.z[i] + s.vz[i] * h;
        k2rx[i] = s.vx[i] + k1vx[i] * h; k2ry[i] = s.vy[i] + k1vy[i] * h; k2rz[i] = s.vz[i] + k1vz[i] * h;
    }
    massive_accel(ng, k2x, k2y, k2z, s.m, k2vx, k2vy, k2vz);
    for (int i = 0; i < ng; ++i) {             /* RK4calc_massive5 */
        k3x[i] = s.x[i] + k2rx[i] * h; k3y[i] = s.y[i] + k2ry[i] * h; k3z[i] = s.z[i] + k2rz[i] * h;
        k3rx[i] = s.vx[i] + k2vx[i] * h; k3ry[i] = s.vy[i] + k2vy[i] * h; k3rz[i] = s.vz[i] + k2vz[i] * h;
    }
    massive_accel(ng, k3x, k3y, k3z, s.m, k3vx, k3vy, k3vz);
    for (int i = 0; i < ng; ++i) {             /* RK4calc_massive7 */
        k4x[i] = s.x[i] + k3rx[i] * dt; k4y[i] = s.y[i] + k3ry[i] * dt; k4z[i] = s.z[i] + k3rz[i] * dt;
        k4rx[i] = s.vx[i] + k3vx[i] * dt; k4ry[i] = s.vy[i] + k3vy[i] * dt; k4rz[i] = s.vz[i] + k3vz[i] * dt;
    }
    massive_accel(ng, k4x, k4y, k4z, s.m, k4vx, k4vy, k4vz);
    /* The massive final update happens after the dust step in the reference
     * (src/grid.cu:387-389); it only reads these arrays, so doing it here, after the stage
     * positions are saved, gives the same result. */
    double d6 = dt / 6.0;      /* src/grid.cu:750 */
    for (int i = 0; i < ng; ++i) {             /* RK4calc_massive_final */
        s.x[i] += d6 * (s.vx[i] + 2.0 * k2rx[i] + 2.0 * k3rx[i] + k4rx[i]);
        s.y[i] += d6 * (s.vy[i] + 2.0 * k2ry[i] + 2.0 * k3ry[i] + k4ry[i]);
        s.z[i] += d6 * (s.vz[i] + 2.0 * k2rz[i] + 2.0 * k3rz[i] + k4rz[i]);
        s.vx[i] += d6 * (k1vx[i] + 2.0 * k2vx[i] + 2.0 * k3vx[i] + k4vx[i]);
        s.vy[i] += d6 * (k1vy[i] + 2.0 * k2vy[i] + 2.0 * k3vy[i] + k4vy[i]);
        s.vz[i] += d6 * (k1vz[i] + 2.0 * k2vz[i] + 2.0 * k3vz[i] + k4vz[i]);
    }
    free(buf);
}

/* ------------------------------------------------------------------------------------
 * Dust: src/gpu_functions.cu:627-943, one tracer, in order.
 * Returns 0 = updated, 1 = removed (N set to 0 at the index the reference uses).
 * ------------------------------------------------------------------------------------ */
static int star_stage(double dx, double dy, double dz, double rx, double ry, double rz,
                      double m0, float bet, float betsw, float qe, double m,
                      const ora_phys *p, double *kx, double *ky, double *kz) {
    double RR = dx * dx + dy * dy + dz * dz;
    double RR3 = RR * sqrt(RR);
    if (RR <= p->Rmin * p->Rmin) return 0;
    double Fg = (1.0 - bet - betsw) * m0 / RR3;
    double Fbase1;
    if (p->SWQ == 1) Fbase1 = m0 / RR * (bet / ORA_LIGHTAU + betsw / p->vsw_AUyr);
    else             Fbase1 = bet * m0 / ORA_LIGHTAU / RR;
    double Fbase2 = (dx * rx + dy * ry + dz * rz) / RR;
    double Fdrx = Fbase1 * (Fbase2 * dx + rx);
    double Fdry = Fbase1 * (Fbase2 * dy + ry);
    double Fdrz = Fbase1 * (Fbase2 * dz + rz);
    double Flx, Fly;
    if (p->FLQ == 1) {
        double Bz = p->Bstar * p->Rstar * p->Rstar * p->Rstar / RR3;
        Flx = qe * (ry - p->Wz * dx) * Bz / m;
        Fly = -qe * (rx + p->Wz * dy) * Bz / m;
    } else {
        Flx = 0; Fly = 0;
    }
    *kx = -Fg * dx - Fdrx + Flx;
    *ky = -Fg * dy - Fdry + Fly;
    *kz = -Fg * dz - Fdrz;
    return 1;
}

static int bodies_stage(int ng, const double *kx_, const double *ky_, const double *kz_,
                        const double *mm, double xt, double yt, double zt,
                        double *kx, double *ky, double *kz) {
    for (int j = 1; j < ng; ++j) {
        double dx = xt - kx_[j];
        double dy = yt - ky_[j];
        double dz = zt - kz_[j];
        double RR = dx * dx + dy * dy + dz * dz;
        if (RR == 0) return 0;
        double f = mm[j] / RR / sqrt(RR);
        *kx += -f * dx;
        *ky += -f * dy;
        *kz += -f * dz;
    }
    return 1;
}

static void dust_one(int ng, int i, ora_state s, const double *kpos, size_t n, double dt,
                     const float *beta, const float *betasw, const float *q,
                     const ora_phys *p, int ref_mode) {
    const double *k1x = kpos + 0 * n, *k1y = kpos + 1 * n, *k1z = kpos + 2 * n;
    const double *k2x = kpos + 3 * n, *k2y = kpos + 4 * n, *k2z = kpos + 5 * n;
    const double *k3x = kpos + 6 * n, *k3y = kpos + 7 * n, *k3z = kpos + 8 * n;
    const double *k4x = kpos + 9 * n, *k4y = kpos + 10 * n, *k4z = kpos + 11 * n;
    int t = ng + i;
    if (s.N[t] == 0) return;
    int id = s.id[t];
    double dt2 = dt / 2.0, dt6 = dt / 6.0;
    double x = s.x[t], y = s.y[t], z = s.z[t], vx = s.vx[t], vy = s.vy[t], vz = s.vz[t];
    float bet = 0.f, betsw = 0.f, qe = 0.f;
    /* The reference reads q[id] even for id < 0 (src/gpu_functions.cu:665), an
     * out-of-bounds read used only with the Lorentz force; 0 is used instead. */
    if (id >= 0) { bet = beta[id]; betsw = betasw[id]; qe = q[id]; }
    double m = s.m[t], m0 = s.m[0];
    double k1vx, k1vy, k1vz, k2vx, k2vy, k2vz, k3vx, k3vy, k3vz, k4vx, k4vy, k4vz;
    double k2rx, k2ry, k2rz, k3rx, k3ry, k3rz, k4rx, k4ry, k4rz, xt, yt, zt;

    /* K1 */
    if (!star_stage(x - k1x[0], y - k1y[0], z - k1z[0], vx, vy, vz, m0, bet, betsw, qe, m, p,
                    &k1vx, &k1vy, &k1vz)) { s.N[t] = 0; return; }
    if (!bodies_stage(ng, k1x, k1y, k1z, s.m, x, y, z, &k1vx, &k1vy, &k1vz)) { s.N[t] = 0; return; }
    /* K2 */
    k2rx = vx + k1vx * dt2; k2ry = vy + k1vy * dt2; k2rz = vz + k1vz * dt2;
    xt = x + vx * dt2; yt = y + vy * dt2; zt = z + vz * dt2;
    if (!star_stage(xt - k2x[0], yt - k2y[0], zt - k2z[0], k2rx, k2ry, k2rz, m0, bet, betsw, qe, m,
                    p, &k2vx, &k2vy, &k2vz)) { s.N[t] = 0; return; }
    if (!bodies_stage(ng, k2x, k2y, k2z, s.m, xt, yt, zt, &k2vx, &k2vy, &k2vz)) { s.N[t] = 0; return; }
    /* K3 */
    k3rx = vx + k2vx * dt2; k3ry = vy + k2vy * dt2; k3rz = vz + k2vz * dt2;
    xt = x + k2rx * dt2; yt = y + k2ry * dt2; zt = z + k2rz * dt2;
    if (!star_stage(xt - k3x[0], yt - k3y[0], zt - k3z[0], k3rx, k3ry, k3rz, m0, bet, betsw, qe, m,
                    p, &k3vx, &k3vy, &k3vz)) { s.N[t] = 0; return; }
    if (!bodies_stage(ng, k3x, k3y, k3z, s.m, xt, yt, zt, &k3vx, &k3vy, &k3vz)) { s.N[t] = 0; return; }
    /* K4 */
    k4rx = vx + k3vx * dt; k4ry = vy + k3vy * dt; k4rz = vz + k3vz * dt;
    xt = x + k3rx * dt; yt = y + k3ry * dt; zt = z + k3rz * dt;
    if (!star_stage(xt - k4x[0], yt - k4y[0], zt - k4z[0], k4rx, k4ry, k4rz, m0, bet, betsw, qe, m,
                    p, &k4vx, &k4vy, &k4vz)) {
        /* src/gpu_functions.cu:878 zeroes N[i] -- the dust-relative index used as an
         * absolute one -- and leaves this grain's state as it was. */
        if (ref_mode) s.N[i] = 0; else s.N[t] = 0;
        return;
    }
    if (!bodies_stage(ng, k4x, k4y, k4z, s.m, xt, yt, zt, &k4vx, &k4vy, &k4vz)) { s.N[t] = 0; return; }
    /* Evolve (src/gpu_functions.cu:927-941) */
    x += dt6 * (vx + 2.0 * (k2rx + k3rx) + k4rx);
    y += dt6 * (vy + 2.0 * (k2ry + k3ry) + k4ry);
    z += dt6 * (vz + 2.0 * (k2rz + k3rz) + k4rz);
    vx += dt6 * (k1vx + 2.0 * (k2vx + k3vx) + k4vx);
    vy += dt6 * (k1vy + 2.0 * (k2vy + k3vy) + k4vy);
    vz += dt6 * (k1vz + 2.0 * (k2vz + k3vz) + k4vz);
    s.x[t] = x; s.y[t] = y; s.z[t] = z;
    s.vx[t] = vx; s.vy[t] = vy; s.vz[t] = vz;
}

/* One step: massive_RK4(dt); small_RK4(dt); massive_final(dt) (src/grid.cu:387-389).
 * kpos_out (optional, 12*n_grav doubles) receives the massive stage positions.
 * nthreads <= 0 leaves the OpenMP default. */
int ora_step(ora_state s, int n_grav, int n_dust, double dt, const float *beta,
             const float *betasw, const float *q, const ora_phys *p, int ref_mode,
             double *kpos_out) {
    if (n_grav < 1 || n_dust < 0) return 1;
    size_t n = (size_t)n_grav;
    double *kpos = kpos_out ? kpos_out : (double *)malloc(sizeof(double) * 12 * n);
    massive_rk4(n_grav, s, dt, kpos, ref_mode);
    int i;
#pragma omp parallel for schedule(dynamic, 256)
    for (i = 0; i < n_dust; ++i) dust_one(n_grav, i, s, kpos, n, dt, beta, betasw, q, p, ref_mode);
    if (!kpos_out) free(kpos);
    return 0;
}

/* The dust half only, with the massive stage positions given (12*n_grav doubles laid out
 * [stage][xyz][body]); used to time or check the dust kernel in isolation. */
int ora_dust(ora_state s, int n_grav, int n_dust, int i0, int i1, double dt, const double *kpos,
             const float *beta, const float *betasw, const float *q, const ora_phys *p,
             int ref_mode) {
    if (n_grav < 1 || i0 < 0 || i1 > n_dust) return 1;
    int i;
#pragma omp parallel for schedule(dynamic, 64)
    for (i = i0; i < i1; ++i) dust_one(n_grav, i, s, kpos, (size_t)n_grav, dt, beta, betasw, q, p, ref_mode);
    return 0;
}

/* ------------------------------------------------------------------------------------
 * Image and SED: src/gpu_functions.cu:983-1156.
 * ------------------------------------------------------------------------------------ */
typedef struct {
    const double *w, *in, *Qabs, *Qsca, *Qpfunc, *Td, *size;
    double Rmin, Rmax;
    int n_grid, n_wav, n_theta;
} ora_optics;

static double temp_of(double R, int id, const ora_optics *o) {
    double f = log(o->Rmax / o->Rmin) / ((double)ORA_NR - 1.0);
    const double *Td = o->Td;
    if (R <= o->Rmin) return Td[id * ORA_NR];
    if (R >= o->Rmax) return Td[id * ORA_NR + ORA_NR - 1];
    int Rid = (int)(log(R / o->Rmin) / f) + 1;
    double Rin = o->Rmin * exp((Rid - 1) * f);
    double Rout = o->Rmin * exp(Rid * f);
    return exp(log(Td[id * ORA_NR + Rid - 1]) +
               log(Td[id * ORA_NR + Rid] / Td[id * ORA_NR + Rid - 1]) * log(R / Rin) / log(Rout / Rin));
}

static double flux_of(double n, int id, int wj, double R, double T, double cossc,
                      const ora_optics *o, double dist) {
    int nwav = o->n_wav, ntheta = o->n_theta;
    double wvl = o->w[wj];
    double I = (2 * ORA_HPLANK * ORA_CSPEED * ORA_CSPEED) /
               (pow(wvl, 5) * (exp(ORA_HPLANK * ORA_CSPEED / (wvl * ORA_KBOLTZ * T)) - 1.0)) * ORA_PI;
    int cosinm = (int)floor(0.5 * (cossc + 1.0) * (ntheta - 1));
    int cosinp = cosinm + 1;
    double cosm = (double)(cosinm)*2.0 / (ntheta - 1) - 1.0;
    double cosp = (double)(cosinp)*2.0 / (ntheta - 1) - 1.0;
    const double *Q = o->Qpfunc;
    double P = exp(log(Q[nwav * (ntheta * id + cosinm) + wj]) +
                   (log(Q[nwav * (ntheta * id + cosinp) + wj]) - log(Q[nwav * (ntheta * id + cosinm) + wj])) *
                       (cossc - cosm) / (cosp - cosm));
    double s = o->size[id];
    double Fscat = o->in[wj] * ORA_PI * s * s * o->Qsca[nwav * id + wj] * P / R / R / ORA_AU / ORA_AU;
    double Fther = I * s * s * o->Qabs[nwav * id + wj] / dist / dist;
    return n * (Fther + Fscat) * 1e26 * wvl * wvl / ORA_CSPEED;
}

/* Pixel of one tracer (src/gpu_functions.cu:1001-1047); returns 0 when outside the image.
 * Also returns R and the scattering-angle cosine. */
static int pixel_of(double x, double y, double z, const ora_view *v, int ntheta, int *xim,
                    int *yim, double *Rout, double *cossc_out, int sed_ref_radius) {
    double rot = v->longitude, incl = v->inc, PA = v->PA, dist = v->dist;
    double phi = atan2(y, x);
    double R = sqrt(x * x + y * y + z * z);
    double Rd = sqrt(x * x + y * y);
    double rr = sed_ref_radius ? R : Rd;
    x = rr * cos(phi + rot);
    y = rr * sin(phi + rot);
    double ly = -dist * sin(incl) - y;
    double lz = dist * cos(incl) - z;
    double cossc = (x * x + (-y) * ly + (-z) * lz) / R / sqrt(x * x + ly * ly + lz * lz);
    if (cossc < -1) cossc = -1.0;
    if (cossc >= 1.0 - 2.0 / ntheta) cossc = 1.0 - 2.0 / ntheta;
    *Rout = R;
    *cossc_out = cossc;
    if (!xim) return 1;
    y = sqrt(y * y + z * z) * cos(atan2(z, y) - incl);
    phi = atan2(y, x);
    Rd = sqrt(x * x + y * y);
    x = Rd * cos(phi + PA);
    y = Rd * sin(phi + PA);
    double psca;
    if (v->xsize >= v->ysize) psca = v->fov / v->xsize;
    else                      psca = v->fov / v->ysize;
    x = x + 0.5 * psca * v->xsize;
    y = y + 0.5 * psca * v->ysize;
    *xim = (int)floor(x / psca);
    *yim = (int)floor(y / psca);
    if (*xim < 0 || *xim > v->xsize - 1 || *yim < 0 || *yim > v->ysize - 1) return 0;
    return 1;
}

/* Images at wj[0..n_img-1]; Fd[img][xsize*ysize] x-major, overwritten.  pix_out
 * (optional, n_dust ints) receives ysize*xim + yim of each tracer, or -1. */
int ora_image(ora_state s, int n_grav, int n_dust, const ora_optics *o, const ora_view *v,
              const int *wj, int n_img, double *Fd, int *pix_out) {
    size_t npix = (size_t)v->xsize * v->ysize;
    memset(Fd, 0, sizeof(double) * npix * n_img);
    for (int i = 0; i < n_dust; ++i) {
        int t = n_grav + i;
        if (pix_out) pix_out[i] = -1;
        int id = s.id[t];
        if (id < 0) continue;
        int xim, yim;
        double R, cossc;
        if (!pixel_of(s.x[t], s.y[t], s.z[t], v, o->n_theta, &xim, &yim, &R, &cossc, 0)) continue;
        if (pix_out) pix_out[i] = v->ysize * xim + yim;
        if (!(R > o->Rmin)) continue;
        double T = temp_of(R, id, o);
        for (int k = 0; k < n_img; ++k)
            Fd[k * npix + (size_t)v->ysize * xim + yim] += flux_of(s.N[t], id, wj[k], R, T, cossc, o, v->dist);
    }
    return 0;
}

/* SED at every table wavelength: Fsed[j] = sum over tracers (src/gpu_functions.cu:1083-1156
 * and :961-981).  ref_mode = 1 rotates by the spherical radius like the reference. */
int ora_sed(ora_state s, int n_grav, int n_dust, const ora_optics *o, const ora_view *v,
            double *Fsed, int ref_mode) {
    int nw = o->n_wav;
    for (int j = 0; j < nw; ++j) Fsed[j] = 0.0;
    int j;
#pragma omp parallel for schedule(static)
    for (j = 0; j < nw; ++j) {
        double acc = 0.0;
        for (int i = 0; i < n_dust; ++i) {
            int t = n_grav + i;
            int id = s.id[t];
            if (id < 0) continue;
            double R, cossc;
            pixel_of(s.x[t], s.y[t], s.z[t], v, o->n_theta, NULL, NULL, &R, &cossc, ref_mode);
            if (!(R > o->Rmin)) continue;
            double T = temp_of(R, id, o);
            acc += flux_of(s.N[t], id, j, R, T, cossc, o, v->dist);
        }
        Fsed[j] = acc;
    }
    return 0;
}

/* ------------------------------------------------------------------------------------
 * Dust-temperature table: Grid::calculate_dust_temp, src/grid.cu:754-834, and the Planck
 * function intens, src/functions.cu:390-397.  Rmax_AU is the largest configured radius
 * (before the reference's factor 2); on return Td[n_grid][100] holds T on the log grid
 * and *Rmin_AU, *Rmax_AU the grid limits in AU.  dist in m.
 * ------------------------------------------------------------------------------------ */
static double intens(double temp, double wvl) {
    return (2 * ORA_HPLANK * ORA_CSPEED * ORA_CSPEED) /
           (pow(wvl, 5) * (exp(ORA_HPLANK * ORA_CSPEED / (wvl * ORA_KBOLTZ * temp)) - 1));
}

int ora_dust_temp(int n_grid, int n_wav, const double *w, const double *in, const double *Qabs,
                  double dist, double *Rmin_AU, double *Rmax_AU, double *Td) {
    double Rmax = *Rmax_AU * 2 * ORA_AU;
    double Rmin = Rmax;
    for (int k = 0; k < n_grid; ++k) {
        double star = 0.0, gflux = 0.0;
        for (int i = 1; i < n_wav; i++)
            star += 0.5 * (w[i] - w[i - 1]) * (Qabs[k * n_wav + i - 1] * in[i - 1] + Qabs[k * n_wav + i] * in[i]) / ORA_PI;
        star *= pow(dist, 2.0);
        for (int i = 1; i < n_wav; i++)
            gflux += 0.5 * (w[i] - w[i - 1]) * (Qabs[k * n_wav + i - 1] * intens(ORA_TSUB, w[i - 1]) + Qabs[k * n_wav + i] * intens(ORA_TSUB, w[i]));
        double Rtmp = 0.5 * sqrt(star / gflux);
        if (Rtmp < Rmin) Rmin = Rtmp;
    }
    int nT = (int)floor((2 * ORA_TSUB - 3) * 0.5) + 1;
    int k;
#pragma omp parallel for schedule(dynamic, 1)
    for (k = 0; k < n_grid; ++k) {
        double *Ra = (double *)malloc(sizeof(double) * nT), *Ta = (double *)malloc(sizeof(double) * nT);
        double star = 0.0;
        for (int i = 1; i < n_wav; i++)
            star += 0.5 * (w[i] - w[i - 1]) * (Qabs[k * n_wav + i - 1] * in[i - 1] + Qabs[k * n_wav + i] * in[i]) / ORA_PI;
        star *= pow(dist, 2.0);
        int j = 0;
        for (double T = 2 * ORA_TSUB; T >= 3.0; T -= 2.0) {
            double gflux = 0.0;
            for (int i = 1; i < n_wav; i++)
                gflux += 0.5 * (w[i] - w[i - 1]) * (Qabs[k * n_wav + i - 1] * intens(T, w[i - 1]) + Qabs[k * n_wav + i] * intens(T, w[i]));
            Ra[j] = 0.5 * sqrt(star / gflux);
            Ta[j] = T;
            j++;
        }
        /* The reference's search has no bounds check; the two guards below only act where
         * it would read outside its arrays. */
        int im = 0, ip = 0;
        for (int i = 0; i < ORA_NR; i++) {
            double R = Rmin * exp(log(Rmax / Rmin) * ((double)i) / ((double)ORA_NR - 1.0));
            while (ip < nT - 1 && Ra[ip] <= R) ip++;
            im = ip - 1;
            if (im < 0) im = 0;
            Td[k * ORA_NR + i] = exp(log(Ta[im]) + log(Ta[ip] / Ta[im]) * log(R / Ra[im]) / log(Ra[ip] / Ra[im]));
            ip--;
            if (ip < 0) ip = 0;
        }
        free(Ra); free(Ta);
    }
    *Rmin_AU = Rmin / ORA_AU;
    *Rmax_AU = Rmax / ORA_AU;
    return 0;
}

/* ------------------------------------------------------------------------------------
 * Time step: Grid::det_step, src/grid.cu:312-342 (PI2 from src/ddyn.cuh:29), over host
 * arrays x, y, z, m of the massive bodies; disks give Rin, blobs (a, ecc, sigma).
 * ------------------------------------------------------------------------------------ */
double ora_det_step(const double *x, const double *y, const double *z, const double *m, int n_grav,
                    int n_step, const double *disk_Rin, int n_disks, const double *blob_a,
                    const double *blob_ecc, const double *blob_sigma, int n_blobs) {
    const double PI2 = 6.28318530717958623200;
    double dtdynmin = 1e137;
    if (n_grav > 1) {
        double R = pow((x[1] - x[0]) * (x[1] - x[0]) + (y[1] - y[0]) * (y[1] - y[0]) +
                           (z[1] - z[0]) * (z[1] - z[0]), 3.0 / 2.0);
        dtdynmin = PI2 * sqrt(R / (m[0] + m[1])) / n_step;
        for (int i = 2; i < n_grav; i++) {
            R = pow((x[i] - x[0]) * (x[i] - x[0]) + (y[i] - y[0]) * (y[i] - y[0]) +
                        (z[i] - z[0]) * (z[i] - z[0]), 3.0 / 2.0);
            double dttmp = PI2 * sqrt(R / (m[0] + m[i])) / n_step;
            if (dttmp < dtdynmin) dtdynmin = dttmp;
        }
    }
    for (int i = 0; i < n_disks; i++) {
        double dttmp = PI2 * sqrt(disk_Rin[i] / (m[0])) / n_step;
        if (dttmp < dtdynmin) dtdynmin = dttmp;
    }
    for (int i = 0; i < n_blobs; i++) {
        double dttmp = PI2 * sqrt((blob_a[i] * (1.0 - blob_ecc[i]) - blob_sigma[i]) / (m[0])) / n_step;
        if (dttmp < dtdynmin) dtdynmin = dttmp;
    }
    return dtdynmin;
}

/* ------------------------------------------------------------------------------------
 * Collision pairs (no reference counterpart; the criterion is the one documented for
 * ddx_collide): live tracers i < j of [i0, i1) with
 *   (xj-xi)^2 + (yj-yi)^2 + (zj-zi)^2 < h^2, left to right, no contraction.
 * ------------------------------------------------------------------------------------ */
static int ora_close(const ora_state *s, int i, int j, double h2) {
    double ex = s->x[j] - s->x[i], ey = s->y[j] - s->y[i], ez = s->z[j] - s->z[i];
    double d2 = ex * ex + ey * ey + ez * ez;
    return d2 < h2;
}

/* Brute force over all pairs.  Writes up to cap pairs (i, j) to out[2k], out[2k+1] in (i, j)
 * order; returns the total number found. */
long long ora_collide_brute(ora_state s, int i0, int i1, double h, int *out, long long cap) {
    double h2 = h * h;
    int n = i1 - i0;
    long long *cnt = (long long *)calloc((size_t)(n > 0 ? n : 1), sizeof(long long));
    int a;
#pragma omp parallel for schedule(dynamic, 64)
    for (a = 0; a < n; ++a) {
        int i = i0 + a;
        if (s.N[i] == 0) continue;
        long long c = 0;
        for (int j = i + 1; j < i1; ++j)
            if (s.N[j] != 0 && ora_close(&s, i, j, h2)) ++c;
        cnt[a] = c;
    }
    long long tot = 0;
    for (a = 0; a < n; ++a) { long long c = cnt[a]; cnt[a] = tot; tot += c; }
#pragma omp parallel for schedule(dynamic, 64)
    for (a = 0; a < n; ++a) {
        int i = i0 + a;
        if (s.N[i] == 0) continue;
        long long k = cnt[a];
        for (int j = i + 1; j < i1; ++j)
            if (s.N[j] != 0 && ora_close(&s, i, j, h2)) {
                if (k < cap) { out[2 * k] = i; out[2 * k + 1] = j; }
                ++k;
            }
    }
    free(cnt);
    return tot;
}

/* The same pairs through a cell list (cell side h(1+1e-9), coordinates clamped to
 * +-(2^20-2)), for sizes where the brute force is too slow. */
typedef struct { long long id; int i; } ora_cell;
static int ora_cell_cmp(const void *a, const void *b) {
    const ora_cell *x = (const ora_cell *)a, *y = (const ora_cell *)b;
    if (x->id != y->id) return x->id < y->id ? -1 : 1;
    return (x->i > y->i) - (x->i < y->i);
}
static long long ora_cc(double x, double inv) {
    double c = floor(x * inv), lim = (double)((1LL << 20) - 2);
    if (c < -lim) c = -lim;
    if (c > lim) c = lim;
    return (long long)c;
}
static long long ora_pack(long long cx, long long cy, long long cz) {
    long long o = 1LL << 20;
    return ((cx + o) << 42) | ((cy + o) << 21) | (cz + o);
}
static int ora_int_cmp(const void *a, const void *b) {
    int x = *(const int *)a, y = *(const int *)b;
    return (x > y) - (x < y);
}

long long ora_collide_grid(ora_state s, int i0, int i1, double h, int *out, long long cap) {
    int n = i1 - i0;
    if (n <= 1) return 0;
    double inv = 1.0 / (h * (1.0 + 1e-9)), h2 = h * h;
    ora_cell *cells = (ora_cell *)malloc(sizeof(ora_cell) * (size_t)n);
    long long *own = (long long *)malloc(sizeof(long long) * (size_t)n);
    int m = 0;
    for (int a = 0; a < n; ++a) {
        int i = i0 + a;
        own[a] = -1;
        if (s.N[i] == 0) continue;
        own[a] = ora_pack(ora_cc(s.x[i], inv), ora_cc(s.y[i], inv), ora_cc(s.z[i], inv));
        cells[m].id = own[a];
        cells[m].i = i;
        ++m;
    }
    qsort(cells, (size_t)m, sizeof(ora_cell), ora_cell_cmp);
    long long *cnt = (long long *)calloc((size_t)n + 1, sizeof(long long));
    for (int pass = 0; pass < 2; ++pass) {
        int a;
#pragma omp parallel for schedule(dynamic, 256)
        for (a = 0; a < n; ++a) {
            if (own[a] < 0) continue;
            int i = i0 + a;
            long long o = 1LL << 20, id = own[a];
            long long cx = ((id >> 42) & 0x1FFFFF) - o, cy = ((id >> 21) & 0x1FFFFF) - o, cz = (id & 0x1FFFFF) - o;
            long long k = pass ? cnt[a] : 0, k0 = k;
            for (int dx = -1; dx <= 1; ++dx)
                for (int dy = -1; dy <= 1; ++dy)
                    for (int dz = -1; dz <= 1; ++dz) {
                        long long nid = ora_pack(cx + dx, cy + dy, cz + dz);
                        int lo = 0, hi = m;           /* first entry with id >= nid */
                        while (lo < hi) { int mid = (lo + hi) / 2; if (cells[mid].id < nid) lo = mid + 1; else hi = mid; }
                        for (int r = lo; r < m && cells[r].id == nid; ++r) {
                            int j = cells[r].i;
                            if (j <= i || !ora_close(&s, i, j, h2)) continue;
                            if (pass && k < cap) { out[2 * k] = i; out[2 * k + 1] = j; }
                            ++k;
                        }
                    }
            if (!pass) cnt[a] = k;
            else if (k0 < cap) {
                long long e = k < cap ? k : cap;
                /* sort this tracer's partners by j */
                int *tmp = (int *)malloc(sizeof(int) * (size_t)(e - k0 > 0 ? e - k0 : 1));
                for (long long q = k0; q < e; ++q) tmp[q - k0] = out[2 * q + 1];
                qsort(tmp, (size_t)(e - k0), sizeof(int), ora_int_cmp);
                for (long long q = k0; q < e; ++q) out[2 * q + 1] = tmp[q - k0];
                free(tmp);
            }
        }
        if (!pass) {
            long long tot = 0;
            for (int b = 0; b < n; ++b) { long long c = cnt[b]; cnt[b] = tot; tot += c; }
            cnt[n] = tot;
        }
    }
    long long tot = cnt[n];
    free(cnt); free(own); free(cells);
    return tot;
}

/* ------------------------------------------------------------------------------------
 * Stellar flux on the table wavelengths and the image wavelength indices:
 * interpolate_stellar_to_grid, src/functions.cu:302-336.  sw, sF: the spectrum file's
 * wavelengths and fluxes (nspec >= 2).  Returns 43, the reference's usage code, if an image
 * wavelength lies outside w.  The reference walks the spectrum with an index that it steps
 * back by one after each table wavelength; that walk is kept, with one guard: where it
 * would read past the last spectrum point (a table wavelength equal to it) it stops there.
 * wj[j] = i - 1 where i is the first index with w[i] >= wavs[j] (at most n_wav - 2), as in
 * the reference, so it is -1 for wavs[j] == w[0].
 * ------------------------------------------------------------------------------------ */
int ora_stellar_grid(int n_wav, const double *w, int nspec, const double *sw, const double *sF, int nwavs,
                     const double *wavs, double *in, int *wj) {
    if (nspec < 2) return -1;
    int ip = 0;
    for (int j = 0; j < n_wav; j++) {
        if (w[j] < sw[0]) {
            in[j] = 0.0;
        } else if (w[j] > sw[nspec - 1]) {
            in[j] = sF[nspec - 1] * pow(sw[nspec - 1] / w[j], 4.0);
        } else {
            while (ip < nspec - 1 && sw[ip] <= w[j]) ip++;
            int im = ip - 1;
            if (sF[im] != 0 && sF[ip] != 0)
                in[j] = exp(log(sF[im]) + log(w[j] / sw[im]) * log(sF[ip] / sF[im]) / log(sw[ip] / sw[im]));
            else
                in[j] = 0.0;
            ip--;
        }
    }
    for (int j = 0; j < nwavs; j++) {
        int i = 0;
        if (wavs[j] < w[0] || wavs[j] > w[n_wav - 1]) return 43;
        while (w[i] < wavs[j] && i < n_wav - 2) i++;
        wj[j] = i - 1;
    }
    return 0;
}

/* ------------------------------------------------------------------------------------
 * Optical tables resampled onto the mass grid and the radiation-pressure and wind-drag
 * tables: interpolate_dust_to_grid, src/functions.cu:243-300, and calculate_beta,
 * :338-388 (Cd = 2, Grav = 4 pi^2, src/ddyn.cuh).  s, Qabs, Qsca, Qpfunc: the optical file's
 * n_dust sizes; a, q, Qa, Qs, Qp, beta, betasw: the n_grid bins.  Returns 54 (the
 * reference's usage code) when the last bin overshoots dmax by more than 1e-12.
 * The size walk is the reference's, with two guards where it would read outside s: a bin
 * at or below s[0] is interpolated on [s[0], s[1]] (the reference reads s[-1] there), and a
 * bin above the last size on the last interval.
 * ------------------------------------------------------------------------------------ */
int ora_dust_grid(int n_dust, int n_wav, int n_theta, const double *s, const double *w, const double *Qabs,
                  const double *Qsca, const double *Qpfunc, const double *in, int n_grid, double amin, double amax,
                  double dmax, double kqe, int radQ, int SWQ, double rho, double dist, double mstar,
                  double mloss, double vsw, double *a, float *q, double *Qa, double *Qs, double *Qp, float *beta,
                  float *betasw, double *Lum, double *betaswconst) {
    if (n_dust < 2 || n_grid < 2) return -1;
    const double f = log(amax / amin) / ((double)n_grid - 1.0);
    int ip = 0;
    for (int i = 0; i < n_grid; i++) {
        a[i] = amin * exp((double)i * f);
        q[i] = kqe * a[i] * 1e9;
        if (i == n_grid - 1 && (a[i] - dmax) > 1e-12) return 54;
        if (i == n_grid - 1 && (a[i] - dmax) < 1e-12 && (a[i] - dmax) > 0) a[i] = dmax;
        while (ip < n_dust - 1 && s[ip] < a[i]) ip++;
        int im = ip - 1;
        if (im < 0) { im = 0; ip = 1; }
        for (int j = 0; j < n_wav; j++) {
            const size_t m = (size_t)im * n_wav + j, p = (size_t)ip * n_wav + j, o = (size_t)i * n_wav + j;
            Qa[o] = exp(log(Qabs[m]) + log(a[i] / s[im]) * log(Qabs[p] / Qabs[m]) / log(s[ip] / s[im]));
            Qs[o] = exp(log(Qsca[m]) + log(a[i] / s[im]) * log(Qsca[p] / Qsca[m]) / log(s[ip] / s[im]));
            for (int k = 0; k < n_theta; k++) {
                const size_t pm = (size_t)n_wav * ((size_t)n_theta * im + k) + j;
                const size_t pp = (size_t)n_wav * ((size_t)n_theta * ip + k) + j;
                Qp[(size_t)n_wav * ((size_t)n_theta * i + k) + j] =
                    exp(log(Qpfunc[pm]) + log(a[i] / s[im]) * log(Qpfunc[pp] / Qpfunc[pm]) / log(s[ip] / s[im]));
            }
        }
        ip--;
    }

    *betaswconst = 3.0 * mloss * 2 * 1.98892e30 * 3.1556926e7 * vsw / 32.0 / ORA_PI / mstar / rho / ORA_AU / ORA_AU /
                   ORA_AU;
    double Star = 0.0;
    for (int j = 0; j < n_wav - 1; j++) Star += 0.5 * (w[j + 1] - w[j]) * (in[j + 1] + in[j]);
    *Lum = Star * 4.0 * ORA_PI * pow(dist, 2.0) / 3.827e26;
    double *Qpr = (double *)malloc(sizeof(double) * n_wav);
    for (int i = 0; i < n_grid; i++) {
        if (radQ == 1) {
            double Qsum = 0.0;
            for (int j = 0; j < n_wav; j++) {
                double g = 0.0, S = 0.0, costm = -1.0;
                for (int k = 1; k < n_theta; k++) {
                    const double costp = (double)k * 2.0 / (n_theta - 1.0) - 1.0;
                    const double P0 = Qp[(size_t)n_wav * ((size_t)n_theta * i + k - 1) + j];
                    const double P1 = Qp[(size_t)n_wav * ((size_t)n_theta * i + k) + j];
                    S += 0.5 * (P0 + P1) * (costp - costm);
                    g += 0.5 * (costm * P0 + costp * P1) * (costp - costm);
                    costm = costp;
                }
                g /= S;
                Qpr[j] = (Qa[(size_t)i * n_wav + j] + Qs[(size_t)i * n_wav + j] * (1.0 - g)) * in[j];
            }
            for (int j = 0; j < n_wav - 1; j++) Qsum += 0.5 * (w[j + 1] - w[j]) * (Qpr[j + 1] + Qpr[j]);
            beta[i] = 0.57 * Qsum / Star * (*Lum / mstar * (4.0 * ORA_PI * ORA_PI)) / a[i] / 1e6 / rho / 1e-3;
        } else {
            beta[i] = 0.0;
        }
        betasw[i] = SWQ == 1 ? *betaswconst / a[i] : 0.0;
    }
    free(Qpr);
    return 0;
}

/* ------------------------------------------------------------------------------------
 * Counter-based set-up draws (the GPU generator of the initial system), restated: the
 * Philox4x32-10 bijection of Salmon, Moraes, Dror and Shaw ("Parallel random numbers: as
 * easy as 1, 2, 3", SC'11), then the orbit draws of genorb_disk / genorb_blob
 * (src/functions.cu:157-232) and coe2rv (:6-46) in the reference's expression order, with
 * libm.  Body i's uniforms come from counters (draw, i lo, i hi, 0x53455455) under the key
 * (seed lo, seed hi), two per counter, each 53 bits mapped to (0, 1].
 * ------------------------------------------------------------------------------------ */
#include <stdint.h>

void ora_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3], k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; r++) {
        if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0, n1 = (uint32_t)p1;
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1, n3 = (uint32_t)p0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

typedef struct { uint32_t k[2], lo, hi, draw; } ora_stream;

static void ora_pair(ora_stream *s, double *u1, double *u2) {
    uint32_t c[4] = {s->draw++, s->lo, s->hi, 0x53455455u}, o[4];
    ora_philox4x32_10(c, s->k, o);
    *u1 = (double)((((uint64_t)(o[0] >> 5)) << 26 | (o[1] >> 6)) + 1) * 0x1.0p-53;
    *u2 = (double)((((uint64_t)(o[2] >> 5)) << 26 | (o[3] >> 6)) + 1) * 0x1.0p-53;
}

#define ORA_PI2 6.28318530717958623200

static double ora_gauss(double u1, double u2) { return sqrt(-2.0 * log(u1)) * cos(ORA_PI2 * u2); }

static void ora_coe2rv(double M, double m, double a, double e, double i, double w, double o, double nu, double *s,
                       double beta) {
    double p = a * (1.0 - e * e), mu = (M + m) * (1.0 - beta);
    double xe = p * cos(nu) / (1.0 + e * cos(nu)), ye = p * sin(nu) / (1.0 + e * cos(nu));
    double vxe = -sqrt(mu / p) * sin(nu), vye = sqrt(mu / p) * (e + cos(nu));
    s[0] = xe * (cos(o) * cos(w) - sin(o) * sin(w) * cos(i)) + ye * (-cos(o) * sin(w) - sin(o) * cos(w) * cos(i));
    s[1] = xe * (sin(o) * cos(w) + cos(o) * sin(w) * cos(i)) + ye * (-sin(o) * sin(w) + cos(o) * cos(w) * cos(i));
    s[2] = xe * sin(w) * sin(i) + ye * cos(w) * sin(i);
    s[3] = vxe * (cos(o) * cos(w) - sin(o) * sin(w) * cos(i)) + vye * (-cos(o) * sin(w) - sin(o) * cos(w) * cos(i));
    s[4] = vxe * (sin(o) * cos(w) + cos(o) * sin(w) * cos(i)) + vye * (-sin(o) * sin(w) + cos(o) * cos(w) * cos(i));
    s[5] = vxe * sin(w) * sin(i) + vye * cos(w) * sin(i);
}

typedef struct { double Rin, Rout, sigmae, gammas, dhdr; } ora_disk;
typedef struct { double a, ecc, inc, w, o, nu, sigma, vkepp; int collcloud; } ora_blob;

/* Bodies first .. first+n-1: kind 0 = disk j[k], 1 = blob j[k]; out[n][6] = x y z vx vy vz.
 * Returns the number of bodies whose rejection draws ran out (1,024 tries). */
long long ora_setup_philox(long long n, long long first, const int *kind, const int *j, const double *m,
                           const double *beta, const ora_disk *disks, const ora_blob *blobs, double M,
                           unsigned long long seed, double *out) {
    long long bad = 0;
    for (long long k = 0; k < n; k++) {
        const long long i = first + k;
        ora_stream rs = {{(uint32_t)seed, (uint32_t)(seed >> 32)}, (uint32_t)i, (uint32_t)((unsigned long long)i >> 32), 0};
        double *s = out + 6 * k, u1, u2;
        int ok = 0;
        if (kind[k] == 0) {
            const ora_disk *d = &disks[j[k]];
            double e = 0.0;
            for (int t = 0; t < 1024 && !ok; t++) {
                ora_pair(&rs, &u1, &u2);
                e = fabs(ora_gauss(u1, u2) * d->sigmae);
                ok = e < 1.0;
            }
            double amin = d->Rin / (1.0 - e), amax = d->Rout / (1.0 + e), g = 2.0 + d->gammas;
            double ua, unu, ui1, ui2, uw, uo;
            ora_pair(&rs, &ua, &unu);
            ora_pair(&rs, &ui1, &ui2);
            ora_pair(&rs, &uw, &uo);
            double a = pow(ua * (pow(amax, g) - pow(amin, g)) + pow(amin, g), 1.0 / g);
            double inc = fabs(ora_gauss(ui1, ui2) * d->dhdr);
            ora_coe2rv(M, m[k], a, e, inc, ORA_PI2 * uw, ORA_PI2 * uo, ORA_PI2 * unu, s, beta[k]);
        } else {
            const ora_blob *b = &blobs[j[k]];
            double a = 0.0;
            for (int t = 0; t < 1024 && !ok; t++) {
                ora_pair(&rs, &u1, &u2);
                a = b->a + ora_gauss(u1, u2) * b->sigma;
                ok = a > 0.0;
            }
            ora_pair(&rs, &u1, &u2);
            double nu = b->nu + ora_gauss(u1, u2) * b->sigma / a;
            ora_coe2rv(M, m[k], a, b->ecc, b->inc, b->w, b->o, nu, s, beta[k]);
            if (b->collcloud == 0) {
                ora_pair(&rs, &u1, &u2);
                double voff = b->vkepp * 0.01 * sqrt(s[3] * s[3] + s[4] * s[4] + s[5] * s[5]);
                double ct = -1.0 + 2.0 * u1, st = sqrt(1.0 - ct * ct), gam = ORA_PI2 * u2;
                s[3] += voff * st * cos(gam);
                s[4] += voff * st * sin(gam);
                s[5] += voff * ct;
            }
        }
        if (!ok) bad++;
    }
    return bad;
}
