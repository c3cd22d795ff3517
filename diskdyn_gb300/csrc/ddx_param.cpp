// DiskDyn parameter files on the host: read_in_param (src/read_in.cu:508-733) with its
// tokeniser (:12-60), star and planet set-up (:63-114, coe2rv src/functions.cu:6-46),
// centre-of-mass correction (:344-375) and disk and blob records (:117-234).
//
// The arithmetic follows the reference operation for operation (this file is compiled
// without floating-point contraction), so the parsed values, including the planets'
// Cartesian states, are the reference's to the bit; tests/test_param_cpu.py checks that
// against the reference's own parser.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../../include/diskdyn_gb300.h"
#include "../../include/diskdyn_gb300_io.h"
#include "ddx_host.h"

namespace ddx_host {

namespace {

// The reference's separator set: '@', space, CR, LF and tab.
bool is_sep(int c) { return c == 64 || c == 32 || c == 13 || c == 10 || c == 9; }

// Drops every double quote of a token, in place.
void drop_quotes(char* s) {
    char* w = s;
    for (char* r = s; *r; ++r)
        if (*r != '"') *w++ = *r;
    *w = 0;
}

}  // namespace

int split(char* buf, char** tok, int max) {
    int n = 0;
    bool in_tok = false, in_quote = false;
    while (*buf && n < max) {
        const bool sep = is_sep(*buf);
        if (!sep && !in_tok) {
            tok[n++] = buf;
            in_tok = true;
            in_quote = (*buf == '"');
            ++buf;
        } else if (in_tok && (!sep || in_quote)) {
            if (*buf == '"') in_quote = !in_quote;
            ++buf;
        } else if (in_tok) {               // a separator ends the token
            *buf++ = 0;
            in_tok = false;
        } else {
            ++buf;
        }
    }
    tok[n] = nullptr;
    for (int k = 0; k < n; ++k) drop_quotes(tok[k]);
    return n;
}

}  // namespace ddx_host

namespace {

using ddx_host::split;

// Constants of src/ddyn.cuh:17-38.
constexpr double kPI = 3.14159265358979323846;
constexpr double kGrav = 4.0 * kPI * kPI;
constexpr double kAU = 1.49598e11;
constexpr double kMSun = 1.98892e30;
constexpr double kRSun = 695700000.0;
constexpr double kYear = 3.1556926e7;
constexpr double kPc = 3.08567758149137e16;
constexpr double kMEarth = 5.97e24;

// sscanf("%lg") / ("%d") / ("%ld") semantics: the target keeps its value when the token
// does not start with a number.
void scan(const char* s, double& v) {
    char* end = nullptr;
    const double r = strtod(s, &end);
    if (end != s) v = r;
}
void scan(const char* s, int& v) {
    char* end = nullptr;
    const long r = strtol(s, &end, 10);
    if (end != s) v = (int)r;
}
void scan(const char* s, long long& v) {
    char* end = nullptr;
    const long long r = strtoll(s, &end, 10);
    if (end != s) v = r;
}

bool is_yes(const char* s) {
    return !strcmp(s, "yes") || !strcmp(s, "Y") || !strcmp(s, "YES") || !strcmp(s, "y") || !strcmp(s, "true") ||
           !strcmp(s, "TRUE");
}
bool is_no(const char* s) {
    return !strcmp(s, "no") || !strcmp(s, "N") || !strcmp(s, "NO") || !strcmp(s, "n") || !strcmp(s, "false") ||
           !strcmp(s, "FALSE");
}

void copy_str(char* dst, const char* src) {
    strncpy(dst, src, DDX_PARAM_STR - 1);
    dst[DDX_PARAM_STR - 1] = 0;
}

}  // namespace

namespace ddx_host {

// Orbital elements to Cartesian state about a central mass, both masses times 4 pi^2
// (src/functions.cu:6-46), expression for expression.
void coe2rv(double M, double m, double a, double e, double i, double w, double o, double nu, double* x,
            double* y, double* z, double* vx, double* vy, double* vz, double beta) {
    const double p = a * (1.0 - e * e);
    const double mu = (M + m) * (1.0 - beta);
    const double xe = p * cos(nu) / (1.0 + e * cos(nu));
    const double ye = p * sin(nu) / (1.0 + e * cos(nu));
    const double ze = 0.0;
    const double vxe = -sqrt(mu / p) * sin(nu);
    const double vye = sqrt(mu / p) * (e + cos(nu));
    const double vze = 0;
    *x = xe * (cos(o) * cos(w) - sin(o) * sin(w) * cos(i)) + ye * (-cos(o) * sin(w) - sin(o) * cos(w) * cos(i)) +
         ze * (sin(o) * sin(i));
    *y = xe * (sin(o) * cos(w) + cos(o) * sin(w) * cos(i)) + ye * (-sin(o) * sin(w) + cos(o) * cos(w) * cos(i)) +
         ze * (-cos(o) * sin(i));
    *z = xe * sin(w) * sin(i) + ye * cos(w) * sin(i) + ze * cos(i);
    *vx = vxe * (cos(o) * cos(w) - sin(o) * sin(w) * cos(i)) + vye * (-cos(o) * sin(w) - sin(o) * cos(w) * cos(i)) +
          vze * (sin(o) * sin(i));
    *vy = vxe * (sin(o) * cos(w) + cos(o) * sin(w) * cos(i)) + vye * (-sin(o) * sin(w) + cos(o) * cos(w) * cos(i)) +
          vze * (-cos(o) * sin(i));
    *vz = vxe * sin(w) * sin(i) + vye * cos(w) * sin(i) + vze * cos(i);
}

}  // namespace ddx_host

namespace {

using ddx_host::coe2rv;

// Shifts the bodies to the centre of mass and gives the star the balancing momentum
// (src/read_in.cu:344-375).
void center_of_mass(ddx_param* p) {
    if (p->n_planets == 1) return;
    double Xc = 0, Yc = 0, Zc = 0, Mtot = 0;
    for (int j = 0; j < p->n_planets; j++) {
        Xc += p->planets[j].m * p->planets[j].x;
        Yc += p->planets[j].m * p->planets[j].y;
        Zc += p->planets[j].m * p->planets[j].z;
        Mtot += p->planets[j].m;
    }
    Xc /= Mtot; Yc /= Mtot; Zc /= Mtot;
    for (int j = 0; j < p->n_planets; j++) {
        p->planets[j].x -= Xc;
        p->planets[j].y -= Yc;
        p->planets[j].z -= Zc;
    }
    double Vx = 0, Vy = 0, Vz = 0;
    for (int j = 1; j < p->n_planets; j++) {
        Vx -= p->planets[j].m * p->planets[j].vx;
        Vy -= p->planets[j].m * p->planets[j].vy;
        Vz -= p->planets[j].m * p->planets[j].vz;
    }
    p->planets[0].vx = Vx / p->planets[0].m;
    p->planets[0].vy = Vy / p->planets[0].m;
    p->planets[0].vz = Vz / p->planets[0].m;
}

struct Fail {
    int status, code;
};

void add_planet(ddx_param* p, char** dat) {
    if (p->n_planets >= DDX_PARAM_MAX_PLANETS) throw Fail{DDX_ERR_RANGE, 0};
    double i = 0, a = 0, e = 0, nu = 0, o = 0, w = 0, m = 0;
    scan(dat[0], i); scan(dat[1], a); scan(dat[2], e); scan(dat[3], nu);
    scan(dat[4], o); scan(dat[5], w); scan(dat[6], m);
    const int j = p->n_planets++;
    i *= kPI / 180.0;
    nu *= kPI / 180.0;
    o *= kPI / 180.0;
    w *= kPI / 180.0;
    m *= kGrav;
    ddx_planet& b = p->planets[j];
    coe2rv(p->planets[0].m, m, a, e, i, w, o, nu, &b.x, &b.y, &b.z, &b.vx, &b.vy, &b.vz, 0.0);
    b.m = m;
}

void add_disk(ddx_param* p, char** dat, int t) {
    if (t < 11) throw Fail{DDX_ERR_ARG, -1};   // the reference reads the missing tokens
    if (p->n_disks >= DDX_PARAM_MAX_DISKS) throw Fail{DDX_ERR_RANGE, 0};
    double Rin = 0, Rout = 0, dhdr = 0, sigmae = 0, amax = 0, amin = 0, etaa = 0, mtot = 0, gammas = 0;
    long long Ngrav = 0, Nsmall = 0;
    scan(dat[0], Rin); scan(dat[1], Rout); scan(dat[2], dhdr); scan(dat[3], sigmae); scan(dat[4], amax);
    scan(dat[5], amin); scan(dat[6], etaa); scan(dat[7], mtot); scan(dat[8], gammas);
    scan(dat[9], Ngrav); scan(dat[10], Nsmall);
    ddx_disk& d = p->disks[p->n_disks++];
    d.Rin = Rin;
    d.Rout = Rout;
    d.dhdr = atan(dhdr);
    d.sigmae = sigmae;
    d.amax = amax * 1000.0;
    d.amin = amin / 1.0e6;
    d.eta = (etaa + 2.0) / 3.0;
    d.Mtot = mtot * kMEarth;
    d.mmax = 4.0 * pow(amax * 1000.0, 3.0) * kPI * p->rho / 3.0;
    d.mmin = 4.0 * pow(amin / 1.0e6, 3.0) * kPI * p->rho / 3.0;
    d.gammas = gammas;
    d.Ngrav = Ngrav;
    d.Nsmall = Nsmall;
}

void add_blob(ddx_param* p, char** dat, int t) {
    if (t < 14) throw Fail{DDX_ERR_ARG, 58};
    if (p->n_blobs >= DDX_PARAM_MAX_BLOBS) throw Fail{DDX_ERR_RANGE, 0};
    double a = 0, ecc = 0, inc = 0, w = 0, o = 0, nu = 0, sigma = 0, amax = 0, amin = 0, etaa = 0, mtot = 0,
           vkepp = 0;
    long long Ngrav = 0, Nsmall = 0;
    int collcloud;
    scan(dat[0], a); scan(dat[1], ecc); scan(dat[2], inc); scan(dat[3], w); scan(dat[4], o); scan(dat[5], nu);
    scan(dat[6], amax); scan(dat[7], amin); scan(dat[8], etaa); scan(dat[9], mtot);
    scan(dat[10], Ngrav); scan(dat[11], Nsmall);
    if (!strcmp(dat[12], "cloud") || !strcmp(dat[12], "Cloud")) {
        collcloud = 1;
        scan(dat[13], sigma);
        vkepp = 0.0;
    } else if (!strcmp(dat[12], "collision") || !strcmp(dat[12], "Collision")) {
        collcloud = 0;
        scan(dat[13], vkepp);
        sigma = 0.0;
    } else {
        throw Fail{DDX_ERR_ARG, 57};
    }
    ddx_blob& b = p->blobs[p->n_blobs++];
    b.a = a;
    b.ecc = ecc;
    b.inc = inc * kPI / 180.0;
    b.w = w * kPI / 180.0;
    b.o = o * kPI / 180.0;
    b.nu = nu * kPI / 180.0;
    b.sigma = sigma;
    b.amax = amax * 1000.0;
    b.amin = amin / 1.0e6;
    b.eta = (etaa + 2.0) / 3.0;
    b.Mtot = mtot * kMEarth;
    b.mmax = 4.0 * pow(amax * 1000.0, 3.0) * kPI * p->rho / 3.0;
    b.mmin = 4.0 * pow(amin / 1.0e6, 3.0) * kPI * p->rho / 3.0;
    b.Ngrav = Ngrav;
    b.Nsmall = Nsmall;
    b.collcloud = collcloud;
    b.vkepp = vkepp;
}

// One non-comment line of section i; i may step back for the list sections, as in the
// reference.
void section(ddx_param* p, int& i, char** dat, int t, double& dtemp, int& itemp) {
    if (i == 0) {
        scan(dat[0], itemp);
        if (itemp < 0) throw Fail{DDX_ERR_ARG, 4};
        p->verb = itemp;
    }
    if (i == 1) {
        scan(dat[0], itemp);
        if (itemp < 0) throw Fail{DDX_ERR_ARG, 6};
        p->gpuid = itemp;
    }
    if (i == 2) {
        if (is_yes(dat[0])) {
            p->gl = 1;
            scan(dat[1], dtemp);
            if (dtemp <= 0) throw Fail{DDX_ERR_ARG, 7};
            p->t_gl = dtemp;
        } else if (is_no(dat[0])) {
            p->gl = 0;
            p->t_gl = 0;
        } else {
            throw Fail{DDX_ERR_ARG, 8};
        }
    }
    if (i == 3) {
        scan(dat[0], dtemp);
        if (dtemp <= 0) throw Fail{DDX_ERR_ARG, 9};
        p->t_write = dtemp;
        scan(dat[1], dtemp);
        if (dtemp <= 0) throw Fail{DDX_ERR_ARG, 9};
        p->t_fits = dtemp;
        scan(dat[2], dtemp);
        if (dtemp <= 0) throw Fail{DDX_ERR_ARG, 9};
        p->t_sed = dtemp;
    }
    if (i == 4) {
        scan(dat[0], dtemp);
        if (dtemp <= 0) throw Fail{DDX_ERR_ARG, 10};
        p->t_end = dtemp;
    }
    if (i == 5) {
        scan(dat[0], itemp);
        if (itemp <= 0) throw Fail{DDX_ERR_ARG, 11};
        p->n_step = itemp;
    }
    if (i == 6) {                            // the star
        if (t < 8) throw Fail{DDX_ERR_ARG, 13};
        scan(dat[0], dtemp);
        if (dtemp <= 0) throw Fail{DDX_ERR_ARG, 12};
        ddx_planet& s = p->planets[p->n_planets++];
        s.x = s.y = s.z = s.vx = s.vy = s.vz = 0.0;
        s.m = dtemp * kGrav;
        copy_str(p->sptype, dat[1]);
        scan(dat[2], dtemp);
        if (dtemp <= 0) throw Fail{DDX_ERR_ARG, 12};
        p->teff = dtemp;
        scan(dat[3], dtemp);
        if (dtemp <= 0) throw Fail{DDX_ERR_ARG, 12};
        p->rstar = dtemp * kRSun / kAU;
        scan(dat[4], dtemp);
        if (dtemp <= 0) throw Fail{DDX_ERR_ARG, 12};
        p->Bstar = dtemp * 1.0e-4 * kYear * kYear / kMSun;
        scan(dat[5], dtemp);
        if (dtemp <= 0) throw Fail{DDX_ERR_ARG, 12};
        p->Wz = 365.2422 / dtemp;
        scan(dat[6], dtemp);
        if (dtemp <= 0) throw Fail{DDX_ERR_ARG, 12};
        p->mloss = dtemp;
        scan(dat[7], dtemp);
        if (dtemp <= 0) throw Fail{DDX_ERR_ARG, 12};
        p->vsw = dtemp * 1000.0;
    }
    if (i == 7) {                            // geometry
        if (t < 7) throw Fail{DDX_ERR_ARG, 36};
        scan(dat[0], dtemp);
        if (dtemp <= 0) throw Fail{DDX_ERR_ARG, 37};
        p->dist = dtemp * kPc;
        scan(dat[1], dtemp);
        if (dtemp <= 0) throw Fail{DDX_ERR_ARG, 38};
        p->fov = dtemp;
        scan(dat[2], dtemp);
        p->PA = dtemp * kPI / 180.0;
        scan(dat[3], dtemp);
        p->inc = dtemp * kPI / 180.0;
        scan(dat[4], dtemp);
        p->longitude = dtemp * kPI / 180.0;
        scan(dat[5], itemp);
        p->xsize = itemp;
        scan(dat[6], itemp);
        p->ysize = itemp;
    }
    if (i == 8) {                            // image wavelengths, micron -> m
        p->nwavs = t;
        for (int k = 0; k < t; k++) scan(dat[k], p->wavs[k]);
        for (int k = 0; k < t; k++) p->wavs[k] *= 1e-6;
    }
    if (i == 9) {                            // stellar spectrum
        if (!strcmp(dat[0], "Library") || !strcmp(dat[0], "library") || !strcmp(dat[0], "LIBRARY")) {
            if (p->teff >= 3375 && p->teff < 10000)
                p->teff = round(p->teff / 250.0) * 250;
            else if (p->teff >= 10000 && p->teff < 13000)
                p->teff = round(p->teff / 500.0) * 500;
            else if (p->teff >= 13000 && p->teff < 35000)
                p->teff = round(p->teff / 1000.0) * 1000;
            else if (p->teff >= 35000 && p->teff < 50000)
                p->teff = round(p->teff / 2500.0) * 2500;
            else
                throw Fail{DDX_ERR_ARG, 40};
            snprintf(p->specfile, DDX_PARAM_STR, "Kurucz/Kurucz_%.0f.dat", p->teff);
        } else {
            copy_str(p->specfile, dat[0]);
        }
    }
    if (i == 10) {                           // physics switches
        if (t < 3) throw Fail{DDX_ERR_ARG, 30};
        int* sw[3] = {&p->radQ, &p->SWQ, &p->FLQ};
        for (int k = 0; k < 3; ++k) {
            if (is_yes(dat[k])) *sw[k] = 1;
            else if (is_no(dat[k])) *sw[k] = 0;
            else throw Fail{DDX_ERR_ARG, 31};
        }
    }
    if (i == 11) {                           // planets
        if (!strcmp(dat[0], "begin_planets")) {
            i--;
        } else if (!strcmp(dat[0], "end_planets")) {
            center_of_mass(p);
        } else {
            if (t < 7) throw Fail{DDX_ERR_ARG, 18};
            add_planet(p, dat);
            i--;
        }
    }
    if (i == 12) {                           // density, composition, charge coefficient
        if (t < 3) throw Fail{DDX_ERR_ARG, 15};
        scan(dat[0], dtemp);
        if (dtemp <= 0) throw Fail{DDX_ERR_ARG, 14};
        p->rho = dtemp * 1000;
        copy_str(p->comp, dat[1]);
        scan(dat[2], dtemp);
        if (dtemp <= 0 && p->FLQ == 1) throw Fail{DDX_ERR_ARG, 32};
        p->kqe = dtemp / kYear;
    }
    if (i == 13) {                           // disks
        if (!strcmp(dat[0], "begin_disks")) i--;
        else if (strcmp(dat[0], "end_disks")) { add_disk(p, dat, t); i--; }
    }
    if (i == 14) {                           // blobs
        if (!strcmp(dat[0], "begin_blobs")) i--;
        else if (strcmp(dat[0], "end_blobs")) { add_blob(p, dat, t); i--; }
    }
    if (i == 15) copy_str(p->name_stub, dat[0]);
}

}  // namespace

extern "C" int ddx_param_read(const char* path, ddx_param* p) {
    if (!path || !p) return DDX_ERR_ARG;
    memset(p, 0, sizeof(*p));
    FILE* f = fopen(path, "rb");
    if (!f) {
        p->usage_code = 3;
        return DDX_ERR_IO;
    }
    char buf[512];
    char* dat[64];
    int i = 0;
    int status = DDX_OK;
    double dtemp = 0;   // kept across lines: a value that fails to scan leaves it as it was
    int itemp = 0;
    try {
        while (!feof(f)) {
            if (fgets(buf, sizeof buf, f) == nullptr) break;
            if (buf[0] == '#') continue;
            const int t = split(buf, dat, 16);
            if (t == 0) continue;
            section(p, i, dat, t, dtemp, itemp);
            i++;
        }
        if (i < 15) throw Fail{DDX_ERR_ARG, 17};
    } catch (const Fail& e) {
        p->usage_code = e.code;
        status = e.status;
    }
    fclose(f);
    return status;
}
