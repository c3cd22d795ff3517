// Output and restart files in the reference's formats, on the host.
//
//  - data file: Grid::writegrid (src/grid.cu:441-673) and its readers read_in_model
//    (src/read_in.cu:736-1014) and Grid::read_in (src/grid.cu:205-310).  The layout is a
//    file format: every header line, its order and its printf conversion are the
//    reference's, so either program reads the other's files;
//  - SED file: Grid::write_sed (src/grid.cu:675-691);
//  - FITS image: Grid::write_image (src/fits.cu:9-85), written here without cfitsio:
//    2880-byte blocks of 80-character cards, big-endian IEEE doubles.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include "../../include/diskdyn_gb300.h"
#include "../../include/diskdyn_gb300_io.h"
#include "ddx_host.h"

namespace {

using ddx_host::split;

constexpr double kPI = 3.14159265358979323846;
constexpr double kGrav = 4.0 * kPI * kPI;
constexpr double kAU = 1.49598e11;
constexpr double kMSun = 1.98892e30;
constexpr double kRSun = 695700000.0;
constexpr double kYear = 3.1556926e7;
constexpr double kPc = 3.08567758149137e16;
constexpr double kCspeed = 299792458.0;

struct File {
    FILE* f;
    explicit File(const char* path, const char* mode) : f(fopen(path, mode)) {}
    ~File() { if (f) fclose(f); }
};

// ---------------------------------------------------------------------------------------
// data file writer
// ---------------------------------------------------------------------------------------

template <typename T, typename F>
void row(FILE* fw, const char* label, int n, const T* items, F field, const char* fmt) {
    fputs(label, fw);
    for (int i = 0; i < n; i++) fprintf(fw, fmt, field(items[i]));
    fputs("\n", fw);
}

void write_header(FILE* fw, const char* ver, const ddx_param* c, const ddx_dat_run* r) {
    fprintf(fw, "#\n");
    fprintf(fw, "#Calculated_with_DiskDyn_Version %s\n", ver);
    fprintf(fw, "#\n");
    fprintf(fw, "#Config file parameters\n");
    fprintf(fw, "#Verbose\t\t\t%d\n", c->verb);
    fprintf(fw, "#GPUID\t\t\t\t%d\n", c->gpuid);
    fprintf(fw, "#Graphical_Output\t\t%d\n", c->gl);
    fprintf(fw, "#Time_Out_for_Graphics\t\t%.3f\n", c->t_gl);
    fprintf(fw, "#Time_Out_for_Data\t\t%.3f\n", c->t_write);
    fprintf(fw, "#Time_Out_for_SED\t\t%.3f\n", c->t_sed);
    fprintf(fw, "#Time_Out_for_FITS\t\t%.3f\n", c->t_fits);
    fprintf(fw, "#Time_End_for_model\t\t%.3f\n", c->t_end);
    fprintf(fw, "#N_step_per_orbit\t\t%d\n", c->n_step);
    fprintf(fw, "#Spectral-type_of_star\t\t%s\n", c->sptype);
    fprintf(fw, "#Temperature_of_star\t\t%.2f\n", c->teff);
    fprintf(fw, "#Radius_of_star\t\t\t%.5f\n", c->rstar * kAU / kRSun);
    fprintf(fw, "#Magnetic_field_of_star\t\t%.5e\n", c->Bstar * kMSun * 1.0e4 / kYear / kYear);
    fprintf(fw, "#Stellar_rotation_of_star\t%.5f\n", 365.2422 / c->Wz);
    fprintf(fw, "#Stellar_mass_loss\t\t%.5e\n", c->mloss);
    fprintf(fw, "#Stellar_wind_speed\t\t%.5e\n", c->vsw);
    fprintf(fw, "#Include_rad_press\t\t%d\n", c->radQ);
    fprintf(fw, "#Include_SWD\t\t\t%d\n", c->SWQ);
    fprintf(fw, "#Include_Lorentz\t\t%d\n", c->FLQ);
    fprintf(fw, "#Bulk_density\t\t\t%.3f\n", c->rho);
    fprintf(fw, "#Electric_charge_coeff\t\t%.3f\n", c->kqe * kYear);
    fprintf(fw, "#Name_Stub\t\t\t%s\n", c->name_stub);
    fprintf(fw, "#Distance\t\t\t%.5f\n", c->dist / kPc);
    fprintf(fw, "#Field_of_View\t\t\t%.6f\n", c->fov);
    fprintf(fw, "#Position_Angle\t\t\t%.5f\n", c->PA * 180.0 / kPI);
    fprintf(fw, "#Inclination_Angle\t\t%.5f\n", c->inc * 180.0 / kPI);
    fprintf(fw, "#Longitude_Angle\t\t%.5f\n", c->longitude * 180.0 / kPI);
    fprintf(fw, "#Image_x_size\t\t\t%d\n", c->xsize);
    fprintf(fw, "#Image_y_size\t\t\t%d\n", c->ysize);
    fprintf(fw, "#Spectral-file\t\t\t%s\n", c->specfile);
    fprintf(fw, "#Minimum_particle_size\t\t%.8e\n", c->amin);
    fprintf(fw, "#Maximum_particle_size\t\t%.8e\n", c->amax);
    fprintf(fw, "#Minimum_particle_mass\t\t%.8e\n", c->mmin);
    fprintf(fw, "#Maximum_particle_mass\t\t%.8e\n", c->mmax);
    fprintf(fw, "#Number_of_dust_grids\t\t%d\n", c->n_grid);
    fprintf(fw, "#Mass_grid_ratio\t\t%.8e\n", c->f);
    fprintf(fw, "#Optical_composition_file\t%s\n", c->comp);
    fprintf(fw, "#Wavelengths_in_interpolation\t%d\n", c->n_wav);
    fprintf(fw, "#Number_of_thetas\t\t%d\n", c->n_theta);
    fprintf(fw, "#Number_of_dust_grids\t\t%d\n", c->n_dust);
    fprintf(fw, "#Number_of_planets\t\t%d\n", c->n_planets);
    fprintf(fw, "#Number_of_disks\t\t%d\n", c->n_disks);
    fprintf(fw, "#Number_of_blobs\t\t%d\n", c->n_blobs);
    fprintf(fw, "#Image_wavelengths\t");
    for (int i = 0; i < c->nwavs; i++) fprintf(fw, "\t%.3f", c->wavs[i] * 1e6);
    fprintf(fw, "\n");
    fprintf(fw, "#Seed_of_model\t\t\t%lld\n", c->seed);
    const ddx_disk* D = c->disks;
    const int nd = c->n_disks;
    row(fw, "#Disk_Rin\t", nd, D, [](const ddx_disk& d) { return d.Rin; }, "\t\t%.3f");
    row(fw, "#Disk_Rout\t", nd, D, [](const ddx_disk& d) { return d.Rout; }, "\t\t%.3f");
    row(fw, "#Disk_dhdr\t", nd, D, [](const ddx_disk& d) { return d.dhdr; }, "\t\t%.4f");
    row(fw, "#Disk_sigmae\t", nd, D, [](const ddx_disk& d) { return d.sigmae; }, "\t\t%.4f");
    row(fw, "#Disk_amax\t\t", nd, D, [](const ddx_disk& d) { return d.amax; }, "\t%.6e");
    row(fw, "#Disk_mmax\t\t", nd, D, [](const ddx_disk& d) { return d.mmax; }, "\t%.6e");
    row(fw, "#Disk_amin\t\t", nd, D, [](const ddx_disk& d) { return d.amin; }, "\t%.6e");
    row(fw, "#Disk_mmin\t\t", nd, D, [](const ddx_disk& d) { return d.mmin; }, "\t%.6e");
    row(fw, "#Disk_dmax\t\t", nd, D, [](const ddx_disk& d) { return d.dmax; }, "\t%.6e");
    row(fw, "#Disk_dmmax\t\t", nd, D, [](const ddx_disk& d) { return d.dmmax; }, "\t%.6e");
    row(fw, "#Disk_eta\t", nd, D, [](const ddx_disk& d) { return d.eta; }, "\t\t%.4f");
    row(fw, "#Disk_gammas\t", nd, D, [](const ddx_disk& d) { return d.gammas; }, "\t\t%.3f");
    row(fw, "#Disk_C\t\t\t", nd, D, [](const ddx_disk& d) { return d.C; }, "\t%.8e");
    row(fw, "#Disk_Mtot\t\t", nd, D, [](const ddx_disk& d) { return d.Mtot; }, "\t%.8e");
    row(fw, "#Disk_Ngrav\t", nd, D, [](const ddx_disk& d) { return (long long)d.Ngrav; }, "\t\t%lld");
    row(fw, "#Disk_Nsmall\t", nd, D, [](const ddx_disk& d) { return (long long)d.Nsmall; }, "\t\t%lld");
    const ddx_blob* B = c->blobs;
    const int nb = c->n_blobs;
    row(fw, "#Blob_a\t\t", nb, B, [](const ddx_blob& b) { return b.a; }, "\t\t%.5f");
    row(fw, "#Blob_ecc\t", nb, B, [](const ddx_blob& b) { return b.ecc; }, "\t\t%.5f");
    row(fw, "#Blob_inc\t", nb, B, [](const ddx_blob& b) { return b.inc; }, "\t\t%.5f");
    row(fw, "#Blob_w\t\t", nb, B, [](const ddx_blob& b) { return b.w; }, "\t\t%.5f");
    row(fw, "#Blob_o\t", nb, B, [](const ddx_blob& b) { return b.o; }, "\t\t%.5f");
    row(fw, "#Blob_nu\t", nb, B, [](const ddx_blob& b) { return b.nu; }, "\t\t%.5f");
    row(fw, "#Blob_sigma\t", nb, B, [](const ddx_blob& b) { return b.sigma; }, "\t\t%.3f");
    row(fw, "#Blob_amax\t\t", nb, B, [](const ddx_blob& b) { return b.amax; }, "\t%.6e");
    row(fw, "#Blob_mmax\t\t", nb, B, [](const ddx_blob& b) { return b.mmax; }, "\t%.6e");
    row(fw, "#Blob_amin\t\t", nb, B, [](const ddx_blob& b) { return b.amin; }, "\t%.6e");
    row(fw, "#Blob_mmin\t\t", nb, B, [](const ddx_blob& b) { return b.mmin; }, "\t%.6e");
    row(fw, "#Blob_dmax\t\t", nb, B, [](const ddx_blob& b) { return b.dmax; }, "\t%.6e");
    row(fw, "#Blob_dmmax\t\t", nb, B, [](const ddx_blob& b) { return b.dmmax; }, "\t%.6e");
    row(fw, "#Blob_eta\t", nb, B, [](const ddx_blob& b) { return b.eta; }, "\t\t%.3f");
    row(fw, "#Blob_C\t\t\t", nb, B, [](const ddx_blob& b) { return b.C; }, "\t%.8e");
    row(fw, "#Blob_Mtot\t\t", nb, B, [](const ddx_blob& b) { return b.Mtot; }, "\t%.8e");
    row(fw, "#Blob_Ngrav\t", nb, B, [](const ddx_blob& b) { return (long long)b.Ngrav; }, "\t\t%lld");
    row(fw, "#Blob_Nsmall\t", nb, B, [](const ddx_blob& b) { return (long long)b.Nsmall; }, "\t\t%lld");
    row(fw, "#Blob_collcloud\t", nb, B, [](const ddx_blob& b) { return b.collcloud; }, "\t\t%d");
    row(fw, "#Blob_vkepp\t", nb, B, [](const ddx_blob& b) { return b.vkepp; }, "\t\t%.5f");
    fprintf(fw, "#\n");
    fprintf(fw, "# t=0 positions and velocities of planets and Star\n");
    const ddx_planet* P = c->planets;
    const int np = c->n_planets;
    row(fw, "#Planet_x\t", np, P, [](const ddx_planet& b) { return b.x; }, "\t\t%.4f");
    row(fw, "#Planet_y\t", np, P, [](const ddx_planet& b) { return b.y; }, "\t\t%.4f");
    row(fw, "#Planet_z\t", np, P, [](const ddx_planet& b) { return b.z; }, "\t\t%.4f");
    row(fw, "#Planet_vx\t", np, P, [](const ddx_planet& b) { return b.vx; }, "\t\t%.4f");
    row(fw, "#Planet_vy\t", np, P, [](const ddx_planet& b) { return b.vy; }, "\t\t%.4f");
    row(fw, "#Planet_vz\t", np, P, [](const ddx_planet& b) { return b.vz; }, "\t\t%.4f");
    row(fw, "#Planet_m\t\t", np, P, [](const ddx_planet& b) { return b.m; }, "\t%.6e");
    fprintf(fw, "#NR_used\t\t\t%d\n", r->nR);
    fprintf(fw, "#\n");
    fprintf(fw, "# Remaining parameters and data are for Grid class read-in\n");
    fprintf(fw, "#\n");
    fprintf(fw, "#Time_of_model\t\t\t%.8f\n", r->time);
    fprintf(fw, "#dt_of_model\t\t\t%.8f\n", r->dt);
    fprintf(fw, "#Last_t_of_data\t\t\t%.8f\n", r->tlastd);
    fprintf(fw, "#Last_t_of_fits\t\t\t%.8f\n", r->tlastf);
    fprintf(fw, "#Last_t_of_SED\t\t\t%.8f\n", r->tlasts);
    fprintf(fw, "#Number_of_grav_bodies\t\t%d\n", r->n_mass);
    fprintf(fw, "#Number_of_dust_particles\t%d\n", r->n_dust);
    fprintf(fw, "#Number_of_all_particles\t%d\n", r->n_all);
}

// ---------------------------------------------------------------------------------------
// data file reader: the reference's tokeniser (ddx_host::split) and line numbering
// ---------------------------------------------------------------------------------------

void scan(const char* s, double& v) {
    if (!s) return;
    char* e = nullptr;
    const double r = strtod(s, &e);
    if (e != s) v = r;
}
void scan(const char* s, int& v) {
    if (!s) return;
    char* e = nullptr;
    const long r = strtol(s, &e, 10);
    if (e != s) v = (int)r;
}
void scan(const char* s, long long& v) {
    if (!s) return;
    char* e = nullptr;
    const long long r = strtoll(s, &e, 10);
    if (e != s) v = r;
}

void copy_str(char* dst, const char* src) {
    strncpy(dst, src ? src : "", DDX_PARAM_STR - 1);
    dst[DDX_PARAM_STR - 1] = 0;
}

struct Fail {
    int status, code;
};

// Header line i (counting non-empty lines from 0), tokens dat[0..t).
void header_line(int i, char** dat, int t, const char* ver, ddx_param* c, ddx_dat_run* r, double& dtemp, int& itemp) {
    auto d1 = [&]() { scan(dat[1], dtemp); return dtemp; };
    auto i1 = [&]() { scan(dat[1], itemp); return itemp; };
    switch (i) {
        case 1: if (t < 2 || strcmp(ver, dat[1]) != 0) throw Fail{DDX_ERR_ARG, 55}; break;
        case 4: if (i1() < 0) throw Fail{DDX_ERR_ARG, 4}; c->verb = itemp; break;
        case 5: if (i1() < 0) throw Fail{DDX_ERR_ARG, 6}; c->gpuid = itemp; break;
        case 6: c->gl = i1(); break;
        case 7: c->t_gl = d1(); break;
        case 8: c->t_write = d1(); break;
        case 9: c->t_sed = d1(); break;
        case 10: c->t_fits = d1(); break;
        case 11: c->t_end = d1(); break;
        case 12: c->n_step = i1(); break;
        case 13: copy_str(c->sptype, dat[1]); break;
        case 14: c->teff = d1(); break;
        case 15: c->rstar = d1() * kRSun / kAU; break;
        case 16: c->Bstar = d1() * kYear * kYear * 1.0e-4 / kMSun; break;
        case 17: c->Wz = 365.2422 / d1(); break;
        case 18: c->mloss = d1(); break;
        case 19: c->vsw = d1(); break;
        case 20: c->radQ = i1(); break;
        case 21: c->SWQ = i1(); break;
        case 22: c->FLQ = i1(); break;
        case 23: c->rho = d1(); break;
        case 24: c->kqe = d1() / kYear; break;
        case 25: copy_str(c->name_stub, dat[1]); break;
        case 26: c->dist = d1() * kPc; break;
        case 27: c->fov = d1(); break;
        case 28: c->PA = d1() * kPI / 180.0; break;
        case 29: c->inc = d1() * kPI / 180.0; break;
        case 30: c->longitude = d1() * kPI / 180.0; break;
        case 31: c->xsize = i1(); break;
        case 32: c->ysize = i1(); break;
        case 33: copy_str(c->specfile, dat[1]); break;
        case 34: c->amin = d1(); break;
        case 35: c->amax = d1(); break;
        case 36: c->mmin = d1(); break;
        case 37: c->mmax = d1(); break;
        case 38: c->n_grid = i1(); break;
        case 39: c->f = d1(); break;
        case 40: copy_str(c->comp, dat[1]); break;
        case 41: c->n_wav = i1(); break;
        case 42: c->n_theta = i1(); break;
        case 43: c->n_dust = i1(); break;
        case 44:
            c->n_planets = i1();
            if (c->n_planets < 0 || c->n_planets > DDX_PARAM_MAX_PLANETS) throw Fail{DDX_ERR_RANGE, 0};
            break;
        case 45:
            c->n_disks = i1();
            if (c->n_disks < 0 || c->n_disks > DDX_PARAM_MAX_DISKS) throw Fail{DDX_ERR_RANGE, 0};
            break;
        case 46:
            c->n_blobs = i1();
            if (c->n_blobs < 0 || c->n_blobs > DDX_PARAM_MAX_BLOBS) throw Fail{DDX_ERR_RANGE, 0};
            break;
        case 47:
            if (t < 2) throw Fail{DDX_ERR_ARG, 41};
            if (t - 1 > DDX_PARAM_MAX_WAVS) throw Fail{DDX_ERR_RANGE, 0};
            c->nwavs = t - 1;
            for (int k = 1; k < t; k++) scan(dat[k], c->wavs[k - 1]);
            for (int k = 1; k < t; k++) c->wavs[k - 1] *= 1e-6;
            break;
        case 48: c->seed = i1(); break;   // Grid::read_in reads the seed with %d
        case 94:
            if (i1() != r->nR) throw Fail{DDX_ERR_ARG, 56};
            break;
        case 98: r->time = d1(); break;
        case 99: r->dt = d1(); break;
        case 100: r->tlastd = d1(); break;
        case 101: r->tlastf = d1(); break;
        case 102: r->tlasts = d1(); break;
        case 103: r->n_mass = i1(); break;
        case 104: r->n_dust = i1(); break;
        case 105: r->n_all = i1(); break;
        default: break;
    }
    // the per-disk, per-blob and per-planet rows (lines 49-93)
    auto each = [&](int n, auto set) {
        for (int k = 1; k < t && k - 1 < n; k++) set(k - 1, dat[k]);
    };
    ddx_disk* D = c->disks;
    ddx_blob* B = c->blobs;
    ddx_planet* P = c->planets;
    const int nd = c->n_disks, nb = c->n_blobs, np = c->n_planets;
    switch (i) {
        case 49: each(nd, [&](int k, const char* s) { scan(s, D[k].Rin); }); break;
        case 50: each(nd, [&](int k, const char* s) { scan(s, D[k].Rout); }); break;
        case 51: each(nd, [&](int k, const char* s) { scan(s, D[k].dhdr); }); break;
        case 52: each(nd, [&](int k, const char* s) { scan(s, D[k].sigmae); }); break;
        case 53: each(nd, [&](int k, const char* s) { scan(s, D[k].amax); }); break;
        case 54: each(nd, [&](int k, const char* s) { scan(s, D[k].mmax); }); break;
        case 55: each(nd, [&](int k, const char* s) { scan(s, D[k].amin); }); break;
        case 56: each(nd, [&](int k, const char* s) { scan(s, D[k].mmin); }); break;
        case 57: each(nd, [&](int k, const char* s) { scan(s, D[k].dmax); }); break;
        case 58: each(nd, [&](int k, const char* s) { scan(s, D[k].dmmax); }); break;
        case 59: each(nd, [&](int k, const char* s) { scan(s, D[k].eta); }); break;
        case 60: each(nd, [&](int k, const char* s) { scan(s, D[k].gammas); }); break;
        case 61: each(nd, [&](int k, const char* s) { scan(s, D[k].C); }); break;
        case 62: each(nd, [&](int k, const char* s) { scan(s, D[k].Mtot); }); break;
        case 63: each(nd, [&](int k, const char* s) { scan(s, D[k].Ngrav); }); break;
        case 64: each(nd, [&](int k, const char* s) { scan(s, D[k].Nsmall); }); break;
        case 65: each(nb, [&](int k, const char* s) { scan(s, B[k].a); }); break;
        case 66: each(nb, [&](int k, const char* s) { scan(s, B[k].ecc); }); break;
        case 67: each(nb, [&](int k, const char* s) { scan(s, B[k].inc); }); break;
        case 68: each(nb, [&](int k, const char* s) { scan(s, B[k].w); }); break;
        case 69: each(nb, [&](int k, const char* s) { scan(s, B[k].o); }); break;
        case 70: each(nb, [&](int k, const char* s) { scan(s, B[k].nu); }); break;
        case 71: each(nb, [&](int k, const char* s) { scan(s, B[k].sigma); }); break;
        case 72: each(nb, [&](int k, const char* s) { scan(s, B[k].amax); }); break;
        case 73: each(nb, [&](int k, const char* s) { scan(s, B[k].mmax); }); break;
        case 74: each(nb, [&](int k, const char* s) { scan(s, B[k].amin); }); break;
        case 75: each(nb, [&](int k, const char* s) { scan(s, B[k].mmin); }); break;
        case 76: each(nb, [&](int k, const char* s) { scan(s, B[k].dmax); }); break;
        case 77: each(nb, [&](int k, const char* s) { scan(s, B[k].dmmax); }); break;
        case 78: each(nb, [&](int k, const char* s) { scan(s, B[k].eta); }); break;
        case 79: each(nb, [&](int k, const char* s) { scan(s, B[k].C); }); break;
        case 80: each(nb, [&](int k, const char* s) { scan(s, B[k].Mtot); }); break;
        case 81: each(nb, [&](int k, const char* s) { scan(s, B[k].Ngrav); }); break;
        case 82: each(nb, [&](int k, const char* s) { scan(s, B[k].Nsmall); }); break;
        case 83: each(nb, [&](int k, const char* s) { scan(s, B[k].collcloud); }); break;
        case 84: each(nb, [&](int k, const char* s) { scan(s, B[k].vkepp); }); break;
        case 87: each(np, [&](int k, const char* s) { scan(s, P[k].x); }); break;
        case 88: each(np, [&](int k, const char* s) { scan(s, P[k].y); }); break;
        case 89: each(np, [&](int k, const char* s) { scan(s, P[k].z); }); break;
        case 90: each(np, [&](int k, const char* s) { scan(s, P[k].vx); }); break;
        case 91: each(np, [&](int k, const char* s) { scan(s, P[k].vy); }); break;
        case 92: each(np, [&](int k, const char* s) { scan(s, P[k].vz); }); break;
        case 93: each(np, [&](int k, const char* s) { scan(s, P[k].m); }); break;
        default: break;
    }
}

void put_be64(unsigned char* dst, double v) {
    uint64_t b;
    memcpy(&b, &v, 8);
    for (int k = 7; k >= 0; --k) {
        dst[k] = (unsigned char)(b & 0xff);
        b >>= 8;
    }
}

// One 80-character FITS header card.
void card(std::string& h, const char* text) {
    char c[81];
    snprintf(c, sizeof c, "%-80s", text);
    h.append(c, 80);
}

}  // namespace

extern "C" int ddx_dat_write(const char* path, const char* version, const ddx_param* p, const ddx_dat_run* run,
                             const ddx_host_state* s, const float* beta) {
    if (!path || !version || !p || !run || !s || !s->x || !s->y || !s->z || !s->vx || !s->vy || !s->vz || !s->N ||
        !s->m || !s->id || run->n_all < p->n_planets || (p->n_grid > 0 && !beta))
        return DDX_ERR_ARG;
    File fw(path, "wb");
    if (!fw.f) return DDX_ERR_IO;
    write_header(fw.f, version, p, run);
    fprintf(fw.f, "#Data: x[AU] y[AU] z[AU] vx[AU/yr] vy[AU/yr] vz[AU/yr] N m[kg] r[m] beta\n");
    fprintf(fw.f, "#Planets:\n");
    for (int i = 0; i < p->n_planets; i++)
        fprintf(fw.f, "% .8e % .8e % .8e % .8e % .8e % .8e %.12e %.8e %d\n", s->x[i], s->y[i], s->z[i], s->vx[i],
                s->vy[i], s->vz[i], 1.0, s->m[i] * kMSun / kGrav, s->id[i]);
    fprintf(fw.f, "#Bodies:\n");
    for (int i = p->n_planets; i < run->n_all; i++) {
        const double R = s->x[i] * s->x[i] + s->y[i] * s->y[i] + s->z[i] * s->z[i];
        if (R > run->Rmax * run->Rmax) fprintf(fw.f, "## ");
        if (R < p->rstar * p->rstar) fprintf(fw.f, "## ");
        const int id = s->id[i];
        // the reference reads beta[id] also for id = -1 (outside its table); 0 here
        const double b = (id >= 0 && id < p->n_grid) ? beta[id] : 0.0;
        fprintf(fw.f, "% .8e % .8e % .8e % .8e % .8e % .8e %.12e %.8e %.8e %.8e %d\n", s->x[i], s->y[i], s->z[i],
                s->vx[i], s->vy[i], s->vz[i], s->N[i], s->m[i] * kMSun / kGrav,
                pow(3.0 * s->m[i] * kMSun / kGrav / 4.0 / kPI / p->rho, 1.0 / 3.0), b, id);
    }
    return ferror(fw.f) ? DDX_ERR_IO : DDX_OK;
}

extern "C" int ddx_dat_read(const char* path, const char* version, ddx_param* p, ddx_dat_run* run,
                            ddx_host_state* s) {
    if (!path || !version || !p || !run) return DDX_ERR_ARG;
    const int nR = run->nR;          // inputs: the radius grid to check against, and the
    const double Rmax = run->Rmax;   // temperature table's outer radius (not in the file)
    memset(p, 0, sizeof(*p));
    memset(run, 0, sizeof(*run));
    run->nR = nR;
    run->Rmax = Rmax;
    File fr(path, "rb");
    if (!fr.f) {
        p->usage_code = 3;
        return DDX_ERR_IO;
    }
    const bool bodies = s && s->x && s->y && s->z && s->vx && s->vy && s->vz && s->N && s->m && s->id;
    std::vector<char> buf(2048);
    char* dat[64];
    double dtemp = 0;
    int itemp = 0;
    long long n = 0;   // bodies read
    try {
        int i = 0;
        while (!feof(fr.f)) {
            if (!fgets(buf.data(), (int)buf.size(), fr.f)) break;
            const int t = split(buf.data(), dat, 32);
            if (t == 0) continue;
            if (i <= 105) header_line(i, dat, t, version, p, run, dtemp, itemp);
            if (i == 105 && (!bodies || s->cap < run->n_all)) return DDX_OK;   // header only
            const bool planet = i >= 108 && i < 108 + p->n_planets;
            const bool body = i >= 108 + p->n_planets + 1;
            if (planet || body) {
                if (n >= run->n_all) throw Fail{DDX_ERR_RANGE, 0};
                const int off = strcmp(dat[0], "##") == 0 ? 1 : 0;
                double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
                for (int k = 0; k < 8; ++k) scan(k + off < t ? dat[k + off] : nullptr, v[k]);
                s->x[n] = v[0]; s->y[n] = v[1]; s->z[n] = v[2];
                s->vx[n] = v[3]; s->vy[n] = v[4]; s->vz[n] = v[5];
                s->N[n] = v[6];
                s->m[n] = v[7] * kGrav / kMSun;
                int id = -1;
                if (body) {
                    id = (int)round(log(v[7] / p->mmin) / p->f);
                    if (id > p->n_grid - 1) id = -1;
                }
                s->id[n] = id;
                ++n;
            }
            i++;
        }
    } catch (const Fail& e) {
        p->usage_code = e.code;
        return e.status;
    }
    if (bodies && n != run->n_all) return DDX_ERR_IO;   // a truncated file
    return DDX_OK;
}

extern "C" int ddx_sed_write(const char* path, const char* version, int n_wav, const double* w, const double* in,
                             const double* exc) {
    if (!path || !version || n_wav < 0 || (n_wav > 0 && (!w || !in || !exc))) return DDX_ERR_ARG;
    File fw(path, "wb");
    if (!fw.f) return DDX_ERR_IO;
    fprintf(fw.f, "#Calculated with DiskDyn Version %s\n", version);
    fprintf(fw.f, "#Wav[mu]\tFlux_star[Jy]\tFlux_exc[Jy]\n");
    for (int j = 0; j < n_wav; j++)
        fprintf(fw.f, "%.3f %.6e %.6e\n", w[j] * 1e6, in[j] * 1e26 * w[j] * w[j] / kCspeed, exc[j]);
    return ferror(fw.f) ? DDX_ERR_IO : DDX_OK;
}

extern "C" int ddx_fits_write(const char* path, const char* version, int xsize, int ysize, const double* F,
                              double wavelength_m, double fov_AU, double dist_m) {
    if (!path || !version || !F || xsize < 1 || ysize < 1 || !(dist_m > 0.0)) return DDX_ERR_ARG;
    const size_t npix = (size_t)xsize * ysize;
    double Ptot = 0;   // in the reference's summation order: y outer, x inner
    for (int y = 0; y < ysize; y++)
        for (int x = 0; x < xsize; x++) Ptot += F[(size_t)ysize * x + y];
    const int size = xsize >= ysize ? xsize : ysize;
    const float pxscale = (float)(fov_AU / dist_m * kPc / size);
    const float lambda = (float)(wavelength_m * 1e6);
    char t[96];
    std::string h;
    card(h, "SIMPLE  =                    T / file does conform to FITS standard");
    card(h, "BITPIX  =                  -64 / number of bits per data pixel");
    card(h, "NAXIS   =                    2 / number of data axes");
    snprintf(t, sizeof t, "NAXIS1  = %20d / length of data axis 1", xsize);
    card(h, t);
    snprintf(t, sizeof t, "NAXIS2  = %20d / length of data axis 2", ysize);
    card(h, t);
    card(h, "EXTEND  =                    T / FITS dataset may contain extensions");
    snprintf(t, sizeof t, "WAVELENG= %20.7G / [micron] Wavelength of dataset", (double)lambda);
    card(h, t);
    snprintf(t, sizeof t, "FLUX    = %20.15G / [Jy] Total flux detected", Ptot);
    card(h, t);
    snprintf(t, sizeof t, "PIXELSCA= %20.7G / [''/px] pixel scale of instrument setup", (double)pxscale);
    card(h, t);
    std::string v = "'";
    for (const char* c = version; *c && v.size() < 60; ++c) v += (*c == '\'') ? std::string("''") : std::string(1, *c);
    v += "'";
    while (v.size() < 10) v.insert(v.size() - 1, " ");
    snprintf(t, sizeof t, "VERSION = %-20s / DiskDyn version", v.c_str());
    card(h, t);
    card(h, "HISTORY Created with DiskDyn");
    const time_t now = time(nullptr);
    struct tm g;
    gmtime_r(&now, &g);
    snprintf(t, sizeof t, "DATE    = '%04d-%02d-%02dT%02d:%02d:%02d' / file creation date (YYYY-MM-DDThh:mm:ss UT)",
             g.tm_year + 1900, g.tm_mon + 1, g.tm_mday, g.tm_hour, g.tm_min, g.tm_sec);
    card(h, t);
    card(h, "END");
    h.append((2880 - h.size() % 2880) % 2880, ' ');
    // data: rows of x for each y (the transpose of the x-major image), big-endian
    std::vector<unsigned char> d(npix * 8);
    size_t k = 0;
    for (int y = 0; y < ysize; y++)
        for (int x = 0; x < xsize; x++, k += 8) put_be64(&d[k], F[(size_t)ysize * x + y]);
    d.resize(d.size() + (2880 - d.size() % 2880) % 2880, 0);
    File fw(path, "wb");
    if (!fw.f) return DDX_ERR_IO;
    if (fwrite(h.data(), 1, h.size(), fw.f) != h.size() || fwrite(d.data(), 1, d.size(), fw.f) != d.size())
        return DDX_ERR_IO;
    return DDX_OK;
}
