// Optical-table and stellar-spectrum input on the host:
//  - ddx_optical_read: the Mie table file (add_optical_data, src/read_in.cu:419-505);
//  - ddx_spec_read: the stellar spectrum (add_specfile, src/read_in.cu:377-417);
//  - ddx_stellar_grid: the spectrum on the table wavelengths and the image wavelength
//    indices (interpolate_stellar_to_grid, src/functions.cu:302-336).
//
// The text is read the way the reference reads it (254-character fgets pieces, its
// tokeniser, sscanf's keep-the-old-value rule for tokens that are not numbers) and the
// arithmetic follows it operation for operation (compiled without floating-point
// contraction), so every value is the reference's to the bit.  Where the reference would
// read or write outside its arrays, these calls stop with an error or a documented guard.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../../include/diskdyn_gb300.h"
#include "../../include/diskdyn_gb300_io.h"
#include "ddx_host.h"

namespace {

constexpr double kAU = 1.49598e11;
constexpr int kLine = 255;   // the reference's fgets size

// sscanf "%lf" / "%d": the target keeps its value when the token does not start with a
// number (and a missing token converts nothing).
void scan(const char* s, double& v) {
    if (!s) return;
    char* e = nullptr;
    const double r = strtod(s, &e);
    if (e != s) v = r;
}

bool scan_ok(const char* s, double& v) {
    if (!s) return false;
    char* e = nullptr;
    const double r = strtod(s, &e);
    if (e == s) return false;
    v = r;
    return true;
}

void scan(const char* s, int& v) {
    if (!s) return;
    char* e = nullptr;
    const long r = strtol(s, &e, 10);
    if (e != s) v = (int)r;
}

struct File {
    FILE* f;
    explicit File(const char* p) : f(fopen(p, "rb")) {}
    ~File() {
        if (f) fclose(f);
    }
};

}  // namespace

extern "C" int ddx_optical_read(const char* path, ddx_optical_table* t, double* w, double* dmin, double* dmax) {
    if (!path || !t || !dmin || !dmax) return DDX_ERR_ARG;
    const bool header_only = (t->s == nullptr);
    if (!header_only && (!w || !t->Qabs || !t->Qsca || !t->Qpfunc)) return DDX_ERR_ARG;
    File fr(path);
    if (!fr.f) return DDX_ERR_IO;
    char buf[512];
    char* dat[16];
    int i = 0, j = 0, nw = 0, l = 0;
    int n_wav = 0, n_theta = 0, n_dust = 0;
    double dtemp = 0.0;
    int itemp = 0;
    while (!feof(fr.f)) {
        if (fgets(buf, kLine, fr.f) == nullptr) break;
        if (i == 0) {
            i++;
            continue;
        }
        const int tk = ddx_host::split(buf, dat, 12);
        if (i == 1) {                                     // the header line
            if (tk < 6) return DDX_ERR_ARG;
            scan(dat[1], itemp); n_wav = itemp;
            scan(dat[2], itemp); n_theta = itemp;
            scan(dat[3], itemp); n_dust = itemp;
            scan(dat[4], dtemp); *dmin = dtemp * 1e-6;
            scan(dat[5], dtemp); *dmax = dtemp * 1e-6;
            if (n_wav < 1 || n_theta < 1 || n_dust < 1) return DDX_ERR_ARG;
            if (header_only) {
                t->n_size = n_dust;
                t->n_wav = n_wav;
                t->n_theta = n_theta;
                return DDX_OK;
            }
            if (t->n_size != n_dust || t->n_wav != n_wav || t->n_theta != n_theta) return DDX_ERR_ARG;
        }
        const size_t per_size = (size_t)n_theta * n_wav;
        if (i > 1 && buf[0] == '#') {                     // a new grain size
            if (j > 0 && (nw != n_wav || (size_t)l * 10 != per_size)) return DDX_ERR_ARG;
            if (j >= n_dust || tk < 2) return DDX_ERR_ARG;
            scan(dat[1], dtemp);
            t->s[j] = dtemp * 1e-6;
            j++;
            nw = 0;
            l = 0;
        }
        if (i > 1 && buf[0] != '#' && tk == 3) {          // wavelength, Qabs, Qsca
            if (j == 0 || nw >= n_wav) return DDX_ERR_ARG;
            if (j == 1) {
                scan(dat[0], dtemp);
                w[nw] = dtemp * 1e-6;
            }
            scan(dat[1], dtemp);
            t->Qabs[(size_t)n_wav * (j - 1) + nw] = dtemp;
            scan(dat[2], dtemp);
            t->Qsca[(size_t)n_wav * (j - 1) + nw] = dtemp;
            nw++;
        }
        if (i > 1 && buf[0] != '#' && tk == 10) {         // ten phase-function values
            if (j == 0 || (size_t)l * 10 + 10 > per_size) return DDX_ERR_ARG;
            for (int c = 0; c < 10; ++c) {
                scan(dat[c], dtemp);
                t->Qpfunc[per_size * (j - 1) + (size_t)l * 10 + c] = dtemp;
            }
            l++;
        }
        i++;
    }
    if (i < 2) return DDX_ERR_ARG;
    if (j != n_dust || nw != n_wav || (size_t)l * 10 != (size_t)n_theta * n_wav) return DDX_ERR_ARG;
    return DDX_OK;
}

extern "C" int ddx_spec_read(const char* path, double rstar_AU, double dist_m, int* nspec, double* wvl, double* F,
                             int cap) {
    if (!path || !nspec) return DDX_ERR_ARG;
    File fr(path);
    if (!fr.f) return DDX_ERR_IO;
    // first pass counts, a second one fills when there is room
    const bool fill_wanted = wvl && F;
    for (int pass = 0; pass < 2; ++pass) {
        const bool fill = (pass == 1);
        if (fill) {
            if (!fill_wanted || cap < *nspec) return DDX_OK;
            rewind(fr.f);
        }
        char buf[512];
        char* dat[4];
        int i = 0;
        while (!feof(fr.f)) {
            if (fgets(buf, kLine, fr.f) == nullptr) break;
            if (buf[0] == '#') continue;
            if (ddx_host::split(buf, dat, 2) < 2) continue;
            double w = 0.0, f = 0.0;
            const bool ok_w = scan_ok(dat[0], w);
            const bool ok_f = scan_ok(dat[1], f);
            if (!(ok_w && ok_f)) continue;
            if (fill) {
                wvl[i] = w;
                F[i] = f * pow(rstar_AU * kAU, 2.0) / pow(dist_m, 2.0);
            }
            i++;
        }
        *nspec = i;
    }
    return DDX_OK;
}

extern "C" int ddx_stellar_grid(int n_wav, const double* w, int nspec, const double* spec_w, const double* spec_F,
                                int nwavs, const double* wavs, double* in, int* wj) {
    if (n_wav < 2 || nspec < 2 || nwavs < 0 || !w || !spec_w || !spec_F || !in) return DDX_ERR_ARG;
    if (nwavs > 0 && (!wavs || !wj)) return DDX_ERR_ARG;
    // The reference keeps one spectrum index for all table wavelengths: it walks forward
    // to the first point beyond w[j] and steps back by one afterwards.
    int ip = 0;
    for (int j = 0; j < n_wav; j++) {
        if (w[j] < spec_w[0]) {
            in[j] = 0.0;
        } else if (w[j] > spec_w[nspec - 1]) {
            in[j] = spec_F[nspec - 1] * pow(spec_w[nspec - 1] / w[j], 4.0);
        } else {
            while (ip < nspec - 1 && spec_w[ip] <= w[j]) ip++;
            const int im = ip - 1;
            if (spec_F[im] != 0 && spec_F[ip] != 0)
                in[j] = exp(log(spec_F[im]) +
                            log(w[j] / spec_w[im]) * log(spec_F[ip] / spec_F[im]) / log(spec_w[ip] / spec_w[im]));
            else
                in[j] = 0.0;
            ip--;
        }
    }
    for (int k = 0; k < nwavs; k++) {
        if (wavs[k] < w[0] || wavs[k] > w[n_wav - 1]) return DDX_ERR_RANGE;
        int i = 0;
        while (w[i] < wavs[k] && i < n_wav - 2) i++;
        wj[k] = i - 1;
    }
    return DDX_OK;
}
