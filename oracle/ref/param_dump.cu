// ORACLE -- test infrastructure.  Runs the reference's own parameter-file parser
// (read_in_param, src/read_in.cu, compiled unmodified with its helpers) on one file and
// prints what it set as JSON, every double as a hexadecimal float string so a comparison
// can be exact.  Built by oracle/ref/build_param_ref.py into oracle/_ref/param_dump.
//
// The definitions below are the globals the reference's main translation unit provides
// (src/ddyn.cu:25-33): the configuration and the constant-memory tables it declares.
#include <stdio.h>
#include "ddyn.cuh"

__constant__ double size[nsize];
__constant__ float beta[nsize];
__constant__ float betasw[nsize];
__constant__ float q[nsize];
__device__ double doubletmp;
configdata cconfig;
cudadata ccuda;
cudaconf* prop;

int read_in_param(char* param);
int read_in_model(char* model, const char* ver);

static void hexd(const char* key, double v, bool comma = true) { printf("\"%s\": \"%a\"%s", key, v, comma ? ", " : ""); }
static void str(const char* key, const char* s, bool comma = true) {
    printf("\"%s\": \"%s\"%s", key, s ? s : "", comma ? ", " : "");
}

// param_dump <file.param>             : read_in_param
// param_dump -m <file.dat> <version>   : read_in_model (the data-file header), plus the
//                                        fields only a data file sets
int main(int argc, char** argv) {
    if (argc < 2) return 2;
    const bool model = argc >= 4 && argv[1][0] == '-' && argv[1][1] == 'm';
    if (model) read_in_model(argv[2], argv[3]);
    else read_in_param(argv[1]);
    const configdata* c = &cconfig;
    printf("{");
    if (model) {
        hexd("amin", c->amin); hexd("amax", c->amax); hexd("mmin", c->mmin); hexd("mmax", c->mmax);
        hexd("f", c->f);
        printf("\"n_grid\": %d, \"n_wav\": %d, \"n_theta\": %d, \"n_dust\": %d, ", c->n_grid, c->n_wav, c->n_theta,
               c->n_dust);
        printf("\"disks_extra\": [");
        for (int k = 0; k < c->n_disks; ++k)
            printf("[\"%a\", \"%a\", \"%a\"]%s", c->disks[k].dmax, c->disks[k].dmmax, c->disks[k].C,
                   k + 1 < c->n_disks ? ", " : "");
        printf("], \"blobs_extra\": [");
        for (int k = 0; k < c->n_blobs; ++k)
            printf("[\"%a\", \"%a\", \"%a\"]%s", c->blobs[k].dmax, c->blobs[k].dmmax, c->blobs[k].C,
                   k + 1 < c->n_blobs ? ", " : "");
        printf("], ");
    }
    printf("\"verb\": %d, \"gpuid\": %d, \"gl\": %d, ", c->verb, c->gpuid, c->gl);
    hexd("t_gl", c->t_gl); hexd("t_write", c->t_write); hexd("t_fits", c->t_fits); hexd("t_sed", c->t_sed);
    hexd("t_end", c->t_end);
    printf("\"n_step\": %d, ", c->n_step);
    str("sptype", c->sptype);
    hexd("teff", c->teff); hexd("rstar", c->rstar); hexd("Bstar", c->Bstar); hexd("Wz", c->Wz);
    hexd("mloss", c->mloss); hexd("vsw", c->vsw);
    hexd("dist", c->dist); hexd("fov", c->fov); hexd("PA", c->PA); hexd("inc", c->inc);
    hexd("longitude", c->longitude);
    printf("\"xsize\": %d, \"ysize\": %d, ", c->xsize, c->ysize);
    printf("\"wavs\": [");
    for (int k = 0; k < c->nwavs; ++k) printf("\"%a\"%s", c->wavs[k], k + 1 < c->nwavs ? ", " : "");
    printf("], ");
    str("specfile", c->specfile);
    printf("\"radQ\": %d, \"SWQ\": %d, \"FLQ\": %d, ", c->radQ, c->SWQ, c->FLQ);
    printf("\"planets\": [");
    for (int k = 0; k < c->n_planets; ++k) {
        const planet_cart& b = c->planets[k];
        printf("[\"%a\", \"%a\", \"%a\", \"%a\", \"%a\", \"%a\", \"%a\"]%s", b.x, b.y, b.z, b.vx, b.vy, b.vz, b.m,
               k + 1 < c->n_planets ? ", " : "");
    }
    printf("], ");
    hexd("rho", c->rho); hexd("kqe", c->kqe);
    str("comp", c->comp);
    printf("\"disks\": [");
    for (int k = 0; k < c->n_disks; ++k) {
        const diskconf& d = c->disks[k];
        printf("{\"Rin\": \"%a\", \"Rout\": \"%a\", \"dhdr\": \"%a\", \"sigmae\": \"%a\", \"amax\": \"%a\", "
               "\"mmax\": \"%a\", \"amin\": \"%a\", \"mmin\": \"%a\", \"eta\": \"%a\", \"gammas\": \"%a\", "
               "\"Mtot\": \"%a\", \"Ngrav\": %ld, \"Nsmall\": %ld}%s",
               d.Rin, d.Rout, d.dhdr, d.sigmae, d.amax, d.mmax, d.amin, d.mmin, d.eta, d.gammas, d.Mtot, d.Ngrav,
               d.Nsmall, k + 1 < c->n_disks ? ", " : "");
    }
    printf("], ");
    printf("\"blobs\": [");
    for (int k = 0; k < c->n_blobs; ++k) {
        const blobconf& b = c->blobs[k];
        printf("{\"a\": \"%a\", \"ecc\": \"%a\", \"inc\": \"%a\", \"w\": \"%a\", \"o\": \"%a\", \"nu\": \"%a\", "
               "\"sigma\": \"%a\", \"amax\": \"%a\", \"mmax\": \"%a\", \"amin\": \"%a\", \"mmin\": \"%a\", "
               "\"eta\": \"%a\", \"Mtot\": \"%a\", \"vkepp\": \"%a\", \"Ngrav\": %ld, \"Nsmall\": %ld, "
               "\"collcloud\": %d}%s",
               b.a, b.ecc, b.inc, b.w, b.o, b.nu, b.sigma, b.amax, b.mmax, b.amin, b.mmin, b.eta, b.Mtot, b.vkepp,
               b.Ngrav, b.Nsmall, b.collcloud, k + 1 < c->n_blobs ? ", " : "");
    }
    printf("], ");
    str("name_stub", c->name_stub, false);
    printf("}\n");
    return 0;
}
