// ORACLE -- test infrastructure.  Runs the reference's own optics set-up on a Mie table
// file and a stellar spectrum file: add_optical_data and add_specfile (src/read_in.cu:377-505),
// then interpolate_dust_to_grid, interpolate_stellar_to_grid and calculate_beta
// (src/functions.cu:243-388), in the order Grid::setup calls them (src/grid.cu:74-76), all
// compiled unmodified.  Built with param_dump by oracle/ref/build_param_ref.py.
//
// optics_dump TABLE SPEC OUT n_grid radQ SWQ amin amax kqe rho dist rstar mstar mloss vsw wav...
// (reals in any strtod form, hex floats included; SI units as the reference stores them).
// OUT (little-endian binary): int32 n_dust n_wav n_theta nspec; float64 dmin dmax;
// float64 s[n_dust] w[n_wav] Qabs[n_dust*n_wav] Qsca[n_dust*n_wav] Qpfunc[n_dust*n_theta*n_wav]
// spec_w[nspec] spec_F[nspec] (as read), then float64 in[n_wav]; int32 wj[nwavs];
// float64 s[n_grid]; float32 q[n_grid]; float64 Qabs[n_grid*n_wav] Qsca[n_grid*n_wav]
// Qpfunc[n_grid*n_theta*n_wav]; float32 beta[n_grid] betasw[n_grid]; float64 Lum betaswconst.
#include <stdio.h>
#include <stdlib.h>
#include "ddyn.cuh"

__constant__ double size[nsize];
__constant__ float beta[nsize];
__constant__ float betasw[nsize];
__constant__ float q[nsize];
__device__ double doubletmp;
configdata cconfig;
cudadata ccuda;
cudaconf* prop;

void add_optical_data();
void add_specfile();
void interpolate_dust_to_grid();
void interpolate_stellar_to_grid();
void calculate_beta();

int main(int argc, char** argv) {
    if (argc < 17) return 2;
    configdata* c = &cconfig;
    c->comp = argv[1];
    c->specfile = argv[2];
    c->n_grid = atoi(argv[4]);
    c->radQ = atoi(argv[5]);
    c->SWQ = atoi(argv[6]);
    c->amin = strtod(argv[7], NULL);
    c->amax = strtod(argv[8], NULL);
    c->kqe = strtod(argv[9], NULL);
    c->rho = strtod(argv[10], NULL);
    c->dist = strtod(argv[11], NULL);
    c->rstar = strtod(argv[12], NULL);
    c->n_planets = 1;
    c->planets = (planet_cart*)calloc(1, sizeof(planet_cart));
    c->planets[0].m = strtod(argv[13], NULL);
    c->mloss = strtod(argv[14], NULL);
    c->vsw = strtod(argv[15], NULL);
    c->nwavs = argc - 16;
    c->wavs = (double*)malloc(sizeof(double) * c->nwavs);
    for (int k = 0; k < c->nwavs; ++k) c->wavs[k] = strtod(argv[16 + k], NULL);
    c->wj = (int*)malloc(sizeof(int) * c->nwavs);

    add_optical_data();
    add_specfile();

    FILE* o = fopen(argv[3], "wb");
    if (!o) return 4;
    const size_t nd = c->n_dust, nw = c->n_wav, nt = c->n_theta;
    int h[4] = {c->n_dust, c->n_wav, c->n_theta, c->nspec};
    fwrite(h, sizeof(int), 4, o);
    fwrite(&c->dmin, sizeof(double), 1, o);
    fwrite(&c->dmax, sizeof(double), 1, o);
    fwrite(c->s, sizeof(double), nd, o);
    fwrite(c->w, sizeof(double), nw, o);
    fwrite(c->Qabs, sizeof(double), nd * nw, o);
    fwrite(c->Qsca, sizeof(double), nd * nw, o);
    fwrite(c->Qpfunc, sizeof(double), nd * nt * nw, o);
    for (int k = 0; k < c->nspec; ++k) fwrite(&c->spec[k].wvl, sizeof(double), 1, o);
    for (int k = 0; k < c->nspec; ++k) fwrite(&c->spec[k].F, sizeof(double), 1, o);

    interpolate_dust_to_grid();
    interpolate_stellar_to_grid();
    calculate_beta();

    const size_t ng = c->n_grid;
    fwrite(c->in, sizeof(double), nw, o);
    fwrite(c->wj, sizeof(int), c->nwavs, o);
    fwrite(c->s, sizeof(double), ng, o);
    fwrite(c->q, sizeof(float), ng, o);
    fwrite(c->Qabs, sizeof(double), ng * nw, o);
    fwrite(c->Qsca, sizeof(double), ng * nw, o);
    fwrite(c->Qpfunc, sizeof(double), ng * nt * nw, o);
    fwrite(c->beta, sizeof(float), ng, o);
    fwrite(c->betasw, sizeof(float), ng, o);
    fwrite(&c->Lum, sizeof(double), 1, o);
    fwrite(&c->betaswconst, sizeof(double), 1, o);
    fclose(o);
    return 0;
}
