// ORACLE -- test infrastructure.  Runs the reference's own start-of-run set-up on a
// parameter file, a Mie table file and a spectrum file, in the order its main program and
// Grid::setup run them (src/ddyn.cu:80-101, src/grid.cu:68-166): read_in_param,
// add_optical_data, detminmax, confCdisks, confCblobs, add_specfile,
// interpolate_dust_to_grid, interpolate_stellar_to_grid, calculate_beta, then the body
// generation of Grid::setup with ran3 seeded at -2: planets, the gravitating bodies of each
// disk and blob (getbod + genorb_disk / genorb_blob), and the grains of each disk and blob
// on the mass grid.  The reference's functions are compiled unmodified; the generation
// loop is restated here (src/grid.cu:79-190) because Grid::setup also allocates GPU
// memory.  Built by oracle/ref/build_param_ref.py.
//
// setup_dump PARAM TABLE SPEC OUT
// OUT (little-endian): int32 n_all n_mass n_dust n_grid n_disks n_blobs; float64 amin amax
// mmin mmax f dmin dmax; per disk float64 amin mmin dmax dmmax C; per blob the same five;
// float32 beta[n_grid]; float64 x y z vx vy vz N m [n_all]; int32 id[n_all].
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <vector>
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
void add_optical_data();
void add_specfile();
void detminmax();
void confCdisks();
void confCblobs();
void interpolate_dust_to_grid();
void interpolate_stellar_to_grid();
void calculate_beta();
void getbod(long double* mmax, double* m, double C, double ome);
void genorb_disk(int j, double m, long* rseed, double* x, double* y, double* z, double* vx, double* vy, double* vz,
                 int id);
void genorb_blob(int j, double m, long* rseed, double* x, double* y, double* z, double* vx, double* vy, double* vz,
                 int id);

struct Host {
    std::vector<double> x, y, z, vx, vy, vz, N, m;
    std::vector<int> id;
    void add(double x_, double y_, double z_, double vx_, double vy_, double vz_, double N_, double m_, int id_) {
        x.push_back(x_); y.push_back(y_); z.push_back(z_);
        vx.push_back(vx_); vy.push_back(vy_); vz.push_back(vz_);
        N.push_back(N_); m.push_back(m_); id.push_back(id_);
    }
};

int main(int argc, char** argv) {
    if (argc < 5) return 2;
    configdata* cfg = &cconfig;
    read_in_param(argv[1]);
    cfg->comp = argv[2];
    cfg->specfile = argv[3];
    add_optical_data();
    detminmax();
    confCdisks();
    confCblobs();
    add_specfile();
    interpolate_dust_to_grid();
    interpolate_stellar_to_grid();
    calculate_beta();

    // Grid::setup, src/grid.cu:79-190
    long seed = -2;
    double x, y, z, vx, vy, vz, N, m;
    int n_mass = 0, n_dust = 0;
    for (int j = 0; j < cfg->n_disks; j++) n_mass += cfg->disks[j].Ngrav;
    for (int j = 0; j < cfg->n_blobs; j++) n_mass += cfg->blobs[j].Ngrav;
    Host h;
    for (int j = 0; j < cfg->n_planets; j++)
        h.add(cfg->planets[j].x, cfg->planets[j].y, cfg->planets[j].z, cfg->planets[j].vx, cfg->planets[j].vy,
              cfg->planets[j].vz, 1, cfg->planets[j].m, -1);
    for (int j = 0; j < cfg->n_disks; j++) {
        long double mmax = cfg->disks[j].mmax;
        for (int l = 0; l < cfg->disks[j].Ngrav; l++) {
            getbod(&mmax, &m, cfg->disks[j].C, 1.0 - cfg->disks[j].eta);
            genorb_disk(j, m, &seed, &x, &y, &z, &vx, &vy, &vz, -1);
            h.add(x, y, z, vx, vy, vz, 1, m, -1);
        }
    }
    for (int j = 0; j < cfg->n_blobs; j++) {
        long double mmax = cfg->blobs[j].mmax;
        for (int l = 0; l < cfg->blobs[j].Ngrav; l++) {
            getbod(&mmax, &m, cfg->blobs[j].C, 1.0 - cfg->blobs[j].eta);
            genorb_blob(j, m, &seed, &x, &y, &z, &vx, &vy, &vz, -1);
            h.add(x, y, z, vx, vy, vz, 1, m, -1);
        }
    }
    for (int pop = 0; pop < 2; pop++) {
        const int n = pop == 0 ? cfg->n_disks : cfg->n_blobs;
        for (int j = 0; j < n; j++) {
            const double dmmax = pop == 0 ? cfg->disks[j].dmmax : cfg->blobs[j].dmmax;
            const double pmmin = pop == 0 ? cfg->disks[j].mmin : cfg->blobs[j].mmin;
            const double C = pop == 0 ? cfg->disks[j].C : cfg->blobs[j].C;
            const double eta = pop == 0 ? cfg->disks[j].eta : cfg->blobs[j].eta;
            const long Nsmall = pop == 0 ? cfg->disks[j].Nsmall : cfg->blobs[j].Nsmall;
            double mmax = cfg->mmin * exp(round(log(dmmax / cfg->mmin) / cfg->f) * cfg->f);
            double mmin = cfg->mmin * exp(round(log(pmmin / cfg->mmin) / cfg->f) * cfg->f);
            int Ngrid = round(log(mmax / mmin) / log(mgrid) + 1);
            int Npg = round((double)(Nsmall) / ((double)Ngrid));
            n_dust += Npg * Ngrid;
            for (int l = 0; l < Ngrid; l++) {
                m = mmin * exp((double)l * cfg->f);
                double size = pow(m * 3.0 / 4.0 / PI / cfg->rho, 1.0 / 3.0);
                int id = round(log(m / cfg->mmin) / cfg->f);
                if (size < cfg->dmin) id = -1;
                if (size - cfg->dmax > 1e-9) id = -1;
                double in = mmin * exp(((double)l - 0.5) * cfg->f);
                double ax = mmin * exp(((double)l + 0.5) * cfg->f);
                m *= Grav / MSun;
                if (eta == 0) N = C * (ax - in);
                else if (eta == 1) N = C * log(ax / in);
                else N = C * (pow(ax, 1.0 - eta) - pow(in, 1.0 - eta)) / (1.0 - eta);
                for (int k = 0; k < Npg; k++) {
                    if (pop == 0) genorb_disk(j, m, &seed, &x, &y, &z, &vx, &vy, &vz, id);
                    else genorb_blob(j, m, &seed, &x, &y, &z, &vx, &vy, &vz, id);
                    h.add(x, y, z, vx, vy, vz, N / Npg, m, id);
                }
            }
        }
    }

    FILE* o = fopen(argv[4], "wb");
    if (!o) return 4;
    const int n_all = (int)h.x.size();
    int hd[6] = {n_all, n_mass, n_dust, cfg->n_grid, cfg->n_disks, cfg->n_blobs};
    fwrite(hd, sizeof(int), 6, o);
    double g[7] = {cfg->amin, cfg->amax, cfg->mmin, cfg->mmax, cfg->f, cfg->dmin, cfg->dmax};
    fwrite(g, sizeof(double), 7, o);
    for (int j = 0; j < cfg->n_disks; j++) {
        double v[5] = {cfg->disks[j].amin, cfg->disks[j].mmin, cfg->disks[j].dmax, cfg->disks[j].dmmax,
                       cfg->disks[j].C};
        fwrite(v, sizeof(double), 5, o);
    }
    for (int j = 0; j < cfg->n_blobs; j++) {
        double v[5] = {cfg->blobs[j].amin, cfg->blobs[j].mmin, cfg->blobs[j].dmax, cfg->blobs[j].dmmax,
                       cfg->blobs[j].C};
        fwrite(v, sizeof(double), 5, o);
    }
    fwrite(cfg->beta, sizeof(float), cfg->n_grid, o);
    const std::vector<double>* cols[8] = {&h.x, &h.y, &h.z, &h.vx, &h.vy, &h.vz, &h.N, &h.m};
    for (auto c : cols) fwrite(c->data(), sizeof(double), n_all, o);
    fwrite(h.id.data(), sizeof(int), n_all, o);
    fclose(o);
    return 0;
}
