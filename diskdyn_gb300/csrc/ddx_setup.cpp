// Start-of-run set-up on the host:
//  - ddx_param_grid: the optical size limits, the mass grid and the disk and blob number
//    constants (detminmax and confCdisks / confCblobs, src/read_in.cu:236-342);
//  - the set-up plan shared with the GPU generator: the order of Grid::setup's bodies
//    (src/grid.cu:79-190) as runs ("segments") of bodies with the same generator inputs,
//    the massive bodies' masses (getbod, src/functions.cu:234-239) and each mass bin's
//    mass, size-bin index and grains per tracer;
//  - ddx_setup_host: Grid::setup's generation with the reference's generator, ran3
//    (src/ran3.cu:12-48, the subtractive generator of Knuth as given in Numerical Recipes),
//    and its orbit draws genorb_disk / genorb_blob (src/functions.cu:157-232).
//
// Everything follows the reference operation for operation and is compiled without
// floating-point contraction, so on x86-64 the bodies are the reference's to the bit.
// The gravitating bodies' masses go through long double as in the reference (its getbod
// mixes long double and double), which is 80-bit on x86-64 and 128-bit on Arm.
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/diskdyn_gb300.h"
#include "../../include/diskdyn_gb300_io.h"
#include "../../include/diskdyn_gb300_setup.h"
#include "ddx_host.h"

namespace {

constexpr double kPI = 3.14159265358979323846;
constexpr double kPI2 = 6.28318530717958623200;   // the reference's literal (src/ddyn.cuh)
constexpr double kGrav = 4.0 * kPI * kPI;
constexpr double kMSun = 1.98892e30;
constexpr double kMgrid = 1.1;                     // mass ratio of neighbouring size bins

// ran3: Knuth's subtractive generator (Numerical Recipes' ran3), one state per run rather
// than the reference's function-static one.  The first draw seeds it from |seed|.
class Ran3 {
  public:
    explicit Ran3(long long seed) : seed_(seed) {}
    double next() {
        constexpr long long kBig = 1000000000, kSeed = 161803398;
        if (!started_) {
            started_ = true;
            long long mj = kSeed - (seed_ < 0 ? -seed_ : seed_);
            mj %= kBig;
            ma_[55] = mj;
            long long mk = 1;
            for (int i = 1; i <= 54; i++) {
                const int ii = (21 * i) % 55;
                ma_[ii] = mk;
                mk = mj - mk;
                if (mk < 0) mk += kBig;
                mj = ma_[ii];
            }
            for (int k = 1; k <= 4; k++)
                for (int i = 1; i <= 55; i++) {
                    ma_[i] -= ma_[1 + (i + 30) % 55];
                    if (ma_[i] < 0) ma_[i] += kBig;
                }
            inext_ = 0;
            inextp_ = 31;
        }
        if (++inext_ == 56) inext_ = 1;
        if (++inextp_ == 56) inextp_ = 1;
        long long mj = ma_[inext_] - ma_[inextp_];
        if (mj < 0) mj += kBig;
        ma_[inext_] = mj;
        return mj * (1.0 / kBig);
    }

  private:
    long long seed_;
    long long ma_[56] = {};
    int inext_ = 0, inextp_ = 0;
    bool started_ = false;
};

// N(0, 1) draws as the reference writes them, sqrt(-2 ln u1) cos(2 pi u2): the reference
// leaves the order of the two calls in one expression to its compiler, which draws the
// logarithm's number first.
double gauss(Ran3& r) {
    const double u1 = r.next();
    const double u2 = r.next();
    return sqrt(-2.0 * log(u1)) * cos(kPI2 * u2);
}

// getbod: the next massive body's mass (x 4 pi^2 / Msun) from the running upper limit mmax
// of the cumulative number N(>m) = C m^ome / ome, in the reference's mixed long double /
// double arithmetic.
void getbod(long double& mmax, double& m, double C, double ome) {
    const long double mmin = powl(powl(mmax, (long double)ome) - ome / C, (long double)(1.0 / ome));
    m = (double)(C * (powl(mmax, (long double)(1.0 + ome)) - powl(mmin, (long double)(1.0 + ome))) / (1.0 + ome) /
                 kMSun * kGrav);
    mmax = mmin;
}

// The same chain in double.  Consecutive masses are close, so the difference of the two
// powers is formed without cancellation: with r = mmin / mmax,
//   ln r = log1p(-(ome / C) mmax^-ome) / ome,
//   mmax^(1+ome) - mmin^(1+ome) = -mmax^(1+ome) expm1((1 + ome) ln r).
// ome = 0 keeps the direct form (the chain is degenerate there, as in the reference).
void getbod_fast(double& mmax, double& m, double C, double ome) {
    if (ome == 0.0) {
        const double mmin = pow(pow(mmax, ome) - ome / C, 1.0 / ome);
        m = C * (pow(mmax, 1.0 + ome) - pow(mmin, 1.0 + ome)) / (1.0 + ome) / kMSun * kGrav;
        mmax = mmin;
        return;
    }
    const double lr = log1p(-(ome / C) * pow(mmax, -ome)) / ome;
    m = C * (-pow(mmax, 1.0 + ome) * expm1((1.0 + ome) * lr)) / (1.0 + ome) / kMSun * kGrav;
    mmax = mmax * exp(lr);
}

void orbit_disk(const ddx_disk& d, double M, double m, double beta, Ran3& r, double* o6) {
    double e;
    do {
        e = gauss(r) * d.sigmae;
        if (e < 0) e = -e;
    } while (e >= 1.0);
    const double sem_a_min = d.Rin / (1.0 - e);
    const double sem_a_max = d.Rout / (1.0 + e);
    const double g = 2.0 + d.gammas;
    const double a = pow(r.next() * (pow(sem_a_max, g) - pow(sem_a_min, g)) + pow(sem_a_min, g), 1.0 / g);
    double i = gauss(r) * d.dhdr;
    if (i < 0) i = -i;
    const double nu = kPI2 * r.next();
    const double w = kPI2 * r.next();
    const double o = kPI2 * r.next();
    ddx_host::coe2rv(M, m, a, e, i, w, o, nu, o6, o6 + 1, o6 + 2, o6 + 3, o6 + 4, o6 + 5, beta);
}

void orbit_blob(const ddx_blob& b, double M, double m, double beta, Ran3& r, double* o6) {
    double a;
    do {
        a = b.a + gauss(r) * b.sigma;
    } while (a <= 0.0);
    const double nu = b.nu + gauss(r) * b.sigma / a;
    ddx_host::coe2rv(M, m, a, b.ecc, b.inc, b.w, b.o, nu, o6, o6 + 1, o6 + 2, o6 + 3, o6 + 4, o6 + 5, beta);
    if (b.collcloud == 0) {
        const double voff = b.vkepp * 0.01 * sqrt(o6[3] * o6[3] + o6[4] * o6[4] + o6[5] * o6[5]);
        const double costheta = -1.0 + 2.0 * r.next();
        const double sintheta = sqrt(1.0 - costheta * costheta);
        const double gamma = kPI2 * r.next();
        const double cosgamma = cos(gamma), singamma = sin(gamma);
        o6[3] += voff * sintheta * cosgamma;
        o6[4] += voff * sintheta * singamma;
        o6[5] += voff * costheta;
    }
}

bool plan_ok(const ddx_param* p) {
    return p && p->n_planets >= 1 && p->n_planets <= DDX_PARAM_MAX_PLANETS && p->n_disks >= 0 &&
           p->n_disks <= DDX_PARAM_MAX_DISKS && p->n_blobs >= 0 && p->n_blobs <= DDX_PARAM_MAX_BLOBS &&
           p->n_grid >= 1 && p->f > 0.0 && p->mmin > 0.0 && p->rho > 0.0;
}

}  // namespace

namespace ddx_host {

int plan_setup(const ddx_param& p, double dmin, double dmax, const float* beta, Masses masses, SetupPlan& plan) {
    if (!plan_ok(&p)) return DDX_ERR_ARG;
    plan = SetupPlan{};
    plan.n_planets = p.n_planets;
    long long at = p.n_planets;
    // gravitating bodies: one segment per disk, then per blob
    for (int kind = 0; kind < 2; kind++) {
        const int n = kind == 0 ? p.n_disks : p.n_blobs;
        for (int j = 0; j < n; j++) {
            const long long Ng = kind == 0 ? p.disks[j].Ngrav : p.blobs[j].Ngrav;
            if (Ng < 0) return DDX_ERR_ARG;
            if (Ng == 0) continue;
            SetupSegment s{};
            s.kind = kind;
            s.j = j;
            s.massive = 1;
            s.first = at;
            s.count = Ng;
            s.mass_off = (long long)plan.mass.size();
            s.id = -1;
            s.N = 1.0;
            s.beta = 0.0;
            const double C = kind == 0 ? p.disks[j].C : p.blobs[j].C;
            const double eta = kind == 0 ? p.disks[j].eta : p.blobs[j].eta;
            const double mtop = kind == 0 ? p.disks[j].mmax : p.blobs[j].mmax;
            if (masses == Masses::reference) {
                long double mmax = mtop;
                for (long long l = 0; l < Ng; l++) {
                    double m = 0.0;
                    getbod(mmax, m, C, 1.0 - eta);
                    plan.mass.push_back(m);
                }
            } else if (masses == Masses::fast) {
                double mmax = mtop;
                for (long long l = 0; l < Ng; l++) {
                    double m = 0.0;
                    getbod_fast(mmax, m, C, 1.0 - eta);
                    plan.mass.push_back(m);
                }
            }
            plan.seg.push_back(s);
            at += Ng;
            plan.n_mass += Ng;
        }
    }
    // grains: per disk, then per blob, one segment per mass bin of the grid
    for (int kind = 0; kind < 2; kind++) {
        const int n = kind == 0 ? p.n_disks : p.n_blobs;
        for (int j = 0; j < n; j++) {
            const double dmmax = kind == 0 ? p.disks[j].dmmax : p.blobs[j].dmmax;
            const double pmmin = kind == 0 ? p.disks[j].mmin : p.blobs[j].mmin;
            const double C = kind == 0 ? p.disks[j].C : p.blobs[j].C;
            const double eta = kind == 0 ? p.disks[j].eta : p.blobs[j].eta;
            const long long Nsmall = kind == 0 ? p.disks[j].Nsmall : p.blobs[j].Nsmall;
            const double mmax = p.mmin * exp(round(log(dmmax / p.mmin) / p.f) * p.f);
            const double mmin = p.mmin * exp(round(log(pmmin / p.mmin) / p.f) * p.f);
            const int Ngrid = (int)round(log(mmax / mmin) / log(kMgrid) + 1);
            const int Npg = (int)round((double)(Nsmall) / ((double)Ngrid));
            if (Ngrid < 1 || Npg < 0) return DDX_ERR_ARG;
            for (int l = 0; l < Ngrid && Npg > 0; l++) {
                double m = mmin * exp((double)l * p.f);
                const double size = pow(m * 3.0 / 4.0 / kPI / p.rho, 1.0 / 3.0);
                int id = (int)round(log(m / p.mmin) / p.f);
                if (size < dmin) id = -1;
                if (size - dmax > 1e-9) id = -1;
                if (id >= p.n_grid) return DDX_ERR_RANGE;   // the reference reads past its beta table
                const double in = mmin * exp(((double)l - 0.5) * p.f);
                const double ax = mmin * exp(((double)l + 0.5) * p.f);
                m *= kGrav / kMSun;
                double N;
                if (eta == 0) N = C * (ax - in);
                else if (eta == 1) N = C * log(ax / in);
                else N = C * (pow(ax, 1.0 - eta) - pow(in, 1.0 - eta)) / (1.0 - eta);
                double b = (id < 0 || !beta) ? 0.0 : beta[id];
                if (b >= 0.5) b = 0.0;
                SetupSegment s{};
                s.kind = kind;
                s.j = j;
                s.massive = 0;
                s.first = at;
                s.count = Npg;
                s.mass_off = -1;
                s.m = m;
                s.N = N / Npg;
                s.id = id;
                s.beta = b;
                plan.seg.push_back(s);
                at += Npg;
                plan.n_dust += Npg;
            }
        }
    }
    plan.n_all = at;
    return DDX_OK;
}

}  // namespace ddx_host

extern "C" int ddx_param_grid(ddx_param* p, double dmin, double dmax) {
    if (!p || !(dmin > 0.0) || !(dmax >= dmin) || !(p->rho > 0.0)) return DDX_ERR_ARG;
    const double kappa = 4.0 * kPI * p->rho / 3.0;
    // each disk's and blob's grain range clipped to the optical table's
    for (int i = 0; i < p->n_disks; i++) {
        ddx_disk& d = p->disks[i];
        if (d.amin < dmin) {
            d.amin = dmin;
            d.mmin = kappa * pow(d.amin, 3.0);
        }
        d.dmax = d.amax > dmax ? dmax : d.amax;
        d.dmmax = kappa * pow(d.dmax, 3.0);
    }
    for (int i = 0; i < p->n_blobs; i++) {
        ddx_blob& b = p->blobs[i];
        if (b.amin < dmin) {
            b.amin = dmin;
            b.mmin = kappa * pow(b.amin, 3.0);
        }
        b.dmax = b.amax > dmax ? dmax : b.amax;
        b.dmmax = kappa * pow(b.dmax, 3.0);
    }
    // the global range: the first disk's (else the first blob's, else the table's), widened
    // by every other disk and blob
    double amin, amax;
    if (p->n_disks > 0) {
        amin = p->disks[0].amin;
        amax = p->disks[0].dmax;
    } else if (p->n_blobs > 0) {
        amin = p->blobs[0].amin;
        amax = p->blobs[0].dmax;
    } else {
        amin = dmin;
        amax = dmax;
    }
    for (int i = 1; i < p->n_disks; i++) {
        if (p->disks[i].amin < amin) amin = p->disks[i].amin;
        if (p->disks[i].dmax > amax) amax = p->disks[i].dmax;
    }
    for (int i = 0; i < p->n_blobs; i++) {
        if (p->blobs[i].amin < amin) amin = p->blobs[i].amin;
        if (p->blobs[i].dmax > amax) amax = p->blobs[i].dmax;
    }
    p->amin = amin;
    p->amax = amax;
    p->mmin = kappa * pow(amin, 3.0);
    p->mmax = kappa * pow(amax, 3.0);
    p->n_grid = (int)(log(p->mmax / p->mmin) / log(kMgrid) + 1.0);
    p->f = log(p->mmax / p->mmin) / ((double)p->n_grid - 1.0);
    // number constants: the total mass over the integral of m^(1 - eta) between the limits
    for (int d = 0; d < p->n_disks; d++) {
        ddx_disk& k = p->disks[d];
        k.C = k.Mtot;
        if (k.eta == 1) k.C /= (k.mmax - k.mmin);
        else if (k.eta == 2) k.C /= log(k.mmax / k.mmin);
        else k.C /= (pow(k.mmax, 2.0 - k.eta) - pow(k.mmin, 2.0 - k.eta)) / (2.0 - k.eta);
    }
    for (int d = 0; d < p->n_blobs; d++) {
        ddx_blob& k = p->blobs[d];
        k.C = k.Mtot;
        if (k.eta == 1) k.C /= (k.mmax - k.mmin);
        else if (k.eta == 2) k.C /= log(k.mmax / k.mmin);
        else k.C /= (pow(k.mmax, 2.0 - k.eta) - pow(k.mmin, 2.0 - k.eta)) / (2.0 - k.eta);
    }
    return DDX_OK;
}

extern "C" int ddx_setup_count(const ddx_param* p, double dmin, double dmax, ddx_dat_run* run) {
    if (!p || !run) return DDX_ERR_ARG;
    ddx_host::SetupPlan plan;
    const int r = ddx_host::plan_setup(*p, dmin, dmax, nullptr, ddx_host::Masses::none, plan);
    if (r) return r;
    run->n_mass = (int)plan.n_mass;
    run->n_dust = (int)plan.n_dust;
    run->n_all = (int)plan.n_all;
    return DDX_OK;
}

extern "C" int ddx_setup_host(const ddx_param* p, double dmin, double dmax, const float* beta, long long seed,
                              ddx_host_state* s, ddx_dat_run* run) {
    if (!p || !beta || !s || !run) return DDX_ERR_ARG;
    if (!s->x || !s->y || !s->z || !s->vx || !s->vy || !s->vz || !s->N || !s->m || !s->id) return DDX_ERR_ARG;
    ddx_host::SetupPlan plan;
    int r = ddx_host::plan_setup(*p, dmin, dmax, beta, ddx_host::Masses::reference, plan);
    if (r) return r;
    if (s->cap < plan.n_all) return DDX_ERR_RANGE;
    for (int j = 0; j < p->n_planets; j++) {
        const ddx_planet& b = p->planets[j];
        s->x[j] = b.x; s->y[j] = b.y; s->z[j] = b.z;
        s->vx[j] = b.vx; s->vy[j] = b.vy; s->vz[j] = b.vz;
        s->N[j] = 1;
        s->m[j] = b.m;
        s->id[j] = -1;
    }
    Ran3 rng(seed);
    const double M = p->planets[0].m;
    double o6[6];
    for (const ddx_host::SetupSegment& g : plan.seg) {
        for (long long k = 0; k < g.count; k++) {
            const long long i = g.first + k;
            const double m = g.massive ? plan.mass[g.mass_off + k] : g.m;
            if (g.kind == 0) orbit_disk(p->disks[g.j], M, m, g.beta, rng, o6);
            else orbit_blob(p->blobs[g.j], M, m, g.beta, rng, o6);
            s->x[i] = o6[0]; s->y[i] = o6[1]; s->z[i] = o6[2];
            s->vx[i] = o6[3]; s->vy[i] = o6[4]; s->vz[i] = o6[5];
            s->N[i] = g.N;
            s->m[i] = m;
            s->id[i] = g.id;
        }
    }
    run->n_mass = (int)plan.n_mass;
    run->n_dust = (int)plan.n_dust;
    run->n_all = (int)plan.n_all;
    return DDX_OK;
}
