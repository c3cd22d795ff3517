// Host-side helpers shared by the readers of the reference's text files and by the
// set-up's two generators.
#pragma once

#include <vector>

#include "../../include/diskdyn_gb300_io.h"
#include "../../include/diskdyn_gb300_run.h"

namespace ddx_host {

// A run of consecutive bodies of the initial system that share their generator inputs:
// the gravitating bodies of one disk or blob, or the grains of one mass bin of one.
struct SetupSegment {
    int kind;            // 0 disk, 1 blob
    int j;               // its index
    int massive;         // 1: gravitating bodies, masses in SetupPlan::mass from mass_off
    int id;              // size bin of the grains, -1 for none
    long long first;     // state index of the first body
    long long count;
    long long mass_off;
    double m;            // grain mass x 4 pi^2, Msun
    double N;            // grains per tracer (1 for gravitating bodies)
    double beta;         // beta of the orbit draw (0 for none, and where the bin's is >= 0.5)
};

// Grid::setup's bodies (src/grid.cu:79-190) in its order: the planets, then the
// segments.  mass holds the gravitating bodies' masses of the getbod chain when asked for.
struct SetupPlan {
    std::vector<SetupSegment> seg;
    std::vector<double> mass;
    long long n_planets = 0, n_mass = 0, n_dust = 0, n_all = 0;
};

// The gravitating bodies' masses of a plan: none (counts only), the reference's getbod
// chain in its arithmetic (bit-exact on x86-64), or the same chain in double formed
// without cancellation (accurate to rounding, and fast everywhere; long double is software
// quad precision on Arm).
enum class Masses { none, reference, fast };

// Builds the plan of a parameter file after ddx_param_grid; beta (n_grid entries) may be
// null when only the counts are wanted.  Returns a DDX_* status.
int plan_setup(const ddx_param& p, double dmin, double dmax, const float* beta, Masses masses, SetupPlan& plan);

// The reference's tokeniser (tokenize_spaces with remove_quotes, src/read_in.cu:12-60):
// splits buf in place into at most `max` tokens at the separators '@', space, CR, LF and
// tab outside double quotes, then drops every double quote of each token.  Scanning stops
// once the max-th token has started, so that token runs to the end of the line.  tok needs
// room for max + 1 entries (the list ends with a null pointer).  Returns the token count.
int split(char* buf, char** tok, int max);

// Orbital elements to the Cartesian state about a central mass M, both masses times
// 4 pi^2 in Msun, with the central attraction reduced by the factor 1 - beta (coe2rv,
// src/functions.cu:6-46), expression for expression: a in AU, angles in radians.
void coe2rv(double M, double m, double a, double e, double i, double w, double o, double nu, double* x,
            double* y, double* z, double* vx, double* vy, double* vz, double beta);

// Grid::evolve's clock (src/grid.cu:344-437): the step size dt cut to end on the next
// output time or on t_end, and the outputs due after each step.
struct Clock {
    ddx_cadence c;
    double dt = 0.0, dttmp = 0.0, time = 0.0;
    void start(const ddx_cadence& cad, double dt_);
    bool running() const { return time < c.t_end; }
    // Advances the clock by the current step and returns the outputs now due as a mask of
    // 1 << DDX_OUT_SED, 1 << DDX_OUT_IMAGES, 1 << DDX_OUT_STATE, in that order of writing,
    // with the last-output times updated the way the reference updates them.
    int advance();
};

}  // namespace ddx_host
