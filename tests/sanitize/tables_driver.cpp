// Builds the library's host-side tables (grids, Landau weight factors,
// conservation rows and their inverse Gram matrix, DFT factors, pair and
// window offsets, the LDG band matrix and its LU factors, the dense inverse
// of the Poisson matrix) for small cases; built with AddressSanitizer and
// UndefinedBehaviorSanitizer by tests/test_host_sanitizers.py, which fails
// on any sanitizer report or non-zero exit.
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "lp_tables.h"

static int run(int nx1, int nx2, int nv, int n, double lv, unsigned fixes, int precision, int linear_ei) {
    lp_params p{};
    p.nx1 = nx1; p.nx2 = nx2; p.nv = nv; p.n = n; p.lv = lv; p.lx = 4.0 * 3.14159265358979323846;
    p.nu = 0.05; p.dt = 0.01; p.a_amp = 0.3; p.k_wave = 0.5; p.fixes = fixes; p.precision = precision;
    p.linear_ei = linear_ei;
    lp::Tables t;
    std::string err;
    if (lp::build_tables(p, t, err) != LP_OK) {
        std::fprintf(stderr, "build_tables(%d, %d, %d, %d): %s\n", nx1, nx2, nv, n, err.c_str());
        return 1;
    }
    double s = 0.;
    for (int xi = 0; xi < t.n3; xi += 97)
        for (int om = 0; om < t.n3; om += 89) s += lp::weight_host(t, xi, om);
    for (double x : t.c1) s += x;
    for (double x : t.tfac) s += x;
    std::vector<double> inv;
    lp::poisson_inverse(t.pois, inv);
    for (double x : inv) s += x;
    return std::isfinite(s) ? 0 : 2;
}

int main() {
    int r = 0;
    r |= run(2, 2, 4, 8, 5.25, 0u, LP_PREC_FP64, 0);
    r |= run(4, 1, 6, 8, 5.25, LP_FIX_DEFAULT, LP_PREC_MIXED, 0);
    r |= run(3, 1, 4, 16, 6.0, LP_FIX_DEFAULT, LP_PREC_MIXED, 0);
    r |= run(2, 1, 4, 24, 6.0, LP_FIX_DEFAULT, LP_PREC_FP64, 0);
    r |= run(2, 2, 4, 8, 5.25, LP_FIX_F2 | LP_FIX_F3, LP_PREC_FP64, 1);
    r |= run(5, 3, 5, 6, 5.25, LP_FIX_DEFAULT, LP_PREC_FP64, 0);
    if (r) {
        std::fprintf(stderr, "tables driver: status %d\n", r);
        return r;
    }
    std::printf("ok\n");
    return 0;
}
