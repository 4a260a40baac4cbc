// Drop-in replacements of the reference's hot-path routines over the C ABI.
// See lp_dropin.h.  The globals below are the reference's
// (source/LP_ompi_1.cpp:20-103, source/PoissonVariables.cpp), defined by the
// program that links this file.
#include "lp_dropin.h"

#include <cstdio>
#include <cstring>
#include <vector>

extern int Nx, Nv, N, M;
extern int size_v, size_ft, chunk_Nx;
extern double Lx, Lv, nu, dt, A_amp, k_wave;
extern double **C1, **C2;
extern double CCt[5 * 5];
extern std::vector<double> IE_X, IXE_X, IYE_X, IXXE_X, IXYE_X, IYYE_X;
extern std::vector<double> IE_Y, IXE_Y, IYE_Y, IXXE_Y, IXYE_Y, IYYE_Y;
extern std::vector<double> SE_X, SE_Y;

namespace {

lp_ctx *g_ctx = nullptr;
lp_params g_prm{};
unsigned g_fixes = 0;
lp_status g_status = LP_OK;

bool same(const lp_params &a, const lp_params &b) { return std::memcmp(&a, &b, sizeof(a)) == 0; }

// Context for the current globals (the reference's Nx x Nx grid).
lp_ctx *ctx() {
    lp_params p{};
    p.nx1 = Nx; p.nx2 = Nx; p.nv = Nv; p.n = N;
    p.lv = Lv; p.lx = Lx; p.nu = nu; p.dt = dt; p.a_amp = A_amp; p.k_wave = k_wave;
    p.fixes = g_fixes; p.precision = LP_PREC_FP64;
    if (g_ctx && same(p, g_prm)) return g_ctx;
    if (g_ctx) lp_ctx_destroy(g_ctx);
    g_ctx = nullptr;
    g_status = lp_ctx_create(&p, &g_ctx);
    if (g_status != LP_OK) {
        fprintf(stderr, "lp_dropin: lp_ctx_create failed (%d)\n", (int)g_status);
        g_ctx = nullptr;
        return nullptr;
    }
    g_prm = p;
    return g_ctx;
}

bool check(lp_status s, const char *what) {
    g_status = s;
    if (s != LP_OK) fprintf(stderr, "lp_dropin: %s failed: %s\n", what, g_ctx ? lp_last_error(g_ctx) : "");
    return s == LP_OK;
}

size_t state_len() { return (size_t)Nx * Nx * Nv * Nv * Nv * 7; }

void store_fields(const std::vector<double> &fl) {
    const size_t nc = (size_t)Nx * Nx;
    std::vector<double> *dst[14] = {&IE_X, &IXE_X, &IYE_X, &IXXE_X, &IXYE_X, &IYYE_X, &IE_Y,
                                    &IXE_Y, &IYE_Y, &IXXE_Y, &IXYE_Y, &IYYE_Y, &SE_X, &SE_Y};
    for (int a = 0; a < 14; ++a) dst[a]->assign(fl.begin() + a * nc, fl.begin() + (a + 1) * nc);
}

}  // namespace

extern "C" void lp_dropin_set_fixes(unsigned fixes) { g_fixes = fixes; }
extern "C" lp_status lp_dropin_last_status(void) { return g_status; }

void fft3D(fftw_complex *in, fftw_complex *out) {
    lp_ctx *c = ctx();
    if (c) check(lp_fft3d(c, &in[0][0], &out[0][0]), "fft3D");
}

void FS(fftw_complex *in, fftw_complex *out) {
    lp_ctx *c = ctx();
    if (c) check(lp_fs(c, &in[0][0], &out[0][0]), "FS");
}

// ComputeQ (source/collisionRoutines_1.cpp:739-822); the weights live on the
// device, so conv_weights is not read.
void ComputeQ(double *f, fftw_complex *qHat, double **conv_weights) {
    (void)conv_weights;
    lp_ctx *c = ctx();
    if (c) check(lp_compute_q(c, f, &qHat[0][0]), "ComputeQ");
}

void conserveAllMoments(fftw_complex *qHat) {
    lp_ctx *c = ctx();
    if (c) check(lp_conserve(c, &qHat[0][0]), "conserveAllMoments");
}

// RK4 (source/collisionRoutines_1.cpp:824-906): writes the cell's 5*size_v
// coefficients at dU[(l % chunk_Nx) * size_v * 5].
void RK4(double *f, int l, fftw_complex *qHat, double **conv_weights, std::vector<double> &U_vals, double *dU) {
    (void)conv_weights;
    lp_ctx *c = ctx();
    if (!c) return;
    if (!check(lp_set_state(c, U_vals.data(), state_len()), "RK4 state upload")) return;
    check(lp_rk4_cell(c, f, l, &qHat[0][0], dU + (size_t)(l % chunk_Nx) * size_v * 5), "RK4");
}

// setInit_spectral (source/SetInit_1.cpp:143-163): f[i] for i < Nx.
void setInit_spectral(std::vector<double> &U_vals, double **f) {
    lp_ctx *c = ctx();
    if (!c) return;
    if (!check(lp_set_state(c, U_vals.data(), state_len()), "setInit_spectral state upload")) return;
    const int ncol = (g_fixes & LP_FIX_F3) ? Nx * Nx : Nx;
    std::vector<double> all((size_t)ncol * size_ft);
    if (!check(lp_nodes(c, all.data()), "setInit_spectral")) return;
    for (int i = 0; i < Nx; ++i) std::memcpy(f[i], all.data() + (size_t)i * size_ft, sizeof(double) * size_ft);
}

void generate_conv_weights(double **conv_weights) {
    lp_ctx *c = ctx();
    if (!c || !conv_weights) return;
    for (int r = 0; r < size_ft; ++r)
        if (!check(lp_weights_rows(c, r, r + 1, conv_weights[r]), "generate_conv_weights")) return;
}

// createCCtAndPivot (source/conservationRoutines.cpp:133-209): C1, C2 rows and
// the inverse Gram matrix into the reference's globals.
void createCCtAndPivot() {
    lp_ctx *c = ctx();
    if (!c) return;
    std::vector<double> c1((size_t)5 * size_ft), c2((size_t)5 * size_ft);
    if (!check(lp_conservation_rows(c, c1.data(), c2.data(), CCt), "createCCtAndPivot")) return;
    for (int i = 0; i < M && i < 5; ++i) {
        if (C1 && C1[i]) std::memcpy(C1[i], c1.data() + (size_t)i * size_ft, sizeof(double) * size_ft);
        if (C2 && C2[i]) std::memcpy(C2[i], c2.data() + (size_t)i * size_ft, sizeof(double) * size_ft);
    }
}

// pois2d (source/PoissonFunctions.cpp:1058-1468), including the cell
// integrals of the field in the globals IE_X ... SE_Y.
void pois2d(std::vector<double> &Ut, std::vector<double> &POTC, std::vector<double> &phix, std::vector<double> &phiy) {
    lp_ctx *c = ctx();
    if (!c) return;
    if (!check(lp_set_state(c, Ut.data(), state_len()), "pois2d state upload")) return;
    const size_t nc = (size_t)Nx * Nx;
    POTC.resize(3 * nc); phix.resize(3 * nc); phiy.resize(3 * nc);
    std::vector<double> fl(14 * nc);
    if (!check(lp_poisson(c, POTC.data(), phix.data(), phiy.data(), fl.data()), "pois2d")) return;
    store_fields(fl);
}

// RK3 (source/advection_1.cpp:428-601): one SSP-RK3 step of U in place;
// POTC/phix/phiy and the field integrals hold the last stage's solve, as in
// the reference.
void RK3(std::vector<double> &U_vals, std::vector<double> &POTC, std::vector<double> &phix, std::vector<double> &phiy) {
    lp_ctx *c = ctx();
    if (!c) return;
    if (!check(lp_set_state(c, U_vals.data(), state_len()), "RK3 state upload")) return;
    if (!check(lp_advect_step(c), "RK3")) return;
    if (!check(lp_get_state(c, U_vals.data(), state_len()), "RK3 state download")) return;
    const size_t nc = (size_t)Nx * Nx;
    POTC.resize(3 * nc); phix.resize(3 * nc); phiy.resize(3 * nc);
    std::vector<double> fl(14 * nc);
    if (check(lp_last_fields(c, POTC.data(), phix.data(), phiy.data(), fl.data()), "RK3 fields")) store_fields(fl);
}

void collisionStepGPU(std::vector<double> &U_vals) {
    lp_ctx *c = ctx();
    if (!c) return;
    if (!check(lp_set_state(c, U_vals.data(), state_len()), "collision state upload")) return;
    if (!check(lp_collision_step(c, -1, -1), "collision step")) return;
    check(lp_get_state(c, U_vals.data(), state_len()), "collision state download");
}
