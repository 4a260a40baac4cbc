// C entry points over the Landau-Poisson reference's own routines, for
// generating golden vectors and timing the reference here.  The reference's
// sources are compiled where they lie, unmodified (its main() renamed by a -D
// flag), against the stand-in MPI/FFTW/LAPACK headers in oracle/shim/.  This
// file replaces only the driver: it sets the reference's mutable globals
// (source/LP_ompi_1.cpp:20-103) at run time and performs the set-up sequence of
// main() (source/LP_ompi_1.cpp:154-387), then exposes each hot-path routine.
//
// Built twice: as is (libref.so) and with -DFullandLinear (libref_lin.so, the
// two-species variant with the linear electron-ion operator).
//
// Test infrastructure only; never linked into the shipped library.
#include "LP_ompi.h"
#include "EntropyCalculations.h"
#include "MarginalCreation.h"

#include <cstring>
#include <vector>

static double **g_f = nullptr;            // node values per spatial cell (main's f)
static double **g_conv = nullptr;         // conv_weights (main's local)
#ifdef FullandLinear
static double **g_conv_lin = nullptr;     // conv_weights_linear (main's local)
static fftw_complex *g_qhat_lin = nullptr;
#endif
static fftw_complex *g_qhat = nullptr;    // main's qHat
static int g_have_weights = 0;
static std::vector<double> g_U, g_POTC, g_phix, g_phiy;

template <class T> static void free_rows(T **&p, int n) {
    if (!p) return;
    for (int i = 0; i < n; ++i) free(p[i]);
    free(p);
    p = nullptr;
}

static int g_prev_chunk = 0, g_prev_ft = 0, g_prev_M = 0;

static void release_all() {
    free_rows(g_f, g_prev_chunk);
    free_rows(g_conv, g_prev_ft);
#ifdef FullandLinear
    free_rows(g_conv_lin, g_prev_ft);
    fftw_free(g_qhat_lin); fftw_free(Q1_fft_linear); fftw_free(Q2_fft_linear); fftw_free(Q3_fft_linear);
    g_qhat_lin = Q1_fft_linear = Q2_fft_linear = Q3_fft_linear = nullptr;
#endif
    free_rows(C1, g_prev_M);
    free_rows(C2, g_prev_M);
    free(Utmp); Utmp = nullptr;
    free(output_buffer_vp); output_buffer_vp = nullptr;
    free(cp); free(intE); free(intE1); free(intE2);
    cp = intE = intE1 = intE2 = nullptr;
    free(Q); free(f1); free(Q1); free(Utmp_coll);
    Q = f1 = Q1 = Utmp_coll = nullptr;
    fftw_free(temp); fftw_free(g_qhat); fftw_free(Q1_fft); fftw_free(Q2_fft);
    fftw_free(Q3_fft); fftw_free(fftOut); fftw_free(fftIn);
    temp = g_qhat = Q1_fft = Q2_fft = Q3_fft = fftOut = fftIn = nullptr;
    free(wtN); free(v); free(eta);
    wtN = v = eta = nullptr;
}

// defined in MarginalCreation.cpp:35 without a declaration in its header
double f_marg2D_x1v1(std::vector<double> &U_vals0, int i1, int j1, double x1, double v1);

#ifdef FullandLinear
// The two-species RK4 is defined with a double* state (collisionRoutines_1.cpp:637)
// while its header and main call a vector<double>& version; the forwarder
// below supplies that symbol so the library loads.
void RK4(double *f, int l, fftw_complex *qHat, double **conv_weights, fftw_complex *qHat_linear,
         double **conv_weights_linear, double *U, double *dU);
void RK4(double *f, int l, fftw_complex *qHat, double **conv_weights, fftw_complex *qHat_linear,
         double **conv_weights_linear, std::vector<double> &U_vals, double *dU) {
    RK4(f, l, qHat, conv_weights, qHat_linear, conv_weights_linear, U_vals.data(), dU);
}
void generate_conv_weights_linear(double **conv_weights_linear);
#endif

extern "C" {

// Configure a 2-D (Nx x Nx spatial cells) reference run.  with_weights=0 skips
// the N^6 weight table (ComputeQ/RK4 then unavailable).  Returns 0 on success.
int ref_setup(int nx, int nv, int n_spec, double lv, double lx, double nu_, double dt_,
              double a_amp, double k_w, int with_weights) {
    if (nx + 2 > NXD || nx < 2 || nv < 1 || n_spec < 2) return 1;
    release_all();
    Nx = nx; Nv = nv; N = n_spec;
    size_x = Nx * Nx; size_v = Nv * Nv * Nv; size = size_x * size_v; size_ft = N * N * N;
    NX = Nx; NY = Nx; NYREAL = NY;
    A_amp = a_amp; k_wave = k_w; Lx = lx; Lv = lv;
    dv = 2. * Lv / Nv; dx = Lx / Nx;
    L_v = Lv; R_v = Lv;
    nu = nu_; dt = dt_;
    scaleL = 8 * Lv * Lv * Lv; scalex = dx * dx; scalev = dv * dv * dv;
    myrank_mpi = 0; nprocs_mpi = 1;
    chunksize_dg = size; chunksize_ft = size_ft;
    chunk_Nx = size_x;                          // main: size_x / nprocs_mpi
    nprocs_Nx = (int)((double)Nx / (double)chunk_Nx + 0.5);

    U1.assign(7 * (size_t)size, 0.0);
    U1.shrink_to_fit();
    for (auto *vec : {&IE_X, &IXE_X, &IYE_X, &IXXE_X, &IXYE_X, &IYYE_X, &IE_Y, &IXE_Y,
                      &IYE_Y, &IXXE_Y, &IXYE_Y, &IYYE_Y, &SE_X, &SE_Y})
        vec->assign(NX * NYREAL, 0.0);
    Utmp = (double *)malloc(chunksize_dg * 7 * sizeof(double));
    output_buffer_vp = (double *)malloc(chunksize_dg * 7 * sizeof(double));
    cp = (double *)malloc(Nx * sizeof(double));
    intE = (double *)malloc(Nx * sizeof(double));
    intE1 = (double *)malloc(Nx * sizeof(double));
    intE2 = (double *)malloc(Nx * sizeof(double));

    C1 = (double **)malloc(M * sizeof(double *));
    C2 = (double **)malloc(M * sizeof(double *));
    for (int i = 0; i < M; ++i) {
        C1[i] = (double *)malloc(size_ft * sizeof(double));
        C2[i] = (double *)malloc(size_ft * sizeof(double));
    }
    g_prev_M = M;
    g_f = (double **)malloc(chunk_Nx * sizeof(double *));
    for (int i = 0; i < chunk_Nx; ++i) g_f[i] = (double *)calloc(size_ft, sizeof(double));
    g_prev_chunk = chunk_Nx;
    g_have_weights = with_weights;
    if (with_weights) {
        g_conv = (double **)malloc(size_ft * sizeof(double *));
        for (int i = 0; i < size_ft; ++i) g_conv[i] = (double *)malloc(size_ft * sizeof(double));
#ifdef FullandLinear
        g_conv_lin = (double **)malloc(size_ft * sizeof(double *));
        for (int i = 0; i < size_ft; ++i) g_conv_lin[i] = (double *)malloc(size_ft * sizeof(double));
#endif
        g_prev_ft = size_ft;
    } else {
        g_prev_ft = 0;
    }
    Q = (double *)malloc(size_ft * sizeof(double));
    f1 = (double *)malloc(size_ft * sizeof(double));
    Q1 = (double *)malloc(size_ft * sizeof(double));
    Utmp_coll = (double *)calloc((size_t)chunk_Nx * size_v * 5, sizeof(double));
    temp = (fftw_complex *)fftw_malloc(size_ft * sizeof(fftw_complex));
    g_qhat = (fftw_complex *)fftw_malloc(size_ft * sizeof(fftw_complex));
    p_forward = fftw_plan_dft_3d(N, N, N, temp, temp, FFTW_FORWARD, FFTW_MEASURE);
    p_backward = fftw_plan_dft_3d(N, N, N, temp, temp, FFTW_BACKWARD, FFTW_MEASURE);
    wtN = (double *)malloc(N * sizeof(double));
    v = (double *)malloc(N * sizeof(double));
    eta = (double *)malloc(N * sizeof(double));
    Q1_fft = (fftw_complex *)fftw_malloc(size_ft * sizeof(fftw_complex));
    Q2_fft = (fftw_complex *)fftw_malloc(size_ft * sizeof(fftw_complex));
    Q3_fft = (fftw_complex *)fftw_malloc(size_ft * sizeof(fftw_complex));
    fftOut = (fftw_complex *)fftw_malloc(size_ft * sizeof(fftw_complex));
    fftIn = (fftw_complex *)fftw_malloc(size_ft * sizeof(fftw_complex));
#ifdef FullandLinear
    g_qhat_lin = (fftw_complex *)fftw_malloc(size_ft * sizeof(fftw_complex));
    Q1_fft_linear = (fftw_complex *)fftw_malloc(size_ft * sizeof(fftw_complex));
    Q2_fft_linear = (fftw_complex *)fftw_malloc(size_ft * sizeof(fftw_complex));
    Q3_fft_linear = (fftw_complex *)fftw_malloc(size_ft * sizeof(fftw_complex));
#endif

    scale = 1.0 / sqrt(2.0 * M_PI);
    scale3 = pow(scale, 3.0);
    L_v = Lv;
    L_eta = 0.5 * (double)(N - 1) * PI / L_v;
    h_v = 2.0 * L_v / (double)(N - 1);
    h_eta = 2.0 * L_eta / (double)(N);
    for (int i = 0; i < N; ++i) {
        eta[i] = -L_eta + (double)i * h_eta;
        v[i] = -L_v + (double)i * h_v;
    }
    trapezoidalRule(N, wtN);
    createCCtAndPivot();
    if (with_weights) generate_conv_weights(g_conv);
#ifdef FullandLinear
    if (with_weights) generate_conv_weights_linear(g_conv_lin);
#endif

    // Poisson set-up.  coef_pois writes only the band entries of the static
    // poisab array, so clear the region transmat reads before re-assembling.
    adim();
    setup();
    config();
    setup_pois();
    {
        int nd = 3 * NX * NYREAL;
        int ld = 2 * nsub + nsuper + 1;
        for (int i = 0; i <= ld + 1 && i < 4 * MPD * NYD2; ++i)
            memset(&poisab[i][0], 0, sizeof(double) * (size_t)std::min(nd + 2, MPD * NXD * NYD2));
    }
    setup_matrix();

    g_U.assign(7 * (size_t)size, 0.0);
    g_POTC.assign(3 * NX * NYREAL, 0.0);
    g_phix.assign(3 * NX * NYREAL, 0.0);
    g_phiy.assign(3 * NX * NYREAL, 0.0);
    return 0;
}

// Grids and scalars: v[N], eta[N], wtN[N]; sc = {L_eta, h_eta, h_v, L_v, R_v,
// scale, scale3, scaleL, scalev, dv, dx, Lx, Lv, scalex}.
void ref_get_grid(double *v_out, double *eta_out, double *wt_out, double *sc) {
    for (int i = 0; i < N; ++i) { v_out[i] = v[i]; eta_out[i] = eta[i]; wt_out[i] = wtN[i]; }
    double s[14] = {L_eta, h_eta, h_v, L_v, R_v, scale, scale3, scaleL, scalev, dv, dx, Lx, Lv, scalex};
    memcpy(sc, s, sizeof(s));
}

// C1 and C2 as 5 x size_ft row-major, and the inverted Gram matrix CCt[25].
void ref_get_cons(double *c1, double *c2, double *cct) {
    for (int i = 0; i < 5; ++i) {
        memcpy(c1 + (size_t)i * size_ft, C1[i], sizeof(double) * size_ft);
        memcpy(c2 + (size_t)i * size_ft, C2[i], sizeof(double) * size_ft);
    }
    memcpy(cct, CCt, sizeof(double) * 25);
}

// Rows [r0, r1) of the N^3 x N^3 weight table.
int ref_get_weights(int r0, int r1, double *out) {
    if (!g_have_weights) return 1;
    for (int r = r0; r < r1; ++r) memcpy(out + (size_t)(r - r0) * size_ft, g_conv[r], sizeof(double) * size_ft);
    return 0;
}

double ref_ghat3(double e1, double e2, double e3, double k1, double k2, double k3) {
    return gHat3(e1, e2, e3, k1, k2, k3);
}

void ref_fft3d(const double *in, double *out) {
    memcpy(fftIn, in, sizeof(fftw_complex) * size_ft);
    fft3D(fftIn, fftOut);
    memcpy(out, fftOut, sizeof(fftw_complex) * size_ft);
}

void ref_fs(const double *in, double *out) {
    memcpy(fftIn, in, sizeof(fftw_complex) * size_ft);
    FS(fftIn, fftOut);
    memcpy(out, fftOut, sizeof(fftw_complex) * size_ft);
}

#ifndef FullandLinear
int ref_compute_q(const double *f, double *qhat) {
    if (!g_have_weights) return 1;
    std::vector<double> fcopy(f, f + size_ft);
    ComputeQ(fcopy.data(), g_qhat, g_conv);
    memcpy(qhat, g_qhat, sizeof(fftw_complex) * size_ft);
    return 0;
}

void ref_conserve(double *qhat) {
    memcpy(g_qhat, qhat, sizeof(fftw_complex) * size_ft);
    conserveAllMoments(g_qhat);
    memcpy(qhat, g_qhat, sizeof(fftw_complex) * size_ft);
}

// RK4 for spatial cell l with node values f, conserved qHat and state U
// (7*size doubles); writes the 5*size_v entries of dU for that cell.
int ref_rk4(const double *f, int l, const double *qhat, const double *U, double *dU_cell) {
    if (!g_have_weights) return 1;
    std::vector<double> fcopy(f, f + size_ft);
    memcpy(g_qhat, qhat, sizeof(fftw_complex) * size_ft);
    memcpy(g_U.data(), U, sizeof(double) * 7 * (size_t)size);
    RK4(fcopy.data(), l, g_qhat, g_conv, g_U, Utmp_coll);
    int l_local = l % chunk_Nx;
    memcpy(dU_cell, Utmp_coll + (size_t)l_local * size_v * 5, sizeof(double) * 5 * size_v);
    return 0;
}
#else
// Two-species variant (collisionRoutines_1.cpp:551-737, conservationRoutines.cpp:63-98).
int ref_compute_q_lin(const double *f, double *qhat, double *qhat_lin) {
    if (!g_have_weights) return 1;
    std::vector<double> fcopy(f, f + size_ft);
    ComputeQ(fcopy.data(), g_qhat, g_conv, g_qhat_lin, g_conv_lin);
    memcpy(qhat, g_qhat, sizeof(fftw_complex) * size_ft);
    memcpy(qhat_lin, g_qhat_lin, sizeof(fftw_complex) * size_ft);
    return 0;
}

void ref_conserve_lin(double *qhat, double *qhat_lin) {
    memcpy(g_qhat, qhat, sizeof(fftw_complex) * size_ft);
    memcpy(g_qhat_lin, qhat_lin, sizeof(fftw_complex) * size_ft);
    conserveAllMoments(g_qhat, g_qhat_lin);
    memcpy(qhat, g_qhat, sizeof(fftw_complex) * size_ft);
    memcpy(qhat_lin, g_qhat_lin, sizeof(fftw_complex) * size_ft);
}

void ref_get_cct_lin(double *cct_lin) { memcpy(cct_lin, CCt_linear, sizeof(double) * 4); }

// Rows [r0, r1) of the linear weight table.
int ref_get_weights_lin(int r0, int r1, double *out) {
    if (!g_have_weights) return 1;
    for (int r = r0; r < r1; ++r) memcpy(out + (size_t)(r - r0) * size_ft, g_conv_lin[r], sizeof(double) * size_ft);
    return 0;
}

int ref_rk4_lin(const double *f, int l, const double *qhat, const double *qhat_lin, const double *U,
                double *dU_cell) {
    if (!g_have_weights) return 1;
    std::vector<double> fcopy(f, f + size_ft);
    memcpy(g_qhat, qhat, sizeof(fftw_complex) * size_ft);
    memcpy(g_qhat_lin, qhat_lin, sizeof(fftw_complex) * size_ft);
    memcpy(g_U.data(), U, sizeof(double) * 7 * (size_t)size);
    RK4(fcopy.data(), l, g_qhat, g_conv, g_qhat_lin, g_conv_lin, g_U.data(), Utmp_coll);
    int l_local = l % chunk_Nx;
    memcpy(dU_cell, Utmp_coll + (size_t)l_local * size_v * 5, sizeof(double) * 5 * size_v);
    return 0;
}
#endif

void ref_intmodes(int k1, int k2, int k3, int j1, int j2, int j3, double *out10) {
    IntModes(k1, k2, k3, j1, j2, j3, out10);
}

// setInit_spectral (compiled branch): f_out holds Nx rows of size_ft.
void ref_set_init_spectral(const double *U, double *f_out) {
    memcpy(g_U.data(), U, sizeof(double) * 7 * (size_t)size);
    setInit_spectral(g_U, g_f);
    for (int i = 0; i < Nx; ++i) memcpy(f_out + (size_t)i * size_ft, g_f[i], sizeof(double) * size_ft);
}

void ref_set_init_ld(double *U) {
    std::fill(g_U.begin(), g_U.end(), 0.0);
    SetInit_LD(g_U);
    memcpy(U, g_U.data(), sizeof(double) * 7 * (size_t)size);
}

// pois2d on U; fields = 14 arrays of NX*NYREAL in the order IE_X, IXE_X, IYE_X,
// IXXE_X, IXYE_X, IYYE_X, IE_Y, IXE_Y, IYE_Y, IXXE_Y, IXYE_Y, IYYE_Y, SE_X, SE_Y.
void ref_pois2d(const double *U, double *potc, double *phix, double *phiy, double *fields) {
    memcpy(g_U.data(), U, sizeof(double) * 7 * (size_t)size);
    pois2d(g_U, g_POTC, g_phix, g_phiy);
    int nc = NX * NYREAL;
    memcpy(potc, g_POTC.data(), sizeof(double) * 3 * nc);
    memcpy(phix, g_phix.data(), sizeof(double) * 3 * nc);
    memcpy(phiy, g_phiy.data(), sizeof(double) * 3 * nc);
    if (fields) {
        const std::vector<double> *vs[14] = {&IE_X, &IXE_X, &IYE_X, &IXXE_X, &IXYE_X, &IYYE_X,
                                             &IE_Y, &IXE_Y, &IYE_Y, &IXXE_Y, &IXYE_Y, &IYYE_Y,
                                             &SE_X, &SE_Y};
        for (int a = 0; a < 14; ++a) memcpy(fields + (size_t)a * nc, vs[a]->data(), sizeof(double) * nc);
    }
}

// Band matrix after dgbtrf: dims = {ndim, nsub, nsuper, ldab}; ab is ldab*ndim.
void ref_get_band(int *dims, double *ab, int *piv) {
    dims[0] = ndim; dims[1] = nsub; dims[2] = nsuper; dims[3] = ldab;
    if (ab) memcpy(ab, poiscab, sizeof(double) * (size_t)ldab * ndim);
    if (piv) memcpy(piv, ipiv, sizeof(int) * ndim);
}

// One SSP-RK3 advection step (source/advection_1.cpp:428-601) on U in place.
void ref_rk3(double *U, double *potc, double *phix, double *phiy) {
    memcpy(g_U.data(), U, sizeof(double) * 7 * (size_t)size);
    RK3(g_U, g_POTC, g_phix, g_phiy);
    memcpy(U, g_U.data(), sizeof(double) * 7 * (size_t)size);
    int nc = NX * NYREAL;
    if (potc) memcpy(potc, g_POTC.data(), sizeof(double) * 3 * nc);
    if (phix) memcpy(phix, g_phix.data(), sizeof(double) * 3 * nc);
    if (phiy) memcpy(phiy, g_phiy.data(), sizeof(double) * 3 * nc);
}

// The collision sequence of main for spatial cells [l0, l1) (source/
// LP_ompi_1.cpp:502-516): setInit_spectral, then per cell ComputeQ,
// conserveAllMoments, RK4.  dU_out receives (l1-l0)*size_v*5 doubles.
#ifndef FullandLinear
int ref_collision_cells(const double *U, int l0, int l1, double *dU_out) {
    if (!g_have_weights) return 1;
    memcpy(g_U.data(), U, sizeof(double) * 7 * (size_t)size);
    setInit_spectral(g_U, g_f);
    for (int l = l0; l < l1; ++l) {
        ComputeQ(g_f[l % chunk_Nx], g_qhat, g_conv);
        conserveAllMoments(g_qhat);
        RK4(g_f[l % chunk_Nx], l, g_qhat, g_conv, g_U, Utmp_coll);
        if (dU_out)
            memcpy(dU_out + (size_t)(l - l0) * size_v * 5, Utmp_coll + (size_t)(l % chunk_Nx) * size_v * 5,
                   sizeof(double) * 5 * size_v);
    }
    return 0;
}
#endif

// Moments of the reference: out = {mass, p1, p2, p3, KiE, EleE(phix, phiy)}.
void ref_moments(const double *U, const double *phix, const double *phiy, double *out) {
    memcpy(g_U.data(), U, sizeof(double) * 7 * (size_t)size);
    int nc = NX * NYREAL;
    memcpy(g_phix.data(), phix, sizeof(double) * 3 * nc);
    memcpy(g_phiy.data(), phiy, sizeof(double) * 3 * nc);
    double a[3];
    out[0] = computeMass(g_U);
    computeMomentum(g_U, a);
    out[1] = a[0]; out[2] = a[1]; out[3] = a[2];
    out[4] = computeKiE(g_U);
    out[5] = computeEleE(g_phix, g_phiy);
}

// Entropy (computeEntropy, EntropyCalculations.cpp:11) of U.
double ref_entropy(const double *U) {
    memcpy(g_U.data(), U, sizeof(double) * 7 * (size_t)size);
    return computeEntropy(g_U);
}


// The (x1, v1) marginal values PrintMarginal writes (MarginalCreation.cpp:174-197),
// out[(i1*4 + nx) * (Nv*4) + j1*4 + nv].
void ref_marginal_x1v1(const double *U, double *out) {
    memcpy(g_U.data(), U, sizeof(double) * 7 * (size_t)size);
    const int np = 4;
    const double ddx = dx / np, ddv = dv / np;
    size_t o = 0;
    for (int i1 = 0; i1 < Nx; i1++) {
        const double x1_0 = Gridx((double)i1 - 0.5);
        for (int nx = 0; nx < np; nx++) {
            const double x1_val = x1_0 + nx * ddx;
            for (int j1 = 0; j1 < Nv; j1++) {
                const double v1_0 = Gridv((double)j1 - 0.5);
                for (int nv = 0; nv < np; nv++) out[o++] = f_marg2D_x1v1(g_U, i1, j1, x1_val, v1_0 + nv * ddv);
            }
        }
    }
}

}  // extern "C"
