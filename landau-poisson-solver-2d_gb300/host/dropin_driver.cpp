// Exercises the drop-in routines the way the reference's main does: it
// defines the reference's globals (source/LP_ompi_1.cpp:20-103), reads
// inputs written by the test, calls each replaced routine and writes the
// outputs for comparison with the CPU oracle.
//
//   dropin_driver <in.bin> <out.bin> Nx Nv N Lv Lx nu dt A k
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "lp_dropin.h"

// ---- the reference's globals used by the hot path -----------------------
int Nx, Nv, N, M = 5, size_v, size_ft, chunk_Nx;
double Lx, Lv, nu, dt, A_amp, k_wave;
double **C1, **C2;
double CCt[5 * 5];
std::vector<double> IE_X, IXE_X, IYE_X, IXXE_X, IXYE_X, IYYE_X;
std::vector<double> IE_Y, IXE_Y, IYE_Y, IXXE_Y, IXYE_Y, IYYE_Y;
std::vector<double> SE_X, SE_Y;

static FILE *g_out = nullptr;
static void put(const char *name, const double *d, size_t n) {
    char nm[16] = {0};
    std::strncpy(nm, name, 15);
    long long cnt = (long long)n;
    fwrite(nm, 1, 16, g_out);
    fwrite(&cnt, sizeof(cnt), 1, g_out);
    fwrite(d, sizeof(double), n, g_out);
}
static void need_ok(const char *what) {
    if (lp_dropin_last_status() != LP_OK) {
        fprintf(stderr, "%s failed with status %d\n", what, (int)lp_dropin_last_status());
        exit(2);
    }
}

int main(int argc, char **argv) {
    if (argc != 12) {
        fprintf(stderr, "usage: %s in out Nx Nv N Lv Lx nu dt A k\n", argv[0]);
        return 1;
    }
    Nx = atoi(argv[3]); Nv = atoi(argv[4]); N = atoi(argv[5]);
    Lv = atof(argv[6]); Lx = atof(argv[7]); nu = atof(argv[8]); dt = atof(argv[9]);
    A_amp = atof(argv[10]); k_wave = atof(argv[11]);
    size_v = Nv * Nv * Nv; size_ft = N * N * N;
    chunk_Nx = Nx * Nx;  // one rank (LP_ompi_1.cpp:167-171)
    const size_t size = (size_t)Nx * Nx * size_v;
    // inputs: U (7 size), f (size_ft), qhat (2 size_ft), x (2 size_ft)
    std::vector<double> U(7 * size), f(size_ft), qin(2 * size_ft), x(2 * size_ft);
    FILE *in = fopen(argv[1], "rb");
    if (!in || fread(U.data(), 8, U.size(), in) != U.size() || fread(f.data(), 8, f.size(), in) != f.size() ||
        fread(qin.data(), 8, qin.size(), in) != qin.size() || fread(x.data(), 8, x.size(), in) != x.size()) {
        fprintf(stderr, "bad input file\n");
        return 1;
    }
    fclose(in);
    g_out = fopen(argv[2], "wb");
    C1 = (double **)malloc(M * sizeof(double *));
    C2 = (double **)malloc(M * sizeof(double *));
    for (int i = 0; i < M; ++i) {
        C1[i] = (double *)malloc(size_ft * sizeof(double));
        C2[i] = (double *)malloc(size_ft * sizeof(double));
    }
    createCCtAndPivot();
    need_ok("createCCtAndPivot");
    put("c1_0", C1[0], size_ft); put("c1_4", C1[4], size_ft); put("c2_1", C2[1], size_ft);
    put("cct", CCt, 25);
    std::vector<double *> conv(size_ft);
    std::vector<double> conv_store((size_t)size_ft * size_ft);
    for (int r = 0; r < size_ft; ++r) conv[r] = conv_store.data() + (size_t)r * size_ft;
    generate_conv_weights(conv.data());
    need_ok("generate_conv_weights");
    put("w_mid", conv[size_ft / 2], size_ft);
    std::vector<double> out(2 * size_ft);
    fft3D((fftw_complex *)x.data(), (fftw_complex *)out.data());
    need_ok("fft3D");
    put("fft3d", out.data(), out.size());
    FS((fftw_complex *)x.data(), (fftw_complex *)out.data());
    need_ok("FS");
    put("fs", out.data(), out.size());
    std::vector<double> q(2 * size_ft);
    ComputeQ(f.data(), (fftw_complex *)q.data(), conv.data());
    need_ok("ComputeQ");
    put("computeq", q.data(), q.size());
    std::vector<double> qc(qin);
    conserveAllMoments((fftw_complex *)qc.data());
    need_ok("conserveAllMoments");
    put("conserve", qc.data(), qc.size());
    std::vector<double> Uz(7 * size, 0.0), dU((size_t)chunk_Nx * size_v * 5, 0.0);
    RK4(f.data(), 1, (fftw_complex *)qc.data(), conv.data(), Uz, dU.data());
    need_ok("RK4");
    put("rk4", dU.data() + (size_t)1 * size_v * 5, (size_t)size_v * 5);
    std::vector<double *> fr(Nx);
    std::vector<double> fstore((size_t)Nx * size_ft);
    for (int i = 0; i < Nx; ++i) fr[i] = fstore.data() + (size_t)i * size_ft;
    setInit_spectral(U, fr.data());
    need_ok("setInit_spectral");
    put("nodes", fstore.data(), fstore.size());
    std::vector<double> POTC, phix, phiy;
    pois2d(U, POTC, phix, phiy);
    need_ok("pois2d");
    put("potc", POTC.data(), POTC.size()); put("phix", phix.data(), phix.size());
    put("ie_x", IE_X.data(), IE_X.size());
    std::vector<double> U3(U);
    RK3(U3, POTC, phix, phiy);
    need_ok("RK3");
    put("rk3", U3.data(), U3.size()); put("rk3_phix", phix.data(), phix.size());
    std::vector<double> Uc(U);
    collisionStepGPU(Uc);
    need_ok("collisionStepGPU");
    put("collide", Uc.data(), Uc.size());
    fclose(g_out);
    return 0;
}
