/* Stand-in for the FFTW3 subset used by the Landau-Poisson reference
 * (source/LP_ompi.h:24; plans at source/LP_ompi_1.cpp:247-248, executed by
 * fft3D/FS in source/collisionRoutines_1.cpp:163-276).  Semantics follow the
 * published FFTW3 interface: unnormalised complex DFT,
 * X[k] = sum_n x[n] exp(sign * 2 pi i k n / N), row-major (last index
 * fastest), in-place allowed.  The transform itself is our own separable
 * direct DFT (oracle/shim/shim_impl.cpp).  Test infrastructure only. */
#ifndef LP_SHIM_FFTW3_H
#define LP_SHIM_FFTW3_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef double fftw_complex[2];
typedef struct lp_shim_fftw_plan_s *fftw_plan;
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)
fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex *in, fftw_complex *out,
                           int sign, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);
void *fftw_malloc(size_t n);
void fftw_free(void *p);
int fftw_init_threads(void);
void fftw_plan_with_nthreads(int n);
#ifdef __cplusplus
}
#endif
#endif
