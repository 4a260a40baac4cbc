// Drop-in replacements for the Landau-Poisson reference's hot-path routines,
// with the reference's names and signatures (source/collisionRoutines_1.h:36-62,
// source/conservationRoutines.h:31-34, source/advection_1.h:70,
// source/PoissonFunctions.h:35, source/SetInit_1.h:44), running on the GB300
// library through include/lp_gb300.h.  They read the reference's global run
// parameters (source/LP_ompi.h:69-118) and keep its data layout: the state is
// a std::vector<double> of 7 coefficients per record on the Nx x Nx grid,
// spectral arrays are fftw_complex[N^3].
//
// By default the routines reproduce the reference's results including its
// defects F1-F3 (see the defect table of the documentation); call
// lp_dropin_set_fixes(LP_FIX_DEFAULT) to apply the fixes instead.
#pragma once

#include <vector>

#include "lp_gb300.h"

#ifndef FFTW3_H
typedef double fftw_complex[2];
#endif

void ComputeQ(double *f, fftw_complex *qHat, double **conv_weights);
void conserveAllMoments(fftw_complex *qHat);
void RK4(double *f, int l, fftw_complex *qHat, double **conv_weights, std::vector<double> &U_vals, double *dU);
void RK3(std::vector<double> &U_vals, std::vector<double> &POTC, std::vector<double> &phix, std::vector<double> &phiy);
void pois2d(std::vector<double> &Ut, std::vector<double> &POTC, std::vector<double> &phix, std::vector<double> &phiy);
void setInit_spectral(std::vector<double> &U_vals, double **f);
void generate_conv_weights(double **conv_weights);
void createCCtAndPivot();
void fft3D(fftw_complex *in, fftw_complex *out);
void FS(fftw_complex *in, fftw_complex *out);

// The batched replacement of the per-cell collision loop and the dU scatter
// of main (source/LP_ompi_1.cpp:502-567): one call collides every spatial
// cell on the GPU and updates U in place.
void collisionStepGPU(std::vector<double> &U_vals);

extern "C" {
// LP_FIX_* bits applied by the drop-in routines (default 0: the reference's behaviour).
void lp_dropin_set_fixes(unsigned fixes);
// Last status of a drop-in routine (the reference's routines return void).
lp_status lp_dropin_last_status(void);
}
