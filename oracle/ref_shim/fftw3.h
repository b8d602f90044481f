// TEST INFRASTRUCTURE ONLY -- stand-in for the FFTW3 header, used only when
// the reference's own CPU sources are compiled as a second oracle
// (oracle/build_ref.py).  It declares the subset of the FFTW3 API that
// TW_paDIC_FFTCC2D_CPU.cpp calls (single-precision 2D r2c / c2r plans,
// execute, destroy, malloc / free).  The transforms are implemented in
// ref_shim.cpp as direct DFTs evaluated in double precision and rounded once
// to float (FFTW3's definition of the unnormalised forward and backward
// transforms; FFTW's own rounding pattern is not reproduced).
#ifndef TWREF_FFTW3_STANDIN_H
#define TWREF_FFTW3_STANDIN_H

#include <cstddef>

extern "C" {

typedef float fftwf_complex[2];
typedef double fftw_complex[2];
typedef struct twref_fftwf_plan_s* fftwf_plan;
typedef struct twref_fftw_plan_s* fftw_plan;

#define FFTW_ESTIMATE (1U << 6)

void* fftw_malloc(size_t n);
void fftw_free(void* p);
void* fftwf_malloc(size_t n);
void fftwf_free(void* p);

// n0 x n1 real array (row-major, n1 fastest) -> n0 x (n1/2 + 1) spectrum
fftwf_plan fftwf_plan_dft_r2c_2d(int n0, int n1, float* in, fftwf_complex* out, unsigned flags);
// n0 x (n1/2 + 1) Hermitian half spectrum -> n0 x n1 real array, unnormalised
fftwf_plan fftwf_plan_dft_c2r_2d(int n0, int n1, fftwf_complex* in, float* out, unsigned flags);
void fftwf_execute(const fftwf_plan p);
void fftwf_destroy_plan(fftwf_plan p);
}

#endif
