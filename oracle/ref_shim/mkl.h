// TEST INFRASTRUCTURE ONLY -- stand-in for the MKL header, used only when the
// reference's own CPU sources are compiled as a second oracle
// (oracle/build_ref.py).  TW_paDIC_ICGN2D_CPU.cpp calls LAPACKE_spotrf and
// LAPACKE_spotrs in row-major layout with uplo 'L'.  ref_shim.cpp implements
// the LAPACKE row-major convention (transpose to column-major, call the
// Fortran routine, transpose back) over the Fortran spotrf_ / spotrs_ of the
// LAPACK library that the test process hands over at start-up
// (twref_set_lapack), i.e. the LAPACK that scipy links.
#ifndef TWREF_MKL_STANDIN_H
#define TWREF_MKL_STANDIN_H

typedef int MKL_INT;

#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102

extern "C" {
int LAPACKE_spotrf(int matrix_layout, char uplo, int n, float* a, int lda);
int LAPACKE_spotrs(int matrix_layout, char uplo, int n, int nrhs, const float* a, int lda, float* b, int ldb);
int LAPACKE_dpotrf(int matrix_layout, char uplo, int n, double* a, int lda);
int LAPACKE_dpotrs(int matrix_layout, char uplo, int n, int nrhs, const double* a, int lda, double* b, int ldb);
}

#endif
