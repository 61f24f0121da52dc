/* CBLAS prototypes for building the mpsxx reference against the OpenBLAS that the
 * scipy wheel bundles (its symbols carry a "scipy_" prefix; LP64 integers).  Only
 * the routines the reference's include/blas wrappers call are declared.  Oracle
 * test infrastructure. */
#ifndef MPSXX_REF_MKL_CBLAS_H
#define MPSXX_REF_MKL_CBLAS_H
#include <stddef.h>

typedef enum { CblasRowMajor = 101, CblasColMajor = 102 } CBLAS_LAYOUT;
typedef CBLAS_LAYOUT CBLAS_ORDER;
typedef enum { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 } CBLAS_TRANSPOSE;
typedef enum { CblasUpper = 121, CblasLower = 122 } CBLAS_UPLO;
typedef enum { CblasNonUnit = 131, CblasUnit = 132 } CBLAS_DIAG;
typedef enum { CblasLeft = 141, CblasRight = 142 } CBLAS_SIDE;
typedef int MKL_INT;

#define MPSXX_REAL_L1(p, T)                                                                    \
  void scipy_cblas_##p##axpby(MKL_INT, T, const T*, MKL_INT, T, T*, MKL_INT);                \
  void scipy_cblas_##p##axpy(MKL_INT, T, const T*, MKL_INT, T*, MKL_INT);                    \
  void scipy_cblas_##p##copy(MKL_INT, const T*, MKL_INT, T*, MKL_INT);                       \
  T scipy_cblas_##p##dot(MKL_INT, const T*, MKL_INT, const T*, MKL_INT);                     \
  T scipy_cblas_##p##nrm2(MKL_INT, const T*, MKL_INT);                                       \
  void scipy_cblas_##p##scal(MKL_INT, T, T*, MKL_INT);                                       \
  void scipy_cblas_##p##gemv(CBLAS_LAYOUT, CBLAS_TRANSPOSE, MKL_INT, MKL_INT, T, const T*,   \
                             MKL_INT, const T*, MKL_INT, T, T*, MKL_INT);                    \
  void scipy_cblas_##p##ger(CBLAS_LAYOUT, MKL_INT, MKL_INT, T, const T*, MKL_INT, const T*,  \
                            MKL_INT, T*, MKL_INT);                                           \
  void scipy_cblas_##p##gemm(CBLAS_LAYOUT, CBLAS_TRANSPOSE, CBLAS_TRANSPOSE, MKL_INT,        \
                             MKL_INT, MKL_INT, T, const T*, MKL_INT, const T*, MKL_INT, T,   \
                             T*, MKL_INT);

#define MPSXX_CPLX_L1(p, R)                                                                    \
  void scipy_cblas_##p##axpby(MKL_INT, const void*, const void*, MKL_INT, const void*, void*, \
                              MKL_INT);                                                      \
  void scipy_cblas_##p##axpy(MKL_INT, const void*, const void*, MKL_INT, void*, MKL_INT);    \
  void scipy_cblas_##p##copy(MKL_INT, const void*, MKL_INT, void*, MKL_INT);                 \
  void scipy_cblas_##p##dotc_sub(MKL_INT, const void*, MKL_INT, const void*, MKL_INT, void*); \
  void scipy_cblas_##p##dotu_sub(MKL_INT, const void*, MKL_INT, const void*, MKL_INT, void*); \
  void scipy_cblas_##p##scal(MKL_INT, const void*, void*, MKL_INT);                          \
  void scipy_cblas_##p##gemv(CBLAS_LAYOUT, CBLAS_TRANSPOSE, MKL_INT, MKL_INT, const void*,   \
                             const void*, MKL_INT, const void*, MKL_INT, const void*, void*, \
                             MKL_INT);                                                       \
  void scipy_cblas_##p##gerc(CBLAS_LAYOUT, MKL_INT, MKL_INT, const void*, const void*,       \
                             MKL_INT, const void*, MKL_INT, void*, MKL_INT);                 \
  void scipy_cblas_##p##geru(CBLAS_LAYOUT, MKL_INT, MKL_INT, const void*, const void*,       \
                             MKL_INT, const void*, MKL_INT, void*, MKL_INT);                 \
  void scipy_cblas_##p##gemm(CBLAS_LAYOUT, CBLAS_TRANSPOSE, CBLAS_TRANSPOSE, MKL_INT,        \
                             MKL_INT, MKL_INT, const void*, const void*, MKL_INT,            \
                             const void*, MKL_INT, const void*, void*, MKL_INT);

MPSXX_REAL_L1(s, float)
MPSXX_REAL_L1(d, double)
MPSXX_CPLX_L1(c, float)
MPSXX_CPLX_L1(z, double)
void scipy_cblas_csscal(MKL_INT, float, void*, MKL_INT);
void scipy_cblas_zdscal(MKL_INT, double, void*, MKL_INT);
float scipy_cblas_scnrm2(MKL_INT, const void*, MKL_INT);
double scipy_cblas_dznrm2(MKL_INT, const void*, MKL_INT);
void scipy_openblas_set_num_threads(int);

#define cblas_saxpby scipy_cblas_saxpby
#define cblas_daxpby scipy_cblas_daxpby
#define cblas_caxpby scipy_cblas_caxpby
#define cblas_zaxpby scipy_cblas_zaxpby
#define cblas_saxpy scipy_cblas_saxpy
#define cblas_daxpy scipy_cblas_daxpy
#define cblas_caxpy scipy_cblas_caxpy
#define cblas_zaxpy scipy_cblas_zaxpy
#define cblas_scopy scipy_cblas_scopy
#define cblas_dcopy scipy_cblas_dcopy
#define cblas_ccopy scipy_cblas_ccopy
#define cblas_zcopy scipy_cblas_zcopy
#define cblas_sdot scipy_cblas_sdot
#define cblas_ddot scipy_cblas_ddot
#define cblas_cdotc_sub scipy_cblas_cdotc_sub
#define cblas_zdotc_sub scipy_cblas_zdotc_sub
#define cblas_cdotu_sub scipy_cblas_cdotu_sub
#define cblas_zdotu_sub scipy_cblas_zdotu_sub
#define cblas_snrm2 scipy_cblas_snrm2
#define cblas_dnrm2 scipy_cblas_dnrm2
#define cblas_scnrm2 scipy_cblas_scnrm2
#define cblas_dznrm2 scipy_cblas_dznrm2
#define cblas_sscal scipy_cblas_sscal
#define cblas_dscal scipy_cblas_dscal
#define cblas_cscal scipy_cblas_cscal
#define cblas_zscal scipy_cblas_zscal
#define cblas_csscal scipy_cblas_csscal
#define cblas_zdscal scipy_cblas_zdscal
#define cblas_sgemv scipy_cblas_sgemv
#define cblas_dgemv scipy_cblas_dgemv
#define cblas_cgemv scipy_cblas_cgemv
#define cblas_zgemv scipy_cblas_zgemv
#define cblas_sger scipy_cblas_sger
#define cblas_dger scipy_cblas_dger
#define cblas_cgerc scipy_cblas_cgerc
#define cblas_zgerc scipy_cblas_zgerc
#define cblas_cgeru scipy_cblas_cgeru
#define cblas_zgeru scipy_cblas_zgeru
#define cblas_sgemm scipy_cblas_sgemm
#define cblas_dgemm scipy_cblas_dgemm
#define cblas_cgemm scipy_cblas_cgemm
#define cblas_zgemm scipy_cblas_zgemm
#endif
