/* LAPACKE prototypes for building the mpsxx reference against scipy's bundled
 * OpenBLAS ("scipy_" symbol prefix, LP64).  Only the routines the reference's
 * include/lapack wrappers call are declared.  Oracle test infrastructure. */
#ifndef MPSXX_REF_MKL_LAPACKE_H
#define MPSXX_REF_MKL_LAPACKE_H
typedef int lapack_int;
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102

#define MPSXX_LAPACKE_REAL(p, T)                                                                  \
  lapack_int scipy_LAPACKE_##p##gesvd(int, char, char, lapack_int, lapack_int, T*, lapack_int, T*, \
                                      T*, lapack_int, T*, lapack_int, T*);                        \
  lapack_int scipy_LAPACKE_##p##syev(int, char, char, lapack_int, T*, lapack_int, T*);           \
  lapack_int scipy_LAPACKE_##p##sygv(int, lapack_int, char, char, lapack_int, T*, lapack_int, T*, \
                                     lapack_int, T*);                                             \
  lapack_int scipy_LAPACKE_##p##geqrf(int, lapack_int, lapack_int, T*, lapack_int, T*);          \
  lapack_int scipy_LAPACKE_##p##gelqf(int, lapack_int, lapack_int, T*, lapack_int, T*);          \
  lapack_int scipy_LAPACKE_##p##orgqr(int, lapack_int, lapack_int, lapack_int, T*, lapack_int,   \
                                      const T*);                                                  \
  lapack_int scipy_LAPACKE_##p##orglq(int, lapack_int, lapack_int, lapack_int, T*, lapack_int,   \
                                      const T*);                                                  \
  lapack_int scipy_LAPACKE_##p##getrf(int, lapack_int, lapack_int, T*, lapack_int, lapack_int*); \
  lapack_int scipy_LAPACKE_##p##getri(int, lapack_int, T*, lapack_int, const lapack_int*);

#define MPSXX_LAPACKE_CPLX(p, C, R)                                                               \
  lapack_int scipy_LAPACKE_##p##gesvd(int, char, char, lapack_int, lapack_int, C*, lapack_int, R*, \
                                      C*, lapack_int, C*, lapack_int, R*);                        \
  lapack_int scipy_LAPACKE_##p##heev(int, char, char, lapack_int, C*, lapack_int, R*);           \
  lapack_int scipy_LAPACKE_##p##geqrf(int, lapack_int, lapack_int, C*, lapack_int, C*);          \
  lapack_int scipy_LAPACKE_##p##gelqf(int, lapack_int, lapack_int, C*, lapack_int, C*);          \
  lapack_int scipy_LAPACKE_##p##ungqr(int, lapack_int, lapack_int, lapack_int, C*, lapack_int,   \
                                      const C*);                                                  \
  lapack_int scipy_LAPACKE_##p##unglq(int, lapack_int, lapack_int, lapack_int, C*, lapack_int,   \
                                      const C*);                                                  \
  lapack_int scipy_LAPACKE_##p##getrf(int, lapack_int, lapack_int, C*, lapack_int, lapack_int*); \
  lapack_int scipy_LAPACKE_##p##getri(int, lapack_int, C*, lapack_int, const lapack_int*);

MPSXX_LAPACKE_REAL(s, float)
MPSXX_LAPACKE_REAL(d, double)
MPSXX_LAPACKE_CPLX(c, lapack_complex_float, float)
MPSXX_LAPACKE_CPLX(z, lapack_complex_double, double)

#define LAPACKE_sgesvd scipy_LAPACKE_sgesvd
#define LAPACKE_dgesvd scipy_LAPACKE_dgesvd
#define LAPACKE_cgesvd scipy_LAPACKE_cgesvd
#define LAPACKE_zgesvd scipy_LAPACKE_zgesvd
#define LAPACKE_ssyev scipy_LAPACKE_ssyev
#define LAPACKE_dsyev scipy_LAPACKE_dsyev
#define LAPACKE_cheev scipy_LAPACKE_cheev
#define LAPACKE_zheev scipy_LAPACKE_zheev
#define LAPACKE_ssygv scipy_LAPACKE_ssygv
#define LAPACKE_dsygv scipy_LAPACKE_dsygv
#define LAPACKE_sgeqrf scipy_LAPACKE_sgeqrf
#define LAPACKE_dgeqrf scipy_LAPACKE_dgeqrf
#define LAPACKE_cgeqrf scipy_LAPACKE_cgeqrf
#define LAPACKE_zgeqrf scipy_LAPACKE_zgeqrf
#define LAPACKE_sgelqf scipy_LAPACKE_sgelqf
#define LAPACKE_dgelqf scipy_LAPACKE_dgelqf
#define LAPACKE_cgelqf scipy_LAPACKE_cgelqf
#define LAPACKE_zgelqf scipy_LAPACKE_zgelqf
#define LAPACKE_sorgqr scipy_LAPACKE_sorgqr
#define LAPACKE_dorgqr scipy_LAPACKE_dorgqr
#define LAPACKE_cungqr scipy_LAPACKE_cungqr
#define LAPACKE_zungqr scipy_LAPACKE_zungqr
#define LAPACKE_sorglq scipy_LAPACKE_sorglq
#define LAPACKE_dorglq scipy_LAPACKE_dorglq
#define LAPACKE_cunglq scipy_LAPACKE_cunglq
#define LAPACKE_zunglq scipy_LAPACKE_zunglq
#define LAPACKE_sgetrf scipy_LAPACKE_sgetrf
#define LAPACKE_dgetrf scipy_LAPACKE_dgetrf
#define LAPACKE_cgetrf scipy_LAPACKE_cgetrf
#define LAPACKE_zgetrf scipy_LAPACKE_zgetrf
#define LAPACKE_sgetri scipy_LAPACKE_sgetri
#define LAPACKE_dgetri scipy_LAPACKE_dgetri
#define LAPACKE_cgetri scipy_LAPACKE_cgetri
#define LAPACKE_zgetri scipy_LAPACKE_zgetri
#endif
