/* Minimal LAPACKE declarations (LP64) mapped onto scipy's bundled OpenBLAS.
 * Test infrastructure only. */
#ifndef KI_ORACLE_SHIM_LAPACKE_H_
#define KI_ORACLE_SHIM_LAPACKE_H_
#ifndef lapack_int
#define lapack_int int
#endif
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
#ifdef __cplusplus
extern "C" {
#endif
lapack_int scipy_LAPACKE_dgetrf(int, lapack_int, lapack_int, double*, lapack_int, lapack_int*);
lapack_int scipy_LAPACKE_dgetrs(int, char, lapack_int, lapack_int, const double*, lapack_int,
                                const lapack_int*, double*, lapack_int);
lapack_int scipy_LAPACKE_dgeqp3(int, lapack_int, lapack_int, double*, lapack_int, lapack_int*, double*);
lapack_int scipy_LAPACKE_dtrtrs(int, char, char, char, lapack_int, lapack_int, const double*,
                                lapack_int, double*, lapack_int);
lapack_int scipy_LAPACKE_dgecon(int, char, lapack_int, const double*, lapack_int, double, double*);
lapack_int scipy_LAPACKE_dgeev(int, char, char, lapack_int, double*, lapack_int, double*, double*,
                               double*, lapack_int, double*, lapack_int);
#ifdef __cplusplus
}
#endif
#define LAPACKE_dgetrf scipy_LAPACKE_dgetrf
#define LAPACKE_dgetrs scipy_LAPACKE_dgetrs
#define LAPACKE_dgeqp3 scipy_LAPACKE_dgeqp3
#define LAPACKE_dtrtrs scipy_LAPACKE_dtrtrs
#define LAPACKE_dgecon scipy_LAPACKE_dgecon
#define LAPACKE_dgeev scipy_LAPACKE_dgeev
#endif
