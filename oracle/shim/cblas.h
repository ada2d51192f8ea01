/* Minimal CBLAS declarations for compiling the reference CPU solver against
 * the OpenBLAS build that ships inside scipy (its symbols carry a "scipy_"
 * prefix).  Test infrastructure only: nothing in the product links this. */
#ifndef KI_ORACLE_SHIM_CBLAS_H_
#define KI_ORACLE_SHIM_CBLAS_H_
#ifdef __cplusplus
extern "C" {
#endif
enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
typedef enum CBLAS_ORDER CBLAS_LAYOUT;
void scipy_cblas_dgemm(enum CBLAS_ORDER, enum CBLAS_TRANSPOSE, enum CBLAS_TRANSPOSE,
                       int, int, int, double, const double*, int,
                       const double*, int, double, double*, int);
void scipy_openblas_set_num_threads(int);
#ifdef __cplusplus
}
#endif
#define cblas_dgemm scipy_cblas_dgemm
#define openblas_set_num_threads scipy_openblas_set_num_threads
#endif
