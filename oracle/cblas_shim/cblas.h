/*
 * Minimal <cblas.h> for building the reference's BLAS path (TEST
 * INFRASTRUCTURE: the CPU baseline, never shipped).
 *
 * The reference includes <cblas.h> under -DUSE_OPENBLAS and calls exactly
 * cblas_sgemv / cblas_dgemv (matrix_times_vector.h:190-262) and
 * openblas_set_num_threads / openblas_get_num_threads
 * (tensor_times_vector.h:91-113).  No system BLAS is installed on these
 * hosts; NumPy's wheel ships OpenBLAS with renamed ILP64 symbols (for NumPy 2:
 * scipy_cblas_sgemv64_, scipy_openblas_set_num_threads64_; for NumPy 1:
 * cblas_sgemv64_, openblas_set_num_threads64_).  This header declares the
 * standard CBLAS enumerations and forwards the four calls to the renamed
 * symbols, whose prefix and suffix the build passes in:
 *     -DTTVREF_BLAS_PREFIX=scipy_ -DTTVREF_BLAS_SUFFIX=64_
 * Sizes are 64-bit (ILP64) when the suffix is 64_, else int.
 */
#ifndef TTVREF_CBLAS_SHIM_H
#define TTVREF_CBLAS_SHIM_H

#include <stdint.h>

#ifndef TTVREF_BLAS_PREFIX
#define TTVREF_BLAS_PREFIX
#endif
#ifndef TTVREF_BLAS_SUFFIX
#define TTVREF_BLAS_SUFFIX
#endif
#ifdef TTVREF_BLAS_ILP64
typedef int64_t ttvref_blasint;
#else
typedef int ttvref_blasint;
#endif

#define TTVREF_CAT3_(a, b, c) a##b##c
#define TTVREF_CAT3(a, b, c) TTVREF_CAT3_(a, b, c)
#define TTVREF_SYM(name) TTVREF_CAT3(TTVREF_BLAS_PREFIX, name, TTVREF_BLAS_SUFFIX)

enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };

#ifdef __cplusplus
extern "C" {
#endif
void TTVREF_SYM(cblas_sgemv)(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE trans, ttvref_blasint m,
                             ttvref_blasint n, float alpha, const float* a, ttvref_blasint lda,
                             const float* x, ttvref_blasint incx, float beta, float* y,
                             ttvref_blasint incy);
void TTVREF_SYM(cblas_dgemv)(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE trans, ttvref_blasint m,
                             ttvref_blasint n, double alpha, const double* a, ttvref_blasint lda,
                             const double* x, ttvref_blasint incx, double beta, double* y,
                             ttvref_blasint incy);
void TTVREF_SYM(openblas_set_num_threads)(int num);
int TTVREF_SYM(openblas_get_num_threads)(void);
#ifdef __cplusplus
}
#endif

#ifdef TTVREF_BLAS_RENAMED
/* the names the reference calls, forwarding to the renamed library symbols */
static inline void cblas_sgemv(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE trans, ttvref_blasint m,
                               ttvref_blasint n, float alpha, const float* a, ttvref_blasint lda,
                               const float* x, ttvref_blasint incx, float beta, float* y,
                               ttvref_blasint incy)
{
    TTVREF_SYM(cblas_sgemv)(order, trans, m, n, alpha, a, lda, x, incx, beta, y, incy);
}
static inline void cblas_dgemv(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE trans, ttvref_blasint m,
                               ttvref_blasint n, double alpha, const double* a, ttvref_blasint lda,
                               const double* x, ttvref_blasint incx, double beta, double* y,
                               ttvref_blasint incy)
{
    TTVREF_SYM(cblas_dgemv)(order, trans, m, n, alpha, a, lda, x, incx, beta, y, incy);
}
static inline void openblas_set_num_threads(int num) { TTVREF_SYM(openblas_set_num_threads)(num); }
static inline int openblas_get_num_threads(void) { return TTVREF_SYM(openblas_get_num_threads)(); }
#endif

#endif /* TTVREF_CBLAS_SHIM_H */
