/*
 * CPU oracle for the mode-q tensor-times-vector path (TEST INFRASTRUCTURE ONLY).
 *
 * This is a plain-C restatement of the reference library's algorithm for
 *   C = A x_q b
 * used as the checker for the CUDA engine (and as the timed CPU baseline of
 * the benchmark).  Nothing in the product path links or calls it.
 *
 * Parity: pinned.  The restatement is checked bit-for-bit against the
 * reference headers compiled from source (oracle/ref_shim.cpp -> oracle/_ref)
 * and against the reference's own known-answer tests (restated in tests/).
 *
 * Reference files restated here (paths inside the reference project):
 *   include/tlib/detail/shape.h      shape predicates, output shape
 *   include/tlib/detail/layout.h     layout predicates, k-order / output layout
 *   include/tlib/detail/strides.h    stride generation and validation
 *   include/tlib/detail/cases.h      the eight (p, q, pi) cases
 *   include/tlib/ttv.h:64-89         argument validation of the low-level call
 *   include/tlib/detail/tensor_times_vector.h:147-168  pic/pia consistency
 *   include/tlib/detail/tensor_times_vector.h:934-968  seq/subtensor/none
 *   include/tlib/detail/tensor_times_vector.h:1208-1256 par_loop/subtensor/all
 *   include/tlib/detail/tensor_times_vector.h:706-772  par_loop/slice/all
 *   include/tlib/detail/matrix_times_vector.h:52-127,265-330  gemv_row/gemv_col/dot/mtv
 */
#ifndef TTV_ORACLE_H
#define TTV_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- metadata (shape.h / layout.h / strides.h) ---- */
int  orc_is_valid_shape(const size_t* n, size_t len);
int  orc_is_valid_layout(const size_t* pi, size_t len);
/* 1 valid, 0 invalid, -1 the layout itself is invalid (the reference throws) */
int  orc_is_valid_strides(const size_t* pi, size_t len, const size_t* w);
/* 0 ok, nonzero error (reference throws) */
int  orc_output_shape(const size_t* na, size_t p, size_t q, size_t* nc);
int  orc_output_layout(const size_t* pia, size_t p, size_t q, size_t* pic);
int  orc_strides(const size_t* n, const size_t* pi, size_t p, size_t* w);
int  orc_k_order_layout(size_t p, size_t k, size_t* pi);
size_t orc_inverse_mode(const size_t* pi, size_t p, size_t mode);
int  orc_case(size_t p, size_t q, const size_t* pi);

/* ---- argument validation of the low-level call (ttv.h:64-89) ----
 * Returns 0 when the call is valid, else the 1-based index of the first
 * failing check; orc_check_message() gives the reference's exception text. */
int orc_check(size_t q, size_t p, int a_nonnull, const size_t* na, const size_t* wa,
              const size_t* pia, int b_nonnull, const size_t* nb, int c_nonnull,
              const size_t* nc, const size_t* wc, const size_t* pic);
const char* orc_check_message(int code);
/* pic/pia consistency of case 8 (tensor_times_vector.h:147-168):
 * 0 ok, 1 "beginning" error, 2 "end" error */
int orc_check_pic(const size_t* pia, const size_t* pic, size_t p, size_t q);

/* ---- canonical view: A = (S, nq, P) row-major, C = (S, P) ---- */
void orc_canonical(size_t p, size_t q, const size_t* na, const size_t* pia,
                   uint64_t* P, uint64_t* nq, uint64_t* S);

/* ---- restated execution paths (C must be zero on entry, as the
 *      reference's callers guarantee) ----
 * policy: 0 seq/subtensor/none, 1 par_loop/subtensor/all, 2 par_loop/slice/all
 * Returns 0, or the orc_check / pic error (C untouched then). */
int orc_ttv_f32(int policy, size_t q, size_t p, const float* a, const size_t* na,
                const size_t* wa, const size_t* pia, const float* b, const size_t* nb,
                float* c, const size_t* nc, const size_t* wc, const size_t* pic);
int orc_ttv_f64(int policy, size_t q, size_t p, const double* a, const size_t* na,
                const size_t* wa, const size_t* pia, const double* b, const size_t* nb,
                double* c, const size_t* nc, const size_t* wc, const size_t* pic);

/* ---- canonical batched column/row products with the reference's
 *      accumulation order, OpenMP over outputs (CPU baseline) ---- */
void orc_canon_f32(uint64_t S, uint64_t nq, uint64_t P, const float* a, const float* b, float* c);
void orc_canon_f64(uint64_t S, uint64_t nq, uint64_t P, const double* a, const double* b, double* c);

/* ---- high-precision truth and error normaliser ----
 * ref[o]  = sum_i a[s,i,j] * b[i]   (double-double accumulation, rounded to double)
 * absn[o] = sum_i |a[s,i,j] * b[i]| (double)
 * bf16 variant takes A as raw bf16 bit patterns (uint16). */
void orc_truth_f32(uint64_t S, uint64_t nq, uint64_t P, const float* a, const float* b,
                   double* ref, double* absn);
void orc_truth_f64(uint64_t S, uint64_t nq, uint64_t P, const double* a, const double* b,
                   double* ref, double* absn);
void orc_truth_bf16a(uint64_t S, uint64_t nq, uint64_t P, const uint16_t* a, const float* b,
                     double* ref, double* absn);

int orc_num_threads(void);

#ifdef __cplusplus
}
#endif
/* truth of the multi-vector chain (every mode but q), canonical (S, nq, P)
 * view of A, Kronecker weights wS (S) and wP (P) in double */
void orc_truth_ttvs_f32(uint64_t S, uint64_t nq, uint64_t P, const float* a, const double* wS,
                        const double* wP, double* ref, double* absn);
void orc_truth_ttvs_f64(uint64_t S, uint64_t nq, uint64_t P, const double* a, const double* wS,
                        const double* wP, double* ref, double* absn);
void orc_truth_ttvs_bf16a(uint64_t S, uint64_t nq, uint64_t P, const uint16_t* a, const double* wS,
                          const double* wP, double* ref, double* absn);

#endif
