/*
 * CPU oracle for the mode-q tensor-times-vector path.
 *
 * TEST INFRASTRUCTURE: only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline / reference arm load this file's library.  It is the checker,
 * never the thing measured as the GPU engine and never shipped on the product
 * path.
 *
 * Every function restates one piece of the reference library (bassoy/ttv);
 * the file:line it follows is given beside it.  Parity of this restatement is
 * pinned against the reference compiled from its own headers (ref_shim.cpp)
 * and against the reference's known-answer tests.
 *
 * Built with -ffp-contract=off (both this file and the reference shim) so the
 * restated loops round exactly like the reference on every host.
 */
#include "ttv_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* shape.h                                                                   */
/* ------------------------------------------------------------------------ */

/* shape.h:30-34 */
int orc_is_valid_shape(const size_t* n, size_t len)
{
    if (len == 0) return 0;
    for (size_t r = 0; r < len; ++r)
        if (n[r] == 0) return 0;
    return 1;
}

/* shape.h:38-46 */
static int is_scalar(const size_t* n, size_t len)
{
    if (!orc_is_valid_shape(n, len)) return 0;
    for (size_t r = 0; r < len; ++r)
        if (n[r] != 1) return 0;
    return 1;
}

/* shape.h:49-65: one of the first two extents > 1, one == 1, the rest == 1 */
static int is_vector(const size_t* n, size_t len)
{
    if (!orc_is_valid_shape(n, len)) return 0;
    if (len == 1) return n[0] > 1;
    int any_gt1 = n[0] > 1 || n[1] > 1;
    int any_eq1 = n[0] == 1 || n[1] == 1;
    for (size_t r = 2; r < len; ++r)
        if (n[r] != 1) return 0;
    return any_gt1 && any_eq1;
}

/* shape.h:67-78 */
static int is_matrix(const size_t* n, size_t len)
{
    if (!orc_is_valid_shape(n, len) || len < 2) return 0;
    if (!(n[0] > 1 && n[1] > 1)) return 0;
    for (size_t r = 2; r < len; ++r)
        if (n[r] != 1) return 0;
    return 1;
}

/* shape.h:82-91 */
static int is_tensor(const size_t* n, size_t len)
{
    if (!orc_is_valid_shape(n, len) || len < 3) return 0;
    for (size_t r = 2; r < len; ++r)
        if (n[r] > 1) return 1;
    return 0;
}

/* shape.h:103-123: drop the extent of mode q */
int orc_output_shape(const size_t* na, size_t p, size_t q, size_t* nc)
{
    if (!orc_is_valid_shape(na, p)) return 1;
    if (q == 0 || q > p) return 2;
    size_t o = 0;
    for (size_t r = 0; r < p; ++r)
        if (r != q - 1) nc[o++] = na[r];
    return 0;
}

/* ------------------------------------------------------------------------ */
/* layout.h                                                                  */
/* ------------------------------------------------------------------------ */

/* layout.h:29-55: a permutation of 1..len */
int orc_is_valid_layout(const size_t* pi, size_t len)
{
    if (len == 0) return 0;
    for (size_t r = 0; r < len; ++r) {
        if (pi[r] == 0 || pi[r] > len) return 0;
        for (size_t s = r + 1; s < len; ++s)
            if (pi[s] == pi[r]) return 0;
    }
    return 1;
}

/* layout.h:57-76: k-order layout, k = 0 means last-order */
int orc_k_order_layout(size_t p, size_t k, size_t* pi)
{
    if (p == 0) return 1;
    if (k == 0) k = p;
    size_t m = k > p ? p : k;
    size_t r = 0;
    for (size_t v = m; r < m; --v, ++r) pi[r] = v;
    for (size_t v = m + 1; r < p; ++v, ++r) pi[r] = v;
    return 0;
}

/* layout.h:114-138: one-based position of a mode in the layout */
size_t orc_inverse_mode(const size_t* pi, size_t p, size_t mode)
{
    for (size_t r = 0; r < p; ++r)
        if (pi[r] == mode) return r + 1;
    return 0;
}

/* layout.h:143-172: remove mode q and renumber the modes above q */
int orc_output_layout(const size_t* pia, size_t p, size_t q, size_t* pic)
{
    if (!orc_is_valid_layout(pia, p)) return 1;
    if (q == 0 || q > p) return 2;
    size_t o = 0;
    for (size_t r = 0; r < p; ++r) {
        if (pia[r] == q) continue;
        pic[o++] = pia[r] > q ? pia[r] - 1 : pia[r];
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* strides.h                                                                 */
/* ------------------------------------------------------------------------ */

/* strides.h:31-57 (note: vectors and scalars get all-ones strides) */
int orc_strides(const size_t* n, const size_t* pi, size_t p, size_t* w)
{
    if (!orc_is_valid_shape(n, p)) return 1;
    if (!orc_is_valid_layout(pi, p)) return 2;
    for (size_t r = 0; r < p; ++r) w[r] = 1;
    if (is_vector(n, p) || is_scalar(n, p)) return 0;
    if (!is_matrix(n, p) && !is_tensor(n, p)) return 0;
    for (size_t r = 1; r < p; ++r)
        w[pi[r] - 1] = w[pi[r - 1] - 1] * n[pi[r - 1] - 1];
    return 0;
}

/* strides.h:76-101: strides must not decrease along the layout */
int orc_is_valid_strides(const size_t* pi, size_t len, const size_t* w)
{
    if (!orc_is_valid_layout(pi, len)) return -1;
    if (len == 1 && w[0] == 1) return 1;
    for (size_t r = 0; r + 1 < len; ++r)
        if (w[pi[r] - 1] > w[pi[r + 1] - 1]) return 0;
    return 1;
}

/* ------------------------------------------------------------------------ */
/* cases.h:24-36                                                             */
/* ------------------------------------------------------------------------ */
int orc_case(size_t p, size_t q, const size_t* pi)
{
    if (p == 1) return 1;
    if (p == 2) {
        if (q == 1 && pi[0] == 1) return 2;
        if (q == 2 && pi[0] == 1) return 3;
        if (q == 1 && pi[0] == 2) return 4;
        if (q == 2 && pi[0] == 2) return 5;
        return 0;
    }
    if (pi[0] == q) return 6;
    if (pi[p - 1] == q) return 7;
    return 8;
}

/* ------------------------------------------------------------------------ */
/* ttv.h:64-89 validation                                                    */
/* ------------------------------------------------------------------------ */
static const char* const k_messages[] = {
    "",
    "Error in tlib::tensor_times_vector: input tensor order should be greater zero.",
    "Error in tlib::tensor_times_vector: contraction mode should be greater zero or less than or equal to p.",
    "Error in tlib::tensor_times_vector: pointer to input tensor A should not be zero.",
    "Error in tlib::tensor_times_vector: pointer to input vector B should not be zero.",
    "Error in tlib::tensor_times_vector: pointer to output tensor C should not be zero.",
    "Error in tlib::tensor_times_vector: pointer to input tensor shape vector na should not be zero.",
    "Error in tlib::tensor_times_vector: pointer to input vector shape vector nb should not be zero.",
    "Error in tlib::tensor_times_vector: pointer to output tensor shape vector nc should not be zero.",
    "Error in tlib::tensor_times_vector: pointer to input tensor stride vector wa should not be zero.",
    "Error in tlib::tensor_times_vector: pointer to output tensor stride vector wc should not be zero.",
    "Error in tlib::tensor_times_vector: pointer to input tensor permutation vector pia should not be zero.",
    "Error in tlib::tensor_times_vector: pointer to output tensor permutation vector pic should not be zero.",
    "Error in tlib::tensor_times_vector: contraction dimension of A and B are not equal.",
    "Error in tlib::tensor_times_vector: shape vector of A is not valid.",
    "Error in tlib::tensor_times_vector: shape vector of C is not valid.",
    "Error in tlib::tensor_times_vector: layout vector of A is not valid.",
    "Error in tlib::tensor_times_vector: layout vector of C is not valid.",
    "Error in tlib::tensor_times_vector: stride vector of A is not valid.",
    "Error in tlib::tensor_times_vector: stride vector of C is not valid.",
    "Error in tlib::detail::compute_inverse_pia_m: beginning of layout tuples of both tensors are not correct.",
    "Error in tlib::detail::compute_inverse_pia_m: end of layout tuples of both tensors are not correct.",
    "oracle: the slice path is undefined for unit extents (the reference addresses out of bounds)",
};

const char* orc_check_message(int code)
{
    if (code < 0 || code > 22) return "unknown";
    return k_messages[code];
}

int orc_check(size_t q, size_t p, int a_nonnull, const size_t* na, const size_t* wa,
              const size_t* pia, int b_nonnull, const size_t* nb, int c_nonnull,
              const size_t* nc, const size_t* wc, const size_t* pic)
{
    if (p == 0) return 1;
    if (q == 0 || q > p) return 2;
    if (!a_nonnull) return 3;
    if (!b_nonnull) return 4;
    if (!c_nonnull) return 5;
    if (!na) return 6;
    if (!nb) return 7;
    if (!nc) return 8;
    if (!wa) return 9;
    if (!wc) return 10;
    if (!pia) return 11;
    if (!pic) return 12;
    if (na[q - 1] != nb[0]) return 13;
    if (!orc_is_valid_shape(na, p)) return 14;
    if (!orc_is_valid_shape(nc, p - 1)) return 15;
    if (!orc_is_valid_layout(pia, p)) return 16;
    if (!orc_is_valid_layout(pic, p - 1)) return 17;
    if (orc_is_valid_strides(pia, p, wa) != 1) return 18;
    if (orc_is_valid_strides(pic, p - 1, wc) != 1) return 19;
    return 0;
}

/* tensor_times_vector.h:147-168: pic must be the layout pia induces */
int orc_check_pic(const size_t* pia, const size_t* pic, size_t p, size_t q)
{
    size_t k = orc_inverse_mode(pia, p, q);   /* one-based */
    for (size_t i = 0; i + 1 < k; ++i)
        if ((pia[i] > q && pic[i] + 1 != pia[i]) || (pia[i] < q && pic[i] != pia[i])) return 1;
    for (size_t i = k - 1; i + 1 < p; ++i)
        if ((pia[i + 1] > q && pic[i] + 1 != pia[i + 1]) || (pia[i + 1] < q && pic[i] != pia[i + 1]))
            return 2;
    return 0;
}

void orc_canonical(size_t p, size_t q, const size_t* na, const size_t* pia,
                   uint64_t* P, uint64_t* nq, uint64_t* S)
{
    size_t k = orc_inverse_mode(pia, p, q) - 1;
    uint64_t pre = 1, suf = 1;
    for (size_t r = 0; r < k; ++r) pre *= na[pia[r] - 1];
    for (size_t r = k + 1; r < p; ++r) suf *= na[pia[r] - 1];
    *P = pre;
    *nq = na[q - 1];
    *S = suf;
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* matrix_times_vector.h kernels, restated per element type                  */
/* ------------------------------------------------------------------------ */
/* The generator below instantiates the restated kernels and paths for one
 * element type T with suffix SFX. */
#define ORC_DEFINE_KERNELS(T, SFX)                                                          \
/* matrix_times_vector.h:52-69: row-wise dot products, overwrites c */                      \
static void gemv_row_##SFX(const T* a, const T* b, T* c, size_t M, size_t N, size_t lda)    \
{                                                                                           \
    for (size_t i = 0; i < M; ++i) {                                                        \
        const T* arow = a + i * lda;                                                        \
        T sum = 0;                                                                          \
        _Pragma("omp simd reduction(+:sum)")                                                \
        for (size_t k = 0; k < N; ++k) sum += arow[k] * b[k];                               \
        c[i] = sum;                                                                         \
    }                                                                                       \
}                                                                                           \
/* matrix_times_vector.h:109-127: column-major axpy sweep, accumulates into c */            \
static void gemv_col_##SFX(const T* a, const T* b, T* c, size_t M, size_t N, size_t lda)    \
{                                                                                           \
    for (size_t i = 0; i < N; ++i) {                                                        \
        const T* a0 = a + i * lda;                                                          \
        const T bb = b[i];                                                                  \
        _Pragma("omp simd")                                                                 \
        for (size_t j = 0; j < M; ++j) c[j] += a0[j] * bb;                                  \
    }                                                                                       \
}                                                                                           \
/* matrix_times_vector.h:315-330: cases 2-7 of mtv(seq) (case 1 unreachable, p>=2) */      \
static void mtv_##SFX(size_t m, size_t p, const T* a, const size_t* na, const size_t* pia,   \
                      const T* b, T* c)                                                     \
{                                                                                           \
    size_t full = 1;                                                                        \
    for (size_t r = 0; r < p; ++r) full *= na[r];                                           \
    size_t n = full / na[m - 1];                                                            \
    switch (orc_case(p, m, pia)) {                                                          \
    case 2: gemv_row_##SFX(a, b, c, na[1], na[0], na[0]); break;                            \
    case 3: gemv_col_##SFX(a, b, c, na[0], na[1], na[0]); break;                            \
    case 4: gemv_col_##SFX(a, b, c, na[1], na[0], na[1]); break;                            \
    case 5: gemv_row_##SFX(a, b, c, na[0], na[1], na[1]); break;                            \
    case 6: gemv_row_##SFX(a, b, c, n, na[m - 1], na[m - 1]); break;                        \
    case 7: gemv_col_##SFX(a, b, c, n, na[m - 1], n); break;                                \
    default: break;                                                                         \
    }                                                                                       \
}                                                                                           \
/* tensor_times_vector.h:296-324: recursion over the modes after q in the layout,          \
 * one column-major GEMV per subtensor of the leading modes */                              \
static void subtensors_##SFX(unsigned r, unsigned qq, size_t nn, size_t na_m, size_t wa_m,  \
                             unsigned inv, const T* a, const size_t* na, const size_t* wa,  \
                             const size_t* pia, const T* b, T* c, const size_t* wc,         \
                             const size_t* pic)                                             \
{                                                                                           \
    if (r > 0) {                                                                            \
        if (inv >= r) {                                                                     \
            subtensors_##SFX(r - 1, qq - 1, nn, na_m, wa_m, inv, a, na, wa, pia, b, c, wc,  \
                             pic);                                                          \
        } else {                                                                            \
            const size_t ext = na[pia[r - 1] - 1];                                          \
            const size_t sa = wa[pia[r - 1] - 1];                                           \
            const size_t sc = wc[pic[qq - 1] - 1];                                          \
            for (size_t i = 0; i < ext; ++i)                                                \
                subtensors_##SFX(r - 1, qq - 1, nn, na_m, wa_m, inv, a + i * sa, na, wa,    \
                                 pia, b, c + i * sc, wc, pic);                              \
        }                                                                                   \
    } else {                                                                                \
        gemv_col_##SFX(a, b, c, nn, na_m, wa_m);                                            \
    }                                                                                       \
}                                                                                           \
/* index.h:102-117: fused loop counter -> memory offset (view strides w_view) */           \
static size_t at_at_1_##SFX(size_t np, size_t j, const size_t* wv, const size_t* warr,      \
                            const size_t* pi)                                               \
{                                                                                           \
    size_t k = j, off = 0;                                                                  \
    for (size_t r = np; r-- > 0;) {                                                         \
        size_t q = pi[r] - 1;                                                               \
        size_t i = k / wv[q];                                                               \
        k -= wv[q] * i;                                                                     \
        off += warr[q] * i;                                                                 \
    }                                                                                       \
    return off;                                                                             \
}                                                                                           \
/* tensor_times_vector.h:706-772 + workload_computation.h:36-124: every 2-D slice        \
 * (mode pia[0] x mode q) is one GEMV; all other free modes are fused into one loop */      \
static void slices_all_##SFX(size_t m, size_t p, const T* a, const size_t* na,              \
                             const size_t* wa, const size_t* pia, const T* b, T* c,         \
                             const size_t* wc, const size_t* pic)                           \
{                                                                                           \
    const size_t pi1 = pia[0];                                                              \
    const size_t np = p - 2;                                                                \
    size_t tau[64] = {0}, wa2[64] = {0}, wc2[64] = {0}, na2[64] = {0}, va2[64] = {0};                                \
    /* divide_layout: drop pi1 and m, renumber */                                           \
    for (size_t i = 0, j = 0; i < p; ++i) {                                                 \
        size_t v = pia[i];                                                                  \
        if (v == pi1 || v == m) continue;                                                   \
        tau[j] = v - (v > pi1) - (v > m);                                                   \
        ++j;                                                                                \
    }                                                                                       \
    /* divide(v, pi, p, m): the entries of modes other than pi1 and m, in mode order */     \
    for (size_t i = 0, j = 0; i < p; ++i)                                                   \
        if (i + 1 != pi1 && i + 1 != m) { wa2[j] = wa[i]; na2[j] = na[i]; ++j; }            \
    /* divide(v, pi, p) for C: drop the entry of C's first layout mode */                   \
    for (size_t i = 0, j = 0; i + 1 < p; ++i)                                               \
        if (i + 1 != pic[0]) wc2[j++] = wc[i];                                              \
    orc_strides(na2, tau, np, va2);                                                         \
    size_t nn = 1;                                                                          \
    for (size_t r = 0; r < np; ++r) nn *= na2[r];                                           \
    const size_t na_pia_1 = na[pi1 - 1], na_m = na[m - 1], wa_m = wa[m - 1];                \
    _Pragma("omp parallel for schedule(static)")                                            \
    for (size_t k = 0; k < nn; ++k) {                                                       \
        size_t ka = at_at_1_##SFX(np, k, va2, wa2, tau);                                    \
        size_t kc = at_at_1_##SFX(np, k, va2, wc2, tau);                                    \
        gemv_col_##SFX(a + ka, b, c + kc, na_pia_1, na_m, wa_m);                            \
    }                                                                                       \
}                                                                                           \
int orc_ttv_##SFX(int policy, size_t q, size_t p, const T* a, const size_t* na,              \
                  const size_t* wa, const size_t* pia, const T* b, const size_t* nb, T* c,   \
                  const size_t* nc, const size_t* wc, const size_t* pic)                    \
{                                                                                           \
    int err = orc_check(q, p, a != 0, na, wa, pia, b != 0, nb, c != 0, nc, wc, pic);        \
    if (err) return err;                                                                    \
    if (orc_case(p, q, pia) != 8) {                                                         \
        mtv_##SFX(q, p, a, na, pia, b, c);                                                  \
        return 0;                                                                           \
    }                                                                                       \
    if (policy == 2) {                                                                      \
        /* The slice path never runs compute_inverse_pia_m.  Its fused-index strides come  \
         * from generate_strides, which gives all-ones strides to vector-like sub-shapes;   \
         * with a unit extent among the fused modes the reference then addresses memory    \
         * outside A and C.  Such inputs are refused here instead of reproducing that. */  \
        for (size_t r = 0; r < p; ++r)                                                      \
            if (na[r] == 1) return 22;                                                      \
        slices_all_##SFX(q, p, a, na, wa, pia, b, c, wc, pic);                              \
        return 0;                                                                           \
    }                                                                                       \
    int perr = orc_check_pic(pia, pic, p, q);                                               \
    if (perr) return 19 + perr;                                                             \
    const unsigned inv = (unsigned)orc_inverse_mode(pia, p, q);                             \
    const size_t na_m = na[q - 1], wa_m = wa[q - 1];                                        \
    size_t n = 1;                                                                           \
    for (unsigned r = 0; r + 1 < inv; ++r) n *= na[pia[r] - 1];                             \
    if (policy == 0) {                                                                      \
        subtensors_##SFX((unsigned)p, (unsigned)p - 1, n, na_m, wa_m, inv, a, na, wa, pia,  \
                         b, c, wc, pic);                                                    \
        return 0;                                                                           \
    }                                                                                       \
    /* policy 1, tensor_times_vector.h:1226-1254: one flat loop over the suffix */          \
    size_t num = 1;                                                                         \
    for (size_t i = inv; i < p; ++i) num *= na[pia[i] - 1];                                 \
    const size_t wa_m1 = wa[pia[inv] - 1];                                                  \
    const size_t wc_m1 = wc[pic[inv - 1] - 1];                                              \
    _Pragma("omp parallel for schedule(static)")                                            \
    for (size_t i = 0; i < num; ++i)                                                        \
        subtensors_##SFX(inv - 1, inv - 1, wa_m, na_m, wa_m, inv, a + i * wa_m1, na, wa,    \
                         pia, b, c + i * wc_m1, wc, pic);                                   \
    return 0;                                                                               \
}                                                                                           \
/* Canonical (S, nq, P) form of the same products with the same per-output               \
 * accumulation order, parallel over every output (CPU baseline). */                        \
void orc_canon_##SFX(uint64_t S, uint64_t nq, uint64_t P, const T* a, const T* b, T* c)     \
{                                                                                           \
    if (P == 1) {                                                                           \
        _Pragma("omp parallel for schedule(static)")                                        \
        for (uint64_t s = 0; s < S; ++s) {                                                  \
            const T* arow = a + s * nq;                                                     \
            T sum = 0;                                                                      \
            _Pragma("omp simd reduction(+:sum)")                                            \
            for (uint64_t k = 0; k < nq; ++k) sum += arow[k] * b[k];                        \
            c[s] = sum;                                                                     \
        }                                                                                   \
        return;                                                                             \
    }                                                                                       \
    const uint64_t JB = 2048;                                                               \
    const uint64_t nblk = (P + JB - 1) / JB;                                                \
    _Pragma("omp parallel for schedule(static)")                                            \
    for (uint64_t t = 0; t < S * nblk; ++t) {                                               \
        const uint64_t s = t / nblk, j0 = (t % nblk) * JB;                                  \
        const uint64_t jn = (P - j0) < JB ? (P - j0) : JB;                                  \
        T* cc = c + s * P + j0;                                                             \
        for (uint64_t j = 0; j < jn; ++j) cc[j] = 0;                                        \
        const T* ap = a + s * nq * P + j0;                                                  \
        for (uint64_t i = 0; i < nq; ++i) {                                                 \
            const T* a0 = ap + i * P;                                                       \
            const T bb = b[i];                                                              \
            _Pragma("omp simd")                                                             \
            for (uint64_t j = 0; j < jn; ++j) cc[j] += a0[j] * bb;                          \
        }                                                                                   \
    }                                                                                       \
}

ORC_DEFINE_KERNELS(float, f32)
ORC_DEFINE_KERNELS(double, f64)

/* ------------------------------------------------------------------------ */
/* truth: double-double accumulation (Dekker / Knuth error-free transforms)  */
/* ------------------------------------------------------------------------ */
static inline void dd_add(double* hi, double* lo, double x, double xe)
{
    double s = *hi + x;
    double bb = s - *hi;
    double e = (*hi - (s - bb)) + (x - bb);
    e += *lo + xe;
    double h = s + e;
    *lo = e - (h - s);
    *hi = h;
}

/* Per output the products are added in ascending i, each into a double-double
 * sum; rows (P == 1) one output at a time, columns (P > 1) in blocks of
 * ORC_TRUTH_JB neighbouring outputs that walk their rows together (the same
 * additions in the same order per output, read along the contiguous prefix). */
#define ORC_TRUTH_JB 64
#define ORC_DEFINE_TRUTH(NAME, TA, TB, LOADA, EXACT_PRODUCT)                                \
void NAME(uint64_t S, uint64_t nq, uint64_t P, const TA* a, const TB* b, double* ref,        \
          double* absn)                                                                     \
{                                                                                           \
    const uint64_t nblk = (P + ORC_TRUTH_JB - 1) / ORC_TRUTH_JB;                            \
    _Pragma("omp parallel for schedule(dynamic, 4)")                                        \
    for (uint64_t t = 0; t < S * nblk; ++t) {                                               \
        const uint64_t s = t / nblk, j0 = (t % nblk) * ORC_TRUTH_JB;                        \
        const uint64_t jn = (P - j0) < ORC_TRUTH_JB ? (P - j0) : ORC_TRUTH_JB;              \
        double hi[ORC_TRUTH_JB], lo[ORC_TRUTH_JB], an[ORC_TRUTH_JB];                        \
        for (uint64_t j = 0; j < jn; ++j) hi[j] = lo[j] = an[j] = 0.0;                      \
        const TA* ap = a + s * nq * P + j0;                                                 \
        for (uint64_t i = 0; i < nq; ++i) {                                                 \
            const double bv = (double)b[i];                                                 \
            const TA* row = ap + i * P;                                                     \
            for (uint64_t j = 0; j < jn; ++j) {                                             \
                double av = LOADA(row[j]);                                                  \
                double pr = av * bv;                                                        \
                double pe = EXACT_PRODUCT ? 0.0 : fma(av, bv, -pr);                         \
                dd_add(&hi[j], &lo[j], pr, pe);                                             \
                an[j] += fabs(pr);                                                          \
            }                                                                               \
        }                                                                                   \
        for (uint64_t j = 0; j < jn; ++j) {                                                 \
            ref[s * P + j0 + j] = hi[j] + lo[j];                                            \
            absn[s * P + j0 + j] = an[j];                                                   \
        }                                                                                   \
    }                                                                                       \
}

static inline double load_f32(float v) { return (double)v; }
static inline double load_f64(double v) { return v; }
static inline double load_bf16(uint16_t v)
{
    uint32_t u = ((uint32_t)v) << 16;
    float f;
    memcpy(&f, &u, 4);
    return (double)f;
}

ORC_DEFINE_TRUTH(orc_truth_f32, float, float, load_f32, 1)
ORC_DEFINE_TRUTH(orc_truth_f64, double, double, load_f64, 0)
ORC_DEFINE_TRUTH(orc_truth_bf16a, uint16_t, float, load_bf16, 1)

/* ------------------------------------------------------------------------ */
/* truth of the multi-vector chain (ttvpy.ttvs, wrapped_ttv.cpp:85-199):     */
/* every mode but q contracted.  In the canonical (S, nq, P) view of A,      */
/* c[i] = sum_s sum_j A[s, i, j] wS[s] wP[j] with wS, wP the Kronecker       */
/* products of the suffix and prefix vectors (given in double).  Each        */
/* product a * (wS wP) is added exactly (TwoProduct) into a double-double    */
/* sum per output; absn = sum |a wS wP|.                                     */
/* ------------------------------------------------------------------------ */
#define ORC_DEFINE_TRUTH_TTVS(NAME, TA, LOADA, EXACT_PRODUCT)                               \
void NAME(uint64_t S, uint64_t nq, uint64_t P, const TA* a, const double* wS,               \
          const double* wP, double* ref, double* absn)                                      \
{                                                                                           \
    _Pragma("omp parallel for schedule(dynamic, 1)")                                        \
    for (uint64_t i = 0; i < nq; ++i) {                                                     \
        double hi = 0.0, lo = 0.0, an = 0.0;                                                \
        for (uint64_t s = 0; s < S; ++s) {                                                  \
            const TA* row = a + (s * nq + i) * P;                                           \
            for (uint64_t j = 0; j < P; ++j) {                                              \
                const double w = wS[s] * wP[j];                                             \
                const double av = LOADA(row[j]);                                            \
                const double pr = av * w;                                                   \
                const double pe = fma(av, w, -pr);                                          \
                dd_add(&hi, &lo, pr, pe);                                                   \
                an += fabs(pr);                                                             \
            }                                                                               \
        }                                                                                   \
        ref[i] = hi + lo;                                                                   \
        absn[i] = an;                                                                       \
    }                                                                                       \
}

ORC_DEFINE_TRUTH_TTVS(orc_truth_ttvs_f32, float, load_f32, 1)
ORC_DEFINE_TRUTH_TTVS(orc_truth_ttvs_f64, double, load_f64, 0)
ORC_DEFINE_TRUTH_TTVS(orc_truth_ttvs_bf16a, uint16_t, load_bf16, 1)
