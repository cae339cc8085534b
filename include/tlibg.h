/*
 * tlibg -- GB300-native (sm_103a) mode-q tensor-times-vector engine, C ABI.
 *
 * Computes C = A x_q b for a dense tensor A of runtime order p with extents
 * na, strides wa and layout permutation pia (one-based, as in tlib).  Every
 * entry point takes plain pointers and sizes only, so any FFI (ctypes, cgo,
 * JNI, N-API) can bind it; the C++ drop-in policy lives in tlib/ttv_gpu.h.
 *
 * Conventions shared by all entry points
 *  - a, b, c are DEVICE pointers (except the *_host entry points); na, wa,
 *    pia, nb, nc, wc, pic are HOST arrays read before the call returns.
 *  - work is enqueued on `stream` (a cudaStream_t; NULL = legacy default
 *    stream) and is asynchronous with respect to the host, except where an
 *    entry point says otherwise.
 *  - the return value is a TLIBG_* status; the text of the last failure on
 *    the calling thread is available from tlibg_last_error().  Invalid calls
 *    fail with TLIBG_ERR_ARGUMENT and the exact exception text the reference
 *    throws for the same call, in the same order of checks.
 *  - C is overwritten (the reference's BLAS path uses beta = 0).
 *  - the engine never falls back to the CPU: without a usable GB300 the
 *    compute entry points fail with TLIBG_ERR_CUDA.
 */
#ifndef TLIBG_H
#define TLIBG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define TLIBG_OK               0
#define TLIBG_ERR_ARGUMENT     1  /* invalid call: the reference throws std::runtime_error   */
#define TLIBG_ERR_UNSUPPORTED  2  /* valid for the reference, outside this engine (see text)  */
#define TLIBG_ERR_CUDA         3  /* CUDA runtime error or no usable device                   */
#define TLIBG_ERR_NOMEM        4  /* device scratch could not be allocated                    */
#define TLIBG_ERR_TIMEOUT      5  /* a bounded device-side wait expired (kernel returned)     */

/* ---- element types ---- */
#define TLIBG_F32    0   /* A, b, C float                                      */
#define TLIBG_F64    1   /* A, b, C double                                     */
#define TLIBG_BF16A  2   /* A bfloat16 (raw 16-bit patterns), b and C float    */

/* ---- accumulation ---- */
#define TLIBG_ACC_COMPENSATED  0  /* default.  fp32: per-thread Kahan partials.  fp64: register   */
                                  /*   and row-tile kernels mix native DFMA (half the products)  */
                                  /*   with double-float accumulation on the FP32/INT32 pipes;    */
                                  /*   the streamed kernel, and the row-tile kernel on rows under */
                                  /*   8 elements, use DFMA                                        */
#define TLIBG_ACC_PLAIN        1  /* fp32: plain FMA accumulation; fp64: native DFMA only          */
#define TLIBG_ACC_DOUBLE_FLOAT 2  /* fp64: the mix everywhere (double-float for every in-window   */
                                  /*   product in the streamed kernel)                             */

/* ---- kernel families chosen by the planner ---- */
#define TLIBG_KIND_ROW 0   /* q is the fastest layout mode (prefix P == 1): lane-group dot products */
#define TLIBG_KIND_COL 1   /* q is a middle or outer mode: coalesced column GEMV over the prefix    */
#define TLIBG_KIND_STREAM 2        /* TMA-streamed rows (whole rows of <= 16 KB), any alignment     */
#define TLIBG_KIND_COL_REALIGN 3   /* column GEMV with 16-byte loads realigned by warp shuffles,    */
                                   /*   for prefixes whose rows are not 16-byte aligned (fp32/fp64) */
#define TLIBG_KIND_COL_THIN 4      /* column GEMV for thin prefixes (P / vector width divides 32):  */
                                   /*   several rows per warp step, for few outputs and long q      */
#define TLIBG_KIND_ROW_TILE 5      /* short rows (P == 1, n_q <= 64, no split): tiles of 32-128     */
                                   /*   rows moved to shared memory by TMA, 1-4 rows per lane, any  */
                                   /*   alignment                                                   */
#define TLIBG_KIND_COL_BULK 6      /* column GEMV (P > 1) fed by a TMA producer warp: 4 KB runs of  */
                                   /*   each row in a 3-stage shared-memory ring, any alignment     */
#define TLIBG_KIND_ROW_PANEL 7     /* long q-fastest rows, few of them (P == 1, 16-byte aligned      */
                                   /*   rows): a CTA holds a segment of b in registers and streams  */
                                   /*   that segment of a block of rows, so b is read once per row  */
                                   /*   block; `group` = rows in flight.  On request only           */
#define TLIBG_KIND_ROW_SHIFT 8     /* q-fastest rows that are not whole 16-byte vectors (P == 1,    */
                                   /*   fp32 / fp64): 16-byte loads of each row's aligned body      */
                                   /*   against shifted copies of b in shared memory, head and tail */
                                   /*   elements scalar; `group` = lanes per row.  Default for rows */
                                   /*   of >= 64 elements when the rows fill the lane groups        */

typedef struct tlibg_options {
    int accumulate;   /* TLIBG_ACC_*                                                      */
    int kind;         /* -1: planner; else force TLIBG_KIND_* (must match the problem)    */
    int group;        /* ROW: lanes per output (1..32, power of two); COL: warps along q  */
                      /*   (1, 2, 4 or 8).  0 = planner                                   */
    int vec;          /* elements per vector load (1, 2, 4 or 8); 0 = planner             */
    int split;        /* segments of the contracted mode (two-phase reduce); 0 = planner  */
    int sync;         /* nonzero: synchronise `stream` and check the device error word    */
} tlibg_options;

/* Launch configuration the planner picks for a canonical problem. */
typedef struct tlibg_plan_info {
    uint64_t P, nq, S;   /* prefix before q in the layout, contracted extent, suffix      */
    int kind, group, vec, split, accumulate;
    int grid, block;
} tlibg_plan_info;

/* ---------------------------------------------------------------------------
 * Low-level TTV, one per element type.
 * Replaces: template tlib::ttv::ttv(execution_t, slicing_t, fusion_t, q, p,
 *   a, na, wa, pia, b, nb, c, nc, wc, pic)  -- include/tlib/ttv.h:54-92,
 * dispatched there to detail::ttv (tensor_times_vector.h:416-421, 1208-1256).
 * Same argument meaning, same checks and messages (ttv.h:64-89 and
 * tensor_times_vector.h:160,164).  The slicing / fusion policies of the
 * reference are scheduling hints on the CPU; this engine always folds every
 * free mode into one grid (their `fusion_policy::all`).
 * ------------------------------------------------------------------------- */
int tlibg_ttv_f32(size_t q, size_t p,
                  const float* a, const size_t* na, const size_t* wa, const size_t* pia,
                  const float* b, const size_t* nb,
                  float* c, const size_t* nc, const size_t* wc, const size_t* pic,
                  void* stream);

int tlibg_ttv_f64(size_t q, size_t p,
                  const double* a, const size_t* na, const size_t* wa, const size_t* pia,
                  const double* b, const size_t* nb,
                  double* c, const size_t* nc, const size_t* wc, const size_t* pic,
                  void* stream);

/* A stored as bfloat16 (halves the bytes streamed from HBM), b and C float,
 * fp32 accumulation.  No reference counterpart for the storage type; the
 * call surface is that of ttv.h:54-60 with value_t = float for b and C. */
int tlibg_ttv_bf16a_f32(size_t q, size_t p,
                        const uint16_t* a, const size_t* na, const size_t* wa, const size_t* pia,
                        const float* b, const size_t* nb,
                        float* c, const size_t* nc, const size_t* wc, const size_t* pic,
                        void* stream);

/* Generic form of the three above with explicit options (NULL = defaults). */
int tlibg_ttv_ex(int dtype, size_t q, size_t p,
                 const void* a, const size_t* na, const size_t* wa, const size_t* pia,
                 const void* b, const size_t* nb,
                 void* c, const size_t* nc, const size_t* wc, const size_t* pic,
                 const tlibg_options* opt, void* stream);

/* Extension (no reference counterpart): the same contraction on DEVICE
 * pointers with the natural meaning of every stride, for sliced, padded or
 * transposed views -- A's element (i_1..i_p) at a[sum_r i_r wa[r]] (zero-based
 * indices, strides in elements), b's element i at b[i wb], C's element
 * (j_1..j_{p-1}) at c[sum_r j_r wc[r]], C's modes being A's modes without q.
 * Same checks and messages as tlibg_ttv_f32 for shapes, layouts and monotonic
 * strides; unlike the drop-in calls (whose dense-only rule follows the
 * reference, which gives non-dense strides no single meaning) any stride
 * vector is taken, as long as no two outputs share an element of C
 * (TLIBG_ERR_UNSUPPORTED otherwise) and every offset stays below 2^62.
 * dtype TLIBG_F32 or TLIBG_F64; compensated accumulation; asynchronous on
 * `stream`.  Views that are dense take the dense kernels' speed only through
 * tlibg_ttv_*. */
int tlibg_ttv_strided(int dtype, size_t q, size_t p,
                      const void* a, const size_t* na, const size_t* wa, const size_t* pia,
                      const void* b, const size_t* nb, size_t wb,
                      void* c, const size_t* nc, const size_t* wc, const size_t* pic, void* stream);

/* Same call with HOST pointers a, b, c, as the reference takes them.  A in
 * page-locked memory whose plan reads 512-byte runs per warp load (column
 * tiles with 16-byte loads, rows taken by a whole warp) is read in place by
 * the kernels over the host link (one pass, no staging copy); every
 * other A is staged to the device in chunks overlapped with the kernels
 * (page-locked: copied by the SMs; pageable: by the copy engine).  A page-locked C is written in
 * place by the kernels; b (and a pageable C) go through device buffers.  The
 * call returns when C is complete on the host (the reference's synchronous
 * semantics). */
int tlibg_ttv_host(int dtype, size_t q, size_t p,
                   const void* a, const size_t* na, const size_t* wa, const size_t* pia,
                   const void* b, const size_t* nb,
                   void* c, const size_t* nc, const size_t* wc, const size_t* pic,
                   const tlibg_options* opt);

/* The plan the engine would use for a call (no device work, no CUDA calls
 * except the one-time device-property query). */
int tlibg_plan(int dtype, size_t q, size_t p, const size_t* na, const size_t* pia,
               const tlibg_options* opt, tlibg_plan_info* out);

/* Installs autotuned options for canonical problems (type, P, n_q, S): later
 * calls whose options leave every kernel choice to the planner (or pass NULL)
 * use them.  opt == NULL removes the hint; with P = n_q = S = 0, all hints. */
int tlibg_plan_hint(int dtype, uint64_t P, uint64_t nq, uint64_t S, const tlibg_options* opt);

/* Self-test of the failure path: launches one kernel whose mbarrier wait
 * nothing completes, with a short poll limit (a few milliseconds).  The wait
 * gives up, records it in the device error word and the kernel returns; the
 * call then reports exactly what an expired wait inside a TTV reports:
 * TLIBG_ERR_TIMEOUT with its message.  No trap, no fault: the context stays
 * usable.  Synchronises `stream`. */
int tlibg_selftest_bounded_wait(void* stream);

/* Where a pointer lives: 1 device or managed memory, 0 host memory (pageable
 * or page-locked; every pointer when no device is present), -1 null or
 * unknown.  The compute entry points refuse pageable host pointers
 * (TLIBG_ERR_ARGUMENT) before any launch; host buffers go to tlibg_ttv_host. */
int tlibg_pointer_location(const void* p);

/* Validation only: the checks of the compute entry points (ttv.h:64-89 and
 * tensor_times_vector.h:147-168, in that order, same messages) on the metadata
 * alone, with no data pointers, no device and no launch.  Lets a host wrapper
 * that knows its buffers' sizes check them against the layout once the
 * reference's own checks have passed. */
int tlibg_validate(size_t q, size_t p, const size_t* na, const size_t* wa, const size_t* pia,
                   const size_t* nb, const size_t* nc, const size_t* wc, const size_t* pic);

/* ---------------------------------------------------------------------------
 * Metadata helpers (host only, no device needed).
 * Replace: detail::generate_output_shape (shape.h:103-158),
 * detail::generate_output_layout (layout.h:143-207),
 * detail::generate_strides (strides.h:31-74),
 * detail::generate_k_order_layout (layout.h:57-84),
 * detail::inverse_mode (layout.h:114-138).
 * Return TLIBG_OK or TLIBG_ERR_ARGUMENT with the reference's message.
 * ------------------------------------------------------------------------- */
int tlibg_output_shape(const size_t* na, size_t p, size_t q, size_t* nc);
int tlibg_output_layout(const size_t* pia, size_t p, size_t q, size_t* pic);
int tlibg_strides(const size_t* n, const size_t* pi, size_t p, size_t* w);
int tlibg_k_order_layout(size_t p, size_t k, size_t* pi);
size_t tlibg_inverse_mode(const size_t* pi, size_t p, size_t mode);

/* ---------------------------------------------------------------------------
 * Multi-vector chain: contract every mode of A except q, each with its vector.
 * Replaces: ttvpy.ttvs(q, A, bs, order) -- ttvpy/src/wrapped_ttv.cpp:85-199,
 * which runs p - 1 TTVs one after another.  bs (HOST array of p - 1 DEVICE
 * pointers) holds the vectors in mode order without mode q (bs[r] belongs to
 * mode r + 1 for r < q - 1, else mode r + 2); nbs (HOST) their lengths; c
 * (DEVICE) receives na[q-1] elements.  A is any dense layout (na, wa, pia as
 * in the single call).  The chain reads A once, whatever order the reference
 * would contract in: a first stage over the fastest modes (rows) or the
 * slowest (columns) reads A, one to three stages over the much smaller
 * intermediates follow; stages over several modes use Kronecker weights built
 * by one kernel, a stage over one mode reads its vector in place.  No host
 * synchronisation; intermediates in the stream's cached scratch; each launch
 * after the first is a programmatic dependent of the one before.  Same
 * messages as ttvpy for bad q, order or vector lengths.  dtype TLIBG_BF16A:
 * A bfloat16, vectors and c float.
 * ------------------------------------------------------------------------- */
int tlibg_ttvs(int dtype, size_t q, size_t p,
               const void* a, const size_t* na, const size_t* wa, const size_t* pia,
               const void* const* bs, const size_t* nbs, void* c, void* stream);

/* ---------------------------------------------------------------------------
 * Allocation-free fp32 TTV.  No counterpart in the reference.
 *
 * For callers that cannot have device memory allocated on their behalf:
 * frameworks whose caching allocator owns and accounts for every device byte,
 * memory-budgeted or multi-tenant processes, and latency-critical loops that
 * cannot absorb the implicit device synchronisation of cudaMalloc/cudaFree.
 * Same arguments and checks as tlibg_ttv_f32; the caller passes a, b and c.
 * The split-n_q partial sums live in one fixed array of
 * TLIBG_NOALLOC_SCRATCH_BYTES compiled into the library, which every device
 * that loads the library holds until the process exits.  The call never
 * allocates or frees memory (tlibg_device_alloc_count does not move).
 *  - When the planner's split needs more scratch than the array, the call
 *    plans again with fewer segments (the most that fit), then with none;
 *    problems that fit neither way are refused with TLIBG_ERR_UNSUPPORTED and
 *    a message giving both sizes.
 *  - The first call on each device (and again after a new context, e.g. after
 *    cudaDeviceReset) looks up the array's device address with that device
 *    current; make that first call before any stream capture.
 *  - All calls share the one array: calls that overlap on the GPU (different
 *    streams, or host threads) race on it and must be serialised by the caller.
 *    Nothing in it needs to start at zero; each call writes every slot it reads.
 * ------------------------------------------------------------------------- */
#define TLIBG_NOALLOC_SCRATCH_BYTES (8u << 20)
int tlibg_ttv_f32_noalloc(size_t q, size_t p,
                          const float* a, const size_t* na, const size_t* wa, const size_t* pia,
                          const float* b, const size_t* nb,
                          float* c, const size_t* nc, const size_t* wc, const size_t* pic,
                          void* stream);

/* ---------------------------------------------------------------------------
 * Batched TTVs: thousands of independent fp32 problems (uneven order, extents,
 * q and layout) in one persistent launch fed by a device-side work queue,
 * captured once in a CUDA graph and replayed.  No reference counterpart (the
 * reference runs one call at a time); each problem has the argument meaning
 * of ttv.h:54-60 and is validated like tlibg_ttv_f32.
 * ------------------------------------------------------------------------- */
typedef struct tlibg_problem {
    size_t q, p;
    const void* a; const size_t* na; const size_t* wa; const size_t* pia;
    const void* b; const size_t* nb;
    void* c; const size_t* nc; const size_t* wc; const size_t* pic;
} tlibg_problem;

#define TLIBG_SELECT_HEURISTIC 0  /* fixed rule of the engine                                 */
#define TLIBG_SELECT_LEARNED   1  /* cost-model MLP scores every variant on the device         */
#define TLIBG_SELECT_FIXED     2  /* every problem runs `variant`                              */
#define TLIBG_SELECT_GIVEN     3  /* per-problem `variants` (e.g. from exhaustive tuning)      */
/* Variants of a batched problem: v = 2 g + s for v < 8 (row form: 1 << g lanes
 * per row; column form: 1 << g warps along q; s = 1: q split into up to four
 * segments); v = 8: q-fastest rows of at most 64 elements staged through
 * shared memory by TMA bulk copies, one lane per row (row form only; a
 * column problem given it runs the fixed rule's variant). */
#define TLIBG_NVARIANT 9

typedef struct tlibg_batch_options {
    int select;            /* TLIBG_SELECT_*; LEARNED without a model falls back to GIVEN, then HEURISTIC */
    int variant;           /* TLIBG_SELECT_FIXED                                              */
    int accumulate;        /* TLIBG_ACC_*                                                     */
    int no_graph;          /* nonzero: launch the kernels directly instead of a CUDA graph    */
    const int* variants;   /* one per problem (TLIBG_SELECT_GIVEN), or NULL                   */
    int record_costs;      /* nonzero: the executor sums each problem's SM clock cycles       */
} tlibg_batch_options;

typedef struct tlibg_batch tlibg_batch;

/* Builds device descriptors (synchronises `stream` once) and, unless no_graph,
 * instantiates the CUDA graph of one launch.  Problem buffers must stay valid
 * for the lifetime of the batch. */
int tlibg_batch_create(int dtype, const tlibg_problem* probs, size_t count,
                       const tlibg_batch_options* opt, void* stream, tlibg_batch** out);
/* Runs every problem of the batch once (asynchronous on `stream`). */
int tlibg_batch_launch(tlibg_batch* batch, void* stream);
/* Changes the forced variant of a TLIBG_SELECT_FIXED batch created with
 * no_graph (the autotuner's loop over variants). */
int tlibg_batch_set_variant(tlibg_batch* batch, int variant);
/* SM cycles each problem's work units took in the last launch of a batch
 * created with record_costs: the units' clock cycles divided by the units
 * resident per SM (CTAs, or warps for staged rows), so that costs of either
 * executor add up to the launch time (the autotuner's per-problem cost inside
 * a mixed batch; synchronises). */
int tlibg_batch_costs(tlibg_batch* batch, uint64_t* cycles, void* stream);
/* The variant each problem ran with in the last launch (synchronises). */
int tlibg_batch_variants(tlibg_batch* batch, int* out, void* stream);
int tlibg_batch_destroy(tlibg_batch* batch);
/* fp32 batch in one call with the learned selection (the installed cost
 * model, else the fixed rule); synchronous.  Same as tlibg_ttv_batch with
 * TLIBG_F32 and TLIBG_SELECT_LEARNED. */
int tlibg_ttv_batch_f32(const tlibg_problem* probs, int n, void* stream);
/* create + launch + destroy (synchronous). */
int tlibg_ttv_batch(int dtype, const tlibg_problem* probs, size_t count,
                    const tlibg_batch_options* opt, void* stream);
/* The plain alternative: one tlibg_ttv_ex launch per problem, in order. */
int tlibg_ttv_percall(int dtype, const tlibg_problem* probs, size_t count, void* stream);
/* Cost-model features of each problem (TLIBG_MLP_FEATURES floats per problem:
 * p/8, position of q in the layout/(p-1), log2 P/24, log2 n_q/24, log2 S/24,
 * dtype (0 = fp32), log2 batch size/16, widest legal load/4),
 * its kernel family and the fixed rule's variant (kind / heuristic may be NULL). */
int tlibg_batch_features(const tlibg_problem* probs, size_t count, float* feat, int* kind,
                         int* heuristic);
/* Reads and clears the batched executor's device error word. */
unsigned int tlibg_batch_device_error(void);

/* ---------------------------------------------------------------------------
 * Learned cost model: an MLP (TLIBG_MLP_IN inputs = features + one-hot
 * variant, three hidden layers of 64 ReLU units, one output = predicted
 * log2 cost per problem) trained by the engine's own CUDA kernels.  All
 * buffers are device pointers unless stated.
 * ------------------------------------------------------------------------- */
#define TLIBG_MLP_FEATURES 8
#define TLIBG_MLP_IN 17
#define TLIBG_MLP_HIDDEN 64
#define TLIBG_MLP_PARAMS 9537
/* loss = (1/n) sum 0.5 (f(x)-y)^2 and its gradient (grad[TLIBG_MLP_PARAMS], loss[1]) */
int tlibg_mlp_loss_grad(const float* params, const float* x, const float* y, size_t n, float* grad,
                        float* loss, void* stream);
/* one Adam step (step counts from 1) */
int tlibg_mlp_adam(float* params, const float* grad, float* m, float* v, uint64_t step, float lr,
                   float beta1, float beta2, float eps, void* stream);
int tlibg_mlp_predict(const float* params, const float* x, size_t n, float* y, void* stream);
/* minibatch Adam over `epochs` shuffled passes; epoch_loss (HOST, epochs floats) may be NULL */
int tlibg_mlp_train(float* params, float* m, float* v, const float* x, const float* y, size_t n,
                    int epochs, int batch, float lr, uint64_t seed, float* epoch_loss, void* stream);
/* Installs (HOST array of TLIBG_MLP_PARAMS floats) or clears (NULL) the model
 * TLIBG_SELECT_LEARNED uses for batches created afterwards.  A problem leaves
 * the fixed rule's variant only when the model predicts the new one costs
 * less than (1 - margin) of it. */
int tlibg_set_cost_model(const float* params, size_t count, float margin);

/* ---- diagnostics ---- */
/* Copies the calling thread's last error text into buf (NUL-terminated,
 * truncated to len); returns the full text length. */
size_t tlibg_last_error(char* buf, size_t len);
/* Reads and clears the device error word set by bounded waits that expired
 * (synchronises the device).  0 = no device-side error. */
int tlibg_device_error(void);
/* Number of kernels this library launched since load (all entry points). */
uint64_t tlibg_launch_count(void);
/* Number of device allocations (cudaMalloc) this library made since load:
 * split scratch, host-path staging buffers, batch descriptors, training
 * buffers.  tlibg_ttv_f32_noalloc never adds to it. */
uint64_t tlibg_device_alloc_count(void);
/* Library version string. */
const char* tlibg_version(void);

#ifdef __cplusplus
}
#endif
#endif /* TLIBG_H */
