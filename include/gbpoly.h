/*
 * gbpoly.h — C ABI of the GB300 (sm_103a) PolyBench dense-contraction library.
 *
 * This is the boundary that replaces the SYCL device queue of sycl-bench's
 * polybench/{gemm,2mm,3mm,syrk,syr2k}.cpp (the dense contractions), and of
 * their neighbours polybench/{covariance,correlation}.cpp (column
 * statistics + a symmetric contraction), runtime/matmulchain.cpp (chained
 * contractions) and polybench/{atax,bicg,mvt,gesummv}.cpp (matrix-vector
 * products).  Every entry point takes plain
 * pointers and sizes, returns a gbpoly_status, and never throws.  Device
 * pointers are opaque to the caller and owned by the caller.  A context is
 * bound to one device and one CUDA stream; calls on one context are not
 * thread-safe (the reference harness drives one queue from one thread,
 * include/command_line.h:129-140).
 *
 * All matrices are dense and row-major: element (r, c) of a matrix with
 * leading dimension ld lives at base[r * ld + c].  This is the layout of the
 * reference's sycl::buffer<float, 2>(range<2>(N, N)) (polybench/gemm.cpp:69-71).
 */
#ifndef GBPOLY_H
#define GBPOLY_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  GBPOLY_OK is 0; everything else is an error whose text is
 * returned by gbpoly_last_error().  The reference reports errors by throwing
 * sycl::exception (include/common.h:208-212); the C++ harness turns a non-zero
 * status back into an exception at the same place. */
typedef enum {
  GBPOLY_OK = 0,
  GBPOLY_ERR_INVALID = 1,     /* bad argument (null pointer, negative size, bad enum) */
  GBPOLY_ERR_CUDA = 2,        /* a CUDA runtime/driver call failed */
  GBPOLY_ERR_NOMEM = 3,       /* device or pinned host allocation failed */
  GBPOLY_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up (kernel returned early) */
  GBPOLY_ERR_UNSUPPORTED = 5, /* valid request this build or device cannot serve */
  GBPOLY_ERR_STATE = 6        /* call out of order (e.g. graph end without begin) */
} gbpoly_status;

/* Arithmetic form of a contraction. */
typedef enum {
  GBPOLY_PREC_FP32 = 0,   /* plain FP32 SIMT FFMA kernels: the drop-in form */
  GBPOLY_PREC_BF16X3 = 1, /* split-BF16: hi*hi + hi*lo + lo*hi on tcgen05, FP32 accumulation in TMEM */
  GBPOLY_PREC_TF32 = 2,   /* tcgen05 kind::tf32, FP32 accumulation */
  GBPOLY_PREC_FP8 = 3,    /* e4m3 with one scale per 128x128 operand tile */
  GBPOLY_PREC_TF32X3 = 4, /* split-TF32: hi*hi + hi*lo + lo*hi on kind::tf32 (hi+lo keep ~24 bits: FP32-level error) */
  GBPOLY_PREC_BF16X6 = 5, /* three-way split-BF16: the 6 products of order <= 2^-16 (FP32-level error) */
  GBPOLY_PREC_FP16X3 = 6  /* split-FP16 with one power-of-two scale per 64x64 operand block: hi*hi + hi*lo + lo*hi
                             (hi+lo keep 22 bits: FP32-level error at bf16x3's speed) */
} gbpoly_precision;

/* Operand transposition: OP_N uses the matrix as stored, OP_T its transpose. */
typedef enum { GBPOLY_OP_N = 0, GBPOLY_OP_T = 1 } gbpoly_op;

typedef struct gbpoly_ctx gbpoly_ctx;

/* ---------------------------------------------------------------- context -- */

/* Create a context on CUDA device `device` with its own non-blocking stream.
 * Replaces the queue construction of include/command_line.h:183-202. */
gbpoly_status gbpoly_init(int device, gbpoly_ctx** out_ctx);

/* Synchronise, release the context's workspace, stream and events. */
gbpoly_status gbpoly_destroy(gbpoly_ctx* ctx);

/* Text of the last error on this thread ("" if none).  Valid until the next call. */
const char* gbpoly_last_error(void);

/* Device name, as the reference reads it with
 * get_info<sycl::info::device::name>() (include/common.h:42-43). */
gbpoly_status gbpoly_device_name(gbpoly_ctx* ctx, char* buf, size_t buflen);

/* Number of SMs, current max SM clock (kHz) and compute capability. */
gbpoly_status gbpoly_device_props(gbpoly_ctx* ctx, int* sm_count, int* sm_clock_khz, int* cc_major, int* cc_minor);

/* Block until all work queued on the context's stream has finished, then
 * report any device-side error word (a bounded wait that timed out).
 * Replaces queue::wait_and_throw() (include/common.h:61, :75). */
gbpoly_status gbpoly_synchronize(gbpoly_ctx* ctx);

/* Use a caller-owned cudaStream_t (passed as void*) for all later work;
 * NULL restores the context's own stream. */
gbpoly_status gbpoly_set_stream(gbpoly_ctx* ctx, void* cuda_stream);

/* ----------------------------------------------------------------- memory -- */

/* Device buffers.  Together with gbpoly_memcpy_h2d they replace
 * PrefetchedBuffer::initialize + forceDataTransfer (include/memory_wrappers.h:21-28, :47-51). */
gbpoly_status gbpoly_malloc(gbpoly_ctx* ctx, void** dptr, size_t bytes);
gbpoly_status gbpoly_free(gbpoly_ctx* ctx, void* dptr);

/* Page-locked host buffers, for copies that overlap and run at full link speed. */
gbpoly_status gbpoly_host_alloc(gbpoly_ctx* ctx, void** hptr, size_t bytes);
gbpoly_status gbpoly_host_free(gbpoly_ctx* ctx, void* hptr);

/* Copies are queued on the context's stream (asynchronous with respect to the
 * host for pinned memory); gbpoly_synchronize() waits for them.  d2h replaces
 * buffer::get_host_access() (polybench/gemm.cpp:99). */
gbpoly_status gbpoly_memcpy_h2d(gbpoly_ctx* ctx, void* dst, const void* src, size_t bytes);
gbpoly_status gbpoly_memcpy_d2h(gbpoly_ctx* ctx, void* dst, const void* src, size_t bytes);
gbpoly_status gbpoly_memcpy_d2d(gbpoly_ctx* ctx, void* dst, const void* src, size_t bytes);
gbpoly_status gbpoly_memset(gbpoly_ctx* ctx, void* dst, int value, size_t bytes);

/* Make the context workspace (split panels of the tensor-core forms) at
 * least `bytes` large now, so that later calls of that size do not allocate.
 * Needed before capturing tensor-core calls into a graph.  Synchronises. */
gbpoly_status gbpoly_workspace_reserve(gbpoly_ctx* ctx, size_t bytes);
/* Workspace bytes a contraction of this shape and form needs (fp32: the
 * partial products of its K split, used when the output tiles are too few
 * to fill the device; 0 otherwise). */
gbpoly_status gbpoly_workspace_query(gbpoly_precision prec, int64_t M, int64_t N, int64_t K, int same_operand,
    size_t* bytes);

/* -------------------------------------------------------------- autotuner -- */

/* Each tensor-core form has a few compiled tile configurations: tile width,
 * K bytes per pipeline stage, pipeline depth and cluster size (tf32, bf16x3,
 * tf32x3, bf16x6: configurations 3, 4 and 5 run CTA pairs, cta_group::2 MMAs
 * on 256 x 256 tiles; 5 keeps the C tile in shared memory, loaded and stored
 * by TMA, for short K, and runs as 3 for symmetric products or C rows that
 * do not start and end on 16-byte boundaries).  The context keeps one per (form, ceil(log2) of
 * M, N, K); unless tuned or set, a shape whose 256 x 256 tiles give every SM
 * pair a tile uses configuration 5 up to K = 256 (tf32: 512, tf32x3: 128)
 * and 3 beyond, smaller ones a 128 x 128 configuration.  fp8: configuration
 * 1 (128 x 256 tiles) when its tiles give every SM one, else 0 (128 x 128,
 * also every symmetric product). */
gbpoly_status gbpoly_gemm_config_count(gbpoly_precision prec, int* count);
gbpoly_status gbpoly_gemm_config_set(gbpoly_ctx* ctx, gbpoly_precision prec, int64_t M, int64_t N, int64_t K,
    int config);
gbpoly_status gbpoly_gemm_config_get(gbpoly_ctx* ctx, gbpoly_precision prec, int64_t M, int64_t N, int64_t K,
    int* config);
/* Times every configuration of `prec` on an M x N x K problem (allocates its
 * own operands), `reps` launches each, keeps the fastest for that shape
 * bucket and returns it.  Synchronous. */
gbpoly_status gbpoly_autotune_gemm(gbpoly_ctx* ctx, gbpoly_precision prec, int64_t M, int64_t N, int64_t K, int reps,
    int* best_config, float* best_ms);
/* Persist / restore the tuned table as text lines keyed by device name and
 * driver version (entries of other devices in the file are kept). */
gbpoly_status gbpoly_autotune_save(gbpoly_ctx* ctx, const char* path);
gbpoly_status gbpoly_autotune_load(gbpoly_ctx* ctx, const char* path, int* loaded);
/* K-split tail (CTA-pair configurations, on by default): when the last round
 * of 256 x 256 tiles would leave at least half the resident SM pairs idle,
 * each tile of that round runs as two halves of its K range on two pairs;
 * the first half adds the second half's partial sums (in a fixed order, so
 * results are the same on every run) and writes C.  The workspace query
 * includes the partial sums. */
gbpoly_status gbpoly_tail_split_enable(gbpoly_ctx* ctx, int enable);

/* ----------------------------------------------------------------- graphs -- */

/* Capture the work later calls queue on the context's stream into a CUDA
 * graph, then replay it with one launch.  This is how the multi-kernel
 * benchmarks (2mm.cpp:94-123, 3mm.cpp:115-158, which the reference submits as
 * separate command groups) run as one launch.  Between begin and end no call
 * may allocate: reserve the workspace first (a tensor-core call that would
 * grow it returns GBPOLY_ERR_STATE). */
typedef struct gbpoly_graph gbpoly_graph;
gbpoly_status gbpoly_graph_begin(gbpoly_ctx* ctx);
gbpoly_status gbpoly_graph_end(gbpoly_ctx* ctx, gbpoly_graph** graph);
gbpoly_status gbpoly_graph_launch(gbpoly_ctx* ctx, gbpoly_graph* graph);
gbpoly_status gbpoly_graph_destroy(gbpoly_ctx* ctx, gbpoly_graph* graph);

/* --------------------------------------------------------- stream hold -- */
/* Hold the context's stream: work queued after gbpoly_stream_hold starts only
 * once gbpoly_stream_release is called, or once `timeout_us` microseconds
 * have passed (a small kernel waits, bounded, on a mapped host word).  The
 * harness brackets each command group with it so that the command's start
 * event is timestamped when the command's kernels are already queued: the
 * event pair then measures device execution, as the reference's
 * command_start / command_end profiling does (include/common.h:86-99),
 * instead of including the host's launch latency.  Not for use inside a
 * graph capture. */
gbpoly_status gbpoly_stream_hold(gbpoly_ctx* ctx, uint32_t timeout_us);
gbpoly_status gbpoly_stream_release(gbpoly_ctx* ctx);

/* ------------------------------------------------------------ diagnostics -- */
/* Failure paths, exercised without any fault on the GPU.
 *
 * gbpoly_wait_probe queues one small kernel whose bounded wait, made by the
 * same routine as every pipeline wait of the contraction kernels, is on an
 * mbarrier that nothing completes: after limit_us it records its code in the
 * context's error word and returns.  The next gbpoly_synchronize then returns
 * GBPOLY_ERR_TIMEOUT (and clears the word), exactly as it does when a
 * kernel's pipeline stalls past its 2 s limit, and the context stays usable.
 * This is the device side of the error the reference throws from
 * queue::wait_and_throw() and catches per benchmark (include/common.h:61,
 * :208-212).
 *
 * Host-side fault injection (environment variable GBPOLY_FAULT_INJECT, read
 * by gbpoly_init): "alloc:N" makes the N-th later gbpoly_malloc of the
 * process return GBPOLY_ERR_NOMEM without allocating; "corrupt:N" changes the
 * first 4 bytes of the destination of the N-th later gbpoly_memcpy_d2h once
 * the copy has landed (a float v becomes 2v + 1), so a caller's verification
 * sees a wrong element.  Unset, it injects nothing. */
gbpoly_status gbpoly_wait_probe(gbpoly_ctx* ctx, uint32_t limit_us);

/* ----------------------------------------------------------------- events -- */

/* Event handles for kernel-time profiling.  They replace the
 * sycl::event profiling queries of include/common.h:88-96
 * (command_start / command_end). */
typedef struct gbpoly_event gbpoly_event;
gbpoly_status gbpoly_event_create(gbpoly_ctx* ctx, gbpoly_event** ev);
gbpoly_status gbpoly_event_destroy(gbpoly_ctx* ctx, gbpoly_event* ev);
gbpoly_status gbpoly_event_record(gbpoly_ctx* ctx, gbpoly_event* ev);
/* Milliseconds between two recorded events (waits for `end`). */
gbpoly_status gbpoly_event_elapsed_ms(gbpoly_ctx* ctx, gbpoly_event* start, gbpoly_event* end, float* ms);

/* Per-kernel timing.  While enabled, every kernel the library launches on the
 * context's stream is bracketed by CUDA events, so a caller can separate the
 * kernels one contraction call launches (the per-kernel view of the
 * reference's kernel-time, include/common.h:86-99). */
gbpoly_status gbpoly_profile_enable(gbpoly_ctx* ctx, int enable);
/* Waits for the stream, then aggregates the launches recorded since the last
 * read by kernel: names (64 bytes each), launch counts, total milliseconds.
 * *n_entries receives the number of distinct kernels (entries beyond
 * max_entries are dropped).  Clears the record. */
gbpoly_status gbpoly_profile_read(gbpoly_ctx* ctx, int max_entries, char* names, int* counts, double* total_ms,
    int* n_entries);

/* ----------------------------------------------------------- contractions -- */

/* C <- alpha * op(A) * op(B) + beta * C, FP32 in and out.
 * op(A) is M x K, op(B) is K x N, C is M x N.
 * Replaces the kernels polybench/gemm.cpp:82-91 (alpha=32412, beta=2123),
 * polybench/2mm.cpp:99-106 (alpha=1, beta=1) and :114-122 (alpha=1, beta=0),
 * polybench/3mm.cpp:120-157 (alpha=1, beta=1 onto zeroed E/F/G).
 * With beta == 0, C is not read (NaN/Inf in C do not propagate).
 * The call is asynchronous on the context's stream. */
gbpoly_status gbpoly_gemm_f32(gbpoly_ctx* ctx, gbpoly_precision prec, gbpoly_op op_a, gbpoly_op op_b,
    int64_t M, int64_t N, int64_t K, float alpha, const float* A, int64_t lda, const float* B, int64_t ldb,
    float beta, float* C, int64_t ldc);

/* The same contraction with A, B and C in HOST memory (pinned memory from
 * gbpoly_host_alloc reaches full link speed): the operands travel to the
 * device, C comes back, all inside the call, pipelined over row panels of
 * C so that the copies overlap the computation.  This is the whole-job form
 * of the reference's run: setup's upload (PrefetchedBuffer::initialize,
 * include/memory_wrappers.h:47-51), the kernel (polybench/gemm.cpp:82-91)
 * and verify's read-back (polybench/gemm.cpp:99).  Asynchronous on the
 * context's stream; the host buffers must stay valid until
 * gbpoly_synchronize(). */
gbpoly_status gbpoly_gemm_f32_host(gbpoly_ctx* ctx, gbpoly_precision prec, gbpoly_op op_a, gbpoly_op op_b,
    int64_t M, int64_t N, int64_t K, float alpha, const float* A, int64_t lda, const float* B, int64_t ldb,
    float beta, float* C, int64_t ldc);

/* C <- alpha * A * A^T + beta * C over the FULL N x N square (A is N x K).
 * Replaces polybench/syrk.cpp:74-83 (alpha=123, beta=14512). */
gbpoly_status gbpoly_syrk_f32(gbpoly_ctx* ctx, gbpoly_precision prec, int64_t N, int64_t K, float alpha,
    const float* A, int64_t lda, float beta, float* C, int64_t ldc);

/* C <- alpha * (A * B^T + B * A^T) + beta * C over the FULL N x N square
 * (A, B are N x K), both products accumulated in one accumulator.
 * Replaces polybench/syr2k.cpp:78-87 (alpha=1, beta=1). */
gbpoly_status gbpoly_syr2k_f32(gbpoly_ctx* ctx, gbpoly_precision prec, int64_t N, int64_t K, float alpha,
    const float* A, int64_t lda, const float* B, int64_t ldb, float beta, float* C, int64_t ldc);

/* ------------------------------------------------------ matrix-vector -- */
/* The BLAS-2 PolyBench benchmarks, HBM-bound: one pass over the matrix
 * serves every product of a call.  FP32; sums in a fixed order (partials
 * per 1024-column tile and per row group), deterministic but not the
 * reference's sequential order.  Asynchronous on the context's stream; the
 * partial sums use a per-context scratch that grows on the first call of a
 * shape (not during capture). */

/* y <- beta * y + alpha * op(A) x, A rows x cols (op N: x has cols entries,
 * y rows; op T: x has rows entries, y cols).  With beta == 0, y is not read.
 * Replaces Atax1 and Atax2 (polybench/atax.cpp:73-97: tmp += A x, then
 * y += A^T tmp) with alpha = beta = 1. */
gbpoly_status gbpoly_gemv_f32(gbpoly_ctx* ctx, gbpoly_op op, int64_t rows, int64_t cols, float alpha, const float* A,
    int64_t lda, const float* x, float beta, float* y);

/* tmp <- tmp + A x, then y <- y + A^T tmp (the updated tmp).  Replaces
 * Atax1 + Atax2 (polybench/atax.cpp:73-97).  Up to 8192 columns (16-byte
 * aligned rows and x) one kernel reads each row of A from HBM once: a CTA
 * completes a row group's dots, then reads the same rows again (from L2)
 * for the column sums; wider or unaligned matrices take two
 * gbpoly_gemv_f32 passes. */
gbpoly_status gbpoly_atax_f32(gbpoly_ctx* ctx, int64_t rows, int64_t cols, const float* A, int64_t lda, const float* x,
    float* tmp, float* y);

/* One product y <- beta * y + alpha * op(A) x of a pair. */
typedef struct {
  gbpoly_op op;
  float alpha, beta;
  const float* x;
  float* y;
} gbpoly_gemv_term;

/* One or two products of the same A in ONE pass over A (at most one with
 * op T).  Replaces Bicg1 + Bicg2 (polybench/bicg.cpp:77-100: s += A^T r,
 * q += A p) and Mvt1 + Mvt2 (polybench/mvt.cpp:75-98: x1 += A y1,
 * x2 += A y2; the reference's second product uses A, not A^T). */
gbpoly_status gbpoly_gemv_pair_f32(gbpoly_ctx* ctx, int64_t rows, int64_t cols, const float* A, int64_t lda,
    const gbpoly_gemv_term* terms, int count);

/* tmp <- tmp + A x;  y <- alpha * tmp + beta * (y + B x), in one pass over A
 * and B.  Replaces Gesummv (polybench/gesummv.cpp:84-98, alpha = beta = 1). */
gbpoly_status gbpoly_gesummv_f32(gbpoly_ctx* ctx, int64_t rows, int64_t cols, float alpha, const float* A,
    int64_t lda, const float* B, int64_t ldb, const float* x, float beta, float* tmp, float* y);

/* --------------------------------------------------- column statistics -- */
/* The passes of polybench/covariance.cpp and polybench/correlation.cpp that
 * prepare their data matrix (a rows x cols block X, leading dimension ldx)
 * for the X^T * X contraction, which is gbpoly_gemm_f32 with op_a = T,
 * op_b = N and A == B (recognised as symmetric: lower triangle of tiles,
 * mirrored).  FP32 throughout; sums use a fixed two-level order, so results
 * are deterministic but not the reference's sequential row order.
 * Asynchronous on the context's stream; the reductions use a per-context
 * scratch that grows on the first call of a shape (not during capture). */

/* mean[j] = (sum_i X[i][j]) / divisor, j < cols.
 * Replaces CovarianceMean (polybench/covariance.cpp:84-96, divisor float_n)
 * and CorrelationMean (polybench/correlation.cpp:111-124). */
gbpoly_status gbpoly_column_mean_f32(gbpoly_ctx* ctx, int64_t rows, int64_t cols, const float* X, int64_t ldx,
    float divisor, float* mean);

/* s = sqrt((sum_i (X[i][j] - mean[j])^2) / divisor); stddev[j] = s <= eps ? 1 : s.
 * Replaces CorrelationStd (polybench/correlation.cpp:126-142), which divides
 * by the double constant FLOAT_N: passing its float rounding moves the
 * quotient by at most one unit in the last place. */
gbpoly_status gbpoly_column_stddev_f32(gbpoly_ctx* ctx, int64_t rows, int64_t cols, const float* X, int64_t ldx,
    const float* mean, float divisor, float eps, float* stddev);

/* Y[i][j] = X[i][j] - mean[j]                                  (stddev == NULL)
 * Y[i][j] = ((X[i][j] - mean[j]) / scale_div) / stddev[j]     (otherwise)
 * Y may be X itself (same leading dimension) or another buffer, e.g. a
 * packed copy with a 16-byte-aligned leading dimension for the contraction.
 * Replaces CovarianceReduce (polybench/covariance.cpp:98-106) and
 * CorrelationReduce (polybench/correlation.cpp:144-156; scale_div is the
 * float rounding of its sqrt(FLOAT_N)). */
gbpoly_status gbpoly_center_columns_f32(gbpoly_ctx* ctx, int64_t rows, int64_t cols, const float* X, int64_t ldx,
    const float* mean, const float* stddev, float scale_div, float* Y, int64_t ldy);

/* C[j][j] = value, j < n.  Replaces the diagonal stores of CorrelationCorr
 * and Correlation5 (polybench/correlation.cpp:167-186). */
gbpoly_status gbpoly_set_diagonal_f32(gbpoly_ctx* ctx, int64_t n, float value, float* C, int64_t ldc);

/* C (cols x cols) = Y^T . Y with Y the centred (stddev == NULL) or centred
 * and scaled columns of X, as gbpoly_center_columns_f32 defines them: the
 * covariance / correlation contraction of CovarianceReduce + CovarianceCovar
 * (polybench/covariance.cpp:98-126) and CorrelationReduce + CorrelationCorr
 * (polybench/correlation.cpp:144-178) in one call, without a centred copy of
 * X for the split forms (tf32, bf16x3, tf32x3, bf16x6, fp16x3: the split pass centres
 * each element before splitting it, with the same arithmetic, so the result
 * is bitwise that of centring into a copy and contracting it).  fp32 and fp8
 * centre into a context scratch copy and contract it.  The lower triangle of
 * tiles is computed and mirrored, so C is the full symmetric square. */
gbpoly_status gbpoly_covariance_f32(gbpoly_ctx* ctx, gbpoly_precision prec, int64_t rows, int64_t cols, const float* X,
    int64_t ldx, const float* mean, const float* stddev, float scale_div, float* C, int64_t ldc);


/* -------------------------------------------------------------- grouped -- */

/* One contraction of a group: C = alpha * op(A) * op(B) + beta * C. */
typedef struct {
  gbpoly_op op_a, op_b;
  int64_t M, N, K;
  float alpha, beta;
  const float* A;
  int64_t lda;
  const float* B;
  int64_t ldb;
  float* C;
  int64_t ldc;
} gbpoly_gemm_desc;

/* Many independent contractions of uneven shapes.  The reference runs every
 * contraction as its own kernel (e.g. the stages of 3mm.cpp:115-158); a
 * grouped plan runs all of them with the tensor-core forms as one split
 * pass and one persistent launch over all tiles (fp32: one plain launch per
 * problem).  gbpoly_grouped_plan validates the descriptors and prepares
 * everything once (it allocates the term panels and tables and copies them
 * to the device, synchronously); gbpoly_grouped_run only enqueues launches on
 * the context's stream and can be captured into a graph; the operands and
 * outputs must stay at the addresses given to the plan.  count = 0 gives an
 * empty plan (no device memory) whose run launches nothing; fp8 has no
 * grouped form (GBPOLY_ERR_UNSUPPORTED). */
typedef struct gbpoly_grouped gbpoly_grouped;
gbpoly_status gbpoly_grouped_plan(gbpoly_ctx* ctx, gbpoly_precision prec, const gbpoly_gemm_desc* descs, int count,
    gbpoly_grouped** plan);
gbpoly_status gbpoly_grouped_run(gbpoly_ctx* ctx, gbpoly_grouped* plan);
/* Algorithmic FLOPs (sum of 2MNK), output tiles and device bytes of a plan. */
gbpoly_status gbpoly_grouped_info(gbpoly_grouped* plan, int64_t* flops, int* tiles, size_t* device_bytes);
/* The tile configuration a plan runs. */
gbpoly_status gbpoly_grouped_config_of(gbpoly_grouped* plan, int* config);

/* Tile configurations of grouped plans (the tile shape, cluster size and
 * pipeline depth of the persistent grouped kernel): 0 = 1-CTA 128 x 128
 * tiles, 3 stages of 128 bytes of K (bf16x6: 4 stages of 64 bytes); 1 = CTA
 * pairs on 256 x 256 tiles (cta_group::2); bf16x3 also 2 = 1-CTA 128 x 256
 * tiles, 2 stages.  The context keeps one per problem class: the form and
 * ceil(log2) of the problem count and of the median M, N and K.  Untuned, a
 * class uses 1 when its 256 x 256 tiles pad the work at most 5 % more than
 * 128 x 128 tiles and fill every SM pair at least once, else 0.
 * gbpoly_autotune_grouped plans and runs the group with every configuration
 * (`reps` timed runs each, on the caller's operands: C is overwritten), keeps
 * the fastest for the group's class and returns it; gbpoly_autotune_save /
 * _load persist these entries with the single-contraction ones.  There is no
 * such tuner in the reference, whose stages (e.g. 3mm.cpp:115-158) are fixed
 * separate kernels. */
gbpoly_status gbpoly_grouped_config_count(gbpoly_precision prec, int* count);
gbpoly_status gbpoly_grouped_config_set(gbpoly_ctx* ctx, gbpoly_precision prec, const gbpoly_gemm_desc* descs,
    int count, int config);
gbpoly_status gbpoly_grouped_config_get(gbpoly_ctx* ctx, gbpoly_precision prec, const gbpoly_gemm_desc* descs,
    int count, int* config);
gbpoly_status gbpoly_autotune_grouped(gbpoly_ctx* ctx, gbpoly_precision prec, const gbpoly_gemm_desc* descs,
    int count, int reps, int* best_config, float* best_ms);
/* Waits for the context's stream, then frees the plan. */
gbpoly_status gbpoly_grouped_destroy(gbpoly_ctx* ctx, gbpoly_grouped* plan);
/* Plan, run and destroy in one call (synchronous). */
gbpoly_status gbpoly_gemm_grouped_f32(gbpoly_ctx* ctx, gbpoly_precision prec, const gbpoly_gemm_desc* descs,
    int count);

/* Allocation-free split-BF16 contraction: the same contraction as
 * gbpoly_gemm_f32(ctx, GBPOLY_PREC_BF16X3, ...), within split-BF16 rounding
 * (it always runs the fixed 1-CTA 128 x 256 tile configuration 0 over whole
 * tiles: no autotuned choice, no K-split tail, no lower-triangle mirroring,
 * so the sums may round differently), for callers that may not
 * allocate device memory at call time (graph capture in global mode, an
 * application-owned memory pool, allocation-free real-time loops, device
 * memory quotas).  It has no counterpart in the reference.
 * The hi/lo panels live in a fixed 32 MiB device array inside the library
 * (held by every GPU that loads the library until exit) instead of the
 * context workspace, so the call performs no cudaMalloc/cudaFree:
 *   - shapes whose panels exceed it, about (M + N) * round_up(K, 64) * 4 bytes
 *     > 32 MiB, are rejected with GBPOLY_ERR_INVALID and a message;
 *   - the first call on each device looks the array's device address up
 *     (cudaGetSymbolAddress); make that first call before any stream capture.
 *     The address belongs to the device's context: after cudaDeviceReset
 *     (or anything else that replaces the context) the next call looks it up
 *     again, so make that call outside stream capture too;
 *   - all calls share the one array: calls whose work overlaps on the GPU
 *     (several streams or contexts on one device) race and must be ordered
 *     by the caller. */
gbpoly_status gbpoly_gemm_f32_bf16x3_noalloc(gbpoly_ctx* ctx, gbpoly_op op_a, gbpoly_op op_b, int64_t M, int64_t N,
    int64_t K, float alpha, const float* A, int64_t lda, const float* B, int64_t ldb, float beta, float* C,
    int64_t ldc);

/* ------------------------------------------------------------------- FP64 -- */

/* C <- alpha * op(A) * op(B) + beta * C in FP64.  The double variants of the
 * benchmarks (the suite's SYCL_BENCH_HAS_FP64_SUPPORT idiom,
 * single-kernel/nbody.cpp:303-309; polybench/gemm.cpp:14 fixes DATA_TYPE to
 * float, so the reference itself has no double contraction) and the FP64
 * oracle used for error norms at sizes the host loop cannot finish. */
gbpoly_status gbpoly_gemm_f64(gbpoly_ctx* ctx, gbpoly_op op_a, gbpoly_op op_b, int64_t M, int64_t N, int64_t K,
    double alpha, const double* A, int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc);
/* FP64 forms of gbpoly_syrk_f32 / gbpoly_syr2k_f32 (full square). */
gbpoly_status gbpoly_syrk_f64(gbpoly_ctx* ctx, int64_t N, int64_t K, double alpha, const double* A, int64_t lda,
    double beta, double* C, int64_t ldc);
gbpoly_status gbpoly_syr2k_f64(gbpoly_ctx* ctx, int64_t N, int64_t K, double alpha, const double* A, int64_t lda,
    const double* B, int64_t ldb, double beta, double* C, int64_t ldc);

/* dst[i] = (double)src[i] for i < count (device buffers). */
gbpoly_status gbpoly_convert_f32_f64(gbpoly_ctx* ctx, const float* src, double* dst, int64_t count);

/* Error of an FP32 result C against an FP64 reference R over a rows x cols
 * window (device buffers).  Synchronous: waits for queued work, then returns
 *   max_rel      = max|C-R| / max|R|
 *   frob_rel     = ||C-R||_F / ||R||_F
 *   max_elem_rel = max over R != 0 of |C-R| / |R|
 * (+Inf for all three if any C-R is not finite).  This extends the
 * reference's percentDiff verify (polybench/common/polybenchUtilFuncts.h:36-42),
 * which it does not replace.  Any output pointer may be NULL. */
gbpoly_status gbpoly_error_norms(gbpoly_ctx* ctx, const float* C, int64_t ldc, const double* R, int64_t ldr,
    int64_t rows, int64_t cols, double* max_rel, double* frob_rel, double* max_elem_rel);

#ifdef __cplusplus
}
#endif

#endif /* GBPOLY_H */
