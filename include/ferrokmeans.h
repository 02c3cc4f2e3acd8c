/*
 * ferrokmeans.h -- C ABI of the GB300 (sm_103a) KMeans Lloyd library.
 *
 * This is the drop-in boundary for ferrolearn-cluster's KMeans hot path
 * (ferrolearn-cluster/src/kmeans.rs). Every entry point below names the
 * reference item it replaces. Plain pointers and sizes only; arrays are
 * row-major and C-contiguous. Any input or output pointer may be host memory
 * or device memory of the context's GPU: the library checks each pointer and
 * copies only what lives on the host. Calls are synchronous (they return when
 * the results are in the caller's buffers), like the Rust methods.
 *
 * Status codes map one-to-one onto ferrolearn_core::error::FerroError
 * (ferrolearn-core/src/error.rs:30-91) plus CUDA-side failures; the message of
 * the last failure on the calling thread is returned by fk_last_error_message.
 */
#ifndef FERROKMEANS_H
#define FERROKMEANS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum fk_status {
    FK_OK = 0,
    FK_ERR_INVALID_PARAMETER = 1,     /* FerroError::InvalidParameter     */
    FK_ERR_INSUFFICIENT_SAMPLES = 2,  /* FerroError::InsufficientSamples  */
    FK_ERR_SHAPE_MISMATCH = 3,        /* FerroError::ShapeMismatch        */
    FK_ERR_NUMERICAL_INSTABILITY = 4, /* FerroError::NumericalInstability */
    FK_ERR_CUDA = 10,                 /* a CUDA runtime call failed        */
    FK_ERR_OOM = 11,                  /* device allocation failed          */
    FK_ERR_TIMEOUT = 12,              /* a bounded device wait gave up     */
    FK_ERR_UNSUPPORTED = 13,          /* shape/precision not supported     */
    FK_ERR_NULL_POINTER = 14          /* a required pointer was NULL       */
} fk_status;

/* Arithmetic of the distance contraction. The result semantics are always
 * those of the reference's KMeans<F> (F = f64 for the _f64/_f32x64 entry
 * points, F = f32 for _f32):
 *  FK_PRECISION_PLAIN       direct-form sum (x_j - c_j)^2 in F on CUDA cores,
 *                           bit-identical to kmeans.rs:159-163.
 *  FK_PRECISION_MIXED_BF16  BF16 tensor-core contraction (tcgen05, TMEM) with
 *                           a derived per-row error bound; rows whose top-2
 *                           margin is inside the bound are re-scored exactly
 *                           in FP64 direct form.
 *  FK_PRECISION_MIXED_FP8   FP8 E4M3 tensor-core contraction (per-row
 *                           power-of-two scales) with the same bound and
 *                           exact re-check.
 *  Both mixed forms run on the _f32x64 entry points only (F = f64, X stored
 *  as f32); the others return FK_ERR_UNSUPPORTED for them.              */
typedef enum fk_precision {
    FK_PRECISION_PLAIN = 0,
    FK_PRECISION_MIXED_BF16 = 1,
    FK_PRECISION_MIXED_FP8 = 2
} fk_precision;

/* Hyper-parameters of KMeans<F> (kmeans.rs:55-68), plus the explicit-init
 * hooks the reference lacks. */
typedef struct fk_kmeans_params {
    int64_t n_clusters;        /* KMeans::n_clusters                      */
    int64_t max_iter;          /* KMeans::max_iter      (default 300)     */
    double tol;                /* KMeans::tol           (default 1e-4)    */
    int64_t n_init;            /* KMeans::n_init        (default 10)      */
    uint64_t random_state;     /* KMeans::random_state when has_random_state */
    int32_t has_random_state;  /* 0 = None (seed 0, kmeans.rs:451)        */
    int32_t precision;         /* fk_precision                            */
    /* Optional uniform [0,1) stream consumed by k-means++ in place of the
     * per-run generator (one flat stream across runs). NULL = the library's
     * splitmix64 stream seeded with random_state + run (see fk_draws_f64). */
    const double *draws;
    int64_t n_draws;
    int32_t collect_timing;    /* 1 = fill the per-phase device times     */
    int32_t reserved;
} fk_kmeans_params;

/* Diagnostics of one fit / step. All counters are summed over iterations. */
typedef struct fk_fit_report {
    int64_t best_run;          /* index of the run that was kept           */
    int64_t iterations_total;  /* Lloyd iterations over all runs           */
    int64_t rows_assigned;     /* rows x iterations                        */
    int64_t rows_rechecked;    /* mixed: rows whose margin fell inside the
                                  bound and were re-scored (FP32 + FP64)   */
    int64_t rows_full_rescan;  /* mixed: of those, rows whose third score
                                  was also inside the bound                */
    int64_t rows_fp64;         /* mixed: rows that needed FP64 scores      */
    int64_t rows_second_pass;  /* mixed: rows scored again by a second
                                  tensor pass (= rows_full_rescan): BF16
                                  candidate masks after a BF16 main pass,
                                  a BF16 count pass (and masks) after an
                                  FP8 one                                  */
    int64_t rows_few;          /* mixed: of those, rows resolved among at
                                  most 32 candidates                       */
    int64_t rows_exhaustive;   /* mixed: rows re-scored against every
                                  centre after the second pass             */
    int64_t near_tie_rows;     /* mixed: re-scored rows whose FP64 margin
                                  is below 1e-12 relative                  */
    double ms_init;            /* device time, k-means++                   */
    double ms_assign;          /* device time, assignment (+ re-check)     */
    double ms_contract;        /* mixed: device time of the tensor-core
                                  contraction kernel alone                 */
    double ms_update;          /* device time, sort + centroid update      */
    double ms_total;           /* device time of the whole call            */
    int32_t precision_used;
    int32_t reserved;
    int64_t rows_moved;        /* mixed, incremental centroid updates: rows
                                  whose label changed, summed over them    */
    int64_t updates_incremental; /* mixed: iterations whose centroid update
                                  was incremental (the rest were full
                                  passes over X)                           */
    int64_t count_iterations;  /* BF16 fits: iterations whose main pass was
                                  the count pass (thresholds carried from
                                  the previous iteration; the rest ranked
                                  a top-2)                                 */
    double ms_count_pass;      /* device time of those count passes (part
                                  of ms_contract)                          */
} fk_fit_report;

typedef struct fk_ctx fk_ctx;

/* Context: binds a GPU and a CUDA stream (cudaStream_t passed as void*;
 * NULL = the context creates its own non-blocking stream) and caches device
 * buffers across calls. One context per host thread. */
fk_status fk_ctx_create(fk_ctx **out, int32_t device, void *cuda_stream);
fk_status fk_ctx_destroy(fk_ctx *ctx);
/* Message of the last failure on this thread ("" if none). */
const char *fk_last_error_message(void);
const char *fk_version(void);
/* Diagnostics: number of kernel launches this library has issued so far in
 * the process (all contexts). No reference counterpart. */
uint64_t fk_debug_launch_count(void);

/* KMeans::new(n_clusters) defaults (kmeans.rs:76-84). */
void fk_kmeans_params_default(fk_kmeans_params *p, int64_t n_clusters);

/* The library's uniform stream (splitmix64, (u64 >> 11) * 2^-53). Host-only,
 * no GPU needed. k-means++ maps random_range(0..n) to min(floor(u*n), n-1). */
fk_status fk_draws_f64(uint64_t seed, int64_t count, double *out);

/* Fit::fit for KMeans<f64> (kmeans.rs:417-512). x: n*d; init_centers:
 * n_init*k*d explicit initial centres per run, or NULL for k-means++ on the
 * GPU. Outputs: centers_out k*d, labels_out n (usize), inertia_out, n_iter_out.
 * labels/inertia are those of the last assignment of the kept run, against
 * its pre-update centres, exactly as kmeans.rs:470-494. report may be NULL. */
fk_status fk_kmeans_fit_f64(fk_ctx *ctx, const double *x, int64_t n, int64_t d,
                            const fk_kmeans_params *params, const double *init_centers,
                            double *centers_out, uint64_t *labels_out, double *inertia_out,
                            int64_t *n_iter_out, fk_fit_report *report);

/* Fit::fit for KMeans<f32>: every sum, centre and distance in f32. */
fk_status fk_kmeans_fit_f32(fk_ctx *ctx, const float *x, int64_t n, int64_t d,
                            const fk_kmeans_params *params, const float *init_centers,
                            float *centers_out, uint64_t *labels_out, float *inertia_out,
                            int64_t *n_iter_out, fk_fit_report *report);

/* Fit::fit for KMeans<f64> on X stored as f32 (each x widened exactly to f64):
 * identical results to fk_kmeans_fit_f64 on the widened matrix, with half the
 * bytes resident. This is the entry point of the mixed precisions. */
fk_status fk_kmeans_fit_f32x64(fk_ctx *ctx, const float *x, int64_t n, int64_t d,
                               const fk_kmeans_params *params, const double *init_centers,
                               double *centers_out, uint64_t *labels_out, double *inertia_out,
                               int64_t *n_iter_out, fk_fit_report *report);

/* One Lloyd iteration, the loop body of kmeans.rs:468-488: assignment against
 * centers_in (labels_out, inertia_out), then recompute_centroids_into
 * (centers_out; empty clusters keep their centre) and the max centre shift
 * sqrt(max_c ||new-old||^2) (max_shift_out). report may be NULL. */
fk_status fk_lloyd_step_f64(fk_ctx *ctx, const double *x, int64_t n, int64_t d,
                            const double *centers_in, int64_t k, int32_t precision,
                            uint64_t *labels_out, double *centers_out, double *inertia_out,
                            double *max_shift_out, fk_fit_report *report);
fk_status fk_lloyd_step_f32(fk_ctx *ctx, const float *x, int64_t n, int64_t d,
                            const float *centers_in, int64_t k, int32_t precision,
                            uint64_t *labels_out, float *centers_out, float *inertia_out,
                            float *max_shift_out, fk_fit_report *report);
fk_status fk_lloyd_step_f32x64(fk_ctx *ctx, const float *x, int64_t n, int64_t d,
                               const double *centers_in, int64_t k, int32_t precision,
                               uint64_t *labels_out, double *centers_out, double *inertia_out,
                               double *max_shift_out, fk_fit_report *report);

/* Predict::predict (kmeans.rs:538-552): nearest centre per row. d must equal
 * d_fit, else FK_ERR_SHAPE_MISMATCH. */
fk_status fk_kmeans_predict_f64(fk_ctx *ctx, const double *centers, int64_t k, int64_t d_fit,
                                const double *x, int64_t n, int64_t d, int32_t precision,
                                uint64_t *labels_out);
fk_status fk_kmeans_predict_f32(fk_ctx *ctx, const float *centers, int64_t k, int64_t d_fit,
                                const float *x, int64_t n, int64_t d, int32_t precision,
                                uint64_t *labels_out);
fk_status fk_kmeans_predict_f32x64(fk_ctx *ctx, const double *centers, int64_t k, int64_t d_fit,
                                   const float *x, int64_t n, int64_t d, int32_t precision,
                                   uint64_t *labels_out);

/* Transform::transform (kmeans.rs:568-617): out[i*k+c] = sqrt(sum_j (x_ij-c_cj)^2). */
fk_status fk_kmeans_transform_f64(fk_ctx *ctx, const double *centers, int64_t k, int64_t d_fit,
                                  const double *x, int64_t n, int64_t d, double *out);
fk_status fk_kmeans_transform_f32(fk_ctx *ctx, const float *centers, int64_t k, int64_t d_fit,
                                  const float *x, int64_t n, int64_t d, float *out);

/* kmeans_plus_plus (kmeans.rs:169-253) on the GPU: greedy k-means++ with
 * 2+floor(ln k) trials per centre. draws: uniform stream (NULL = splitmix64
 * seeded with seed). draws_used_out (nullable) receives the count consumed. */
fk_status fk_kmeans_plus_plus_f64(fk_ctx *ctx, const double *x, int64_t n, int64_t d, int64_t k,
                                  const double *draws, int64_t n_draws, uint64_t seed,
                                  double *centers_out, int64_t *draws_used_out);
fk_status fk_kmeans_plus_plus_f32(fk_ctx *ctx, const float *x, int64_t n, int64_t d, int64_t k,
                                  const double *draws, int64_t n_draws, uint64_t seed,
                                  float *centers_out, int64_t *draws_used_out);

/* Allocation-free scoring (no counterpart in the reference): nearest-centre
 * labels (uint64) and the inertia (sum of the minimum squared distances,
 * f64) of n rows of x against k centres, with the plain FP64 arithmetic of
 * kmeans.rs (direct form, lowest index on ties). For callers that cannot
 * allocate device memory at call time (serving loops where an allocation
 * would synchronise the device, fixed memory budgets, hosts whose allocator
 * belongs to another framework): x, centers, labels_out and inertia_out must
 * all be device memory of the current device, and the scratch is one
 * fixed-size device array compiled into the library (about 6.3 MB per GPU,
 * held until the process exits). Limits: n <= 524288 rows, else
 * FK_ERR_INVALID_PARAMETER with a message naming the limit. The work is
 * queued on cuda_stream (NULL = the legacy default stream) and the outputs
 * are valid once that stream reaches this point; the call itself does not
 * wait. The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress), so make that first call before any stream capture.
 * That address belongs to the device's primary context (the CUDA runtime's):
 * call with that context current, and not again after cudaDeviceReset.
 * A buffer on another GPU than the current one is refused with
 * FK_ERR_INVALID_PARAMETER naming the argument.
 * All calls share the one array: calls that overlap on the GPU (different
 * streams, or threads without ordering) race and must be serialised by the
 * caller. */
fk_status fk_kmeans_score_f64_noalloc(const double *x, int64_t n, int64_t d, const double *centers,
                                      int64_t k, uint64_t *labels_out, double *inertia_out,
                                      void *cuda_stream);

/* ------------------------------------------------------- batched fits --
 * Many independent KMeans<f32> fits in one call (problems of uneven n, d and
 * k, each with its own n_init runs): Fit::fit (kmeans.rs:417-512) per
 * problem, all runs of all problems at once. Run r of a problem starts from
 * init[r] when init is given, else from k-means++ (kmeans.rs:169-253) on the
 * splitmix64 stream seeded with random_state + r (fk_draws_f64). The best run
 * is the strictly lowest inertia, first run on ties (kmeans.rs:506-511).
 * Distances, the argmin and k-means++ are the reference's f32 arithmetic;
 * the centroid sums follow `reduction`. x and the outputs may be host or
 * device memory. Limits: k <= 1024, d <= 256, k*d <= 32768 (else
 * FK_ERR_UNSUPPORTED); validation errors name the problem index. */
typedef enum fk_reduction {
    FK_REDUCE_REFERENCE = 0, /* row-order f32 sums (kmeans.rs:358-401 for F = f32) */
    FK_REDUCE_F64 = 1        /* each cluster sum formed exactly and rounded once
                                to f64, the mean in f64 rounded once to f32;
                                inertia summed in f64 */
} fk_reduction;

typedef struct fk_batch_problem {
    const float *x;          /* n x d, row-major */
    int64_t n, d;
    int64_t n_clusters;
    int64_t max_iter;
    double tol;
    int64_t n_init;
    uint64_t random_state;
    const float *init;       /* nullable: n_init x k x d initial centres */
    float *centers_out;      /* k x d (best run) */
    uint64_t *labels_out;    /* n (best run) */
    float *inertia_out;
    int64_t *n_iter_out;
    int64_t *best_run_out;   /* nullable */
} fk_batch_problem;

typedef struct fk_batch_report {
    int64_t fits;                /* sum of n_init */
    int64_t iterations_total;    /* Lloyd iterations over all fits */
    int64_t graph_launches;      /* replays of the captured iteration graph */
    int64_t tuned_buckets;       /* (d, k) buckets the autotuner timed in this call */
    int32_t bucket_variant[20];  /* tile shape per bucket d{8,16,32,64,other} x
                                    k{<=16,<=32,<=64,>64}: 0 (1 row, 1 centre per
                                    pass), 1 (2,1), 2 (1,2), 3 (2,2), 4 (4,1);
                                    -1 = bucket absent */
    double ms_upload, ms_init, ms_tune, ms_lloyd, ms_download, ms_total;
    double *fit_inertia;         /* nullable, caller memory: per fit, problem-major */
    int64_t *fit_n_iter;         /* nullable, caller memory: per fit */
} fk_batch_report;

fk_status fk_kmeans_fit_batched_f32(fk_ctx *ctx, fk_batch_problem *problems, int64_t n_problems,
                                    int32_t reduction, fk_batch_report *report);

/* ------------------------------------------------------ MiniBatchKMeans --
 * ferrolearn-cluster/src/mini_batch_kmeans.rs. Builder defaults of
 * MiniBatchKMeans::new (:108-118): batch_size 1024, max_iter 100, tol 0,
 * n_init 3, random_state None, init k-means++. */
typedef enum fk_minibatch_init {
    FK_MB_INIT_KMEANS_PLUS_PLUS = 0, /* MiniBatchKMeansInit::KMeansPlusPlus */
    FK_MB_INIT_RANDOM = 1            /* MiniBatchKMeansInit::Random         */
} fk_minibatch_init;

typedef struct fk_minibatch_params {
    int64_t n_clusters;       /* MiniBatchKMeans::n_clusters             */
    int64_t batch_size;       /* MiniBatchKMeans::batch_size (1024)      */
    int64_t max_iter;         /* MiniBatchKMeans::max_iter   (100)       */
    double tol;               /* MiniBatchKMeans::tol        (0.0)       */
    int64_t n_init;           /* MiniBatchKMeans::n_init     (3)         */
    uint64_t random_state;    /* MiniBatchKMeans::random_state, if set   */
    int32_t has_random_state; /* 0 = None (base seed 0)                  */
    int32_t init;             /* fk_minibatch_init                       */
} fk_minibatch_params;

void fk_minibatch_params_default(fk_minibatch_params *p, int64_t n_clusters);

/* MiniBatchKMeans::fit (:492-591): per run, the initial centres (k-means++
 * or random picks; init_centers, n_init*k*d or NULL, replaces both), then
 * max_iter mini-batches: sample_batch_indices (:451-472), nearest centre of
 * each batch row (direct form, strict < from F::MAX), and
 * update_centers_mini_batch (:410-447) in batch order, stopping when the
 * max centre shift < tol; the kept run has the strictly lowest inertia of
 * assign_clusters_mb (:343-376) over all rows. Random numbers: run r draws
 * the library's uniform stream (fk_draws_f64) seeded with
 * random_state + r * 1000003 (the run seeds of :532), first for the initial
 * centres (as fk_kmeans_plus_plus_*, or k partial Fisher-Yates picks), then
 * for the batches (fk_minibatch_batch_indices). Predict and Transform of the
 * fitted model are those of KMeans (fk_kmeans_predict_* /
 * fk_kmeans_transform_*). best_run_out and report may be NULL. */
fk_status fk_minibatch_fit_f64(fk_ctx *ctx, const double *x, int64_t n, int64_t d,
                               const fk_minibatch_params *params, const double *init_centers,
                               double *centers_out, uint64_t *labels_out, double *inertia_out,
                               int64_t *n_iter_out, int64_t *best_run_out, fk_fit_report *report);
fk_status fk_minibatch_fit_f32(fk_ctx *ctx, const float *x, int64_t n, int64_t d,
                               const fk_minibatch_params *params, const float *init_centers,
                               float *centers_out, uint64_t *labels_out, float *inertia_out,
                               int64_t *n_iter_out, int64_t *best_run_out, fk_fit_report *report);

/* ------------------------------------------------------ BisectingKMeans --
 * ferrolearn-cluster/src/bisecting_kmeans.rs. Builder defaults of
 * BisectingKMeans::new (:93-102): max_iter 300, n_init 10, random_state
 * None, LargestCluster. */
typedef enum fk_bisecting_strategy {
    FK_BISECT_LARGEST_CLUSTER = 0, /* BisectingStrategy::LargestCluster */
    FK_BISECT_LARGEST_SSE = 1      /* BisectingStrategy::LargestSSE     */
} fk_bisecting_strategy;

typedef struct fk_bisecting_params {
    int64_t n_clusters;       /* BisectingKMeans::n_clusters (target)      */
    int64_t max_iter;         /* iterations per 2-means        (300)       */
    int64_t n_init;           /* 2-means restarts per split    (10)        */
    uint64_t random_state;    /* BisectingKMeans::random_state, if set     */
    int32_t has_random_state; /* 0 = None (base seed 0)                    */
    int32_t strategy;         /* fk_bisecting_strategy                     */
} fk_bisecting_params;

void fk_bisecting_params_default(fk_bisecting_params *p, int64_t n_clusters);

/* BisectingKMeans::fit (:326-505): from one cluster of every row, split
 * the cluster with the most rows (or the largest SSE; the last of equal
 * maxima, as Rust's max_by_key / max_by) by the best of n_init 2-means runs
 * (run_2means, :225-312: two distinct rows of the cluster, label 0 when
 * d0 <= d1, row-order sums in F, until no label changes), until n_clusters
 * clusters or none with two rows is left. Run r of split s draws the
 * library's uniform stream seeded with random_state + s * 1000 + r (the
 * seeds of :410-412). Outputs: centers_out (n_clusters * d, the first
 * *n_clusters_out rows filled), labels_out (n, the final cluster of each
 * row, isize in the reference), inertia_out (the clusters' SSE summed in
 * list order). Predict and Transform of the fitted model are those of KMeans
 * (fk_kmeans_predict_* / fk_kmeans_transform_*). d <= 1024, n_init <= 1024. Where the
 * reference would not terminate (the selected cluster's rows are identical,
 * so every split leaves one side empty) the call returns
 * FK_ERR_NUMERICAL_INSTABILITY. */
fk_status fk_bisecting_fit_f64(fk_ctx *ctx, const double *x, int64_t n, int64_t d,
                               const fk_bisecting_params *params, double *centers_out, int64_t *labels_out,
                               double *inertia_out, int64_t *n_clusters_out);
fk_status fk_bisecting_fit_f32(fk_ctx *ctx, const float *x, int64_t n, int64_t d,
                               const fk_bisecting_params *params, float *centers_out, int64_t *labels_out,
                               float *inertia_out, int64_t *n_clusters_out);

/* The batch rows MiniBatchKMeans draws (sample_batch_indices, :451-472)
 * for `iters` iterations from position pos of the uniform stream of seed:
 * out holds iters * min(batch_size, n) row indices. Host-only. */
fk_status fk_minibatch_batch_indices(uint64_t seed, int64_t pos, int64_t n, int64_t batch_size, int64_t iters,
                                     int64_t *out);

/* Diagnostics (no reference counterpart): CUDA-core throughput of this GPU,
 * out[0] FP32 FMA flop/s, [1] FP64 FMA flop/s, [2] FP64 add op/s, [3] FP32
 * add op/s, [4] FP64 add latency in cycles, [5] FP32 add latency. */
fk_status fk_debug_measure_peaks(fk_ctx *ctx, double *out);

/* Diagnostics (no reference counterpart): dense tensor-core throughput of
 * this GPU measured with the contraction's own MMA shape (tcgen05.mma
 * M=128 N=256 from 128-byte-swizzled shared memory into TMEM, one CTA per
 * SM issuing back to back): out[0] BF16 (kind::f16, K=16) flop/s, out[1]
 * E4M3 (kind::f8f6f4, K=32) flop/s. The roofline denominator of the FP8
 * form, for which no library measurement exists. */
fk_status fk_debug_measure_tc_peaks(fk_ctx *ctx, double *out);

/* Diagnostics for the tests (no reference counterpart): one BF16 tensor-core
 * assignment pass of x (n*d f32, device memory) against c (k*d f64, device
 * memory), precision FK_PRECISION_MIXED_BF16 or _FP8. Returns the raw FP32
 * accumulators of the first 128-row tile of the first centre slice (dump:
 * 128 x kp), the quantised operands (xq: first 128 rows x d_pad elements;
 * cq: k_pad x d_pad; aug: k_pad x 16 BF16; xaug (FP8): first 128 rows x 16
 * BF16), the per-slice top-2 records
 * (top: parts x n x 16 bytes) and the plan {d_pad, kp, parts, k_pad, grid,
 * error word}. Buffers are sized by the caller from the plan's upper bounds. */
fk_status fk_debug_tc_probe(fk_ctx *ctx, const float *x_dev, int64_t n, int64_t d, const double *c_dev,
                            int64_t k, int32_t precision, float *dump, void *xq, void *cq, uint16_t *aug,
                            uint16_t *xaug, void *top, int32_t *plan);

/* Diagnostics (no reference counterpart, no GPU needed): the launch plan of
 * one tensor-core pass for a shape -- precision FK_PRECISION_MIXED_BF16 or
 * _FP8, topk 2 (top-2 main pass), 3 (count pass) or 1 (BF16 mask pass), on
 * num_sms SMs. out[0..9] =
 * {d_pad, kp (resident centres per slice), parts (slices), k_pad, nblocks
 * (256-centre accumulator blocks per slice), xst (X ring depth), dynamic
 * shared memory bytes, grid, CTAs per slice, 128-row tiles}. */
fk_status fk_debug_tc_plan(int64_t n, int64_t d, int64_t k, int32_t precision, int32_t topk, int32_t num_sms,
                           int64_t *out);

#ifdef __cplusplus
}
#endif

#endif /* FERROKMEANS_H */
