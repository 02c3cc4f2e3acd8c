/*
 * kmeans_oracle.c -- CPU restatement of ferrolearn-cluster's KMeans Lloyd
 * path, used ONLY as test infrastructure: the parity tests, the smoke check
 * and the CPU-baseline leg of the benchmark call it as the reference result
 * to compare against (or, in the benchmark, to time). Nothing
 * in the product library links or calls this file.
 *
 * It restates ferrolearn-cluster/src/kmeans.rs statement by statement:
 *   squared_euclidean          kmeans.rs:159-163  (left fold from 0, no FMA)
 *   kmeans_plus_plus           kmeans.rs:169-253  (uniform draws injected)
 *   assign_clusters_into       kmeans.rs:279-291
 *   nearest_center             kmeans.rs:295-309  (strict < from F::MAX)
 *   assign_serial/_parallel    kmeans.rs:312-352
 *   recompute_centroids_into   kmeans.rs:358-401  (row-order sums in F)
 *   Fit::fit                   kmeans.rs:417-512  (n_init runs, best strict-<)
 *   Predict::predict           kmeans.rs:538-552
 *   Transform::transform       kmeans.rs:568-617
 * and, for MiniBatchKMeans, ferrolearn-cluster/src/mini_batch_kmeans.rs:
 *   kmeans_plus_plus_mb        :230-321  (same statements as kmeans.rs's)
 *   random_init_mb             :324-338
 *   assign_clusters_mb         :343-376
 *   assign_batch               :381-404
 *   update_centers_mini_batch  :410-447
 *   sample_batch_indices       :451-472
 *   MiniBatchKMeans::fit       :492-591
 * and, for BisectingKMeans, ferrolearn-cluster/src/bisecting_kmeans.rs:
 *   compute_cluster_stats      :192-222
 *   run_2means                 :225-312
 *   BisectingKMeans::fit       :326-505
 *
 * It must be compiled with -ffp-contract=off so that a*b+c is never fused:
 * Rust never contracts, and labels depend on the exact rounding of the
 * direct-form distance.
 *
 * Random numbers: the reference draws from rand 0.9 StdRng (ChaCha12), which
 * is not available here. The oracle instead consumes an explicit stream of
 * uniform doubles in [0,1): random_range(0..n) becomes min(floor(u*n), n-1)
 * and random::<f64>() becomes u. The GPU library consumes the same stream, so
 * both sides start from identical inputs. The default stream is splitmix64
 * (orc_draws_f64 below), identical to the library's host generator.
 *
 * The parallel assignment mirrors assign_parallel's chunking
 * (chunk = max(n/threads, 64)) with OpenMP; the per-chunk inertia partials
 * are folded left to right, which is one of the orders Rayon's reduce can
 * produce. Below the PARALLEL_WORK_THRESHOLD the serial fold is used exactly.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_PARALLEL_WORK_THRESHOLD 100000 /* kmeans.rs:261 */

enum { ORC_OK = 0, ORC_ERR_INVALID_PARAMETER = 1, ORC_ERR_INSUFFICIENT_SAMPLES = 2,
       ORC_ERR_SHAPE_MISMATCH = 3, ORC_ERR_OOM = 11, ORC_ERR_NULL = 14 };

/* ---------------------------------------------------------------- draws -- */
/* splitmix64 stream: state advances by the golden gamma, output mixed. */
typedef struct { uint64_t state; const double *inj; int64_t n_inj; int64_t pos; } orc_draws;

static uint64_t orc_splitmix64(uint64_t *s) {
    uint64_t z = (*s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

static double orc_next(orc_draws *g) {
    if (g->inj) {
        double u = (g->pos < g->n_inj) ? g->inj[g->pos] : 0.0;
        g->pos++;
        return u;
    }
    g->pos++;
    return (double)(orc_splitmix64(&g->state) >> 11) * (1.0 / 9007199254740992.0);
}

static int64_t orc_range(orc_draws *g, int64_t n) {
    double u = orc_next(g);
    int64_t i = (int64_t)floor(u * (double)n);
    if (i < 0) i = 0;
    if (i >= n) i = n - 1;
    return i;
}

/* Exposed so tests can check that the library's host stream is identical. */
void orc_draws_f64(uint64_t seed, int64_t count, double *out) {
    orc_draws g = {seed, NULL, 0, 0};
    for (int64_t i = 0; i < count; i++) out[i] = orc_next(&g);
}

/* ----------------------------------------------------- templated body -- */
#define ORC_DEFINE(T, SUF, TMAX)                                                        \
static T orc_sqeuc_##SUF(const T *a, const T *b, int64_t d) {                          \
    T acc = (T)0;                                                                       \
    for (int64_t j = 0; j < d; j++) { T t = a[j] - b[j]; acc = acc + t * t; }           \
    return acc;                                                                         \
}                                                                                       \
                                                                                        \
static void orc_nearest_##SUF(const T *row, const T *c, int64_t k, int64_t d,          \
                              int64_t *lab, T *dist) {                                 \
    int64_t best = 0; T bd = TMAX;                                                      \
    for (int64_t q = 0; q < k; q++) {                                                   \
        T v = orc_sqeuc_##SUF(row, c + q * d, d);                                       \
        if (v < bd) { bd = v; best = q; }                                               \
    }                                                                                   \
    *lab = best; *dist = bd;                                                            \
}                                                                                       \
                                                                                        \
/* assign_clusters_into (kmeans.rs:279-352): labels + inertia; mind optional */         \
T orc_assign_##SUF(const T *x, int64_t n, int64_t d, const T *c, int64_t k,             \
                   int64_t *labels, T *mind, int nthreads) {                           \
    if (n * d < ORC_PARALLEL_WORK_THRESHOLD || nthreads <= 1) {                         \
        T inertia = (T)0;                                                               \
        for (int64_t i = 0; i < n; i++) {                                               \
            T dist; orc_nearest_##SUF(x + i * d, c, k, d, &labels[i], &dist);           \
            if (mind) mind[i] = dist;                                                   \
            inertia = inertia + dist;                                                   \
        }                                                                               \
        return inertia;                                                                 \
    }                                                                                   \
    int64_t chunk = n / nthreads; if (chunk < 64) chunk = 64;                           \
    int64_t nchunks = (n + chunk - 1) / chunk;                                          \
    T *part = (T *)malloc(sizeof(T) * (size_t)nchunks);                                 \
    _Pragma("omp parallel for schedule(dynamic,1) num_threads(nthreads)")               \
    for (int64_t ch = 0; ch < nchunks; ch++) {                                          \
        int64_t lo = ch * chunk, hi = lo + chunk < n ? lo + chunk : n;                  \
        T loc = (T)0;                                                                   \
        for (int64_t i = lo; i < hi; i++) {                                             \
            T dist; orc_nearest_##SUF(x + i * d, c, k, d, &labels[i], &dist);           \
            if (mind) mind[i] = dist;                                                   \
            loc = loc + dist;                                                           \
        }                                                                               \
        part[ch] = loc;                                                                 \
    }                                                                                   \
    T inertia = (T)0;                                                                   \
    for (int64_t ch = 0; ch < nchunks; ch++) inertia = inertia + part[ch];              \
    free(part);                                                                         \
    return inertia;                                                                     \
}                                                                                       \
                                                                                        \
/* recompute_centroids_into (kmeans.rs:358-401); returns sqrt(max shift^2) */           \
T orc_update_##SUF(const T *x, int64_t n, int64_t d, const int64_t *labels,             \
                   const T *old_c, int64_t k, T *new_c, T *counts) {                    \
    memset(new_c, 0, sizeof(T) * (size_t)(k * d));                                      \
    for (int64_t q = 0; q < k; q++) counts[q] = (T)0;                                   \
    for (int64_t i = 0; i < n; i++) {                                                   \
        int64_t l = labels[i];                                                          \
        counts[l] = counts[l] + (T)1;                                                   \
        for (int64_t j = 0; j < d; j++) new_c[l * d + j] = new_c[l * d + j] + x[i * d + j]; \
    }                                                                                   \
    for (int64_t q = 0; q < k; q++) {                                                   \
        if (counts[q] > (T)0) {                                                         \
            for (int64_t j = 0; j < d; j++) new_c[q * d + j] = new_c[q * d + j] / counts[q]; \
        } else {                                                                        \
            memcpy(new_c + q * d, old_c + q * d, sizeof(T) * (size_t)d);               \
        }                                                                               \
    }                                                                                   \
    T ms = (T)0;                                                                        \
    for (int64_t q = 0; q < k; q++) {                                                   \
        T s = orc_sqeuc_##SUF(new_c + q * d, old_c + q * d, d);                         \
        if (s > ms) ms = s;                                                             \
    }                                                                                   \
    return orc_sqrt_##SUF(ms);                                                          \
}                                                                                       \
                                                                                        \
/* kmeans_plus_plus (kmeans.rs:169-253) with an injected uniform stream */              \
static void orc_kpp_##SUF(const T *x, int64_t n, int64_t d, int64_t k, orc_draws *g,   \
                          T *centers) {                                                 \
    memset(centers, 0, sizeof(T) * (size_t)(k * d));                                    \
    if (n == 0) return;                                                                 \
    int64_t first = orc_range(g, n);                                                    \
    memcpy(centers, x + first * d, sizeof(T) * (size_t)d);                              \
    if (k == 1) return;                                                                 \
    T *mind = (T *)malloc(sizeof(T) * (size_t)n);                                       \
    T *nd = (T *)malloc(sizeof(T) * (size_t)n);                                         \
    T *bestd = (T *)malloc(sizeof(T) * (size_t)n);                                      \
    _Pragma("omp parallel for schedule(static)")                                        \
    for (int64_t i = 0; i < n; i++) mind[i] = orc_sqeuc_##SUF(x + i * d, centers, d);   \
    int64_t n_trials = 2 + (int64_t)floor(log((double)k));                              \
    if (n_trials < 1) n_trials = 1;                                                     \
    for (int64_t c = 1; c < k; c++) {                                                   \
        T total = (T)0;                                                                 \
        for (int64_t i = 0; i < n; i++) total = total + mind[i];                        \
        if (total <= (T)0) {                                                            \
            int64_t idx = orc_range(g, n);                                              \
            memcpy(centers + c * d, x + idx * d, sizeof(T) * (size_t)d);                \
            continue;                                                                   \
        }                                                                               \
        int64_t best_cand = 0; int have = 0; T best_pot = (T)0;                         \
        for (int64_t t = 0; t < n_trials; t++) {                                        \
            T thr = (T)orc_next(g) * total;                                             \
            T cum = (T)0; int64_t cand = n - 1;                                         \
            for (int64_t i = 0; i < n; i++) {                                           \
                cum = cum + mind[i];                                                    \
                if (cum >= thr) { cand = i; break; }                                    \
            }                                                                           \
            /* the distances in parallel, then the potential folded in row order */     \
            _Pragma("omp parallel for schedule(static)")                                \
            for (int64_t i = 0; i < n; i++) {                                           \
                T v = orc_sqeuc_##SUF(x + i * d, x + cand * d, d);                      \
                nd[i] = v < mind[i] ? v : mind[i];                                      \
            }                                                                           \
            T pot = (T)0;                                                               \
            for (int64_t i = 0; i < n; i++) pot = pot + nd[i];                          \
            if (!have || pot < best_pot) {                                              \
                have = 1; best_pot = pot; best_cand = cand;                             \
                T *tmp = bestd; bestd = nd; nd = tmp;                                   \
            }                                                                           \
        }                                                                               \
        memcpy(centers + c * d, x + best_cand * d, sizeof(T) * (size_t)d);             \
        { T *tmp = mind; mind = bestd; bestd = tmp; }                                   \
    }                                                                                   \
    free(mind); free(nd); free(bestd);                                                  \
}                                                                                       \
                                                                                        \
int orc_kmeanspp_##SUF(const T *x, int64_t n, int64_t d, int64_t k,                     \
                       const double *draws, int64_t n_draws, uint64_t seed,            \
                       T *centers, int64_t *draws_used) {                               \
    if (!x || !centers) return ORC_ERR_NULL;                                            \
    orc_draws g = {seed, draws, n_draws, 0};                                            \
    orc_kpp_##SUF(x, n, d, k, &g, centers);                                             \
    if (draws_used) *draws_used = g.pos;                                                \
    return ORC_OK;                                                                      \
}                                                                                       \
                                                                                        \
/* One Lloyd iteration exactly as the body of kmeans.rs:468-488 */                      \
int orc_lloyd_step_##SUF(const T *x, int64_t n, int64_t d, const T *centers, int64_t k, \
                         int64_t *labels, T *new_c, T *inertia, T *max_shift,          \
                         int nthreads) {                                                \
    T *counts = (T *)malloc(sizeof(T) * (size_t)k);                                     \
    if (!counts) return ORC_ERR_OOM;                                                    \
    *inertia = orc_assign_##SUF(x, n, d, centers, k, labels, NULL, nthreads);           \
    *max_shift = orc_update_##SUF(x, n, d, labels, centers, k, new_c, counts);          \
    free(counts);                                                                       \
    return ORC_OK;                                                                      \
}                                                                                       \
                                                                                        \
/* Fit::fit (kmeans.rs:417-512). init: n_init*k*d centers, or NULL for k-means++ */     \
int orc_fit_##SUF(const T *x, int64_t n, int64_t d, int64_t k, int64_t max_iter,        \
                  T tol, int64_t n_init, const T *init, const double *draws,           \
                  int64_t n_draws, uint64_t seed, T *out_c, int64_t *out_labels,        \
                  T *out_inertia, int64_t *out_n_iter, int64_t *out_best_run,          \
                  int nthreads) {                                                       \
    if (k == 0) return ORC_ERR_INVALID_PARAMETER;                                       \
    if (n == 0 || n < k) return ORC_ERR_INSUFFICIENT_SAMPLES;                           \
    if (n_init == 0) return ORC_ERR_INVALID_PARAMETER;                                  \
    T *c = (T *)malloc(sizeof(T) * (size_t)(k * d));                                    \
    T *nc = (T *)malloc(sizeof(T) * (size_t)(k * d));                                   \
    T *counts = (T *)malloc(sizeof(T) * (size_t)k);                                     \
    int64_t *lab = (int64_t *)calloc((size_t)n, sizeof(int64_t));                       \
    if (!c || !nc || !counts || !lab) return ORC_ERR_OOM;                               \
    int have = 0; T best_in = TMAX;                                                     \
    orc_draws g = {0, draws, n_draws, 0};                                               \
    for (int64_t run = 0; run < n_init; run++) {                                        \
        if (init) {                                                                     \
            memcpy(c, init + run * k * d, sizeof(T) * (size_t)(k * d));               \
        } else {                                                                        \
            if (!draws) { g.state = seed + (uint64_t)run; g.pos = 0; }                  \
            orc_kpp_##SUF(x, n, d, k, &g, c);                                           \
        }                                                                               \
        int64_t n_iter = 0; T inertia = TMAX;                                           \
        for (int64_t it = 0; it < max_iter; it++) {                                     \
            inertia = orc_assign_##SUF(x, n, d, c, k, lab, NULL, nthreads);             \
            T ms = orc_update_##SUF(x, n, d, lab, c, k, nc, counts);                    \
            T *tmp = c; c = nc; nc = tmp;                                               \
            n_iter = it + 1;                                                            \
            if (ms < tol) break;                                                        \
        }                                                                               \
        if (!have || inertia < best_in) {                                               \
            have = 1; best_in = inertia;                                                \
            memcpy(out_c, c, sizeof(T) * (size_t)(k * d));                              \
            memcpy(out_labels, lab, sizeof(int64_t) * (size_t)n);                       \
            *out_inertia = inertia; *out_n_iter = n_iter;                               \
            if (out_best_run) *out_best_run = run;                                      \
        }                                                                               \
    }                                                                                   \
    free(c); free(nc); free(counts); free(lab);                                         \
    return ORC_OK;                                                                      \
}                                                                                       \
                                                                                        \
/* Predict::predict (kmeans.rs:538-552) */                                              \
int orc_predict_##SUF(const T *c, int64_t k, int64_t d_fit, const T *x, int64_t n,      \
                      int64_t d, int64_t *labels, int nthreads) {                       \
    if (d != d_fit) return ORC_ERR_SHAPE_MISMATCH;                                      \
    orc_assign_##SUF(x, n, d, c, k, labels, NULL, nthreads);                            \
    return ORC_OK;                                                                      \
}                                                                                       \
                                                                                        \
/* Transform::transform (kmeans.rs:568-617) */                                          \
int orc_transform_##SUF(const T *c, int64_t k, int64_t d_fit, const T *x, int64_t n,    \
                        int64_t d, T *out, int nthreads) {                              \
    if (d != d_fit) return ORC_ERR_SHAPE_MISMATCH;                                      \
    _Pragma("omp parallel for schedule(static) num_threads(nthreads)")                  \
    for (int64_t i = 0; i < n; i++)                                                     \
        for (int64_t q = 0; q < k; q++)                                                 \
            out[i * k + q] = orc_sqrt_##SUF(orc_sqeuc_##SUF(x + i * d, c + q * d, d));  \
    return ORC_OK;                                                                      \
}

static double orc_sqrt_f64(double v) { return sqrt(v); }
static float orc_sqrt_f32(float v) { return sqrtf(v); }

ORC_DEFINE(double, f64, DBL_MAX)
ORC_DEFINE(float, f32, FLT_MAX)

/* ------------------------------------------------------ MiniBatchKMeans -- */
/* ferrolearn-cluster/src/mini_batch_kmeans.rs with the library's uniform
 * stream in place of StdRng: run r draws from splitmix64 seeded with
 * random_state + r * 1000003 (the run seeds of :532); the initial centres
 * come first (kmeans_plus_plus_mb :230-321, the same statements as
 * kmeans.rs:169-253, or random_init_mb :324-338; explicit centres draw
 * nothing), then sample_batch_indices (:451-472) once per iteration.
 * random_range(a..b) is a + min(floor(u (b - a)), b - a - 1). */

/* A stream positioned after `pos` draws of seed: every draw first advances
 * the state by the golden gamma. */
static orc_draws orc_stream_at(uint64_t seed, int64_t pos) {
    orc_draws g = {seed + (uint64_t)pos * 0x9E3779B97F4A7C15ULL, NULL, 0, pos};
    return g;
}

/* sample_batch_indices (:451-472): every row in a random order when
 * batch_size >= n (a full Fisher-Yates pass), else batch_size rows without
 * replacement (a partial Fisher-Yates pass over a fresh pool 0..n). */
static int64_t orc_mb_sample(orc_draws *g, int64_t n, int64_t batch_size, int64_t *pool, int64_t *out) {
    for (int64_t i = 0; i < n; i++) pool[i] = i;
    const int64_t m = batch_size >= n ? n : batch_size;
    for (int64_t i = 0; i < m; i++) {
        int64_t j = i + orc_range(g, n - i);
        int64_t t = pool[i]; pool[i] = pool[j]; pool[j] = t;
        out[i] = pool[i];
    }
    return m;
}

/* The batch indices of `iters` iterations from stream position pos (for the
 * tests of the library's own generator). out: iters * min(batch_size, n). */
int orc_mb_batch_indices(uint64_t seed, int64_t pos, int64_t n, int64_t batch_size, int64_t iters,
                         int64_t *out) {
    if (n <= 0 || batch_size <= 0) return ORC_ERR_INVALID_PARAMETER;
    int64_t *pool = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
    if (!pool) return ORC_ERR_OOM;
    orc_draws g = orc_stream_at(seed, pos);
    const int64_t m = batch_size >= n ? n : batch_size;
    for (int64_t it = 0; it < iters; it++) orc_mb_sample(&g, n, batch_size, pool, out + it * m);
    free(pool);
    return ORC_OK;
}

#define ORC_DEFINE_MB(T, SUF, TMAX)                                                     \
/* random_init_mb (:324-338): k picks of a partial Fisher-Yates pass */                 \
static void orc_mb_random_init_##SUF(const T *x, int64_t n, int64_t d, int64_t k,      \
                                     orc_draws *g, T *centers, int64_t *pool) {         \
    for (int64_t i = 0; i < n; i++) pool[i] = i;                                        \
    for (int64_t i = 0; i < k; i++) {                                                   \
        int64_t j = i + orc_range(g, n - i);                                            \
        int64_t t = pool[i]; pool[i] = pool[j]; pool[j] = t;                            \
        memcpy(centers + i * d, x + pool[i] * d, sizeof(T) * (size_t)d);                \
    }                                                                                   \
}                                                                                       \
                                                                                        \
/* update_centers_mini_batch (:410-447): per sample in batch order,           */        \
/* count += 1, lr = 1 / count, c += lr (x - c); returns the max over centres  */        \
/* of sqrt(||c - c_old||^2) (a NaN shift never wins, as `shift > max`).       */        \
static T orc_mb_update_##SUF(const T *x, const int64_t *idx, const int64_t *lab,        \
                             int64_t m, int64_t d, T *c, int64_t k, int64_t *counts,    \
                             T *old) {                                                  \
    memcpy(old, c, sizeof(T) * (size_t)(k * d));                                        \
    for (int64_t b = 0; b < m; b++) {                                                   \
        const int64_t l = lab[b];                                                       \
        counts[l] += 1;                                                                 \
        const T lr = (T)1 / (T)counts[l];                                               \
        const T *row = x + idx[b] * d;                                                  \
        for (int64_t j = 0; j < d; j++) c[l * d + j] = c[l * d + j] + lr * (row[j] - c[l * d + j]); \
    }                                                                                   \
    T ms = (T)0;                                                                        \
    for (int64_t q = 0; q < k; q++) {                                                   \
        T s = orc_sqrt_##SUF(orc_sqeuc_##SUF(c + q * d, old + q * d, d));               \
        if (s > ms) ms = s;                                                             \
    }                                                                                   \
    return ms;                                                                          \
}                                                                                       \
                                                                                        \
/* MiniBatchKMeans::fit (:492-591). init_mode 0: k-means++, 1: random; init  */         \
/* (n_init * k * d) replaces either when given. Labels and inertia of the    */         \
/* kept run come from assign_clusters_mb (:343-376): nearest centre, strict  */         \
/* < from F::MAX, inertia summed in row order.                               */         \
int orc_minibatch_fit_##SUF(const T *x, int64_t n, int64_t d, int64_t k,               \
                            int64_t batch_size, int64_t max_iter, T tol,               \
                            int64_t n_init, uint64_t seed, int init_mode,              \
                            const T *init, T *out_c, int64_t *out_labels,              \
                            T *out_inertia, int64_t *out_n_iter,                       \
                            int64_t *out_best_run, int64_t *out_run_n_iter,            \
                            T *out_run_inertia) {                                       \
    if (k == 0) return ORC_ERR_INVALID_PARAMETER;                                       \
    if (batch_size == 0) return ORC_ERR_INVALID_PARAMETER;                              \
    if (n_init == 0) return ORC_ERR_INVALID_PARAMETER;                                  \
    if (n == 0 || n < k) return ORC_ERR_INSUFFICIENT_SAMPLES;                           \
    T *c = (T *)malloc(sizeof(T) * (size_t)(k * d));                                    \
    T *old = (T *)malloc(sizeof(T) * (size_t)(k * d));                                  \
    int64_t *counts = (int64_t *)malloc(sizeof(int64_t) * (size_t)k);                   \
    int64_t *pool = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);                     \
    int64_t *idx = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);                      \
    int64_t *blab = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);                     \
    int64_t *lab = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);                      \
    if (!c || !old || !counts || !pool || !idx || !blab || !lab) return ORC_ERR_OOM;    \
    int have = 0; T best_in = TMAX;                                                     \
    for (int64_t run = 0; run < n_init; run++) {                                        \
        orc_draws g = orc_stream_at(seed + (uint64_t)run * 1000003ULL, 0);              \
        if (init) memcpy(c, init + run * k * d, sizeof(T) * (size_t)(k * d));           \
        else if (init_mode == 1) orc_mb_random_init_##SUF(x, n, d, k, &g, c, pool);     \
        else orc_kpp_##SUF(x, n, d, k, &g, c);                                          \
        for (int64_t q = 0; q < k; q++) counts[q] = 1;                                  \
        int64_t n_iter = 0;                                                             \
        for (int64_t it = 0; it < max_iter; it++) {                                     \
            const int64_t m = orc_mb_sample(&g, n, batch_size, pool, idx);              \
            for (int64_t b = 0; b < m; b++) {                                           \
                T dist; orc_nearest_##SUF(x + idx[b] * d, c, k, d, &blab[b], &dist);    \
            }                                                                           \
            T shift = orc_mb_update_##SUF(x, idx, blab, m, d, c, k, counts, old);       \
            n_iter += 1;                                                                \
            if (shift < tol) break;                                                     \
        }                                                                               \
        T inertia = (T)0;                                                               \
        for (int64_t i = 0; i < n; i++) {                                               \
            T dist; orc_nearest_##SUF(x + i * d, c, k, d, &lab[i], &dist);              \
            inertia = inertia + dist;                                                   \
        }                                                                               \
        if (out_run_n_iter) out_run_n_iter[run] = n_iter;                               \
        if (out_run_inertia) out_run_inertia[run] = inertia;                            \
        if (!have || inertia < best_in) {                                               \
            have = 1; best_in = inertia;                                                \
            memcpy(out_c, c, sizeof(T) * (size_t)(k * d));                              \
            memcpy(out_labels, lab, sizeof(int64_t) * (size_t)n);                       \
            *out_inertia = inertia; *out_n_iter = n_iter;                               \
            if (out_best_run) *out_best_run = run;                                      \
        }                                                                               \
    }                                                                                   \
    free(c); free(old); free(counts); free(pool); free(idx); free(blab); free(lab);     \
    return ORC_OK;                                                                      \
}

ORC_DEFINE_MB(double, f64, DBL_MAX)
ORC_DEFINE_MB(float, f32, FLT_MAX)

/* ------------------------------------------------------ BisectingKMeans -- */
/* ferrolearn-cluster/src/bisecting_kmeans.rs with the library's uniform
 * stream in place of StdRng: run r of split s draws from splitmix64 seeded
 * with random_state + s * 1000 + r (wrapping, :410-412). Selection of the
 * cluster to split follows Rust's Iterator::max_by_key / max_by, which keep
 * the LAST of equally maximal elements (:376-396); a cluster whose split
 * leaves one side empty is pushed back unchanged (:466-481), which the
 * reference repeats without end when that cluster stays the one selected:
 * the restatement stops after ORC_BK_MAX_SPLITS splits with
 * ORC_ERR_NO_PROGRESS instead. */
#define ORC_ERR_NUMERICAL 4
#define ORC_ERR_NO_PROGRESS 5
#define ORC_BK_MAX_SPLITS(n, k) (4 * (n) + 4 * (k) + 16)

#define ORC_DEFINE_BK(T, SUF, TMAX)                                                     \
/* compute_cluster_stats (:192-222): row-order sums / n, SSE in row order */            \
static T orc_bk_stats_##SUF(const T *x, int64_t d, const int64_t *idx, int64_t m,       \
                            T *centre) {                                                \
    for (int64_t j = 0; j < d; j++) centre[j] = (T)0;                                   \
    if (m == 0) return (T)0;                                                            \
    const T nf = (T)m;                                                                  \
    for (int64_t i = 0; i < m; i++)                                                     \
        for (int64_t j = 0; j < d; j++) centre[j] = centre[j] + x[idx[i] * d + j];      \
    for (int64_t j = 0; j < d; j++) centre[j] = centre[j] / nf;                         \
    T sse = (T)0;                                                                       \
    for (int64_t i = 0; i < m; i++) sse = sse + orc_sqeuc_##SUF(x + idx[i] * d, centre, d); \
    return sse;                                                                         \
}                                                                                       \
                                                                                        \
/* run_2means (:225-312): two distinct rows of the subset, then assignments */          \
/* (d0 <= d1 -> 0) until no label changes, row-order sums / counts in F    */          \
/* (an empty side keeps its centre); returns the SSE against the final     */          \
/* centres.                                                                */          \
static T orc_bk_2means_##SUF(const T *x, int64_t d, const int64_t *idx, int64_t m,      \
                             int64_t max_iter, orc_draws *g, unsigned char *lab,        \
                             T *c0, T *c1, T *s0, T *s1) {                              \
    const int64_t i0 = orc_range(g, m);                                                 \
    int64_t i1 = orc_range(g, m);                                                       \
    if (m > 1) while (i1 == i0) i1 = orc_range(g, m);                                   \
    memcpy(c0, x + idx[i0] * d, sizeof(T) * (size_t)d);                                \
    memcpy(c1, x + idx[i1] * d, sizeof(T) * (size_t)d);                                \
    memset(lab, 0, (size_t)m);                                                          \
    for (int64_t it = 0; it < max_iter; it++) {                                         \
        int changed = 0;                                                                \
        for (int64_t i = 0; i < m; i++) {                                               \
            const T *row = x + idx[i] * d;                                              \
            const T d0 = orc_sqeuc_##SUF(row, c0, d), d1 = orc_sqeuc_##SUF(row, c1, d); \
            const unsigned char nl = d0 <= d1 ? 0 : 1;                                  \
            if (nl != lab[i]) { lab[i] = nl; changed = 1; }                             \
        }                                                                               \
        if (!changed) break;                                                            \
        T n0 = (T)0, n1 = (T)0;                                                         \
        for (int64_t j = 0; j < d; j++) { s0[j] = (T)0; s1[j] = (T)0; }                 \
        for (int64_t i = 0; i < m; i++) {                                               \
            const T *row = x + idx[i] * d;                                              \
            if (lab[i] == 0) {                                                          \
                n0 = n0 + (T)1;                                                         \
                for (int64_t j = 0; j < d; j++) s0[j] = s0[j] + row[j];                 \
            } else {                                                                    \
                n1 = n1 + (T)1;                                                         \
                for (int64_t j = 0; j < d; j++) s1[j] = s1[j] + row[j];                 \
            }                                                                           \
        }                                                                               \
        if (n0 > (T)0) for (int64_t j = 0; j < d; j++) c0[j] = s0[j] / n0;              \
        if (n1 > (T)0) for (int64_t j = 0; j < d; j++) c1[j] = s1[j] / n1;              \
    }                                                                                   \
    T sse = (T)0;                                                                       \
    for (int64_t i = 0; i < m; i++)                                                     \
        sse = sse + orc_sqeuc_##SUF(x + idx[i] * d, lab[i] ? c1 : c0, d);               \
    return sse;                                                                         \
}                                                                                       \
                                                                                        \
/* BisectingKMeans::fit (:326-505). strategy 0: LargestCluster, 1:           */        \
/* LargestSSE. Outputs: out_c (k*d, the first *out_n_clusters rows used),    */        \
/* labels (cluster order of the final list), inertia (sum of the clusters'  */        \
/* SSE in list order).                                                       */        \
int orc_bisecting_fit_##SUF(const T *x, int64_t n, int64_t d, int64_t k,               \
                            int64_t max_iter, int64_t n_init, uint64_t seed,           \
                            int strategy, T *out_c, int64_t *out_labels,               \
                            T *out_inertia, int64_t *out_n_clusters) {                  \
    if (k == 0) return ORC_ERR_INVALID_PARAMETER;                                       \
    if (n_init == 0) return ORC_ERR_INVALID_PARAMETER;                                  \
    if (n == 0 || n < k) return ORC_ERR_INSUFFICIENT_SAMPLES;                           \
    int64_t **cidx = (int64_t **)calloc((size_t)k + 1, sizeof(int64_t *));              \
    int64_t *cm = (int64_t *)calloc((size_t)k + 1, sizeof(int64_t));                    \
    T *ccen = (T *)malloc(sizeof(T) * (size_t)((k + 1) * d + 1));                       \
    T *csse = (T *)malloc(sizeof(T) * (size_t)(k + 1));                                 \
    unsigned char *lab = (unsigned char *)malloc((size_t)n + 1);                        \
    unsigned char *blab = (unsigned char *)malloc((size_t)n + 1);                       \
    T *w = (T *)malloc(sizeof(T) * (size_t)(6 * d + 6));                                \
    if (!cidx || !cm || !ccen || !csse || !lab || !blab || !w) return ORC_ERR_OOM;      \
    T *c0 = w, *c1 = w + d, *s0 = w + 2 * d, *s1 = w + 3 * d, *b0 = w + 4 * d, *b1 = w + 5 * d; \
    int rc = ORC_OK;                                                                    \
    int64_t nc = 1;                                                                     \
    cidx[0] = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);                           \
    for (int64_t i = 0; i < n; i++) cidx[0][i] = i;                                     \
    cm[0] = n;                                                                          \
    csse[0] = orc_bk_stats_##SUF(x, d, cidx[0], n, ccen);                               \
    uint64_t split_count = 0;                                                           \
    while (nc < k) {                                                                    \
        if ((int64_t)split_count > ORC_BK_MAX_SPLITS(n, k)) { rc = ORC_ERR_NO_PROGRESS; break; } \
        int64_t t = -1;                                                                 \
        for (int64_t ci = 0; ci < nc; ci++) {                                           \
            if (cm[ci] < 2) continue;                                                   \
            if (t < 0) { t = ci; continue; }                                            \
            if (strategy == 0) { if (!(cm[t] > cm[ci])) t = ci; }                       \
            else { if (!(csse[t] > csse[ci])) t = ci; }                                 \
        }                                                                               \
        if (t < 0) break;                                                               \
        const int64_t m = cm[t];                                                        \
        int have = 0; T best = TMAX;                                                    \
        for (int64_t run = 0; run < n_init; run++) {                                    \
            orc_draws g = orc_stream_at(seed + split_count * 1000ULL + (uint64_t)run, 0); \
            T sse = orc_bk_2means_##SUF(x, d, cidx[t], m, max_iter, &g, lab, c0, c1, s0, s1); \
            if (sse < best) {                                                           \
                best = sse; have = 1;                                                   \
                memcpy(blab, lab, (size_t)m);                                           \
                memcpy(b0, c0, sizeof(T) * (size_t)d); memcpy(b1, c1, sizeof(T) * (size_t)d); \
            }                                                                           \
        }                                                                               \
        split_count++;                                                                  \
        if (!have) { rc = ORC_ERR_NUMERICAL; break; }                                   \
        int64_t m0 = 0;                                                                 \
        for (int64_t i = 0; i < m; i++) m0 += blab[i] == 0;                             \
        int64_t *i0 = (int64_t *)malloc(sizeof(int64_t) * (size_t)(m0 + 1));            \
        int64_t *i1 = (int64_t *)malloc(sizeof(int64_t) * (size_t)(m - m0 + 1));        \
        int64_t p0 = 0, p1 = 0;                                                         \
        for (int64_t i = 0; i < m; i++) {                                               \
            if (blab[i] == 0) i0[p0++] = cidx[t][i]; else i1[p1++] = cidx[t][i];        \
        }                                                                               \
        T sse0 = (T)0, sse1 = (T)0;                                                     \
        for (int64_t i = 0; i < p0; i++) sse0 = sse0 + orc_sqeuc_##SUF(x + i0[i] * d, b0, d); \
        for (int64_t i = 0; i < p1; i++) sse1 = sse1 + orc_sqeuc_##SUF(x + i1[i] * d, b1, d); \
        free(cidx[t]);                                                                  \
        for (int64_t ci = t; ci + 1 < nc; ci++) {                                       \
            cidx[ci] = cidx[ci + 1]; cm[ci] = cm[ci + 1]; csse[ci] = csse[ci + 1];      \
            memcpy(ccen + ci * d, ccen + (ci + 1) * d, sizeof(T) * (size_t)d);          \
        }                                                                               \
        nc -= 1;                                                                        \
        if (p0 > 0) {                                                                   \
            cidx[nc] = i0; cm[nc] = p0; csse[nc] = sse0;                                \
            memcpy(ccen + nc * d, b0, sizeof(T) * (size_t)d); nc++;                     \
        } else free(i0);                                                                \
        if (p1 > 0) {                                                                   \
            cidx[nc] = i1; cm[nc] = p1; csse[nc] = sse1;                                \
            memcpy(ccen + nc * d, b1, sizeof(T) * (size_t)d); nc++;                     \
        } else free(i1);                                                                \
    }                                                                                   \
    if (rc == ORC_OK) {                                                                 \
        T inertia = (T)0;                                                               \
        for (int64_t ci = 0; ci < nc; ci++) {                                           \
            memcpy(out_c + ci * d, ccen + ci * d, sizeof(T) * (size_t)d);               \
            for (int64_t i = 0; i < cm[ci]; i++) out_labels[cidx[ci][i]] = ci;          \
            inertia = inertia + csse[ci];                                               \
        }                                                                               \
        *out_inertia = inertia;                                                         \
        *out_n_clusters = nc;                                                           \
    }                                                                                   \
    for (int64_t ci = 0; ci < nc; ci++) free(cidx[ci]);                                 \
    free(cidx); free(cm); free(ccen); free(csse); free(lab); free(blab); free(w);       \
    return rc;                                                                          \
}

ORC_DEFINE_BK(double, f64, DBL_MAX)
ORC_DEFINE_BK(float, f32, FLT_MAX)

/* Direct-form FP64 distance from an f32 row to an f64 centre, used for the
 * "X stored f32, oracle in f64" parity cases: the row is widened exactly. */
int orc_widen_f32(const float *x, int64_t count, double *out) {
    for (int64_t i = 0; i < count; i++) out[i] = (double)x[i];
    return ORC_OK;
}

/* --------------------------------------------- batched fits, per run -- */
/* Fit::fit (kmeans.rs:417-512) for F = f32, every run kept: run r seeds
 * k-means++ (kmeans.rs:169-253) with splitmix64(seed + r), or takes
 * init[r]; Lloyd iterations follow kmeans.rs:459-505. wide_sums = 0 is the
 * reference's own f32 arithmetic (recompute_centroids_into, kmeans.rs:358-401,
 * row-order f32 sums); wide_sums = 1 is the batched entry point's FP64
 * reduction variant: each cluster sum formed exactly (128-bit fixed point
 * with F = 124 - bitlen(n) - e fraction bits, 2^e <= max|x| < 2^(e+1)),
 * rounded once to f64, divided by the count in f64 and rounded to f32; the
 * inertia summed in f64 in row order.
 * Outputs per run: centres (k*d), labels (n), inertia (as f64), n_iter. */
static int orc_bitlen(int64_t v) { int b = 0; while (v > 0) { b++; v >>= 1; } return b ? b : 1; }

static float orc_update_f32_wide(const float *x, int64_t n, int64_t d, const int64_t *labels,
                                 const float *old_c, int64_t k, float *new_c, __int128 *sums,
                                 unsigned *flags, int64_t *counts, int F) {
    memset(sums, 0, sizeof(__int128) * (size_t)(k * d));
    memset(flags, 0, sizeof(unsigned) * (size_t)(k * d));
    for (int64_t q = 0; q < k; q++) counts[q] = 0;
    for (int64_t i = 0; i < n; i++) {
        int64_t l = labels[i];
        counts[l] += 1;
        for (int64_t j = 0; j < d; j++) {
            float v = x[i * d + j];
            if (isnan(v)) { flags[l * d + j] |= 1u; continue; }
            if (isinf(v)) { flags[l * d + j] |= v > 0 ? 2u : 4u; continue; }
            int e;
            float fr = frexpf(v, &e);                      /* v = fr * 2^e, 0.5 <= |fr| < 1 */
            int64_t m = (int64_t)ldexpf(fabsf(fr), 24);    /* exact 24-bit integer */
            int s = e - 24 + F;                            /* |v| = m * 2^(s - F) */
            __int128 t = s >= 0 ? ((__int128)m << s) : (s > -64 ? (__int128)(m >> (-s)) : 0);
            sums[l * d + j] += v < 0 ? -t : t;
        }
    }
    for (int64_t q = 0; q < k; q++) {
        if (counts[q] > 0) {
            for (int64_t j = 0; j < d; j++) {
                unsigned fl = flags[q * d + j];
                double sm;
                if ((fl & 1u) || (fl & 6u) == 6u) sm = NAN;
                else if (fl & 2u) sm = INFINITY;
                else if (fl & 4u) sm = -INFINITY;
                else sm = ldexp((double)sums[q * d + j], -F);  /* the conversion rounds to nearest */
                new_c[q * d + j] = (float)(sm / (double)counts[q]);
            }
        } else {
            memcpy(new_c + q * d, old_c + q * d, sizeof(float) * (size_t)d);
        }
    }
    float ms = 0.0f;
    for (int64_t q = 0; q < k; q++) {
        float s = orc_sqeuc_f32(new_c + q * d, old_c + q * d, d);
        if (s > ms) ms = s;
    }
    return sqrtf(ms);
}

int orc_fit_runs_f32(const float *x, int64_t n, int64_t d, int64_t k, int64_t max_iter, float tol,
                     int64_t n_init, const float *init, uint64_t seed, int wide_sums, float *out_c,
                     int64_t *out_labels, double *out_inertia, int64_t *out_n_iter, int nthreads) {
    if (k == 0) return ORC_ERR_INVALID_PARAMETER;
    if (n == 0 || n < k) return ORC_ERR_INSUFFICIENT_SAMPLES;
    if (n_init == 0) return ORC_ERR_INVALID_PARAMETER;
    float *c = (float *)malloc(sizeof(float) * (size_t)(k * d));
    float *nc = (float *)malloc(sizeof(float) * (size_t)(k * d));
    float *counts = (float *)malloc(sizeof(float) * (size_t)k);
    __int128 *sums = (__int128 *)malloc(sizeof(__int128) * (size_t)(k * d));
    unsigned *flags = (unsigned *)malloc(sizeof(unsigned) * (size_t)(k * d));
    int64_t *icounts = (int64_t *)malloc(sizeof(int64_t) * (size_t)k);
    float *mind = (float *)malloc(sizeof(float) * (size_t)n);
    int64_t *lab = (int64_t *)calloc((size_t)n, sizeof(int64_t));
    if (!c || !nc || !counts || !sums || !flags || !icounts || !mind || !lab) return ORC_ERR_OOM;
    float amax = 0.0f;
    for (int64_t i = 0; i < n * d; i++) {
        float a = fabsf(x[i]);
        if (a < INFINITY && a > amax) amax = a;
    }
    int ea = -126;
    if (amax > 0.0f) { frexpf(amax, &ea); ea -= 1; }   /* 2^ea <= amax < 2^(ea+1) */
    const int F = 124 - orc_bitlen(n) - ea;
    for (int64_t run = 0; run < n_init; run++) {
        if (init) {
            memcpy(c, init + run * k * d, sizeof(float) * (size_t)(k * d));
        } else {
            orc_draws g = {seed + (uint64_t)run, NULL, 0, 0};
            orc_kpp_f32(x, n, d, k, &g, c);
        }
        memset(lab, 0, sizeof(int64_t) * (size_t)n);
        int64_t n_iter = 0;
        double inertia = (double)FLT_MAX;
        for (int64_t it = 0; it < max_iter; it++) {
            float ms;
            if (wide_sums) {
                orc_assign_f32(x, n, d, c, k, lab, mind, nthreads);
                double s = 0.0;
                for (int64_t i = 0; i < n; i++) s += (double)mind[i];
                inertia = s;
                ms = orc_update_f32_wide(x, n, d, lab, c, k, nc, sums, flags, icounts, F);
            } else {
                inertia = (double)orc_assign_f32(x, n, d, c, k, lab, NULL, nthreads);
                ms = orc_update_f32(x, n, d, lab, c, k, nc, counts);
            }
            float *tmp = c; c = nc; nc = tmp;
            n_iter = it + 1;
            if (ms < tol) break;
        }
        memcpy(out_c + run * k * d, c, sizeof(float) * (size_t)(k * d));
        memcpy(out_labels + run * n, lab, sizeof(int64_t) * (size_t)n);
        out_inertia[run] = inertia;
        out_n_iter[run] = n_iter;
    }
    free(c); free(nc); free(counts); free(sums); free(flags); free(icounts); free(mind); free(lab);
    return ORC_OK;
}

/* recompute_centroids_into (kmeans.rs:358-401) for KMeans<f64> on f32 rows
 * widened exactly, from given labels, plus the inertia of those labels
 * against the old centres folded in row order (assign_serial,
 * kmeans.rs:312-323). The full-size parity checks of the mixed forms use it:
 * the sums run in row order per (cluster, feature) and the threads split the
 * features, so no rounding differs from the sequential loop. */
int orc_update_given_labels_f32x64(const float *x, int64_t n, int64_t d, const int64_t *labels,
                                   const double *old_c, int64_t k, double *new_c, double *inertia,
                                   int nthreads) {
    if (!x || !labels || !old_c || !new_c || !inertia) return ORC_ERR_NULL;
    for (int64_t i = 0; i < n; i++)
        if (labels[i] < 0 || labels[i] >= k) return ORC_ERR_INVALID_PARAMETER;
    double *counts = (double *)calloc((size_t)k, sizeof(double));
    double *mind = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    if (!counts || !mind) { free(counts); free(mind); return ORC_ERR_OOM; }
    memset(new_c, 0, sizeof(double) * (size_t)(k * d));
    for (int64_t i = 0; i < n; i++) counts[labels[i]] = counts[labels[i]] + 1.0;
    if (nthreads < 1) nthreads = 1;
    _Pragma("omp parallel for schedule(static) num_threads(nthreads)")
    for (int64_t j = 0; j < d; j++)
        for (int64_t i = 0; i < n; i++) {
            const int64_t l = labels[i];
            new_c[l * d + j] = new_c[l * d + j] + (double)x[i * d + j];
        }
    for (int64_t q = 0; q < k; q++) {
        if (counts[q] > 0.0) {
            for (int64_t j = 0; j < d; j++) new_c[q * d + j] = new_c[q * d + j] / counts[q];
        } else {
            memcpy(new_c + q * d, old_c + q * d, sizeof(double) * (size_t)d);
        }
    }
    _Pragma("omp parallel for schedule(static) num_threads(nthreads)")
    for (int64_t i = 0; i < n; i++) {
        const double *c = old_c + labels[i] * d;
        double acc = 0.0;
        for (int64_t j = 0; j < d; j++) {
            const double t = (double)x[i * d + j] - c[j];
            acc = acc + t * t;
        }
        mind[i] = acc;
    }
    double s = 0.0;
    for (int64_t i = 0; i < n; i++) s = s + mind[i];
    *inertia = s;
    free(counts);
    free(mind);
    return ORC_OK;
}

/* The first loop of recompute_centroids_into (kmeans.rs:370-375) for F = f64
 * over the m rows given, continuing the caller's sums and counts: one pass
 * split into consecutive row ranges adds in exactly the single loop's order.
 * The benchmark's reference arm times a full Lloyd iteration this way, a row
 * range per step. */
int orc_update_rows_f64(const double *x, int64_t m, int64_t d, const int64_t *labels, int64_t k, double *sums,
                        double *counts) {
    if (!x || !labels || !sums || !counts) return ORC_ERR_NULL;
    for (int64_t i = 0; i < m; i++) {
        const int64_t l = labels[i];
        if (l < 0 || l >= k) return ORC_ERR_INVALID_PARAMETER;
        counts[l] = counts[l] + 1.0;
        for (int64_t j = 0; j < d; j++) sums[l * d + j] = sums[l * d + j] + x[i * d + j];
    }
    return ORC_OK;
}

/* The rest of recompute_centroids_into (kmeans.rs:377-400): the means (an
 * empty cluster keeps its old centre) and sqrt of the largest squared shift. */
int orc_update_finish_f64(const double *sums, const double *counts, const double *old_c, int64_t k, int64_t d,
                          double *new_c, double *shift) {
    if (!sums || !counts || !old_c || !new_c || !shift) return ORC_ERR_NULL;
    for (int64_t q = 0; q < k; q++) {
        if (counts[q] > 0.0) {
            for (int64_t j = 0; j < d; j++) new_c[q * d + j] = sums[q * d + j] / counts[q];
        } else {
            memcpy(new_c + q * d, old_c + q * d, sizeof(double) * (size_t)d);
        }
    }
    double ms = 0.0;
    for (int64_t q = 0; q < k; q++) {
        const double s = orc_sqeuc_f64(new_c + q * d, old_c + q * d, d);
        if (s > ms) ms = s;
    }
    *shift = sqrt(ms);
    return ORC_OK;
}
