// fk_internal.cuh -- shared declarations of the KMeans Lloyd library.
//
// Layout in HBM (per context, grow-only buffers reused across calls):
//   x        n*d   TX   row-major (TX = float or double), copied once per call
//   centers  k*d   TC   current / next centres (double-buffered)
//   labels   n     int32
//   mind     n     TC   per-row minimum distance of the last assignment
//   members  n     int32  row indices grouped by cluster (stable, row order)
//   seg_hist k*S   int32  per-(cluster, segment) counts / offsets, S segments
//   scalars         one fk_dev_scalars block read back once per iteration
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <string>
#include <vector>

#include "../../include/ferrokmeans.h"

namespace fk {

// ----------------------------------------------------------------- errors --
void set_error(const char *fmt, ...);

struct Error {
    fk_status code;
};

#define FK_CUDA(call)                                                                   \
    do {                                                                                \
        cudaError_t _e = (call);                                                        \
        if (_e != cudaSuccess) {                                                        \
            ::fk::set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(_e),    \
                            __FILE__, __LINE__);                                        \
            throw ::fk::Error{_e == cudaErrorMemoryAllocation ? FK_ERR_OOM : FK_ERR_CUDA}; \
        }                                                                               \
    } while (0)

// Count of kernel launches issued by this library (diagnostics).
extern unsigned long long g_launch_count;
#define FK_LAUNCH_CHECK()                      \
    do {                                       \
        FK_CUDA(cudaGetLastError());           \
        __atomic_add_fetch(&::fk::g_launch_count, 1ULL, __ATOMIC_RELAXED); \
    } while (0)

[[noreturn]] inline void fail(fk_status code) { throw Error{code}; }

// ------------------------------------------------------- device scalars --
// Written by the reduction kernels, read back with one copy per iteration.
struct DevScalars {
    double inertia;                 // deterministic sum of the per-row minima
    unsigned long long shift_bits;  // max_c ||new-old||^2 as raw bits (>= 0)
    unsigned long long recheck_rows;
    unsigned long long full_rows;
    unsigned long long near_tie_rows;
    unsigned long long flag_count;  // number of rows queued for re-check
    unsigned long long full_count;  // number of rows queued for a full re-scan
    unsigned long long quad_count;  // second pass: rows decided among at most 32 candidates
    unsigned long long ex_count;    // second pass: rows re-scored against every centre
    unsigned long long f64_count;   // rows whose remaining candidates are scored in FP64
    unsigned long long error_word;  // nonzero: a bounded device wait gave up
    unsigned long long moved_rows;  // incremental update: rows whose label changed
    unsigned long long incremental; // 1: this iteration's update was incremental
    unsigned long long mask_count;  // FP8 second pass: rows left to its mask pass
};

// --------------------------------------------------- mixed precision --
// Bound ingredients of one assignment (floats rounded up; maxima via atomics).
struct MixedStats {
    float xn_max;  // max_i ||xh_i||           (set once per X)
    float amax;    // max |x_ij| over finite entries (set once per X)
    float tmax;    // max |x_ij - mu_j| over finite entries (set once per X)
    float nonfinite;  // 1 if some row of X holds a non-finite value or overflows ||x|| (set once per X)
    float cn_max;  // max_c ||c' ||            (per iteration from here on)
    float ec_max;  // max_c ||c' - ch||
    float ch_max;  // max_c ||ch||
    float h_max;   // max_c ||c'||^2 / 2
    float co_max;  // max_c ||c||  (uncentred, for the FP64 rounding term)
    float big;     // BIG of this iteration: 1.5 * 2^E, every score lies in [2^E, 2^(E+1))
    float cgrid;   // 3 * 2^(E+6): (T + cgrid) - cgrid rounds T to a multiple of 2^(E-16)
    float ulp;     // 2^(E-23), the unit in the last place of every score
    float tscale;  // FP8: the centres' power-of-two scale t (1 for BF16)
    float inv_t;   // 1 / tscale
};

// Best and second-best score of one row over one slice of the centres, and
// u3, an upper bound of every other score in the slice.
struct alignas(16) Top2 {
    float v1, v2, u3, pad;
    int i1, i2, pad1, pad2;
};

// The same record as the main pass writes it (16 bytes): both centre indices
// relative to the slice's first centre, 16 bits each (0xFFFF: none).
struct alignas(16) SliceTop2 {
    float v1, v2, u3;
    uint32_t ids;
};
__host__ __device__ inline int slice_index(uint32_t local, int base) {
    return local == 0xFFFFu ? -1 : base + (int)local;
}

// One row over one slice in the count pass: the largest score, and the
// centres scoring at least the row's threshold -- their number (low 16 bits
// of meta, saturating) and the first two nonzero 32-centre mask words w1, w2
// with their word indices within the slice (meta bits 16-23 and 24-31, 0xFF:
// none). The words use the mask pass's bit layout.
struct alignas(16) SliceCount {
    float vmax;
    uint32_t meta;
    uint32_t w1, w2;
};


// Launch plan of the tensor-core assignment (fk_tc.cu).
struct MixedPlan {
    int64_t n = -1;
    int d = -1, k = -1;
    int d_pad = 0;        // d rounded up to a multiple of 64 (one 128-byte swizzle atom)
    int k_pad = 0;        // parts * kp
    int parts = 1;        // centre slices, one per CTA group
    int kp = 0;           // centres per slice (multiple of 256)
    int nblocks = 0;      // kp / 256 accumulator blocks
    int64_t tiles = 0;    // ceil(n / 128)
    int ctas_per_part = 0;
    int grid = 0;
    int topk = 2;         // epilogue records: 2 (top-2 main pass), 3 (count pass) or 1 (candidate masks)
    int xst = 2;          // depth of the X tile ring (1 when two stages leave no room for 256 centres)
    int ep = 2;           // epilogue parts per TMEM lane quarter (4 x ep epilogue warps)
    int slots = 3;        // rotating tile-merge slots of the top-2 pass
    size_t smem = 0;
    const void *x = nullptr;
    double mu_norm = 0.0;
    const void *tm_x_ptr = nullptr, *tm_c_ptr = nullptr, *tm_aug_ptr = nullptr, *tm_xaug_ptr = nullptr;
    bool fp8 = false;
    alignas(64) unsigned char tm_xaug[128];
    alignas(64) unsigned char tm_x[128];
    alignas(64) unsigned char tm_c[128];
    alignas(64) unsigned char tm_aug[128];
    alignas(64) unsigned char tm_ones[128];
    void *ones = nullptr;  // 128 x 16 BF16 rows of [1,1,1,0,...] (device)
};

// ---------------------------------------------------------------- context --
enum BufSlot {
    BUF_X = 0, BUF_XC, BUF_C0, BUF_C1, BUF_CBEST, BUF_LABELS, BUF_LBEST, BUF_MIND,
    BUF_MEMBERS, BUF_SEGHIST, BUF_SCAN_TMP, BUF_COUNTS, BUF_PARTIAL, BUF_SCALARS,
    BUF_OUT, BUF_OUT2, BUF_KPP0, BUF_KPP1, BUF_KPP2, BUF_KPP3, BUF_DRAWS,
    BUF_XB, BUF_XNORM, BUF_CB, BUF_CAUX, BUF_TOP2, BUF_FLAGS, BUF_FULL, BUF_CF32, BUF_CF32C, BUF_FIXPART,
    BUF_XB2, BUF_EX, BUF_XAUG, BUF_ROWSCALE, BUF_ROWINFO2, BUF_STATS2, BUF_CB2, BUF_CAUG2,
    BUF_HALF2, BUF_INERTIA2, BUF_C2, BUF_XSTATE, BUF_XCOUNTS, BUF_MOVED, BUF_MOVED_ENT, BUF_MOVED_HIST, BUF_MOVED_TMP,
    BUF_CSPLIT, BUF_RINERT, BUF_F64ITEMS, BUF_INIT,
    BUF_MB_IDX, BUF_MB_XB, BUF_MB_LAB, BUF_MB_OLD, BUF_MB_COUNTS, BUF_MB_PARTV, BUF_MB_PARTI,
    BUF_BK_PERM, BUF_BK_LAB, BUF_BK_CEN, BUF_BK_DIST, BUF_BK_FLAGS, BUF_BK_SCRATCH, BUF_BK_CENTRES, BUF_BK_SEG,
    BUF_BK_FOLD, BUF_BK_LABELS, BUF_BK_XSEG, BUF_BK_CHAINS, BUF_BK_FRES, BUF_BK_FCNT, BUF_FOLD_SUM, BUF_FOLD_CNT,
    BUF_FOLD_MAP, BUF_MASKS, BUF_THRESH, BUF_FLOORS, BUF_SHIFT, BUF_THMAIN, BUF_TH2, BUF_CNT2, BUF_LIST3,
    BUF_SLOT3, BUF_TH3, BUF_XB3,
    BUF_BX, BUF_BFITS, BUF_BSTATE, BUF_BITEMS, BUF_BPART, BUF_BORDER, BUF_BCTR, BUF_BLAB, BUF_BMEM, BUF_BCEN, BUF_BND, BUF_BXOFF,
    BUF_PF_X32, BUF_PF_XERR, BUF_PF_C32, BUF_PF_CERR, BUF_PF_LIST, BUF_PF_CNT,
    BUF_COUNT
};

struct Ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    void *buf[BUF_COUNT] = {};
    size_t cap[BUF_COUNT] = {};
    DevScalars *host_scalars = nullptr;  // pinned
    int num_sms = 0;
    int cc_major = 0, cc_minor = 0;
    void *tmap_fn = nullptr;             // cuTensorMapEncodeTiled entry point
    bool initialized = false;
    struct PendingTimer {
        cudaEvent_t a, b;
        double *acc;
    };
    std::vector<PendingTimer> pending;  // phase timers read after the loop
    MixedPlan mixed;   // main pass
    MixedPlan mixed2;  // second pass (BF16 count pass) over the rows an FP8 main pass left open
    MixedPlan mixedm2; // its mask pass (BF16, the slicing of mixed2)
    MixedPlan mixedm;  // second pass (BF16, candidate masks) over the rows a BF16 main pass left open
    MixedPlan mixedc;  // count pass (main pass from the fourth iteration of a fit)
    // Captured steady-state fit iterations (fk_capi.cu), keyed by what the
    // iteration's launches depend on; a buffer (re)allocation bumps buf_gen,
    // which retires them all (their pointers would be stale).
    struct IterGraph {
        uint64_t key[10];
        cudaGraphExec_t exec;
        unsigned long long launches;  // kernel launches one replay stands for
        int state;                    // 0 not captured yet, 1 captured, 2 not capturable
        int tries;                    // failed captures so far
    };
    std::vector<IterGraph> iter_graphs;
    uint64_t buf_gen = 0, graph_gen = 0;
    int batch_variant[20] = {-1, -1, -1, -1, -1, -1, -1, -1, -1, -1,
                             -1, -1, -1, -1, -1, -1, -1, -1, -1, -1};  // autotuned tile shape per (d, k) bucket
    double *contract_acc = nullptr;  // when set: device time of the contraction kernel
    double *count_acc = nullptr;     // when set: device time of the count passes among those

    void *get(BufSlot s, size_t bytes);  // grow-only device buffer
    void bind();                         // make the device current
};

// Events owned by one call, destroyed on every way out of it (errors are
// thrown as Error and caught at the C boundary).
template <int N>
struct Events {
    cudaEvent_t e[N] = {};
    explicit Events(unsigned flags = cudaEventDefault) {
        for (auto &x : e) FK_CUDA(cudaEventCreateWithFlags(&x, flags));
    }
    ~Events() {
        for (auto x : e)
            if (x) cudaEventDestroy(x);
    }
    Events(const Events &) = delete;
    Events &operator=(const Events &) = delete;
    cudaEvent_t &operator[](int i) { return e[i]; }
};

// Phase timer: records a pair of events on the stream and leaves the
// reading to flush_timers(), so timing never adds a host synchronisation
// inside the Lloyd loop.
struct Timer {
    Ctx *ctx = nullptr;
    cudaEvent_t b = nullptr;
    double *acc = nullptr;
    cudaEvent_t a = nullptr;
    Timer(bool enable, Ctx &c, double *accum) {
        if (!enable || !accum) return;
        ctx = &c;
        acc = accum;
        FK_CUDA(cudaEventCreate(&a));
        FK_CUDA(cudaEventCreate(&b));
        FK_CUDA(cudaEventRecord(a, c.stream));
    }
    ~Timer() {
        if (!ctx) return;
        if (cudaEventRecord(b, ctx->stream) == cudaSuccess) {
            ctx->pending.push_back({a, b, acc});
        } else {
            cudaEventDestroy(a);
            cudaEventDestroy(b);
        }
    }
};

inline void flush_timers(Ctx &ctx) {
    for (auto &p : ctx.pending) {
        float ms = 0.f;
        if (cudaEventSynchronize(p.b) == cudaSuccess && cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess)
            *p.acc += ms;
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    ctx.pending.clear();
}

// ----------------------------------------------------------- kernel APIs --
// Direct-form assignment (kmeans.rs:295-352): labels + per-row minimum in TC.
// TX is the storage type of x, TC the arithmetic type (float or double).
template <typename TX, typename TC>
void launch_assign_direct(const TX *x, int64_t n, int d, const TC *c, int k, int32_t *labels,
                          TC *mind, cudaStream_t s);
// Transform (kmeans.rs:568-617): out[i*k+c] = sqrt(direct distance).
// The assignment with the centres split over `splits` CTA columns (for row
// counts too small to fill the GPU), then an ordered combine: the same labels
// and minima as launch_assign_direct. Scratch: splits x n of each.
// Upper bound, in f32 with upward rounding, of |d32 - D| + |D64 - D| where D
// is the exact real distance and D64 the oracle's FP64 direct form:
// ((d+4) 2^-23 d32 + 2 sqrt(d32) ec + 3 ec^2) * 1.01. 2 sqrt(d32) is bounded
// by d32 / s + s >= 2 sqrt(d32) (any s > 0; with s the power of two 2^(E/2),
// 2^E <= d32, it exceeds 2 sqrt(d32) by at most 25%): two directed-rounding
// operations instead of a correctly rounded square root.
__device__ __forceinline__ float bound32(float d32, float ec, int d) {
    const float dd = d32 > 0.f ? d32 : 0.f;
    const int h = ((int)((__float_as_uint(dd) >> 23) & 0xFFu) - 127) >> 1;  // floor(E / 2), -64..64
    const float sq2 = dd > 0.f ? __fadd_ru(__fmul_ru(dd, __int_as_float((127 - h) << 23)), __int_as_float((h + 127) << 23))
                               : 0.f;
    float e = __fmul_ru((float)(d + 4) * 1.1920929e-07f, dd);
    e = __fadd_ru(e, __fmul_ru(sq2, ec));
    e = __fadd_ru(e, __fmul_ru(3.0f, __fmul_ru(ec, ec)));
    return __fadd_ru(__fmul_ru(e, 1.01f), 1e-30f);
}

template <typename TC>
int assign_splits(int64_t n, int k, int num_sms);
template <typename TX, typename TC>
void launch_assign_direct_split(const TX *x, int64_t n, int d, const TC *c, int k, int32_t *labels, TC *mind,
                                int splits, TC *part_v, int32_t *part_i, cudaStream_t s);
template <typename T>
void launch_transform_direct(const T *x, int64_t n, int d, const T *c, int k, T *out,
                             cudaStream_t s);
// The plain f64 assignment (labels, and mind when set: the FP64 direct form to
// the label, F::MAX for a row with no distance below it) -- the outputs of
// launch_assign_direct<double, double> -- through an FP32 pass with rigorous
// bounds (fk_prefilter.cu): FP64 only for the rows it cannot decide and for
// each row's distance to its label. fresh_x: X changed since the last call
// (its f32 copy is rebuilt).
void launch_assign_f64_filtered(Ctx &ctx, const double *x, int64_t n, int d, const double *c, int k,
                                int32_t *labels, double *mind, bool fresh_x);
// f32 copies of f64 rows and an upper bound of the norm of each row's
// rounding error (the inputs of the FP32 bounds).
void launch_f32_copy(Ctx &ctx, const double *x, int64_t n, int d, float *x32, float *err);
// Deterministic fixed-order sum of v[0..n) in double into *out.
template <typename T>
void launch_sum_fixed(const T *v, int64_t n, double *partial, double *out, cudaStream_t s);
int64_t sum_fixed_partials(int64_t n);

// Stable counting sort of labels into members + per-cluster [start, end).
struct SortPlan {
    int64_t n = 0;
    int k = 0;
    int64_t seg_len = 0;
    int64_t nseg = 0;
    size_t scan_tmp_bytes = 0;
};
SortPlan make_sort_plan(int64_t n, int k);
void launch_sort_by_cluster(const SortPlan &p, const int32_t *labels, int32_t *seg_hist,
                            int32_t *scan_tmp, int32_t *members, cudaStream_t s);

// recompute_centroids_into (kmeans.rs:358-401): per-cluster row-order sums in
// TC, divide, empty -> keep old, then max shift into scalars->shift_bits.
// With inertia_part != nullptr the same pass also accumulates, per (cluster,
// feature), the compensated-f32 sum of (x_ij - c_j)^2 against the old centre.
template <typename TX, typename TC>
void launch_update_centroids(const SortPlan &p, const TX *x, int d, const int32_t *members,
                             const int32_t *seg_hist, const TC *old_c, TC *new_c,
                             DevScalars *scalars, cudaStream_t s, double *inertia_part = nullptr);

// Mixed precisions: exact 128-bit fixed-point cluster sums of an f32 X,
// rounded once to f64, divided by the counts; plus the inertia partials.
size_t update_exact_scratch_bytes(int k, int d);
// Exact 128-bit fixed-point sum of one (cluster, feature) (two's complement).
struct ExactState {
    uint64_t lo, hi;
};
// state / counts (nullable): also keep the exact sums and the cluster sizes,
// which launch_update_centroids_incremental then updates.
void launch_update_centroids_exact(const SortPlan &p, const float *x, int d, const int32_t *members,
                                   const int32_t *seg_hist, const double *old_c, double *new_c, DevScalars *scalars,
                                   const float *amax, double *inertia_part, void *scratch, cudaStream_t s,
                                   ExactState *state = nullptr, long long *counts = nullptr);
// The same new centres from the rows whose label changed since the
// assignment that state / counts describe (they are updated to this one).
// Needs incremental_shape_ok(x, d), a finite X and the two grids of the split
// (-90 <= exponent of max|x| <= 100).
bool incremental_shape_ok(const float *x, int d);
void launch_update_centroids_incremental(Ctx &ctx, const float *x, int64_t n, int d, int k,
                                         const int32_t *prev_labels, const int32_t *labels, const double *old_c,
                                         double *new_c, DevScalars *scalars, const float *amax, ExactState *state,
                                         long long *counts);
// sum_i ||x_i - c_{labels_i}||^2 into scalars->inertia (deterministic).
void launch_row_inertia(Ctx &ctx, const float *x, int64_t n, int d, const int32_t *labels, const double *c, int k,
                        DevScalars *scalars);

void launch_labels_to_u64(const int32_t *l, int64_t n, uint64_t *out, cudaStream_t s);

// MiniBatchKMeans (mini_batch_kmeans.rs): rows idx[0..m) of x into out
// (m x d), and update_centers_mini_batch (:410-447) for one batch -- the
// centres updated in place in batch order, old = the centres before it,
// counts = the running per-centre counts, shift_bits = max_c ||c - old||^2.
template <typename T>
void launch_gather_rows(const T *x, int d, const int32_t *idx, int64_t m, T *out, cudaStream_t s);
template <typename T>
void launch_minibatch_update(const T *xb, const int32_t *labels, int64_t m, int d, int k, T *centres, T *old,
                             long long *counts, unsigned long long *shift_bits, cudaStream_t s);

// BisectingKMeans (bisecting_kmeans.rs): the n_init 2-means runs of one
// split over a segment of the row permutation perm (m rows). Per run: two
// centres (cen, run-major 2 x d), uint8 labels (stride lab_stride), a
// changed flag; active selects the runs still iterating (NULL: every run).
constexpr int BK_MAX_D = 1024;  // 2 d (side, feature) chains per CTA
template <typename T>
void launch_bk_pick(const T *x, int d, const int32_t *perm, const int32_t *picks, int runs, T *cen, cudaStream_t s);
template <typename T>
void launch_bk_assign(const T *x, int d, const int32_t *perm, int64_t m, const T *cen, uint8_t *lab,
                      int64_t lab_stride, const int *active, int *changed, int runs, cudaStream_t s);
template <typename T>
void launch_bk_dist(const T *x, int d, const int32_t *perm, int64_t m, const T *cen, const uint8_t *lab,
                    int64_t lab_stride, T *dist, int64_t dist_stride, int runs, cudaStream_t s);
// Centres from the exact folds of chains (run * 2 + side) * d + feature.
template <typename T>
void launch_bk_centres(const T *sums, const long long *counts, int runs, int d, const int *active, bool whole,
                       int64_t m, T *cen, cudaStream_t s);
size_t bk_partition_scratch_ints(int64_t m);
void launch_bk_partition(int32_t *seg, const uint8_t *lab, int64_t m, int32_t *scratch, int64_t *m0, cudaStream_t s);
void launch_bk_labels(const int32_t *perm, const int64_t *seg, int nclusters, int64_t *labels, cudaStream_t s);
template <typename TS, typename TD>
void launch_convert(const TS *src, int64_t count, TD *dst, cudaStream_t s);

// k-means++ (kmeans.rs:169-253).
// One sequential left fold in F per chain, exactly as the loop
// `acc = acc + v` from zero in index order (fk_fold.cu): chain c folds
// base[i * stride] over i in [0, m) where mask is null or mask[i] == mval,
// and is skipped when active_slot >= 0 and active[active_slot] == 0. chains
// is device memory; result[c] receives the fold, count[c] the values folded.
struct FoldChain {
    const void *base;
    int64_t stride;
    const uint8_t *mask;
    int32_t mval;
    int32_t active_slot;
};
template <typename T>
void run_exact_folds(Ctx &ctx, const FoldChain *chains, int nchains, int64_t m, const int *active, T *result,
                     long long *count);

template <typename T>
void run_kmeanspp(Ctx &ctx, const T *x, int64_t n, int d, int k, const double *draws_dev,
                  int64_t n_draws, T *centers_out, int64_t *draws_used);

// Mixed-precision assignment (BF16 / FP8 tcgen05 approximate pass, FP32 and
// FP64 exact re-check) of X stored as f32. Results identical to the FP64
// direct form.
// With c_prev and labels_prev (the previous iteration's centres and labels,
// and this context's row floors from that iteration's pass), the main pass is
// the count pass.
template <typename TX>
void run_assign_mixed(Ctx &ctx, const TX *x, int64_t n, int d, const double *c, int k,
                      int precision, int32_t *labels, double *mind, DevScalars *scalars,
                      bool x_changed, const double *c_prev = nullptr, const int32_t *labels_prev = nullptr);
// Inertia of the mixed precisions: the per-(cluster, feature) partials of
// the update pass folded in f64 (relative error about 1e-7).
void launch_mixed_inertia(Ctx &ctx, const double *part, int64_t m, DevScalars *scalars);

// Tensor-core assignment (fk_tc.cu): plan, then one persistent launch that
// writes per (slice, row) a SliceTop2 (topk 2) or SliceCount (topk 3)
// record, or per row its candidate mask words (topk 1).
void plan_tc(Ctx &ctx, MixedPlan &mp, int64_t n, int d, int k, bool fp8, int topk, int kp_fixed = 0);
// Dense BF16 (out[0]) and E4M3 (out[1]) flop/s of a tensor-core MMA loop (fk_tc.cu).
void measure_tc_peaks(Ctx &ctx, double *out);
// dump (tests only, nullable): raw accumulators of CTA 0's first tile.
// n_dev (nullable): the row count is read there at launch (mp.n is then the
// capacity). FP8 (mp.fp8): xaug is the per-row augmentation tensor (n x 16
// BF16) and rowscale the per-row power of two mapping scores to the row's
// accumulator units.
// Launch shape only (host arithmetic, no device work); plan_tc adds the
// device-side constants.
void plan_shape(MixedPlan &mp, int64_t n, int d, int k, bool fp8, int topk, int sms, int kp_fixed = 0);
void launch_tc_assign(Ctx &ctx, MixedPlan &mp, const void *xb, const void *cb, const void *caug, SliceTop2 *out,
                      DevScalars *sc, const MixedStats *stats, float *dump = nullptr,
                      const unsigned long long *n_dev = nullptr, const void *xaug = nullptr,
                      const float *rowscale = nullptr, uint32_t *masks = nullptr, const float *thresh = nullptr,
                      SliceCount *outc = nullptr);

// Batched KMeans<f32> fits (fk_batched.cu).
fk_status batched_fit_impl(Ctx &ctx, fk_batch_problem *problems, int64_t n_problems, int reduction,
                           fk_batch_report *report);
int kpp_trials_host(int64_t k);

void measure_peaks(Ctx &ctx, double *out);
void debug_tc_probe(Ctx &ctx, const float *x, int64_t n, int d, const double *c, int k, int precision,
                    float *dump_out, void *xq_out, void *cq_out, uint16_t *aug_out, uint16_t *xaug_out,
                    Top2 *top_out, int *plan_out);

}  // namespace fk
