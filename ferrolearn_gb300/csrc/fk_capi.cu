// fk_capi.cu -- the extern "C" boundary and the host side of the Lloyd loop.
//
// The host side restates Fit::fit (kmeans.rs:417-512) on the GPU: validation in
// the reference's order, n_init runs seeded base+run, the Lloyd loop whose
// labels/inertia come from the assignment against the pre-update centres
// while the returned centres are the post-update ones, convergence when
// sqrt(max shift^2) < tol (absolute), and the strictly-lowest inertia run
// kept (earliest wins ties). All per-iteration work stays on the device; the
// only host traffic per iteration is one 64-byte scalar block read back.
#include <cmath>
#include <cstdarg>
#include <algorithm>
#include <cstring>
#include <memory>
#include <unordered_map>
#include <vector>

#include "fk_internal.cuh"

namespace fk {

static thread_local std::string g_last_error;
unsigned long long g_launch_count = 0;

void set_error(const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
}

// CUDA is first touched here, not at context creation, so argument errors
// are reported the same way on machines without a GPU.
void Ctx::bind() {
    FK_CUDA(cudaSetDevice(device));
    if (initialized) return;
    cudaDeviceProp prop;
    FK_CUDA(cudaGetDeviceProperties(&prop, device));
    num_sms = prop.multiProcessorCount;
    cc_major = prop.major;
    cc_minor = prop.minor;
    if (!stream) {
        FK_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        own_stream = true;
    }
    FK_CUDA(cudaMallocHost((void **)&host_scalars, 3 * sizeof(DevScalars)));  // [0]: reads; [1], [2]: pipelined fits
    initialized = true;
}

void *Ctx::get(BufSlot s, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (cap[s] >= bytes) return buf[s];
    if (buf[s]) {
        FK_CUDA(cudaStreamSynchronize(stream));
        FK_CUDA(cudaFree(buf[s]));
        buf[s] = nullptr;
        cap[s] = 0;
    }
    size_t want = bytes + bytes / 8;  // headroom for slightly larger calls
    void *p = nullptr;
    buf_gen++;  // captured iterations that used the old buffer are retired
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        e = cudaMalloc(&p, bytes);
        want = bytes;
    }
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        set_error("cudaMalloc of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
        fail(FK_ERR_OOM);
    }
    buf[s] = p;
    cap[s] = want;
    return p;
}

// n_trials of kmeans.rs:198 (2 + floor(ln k), at least 1).
int kpp_trials_host(int64_t k) {
    long long t = 2 + (long long)std::floor(std::log((double)k));
    return t < 1 ? 1 : (int)t;
}

// First iteration whose main pass may be the count pass (it needs the row
// floors of a previous pass, and the centres' shifts to have settled).
#ifndef FK_COUNT_FROM
#define FK_COUNT_FROM 3
#endif

namespace {

// True for device (or managed) memory the call can use in place, false for
// host memory. Device memory of another GPU than the context's is refused
// with FK_ERR_INVALID_PARAMETER: without peer access a kernel reading it
// would fault instead of returning an error.
bool is_device_ptr(const void *p) {
    if (!p) return false;
    cudaPointerAttributes a;
    cudaError_t e = cudaPointerGetAttributes(&a, p);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeDevice) {
        int cur = 0;
        FK_CUDA(cudaGetDevice(&cur));
        if (a.device != cur) {
            set_error("buffer %p is device memory of GPU %d, but the call runs on GPU %d", p, a.device, cur);
            fail(FK_ERR_INVALID_PARAMETER);
        }
        return true;
    }
    return a.type == cudaMemoryTypeManaged;
}

template <typename T>
const T *stage_in(Ctx &ctx, BufSlot slot, const T *p, size_t count) {
    if (is_device_ptr(p)) return p;
    T *d = (T *)ctx.get(slot, sizeof(T) * count);
    if (count) FK_CUDA(cudaMemcpyAsync(d, p, sizeof(T) * count, cudaMemcpyHostToDevice, ctx.stream));
    return d;
}

template <typename T>
void copy_out(Ctx &ctx, T *dst, const T *dev_src, size_t count) {
    if (!count || !dst) return;
    FK_CUDA(cudaMemcpyAsync(dst, dev_src, sizeof(T) * count, cudaMemcpyDefault, ctx.stream));
}

template <typename T> struct FMax;
template <> struct FMax<double> { static double v() { return 1.7976931348623157e308; } };
template <> struct FMax<float> { static float v() { return 3.40282347e38f; } };

template <typename TC>
TC shift_from_bits(unsigned long long bits);
template <>
double shift_from_bits<double>(unsigned long long bits) {
    double v;
    memcpy(&v, &bits, sizeof v);
    return std::sqrt(v);
}
template <>
float shift_from_bits<float>(unsigned long long bits) {
    uint32_t b = (uint32_t)bits;
    float v;
    memcpy(&v, &b, sizeof v);
    return std::sqrt(v);
}

uint64_t splitmix64(uint64_t *s) {
    uint64_t z = (*s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

void host_draws(uint64_t seed, int64_t count, double *out) {
    uint64_t st = seed;
    for (int64_t i = 0; i < count; i++) out[i] = (double)(splitmix64(&st) >> 11) * (1.0 / 9007199254740992.0);
}


// Plain: every entry point. BF16 and FP8: f64 semantics on X stored as f32
// (the f32x64 entry points), the form whose rows the tensor-core operands,
// the exact integer centroid sums and the re-check cascade are built for.
template <typename TX, typename TC>
bool precision_ok(int prec) {
    constexpr bool mixed_ok = std::is_same<TC, double>::value && std::is_same<TX, float>::value;
    if (prec == FK_PRECISION_PLAIN) return true;
    if (prec == FK_PRECISION_MIXED_BF16 || prec == FK_PRECISION_MIXED_FP8) return mixed_ok;
    return false;
}

void precision_error(int prec) {
    if (prec == FK_PRECISION_MIXED_BF16 || prec == FK_PRECISION_MIXED_FP8)
        set_error("precision %d (tensor-core form) reads X stored as f32 with f64 semantics: use the f32x64 "
                  "entry points", prec);
    else
        set_error("precision %d is not available for this entry point", prec);
}

// The ranges every entry point accepts: rows index int32 labels, and the
// kernels index features and clusters with 32-bit integers. Checked before
// CUDA is touched, like the reference's own argument errors.
fk_status check_shape(int64_t n, int64_t d, int64_t k) {
    if (d < 0) {
        set_error("Invalid parameter `d`: negative");
        return FK_ERR_INVALID_PARAMETER;
    }
    if (k > (1 << 20) || n > INT32_MAX || d > (1 << 16)) {
        set_error("shape n=%lld d=%lld k=%lld exceeds the supported range", (long long)n, (long long)d, (long long)k);
        return FK_ERR_UNSUPPORTED;
    }
    return FK_OK;
}

// ------------------------------------------------------------ one step --
// Update modes of the mixed path with f32 X: the full exact pass (optionally
// keeping its exact sums), or the incremental one from the rows whose label
// changed since the previous assignment (no inertia: the fit computes it
// once, for the assignment it keeps).
enum UpdateMode { UPDATE_FULL = 0, UPDATE_FULL_STATE = 1, UPDATE_INCREMENTAL = 2 };

// One fit iteration through a CUDA graph: the first time a key is seen the
// body is captured (relaxed mode; nothing runs while capturing) and launched
// as a graph, and every later time the graph is replayed -- one launch for
// the iteration's twenty-odd kernels, memsets and copies. A capture that
// fails (a first use that allocates a buffer or plans a pass, which
// synchronises) runs the body as usual and is tried once more at the key's
// next occurrence, then given up.
template <typename Body>
void run_graphed(Ctx &ctx, const uint64_t (&key)[10], Body &&body) {
    if (ctx.graph_gen != ctx.buf_gen || ctx.iter_graphs.size() > 64) {
        for (auto &g : ctx.iter_graphs)
            if (g.exec) cudaGraphExecDestroy(g.exec);
        ctx.iter_graphs.clear();
        ctx.graph_gen = ctx.buf_gen;
    }
    Ctx::IterGraph *e = nullptr;
    for (auto &g : ctx.iter_graphs)
        if (memcmp(g.key, key, sizeof(g.key)) == 0) e = &g;
    if (!e) {
        Ctx::IterGraph g{};
        memcpy(g.key, key, sizeof(g.key));
        g.exec = nullptr;
        g.launches = 0;
        g.state = 0;
        g.tries = 0;
        ctx.iter_graphs.push_back(g);
        e = &ctx.iter_graphs.back();
    }
    if (e->state == 1) {
        FK_CUDA(cudaGraphLaunch(e->exec, ctx.stream));
        __atomic_add_fetch(&g_launch_count, e->launches, __ATOMIC_RELAXED);
        return;
    }
    if (e->state == 2) {
        body();
        return;
    }
    const uint64_t gen0 = ctx.buf_gen;
    const unsigned long long l0 = __atomic_load_n(&g_launch_count, __ATOMIC_RELAXED);
    FK_CUDA(cudaStreamBeginCapture(ctx.stream, cudaStreamCaptureModeRelaxed));
    bool ok = true;
    try {
        body();
    } catch (const Error &) {
        ok = false;
    }
    cudaGraph_t graph = nullptr;
    cudaError_t err = cudaStreamEndCapture(ctx.stream, &graph);
    cudaGraphExec_t exec = nullptr;
    if (err == cudaSuccess && graph && ok && ctx.buf_gen == gen0) err = cudaGraphInstantiate(&exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    // the entry may have moved if body() grew the cache: find it again
    for (auto &g : ctx.iter_graphs)
        if (memcmp(g.key, key, sizeof(g.key)) == 0) e = &g;
    if (err != cudaSuccess || !exec || !ok || ctx.buf_gen != gen0) {
        (void)cudaGetLastError();
        if (exec) cudaGraphExecDestroy(exec);
        g_last_error.clear();
        __atomic_store_n(&g_launch_count, l0, __ATOMIC_RELAXED);
        e->state = ++e->tries >= 2 ? 2 : 0;
        body();
        return;
    }
    e->exec = exec;
    e->launches = __atomic_load_n(&g_launch_count, __ATOMIC_RELAXED) - l0;
    e->state = 1;
    FK_CUDA(cudaGraphLaunch(exec, ctx.stream));
}

// Assignment against c (labels, inertia into scalars), then the update into
// nc (+ shift bits). Mixed precisions fold the inertia into the update pass.
template <typename TX, typename TC>
void lloyd_iteration(Ctx &ctx, const TX *x, int64_t n, int d, const TC *c, int k, int prec, TC *nc,
                     int32_t *labels, DevScalars *sc, const SortPlan &plan, bool x_changed, fk_fit_report *rep,
                     bool timing, int mode = UPDATE_FULL, const int32_t *prev_labels = nullptr,
                     const TC *prev_c = nullptr) {
    cudaStream_t s = ctx.stream;
    int32_t *members = (int32_t *)ctx.get(BUF_MEMBERS, sizeof(int32_t) * (size_t)n);
    int32_t *seg = (int32_t *)ctx.get(BUF_SEGHIST, sizeof(int32_t) * (size_t)plan.k * plan.nseg);
    int32_t *tmp = (int32_t *)ctx.get(BUF_SCAN_TMP, plan.scan_tmp_bytes);
    // the contraction's timer writes into this call's report: set only for
    // the assignment below (a pointer left behind would outlive the report)
    ctx.contract_acc = (timing && rep) ? &rep->ms_contract : nullptr;
    ctx.count_acc = (timing && rep) ? &rep->ms_count_pass : nullptr;
    {
        Timer t(timing, ctx, rep ? &rep->ms_assign : nullptr);
        if (prec == FK_PRECISION_PLAIN) {
            TC *mind = (TC *)ctx.get(BUF_MIND, sizeof(TC) * (size_t)n);
            double *part = (double *)ctx.get(BUF_PARTIAL, sizeof(double) * (size_t)sum_fixed_partials(n));
            if constexpr (std::is_same<TX, double>::value && std::is_same<TC, double>::value)
                launch_assign_f64_filtered(ctx, x, n, d, c, k, labels, mind, x_changed);
            else
                launch_assign_direct<TX, TC>(x, n, d, c, k, labels, mind, s);
            launch_sum_fixed<TC>(mind, n, part, &sc->inertia, s);
        } else {
            if constexpr (std::is_same<TX, float>::value && std::is_same<TC, double>::value) {
                run_assign_mixed(ctx, x, n, d, c, k, prec, labels, nullptr, sc, x_changed, prev_c,
                                 prev_c ? prev_labels : nullptr);
            }
        }
    }
    ctx.contract_acc = nullptr;
    ctx.count_acc = nullptr;
    {
        Timer t(timing, ctx, rep ? &rep->ms_update : nullptr);
        if constexpr (std::is_same<TX, float>::value && std::is_same<TC, double>::value) {
            if (mode != UPDATE_FULL) {
                const MixedStats *st = (const MixedStats *)ctx.get(BUF_CF32, sizeof(MixedStats));
                ExactState *state = (ExactState *)ctx.get(BUF_XSTATE, sizeof(ExactState) * (size_t)k * d);
                long long *counts = (long long *)ctx.get(BUF_XCOUNTS, sizeof(long long) * (size_t)k);
                if (mode == UPDATE_INCREMENTAL) {
                    launch_update_centroids_incremental(ctx, x, n, d, k, prev_labels, labels, c, nc, sc, &st->amax,
                                                        state, counts);
                } else {
                    launch_sort_by_cluster(plan, labels, seg, tmp, members, s);
                    double *part = (double *)ctx.get(BUF_OUT2, sizeof(double) * (size_t)plan.k * d + 64);
                    void *scratch = ctx.get(BUF_FIXPART, update_exact_scratch_bytes(plan.k, d));
                    launch_update_centroids_exact(plan, x, d, members, seg, c, nc, sc, &st->amax, part, scratch, s,
                                                  state, counts);
                    launch_mixed_inertia(ctx, part, (int64_t)plan.k * d, sc);
                }
                return;
            }
        }
        launch_sort_by_cluster(plan, labels, seg, tmp, members, s);
        if constexpr (std::is_same<TX, float>::value && std::is_same<TC, double>::value) {
            if (prec != FK_PRECISION_PLAIN) {
                double *part = (double *)ctx.get(BUF_OUT2, sizeof(double) * (size_t)plan.k * d + 64);
                const MixedStats *st = (const MixedStats *)ctx.get(BUF_CF32, sizeof(MixedStats));
                void *scratch = ctx.get(BUF_FIXPART, update_exact_scratch_bytes(plan.k, d));
                launch_update_centroids_exact(plan, x, d, members, seg, c, nc, sc, &st->amax, part, scratch, s);
                launch_mixed_inertia(ctx, part, (int64_t)plan.k * d, sc);
                return;
            }
        }
        launch_update_centroids<TX, TC>(plan, x, d, members, seg, c, nc, sc, s);
    }
}

void read_scalars(Ctx &ctx, DevScalars *dev) {
    FK_CUDA(cudaMemcpyAsync(ctx.host_scalars, dev, sizeof(DevScalars), cudaMemcpyDeviceToHost, ctx.stream));
    FK_CUDA(cudaStreamSynchronize(ctx.stream));
    if (ctx.host_scalars->error_word) {
        set_error("a bounded device wait gave up (code %llu)", ctx.host_scalars->error_word);
        fail(FK_ERR_TIMEOUT);
    }
}

void accumulate_report(fk_fit_report *rep, const DevScalars &h, int64_t n) {
    if (!rep) return;
    rep->rows_assigned += n;
    rep->rows_rechecked += (int64_t)(h.flag_count + h.full_count);
    rep->rows_full_rescan += (int64_t)h.full_count;
    rep->rows_fp64 += (int64_t)h.recheck_rows;
    rep->rows_second_pass += (int64_t)h.full_count;
    rep->rows_few += (int64_t)h.quad_count;
    rep->rows_exhaustive += (int64_t)h.ex_count;
    rep->near_tie_rows += (int64_t)h.near_tie_rows;
    rep->rows_moved += (int64_t)h.moved_rows;
    rep->updates_incremental += (int64_t)h.incremental;
}

// ------------------------------------------------------------------ fit --
template <typename TX, typename TC>
fk_status fit_impl(fk_ctx *ctxp, const TX *x_in, int64_t n, int64_t d, const fk_kmeans_params *p,
                   const TC *init_in, TC *centers_out, uint64_t *labels_out, TC *inertia_out, int64_t *n_iter_out,
                   fk_fit_report *rep) {
    Ctx &ctx = *reinterpret_cast<Ctx *>(ctxp);
    const int64_t k = p->n_clusters;
    // Validation order of kmeans.rs:421-449.
    if (k <= 0) {
        set_error("Invalid parameter `n_clusters`: must be at least 1");
        return FK_ERR_INVALID_PARAMETER;
    }
    if (n <= 0) {
        set_error("Insufficient samples: need at least %lld, got 0 (KMeans requires at least n_clusters samples)",
                  (long long)k);
        return FK_ERR_INSUFFICIENT_SAMPLES;
    }
    if (n < k) {
        set_error("Insufficient samples: need at least %lld, got %lld (KMeans requires at least n_clusters samples)",
                  (long long)k, (long long)n);
        return FK_ERR_INSUFFICIENT_SAMPLES;
    }
    if (p->n_init <= 0) {
        set_error("Invalid parameter `n_init`: must be at least 1");
        return FK_ERR_INVALID_PARAMETER;
    }
    if (p->max_iter < 0) {
        set_error("Invalid parameter `max_iter`: negative");
        return FK_ERR_INVALID_PARAMETER;
    }
    if (d < 0) {
        set_error("Invalid parameter `d`: negative");
        return FK_ERR_INVALID_PARAMETER;
    }
    if (!x_in || !centers_out || !labels_out || !inertia_out || !n_iter_out) {
        set_error("required pointer is NULL");
        return FK_ERR_NULL_POINTER;
    }
    if (!precision_ok<TX, TC>(p->precision)) {
        precision_error(p->precision);
        return FK_ERR_UNSUPPORTED;
    }
    if (!init_in && p->draws && p->n_draws < 0) {
        set_error("Invalid parameter `n_draws`: negative");
        return FK_ERR_INVALID_PARAMETER;
    }
    if (fk_status st = check_shape(n, d, k)) return st;
    ctx.bind();
    if (rep) {
        memset(rep, 0, sizeof(*rep));
        rep->precision_used = p->precision;
    }
    const bool timing = p->collect_timing != 0 && rep != nullptr;
    cudaStream_t s = ctx.stream;
    std::unique_ptr<Events<2>> tev;  // whole-call timing: [0] begin, [1] end
    if (timing) {
        tev.reset(new Events<2>());
        FK_CUDA(cudaEventRecord((*tev)[0], s));
    }
    const size_t kd = (size_t)k * d;
    const TX *x = stage_in<TX>(ctx, BUF_X, x_in, (size_t)n * d);
    // Three rotating centre buffers: iteration it reads cb3[it % 3] and writes
    // cb3[(it + 1) % 3], so neither the kept iteration's input nor its output
    // is overwritten by the successor queued before the convergence test.
    TC *cb3[3] = {(TC *)ctx.get(BUF_C0, sizeof(TC) * kd), (TC *)ctx.get(BUF_C1, sizeof(TC) * kd),
                  (TC *)ctx.get(BUF_C2, sizeof(TC) * kd)};
    TC *c = cb3[0];
    TC *cbest = (TC *)ctx.get(BUF_CBEST, sizeof(TC) * kd);
    // labels alternate between iterations: the next iteration is queued
    // before the previous one's convergence test has been read back
    int32_t *labels2 = (int32_t *)ctx.get(BUF_LABELS, sizeof(int32_t) * 2 * (size_t)n);
    int32_t *lbest = (int32_t *)ctx.get(BUF_LBEST, sizeof(int32_t) * (size_t)n);
    DevScalars *sc = (DevScalars *)ctx.get(BUF_SCALARS, sizeof(DevScalars));
    FK_CUDA(cudaMemsetAsync(labels2, 0, sizeof(int32_t) * 2 * (size_t)n, s));
    SortPlan plan = make_sort_plan(n, (int)k);
    Events<2> iter_done(cudaEventDisableTiming);

    // a slot of its own: the runs after the first read it while the mixed
    // updates use their own scratch (which may grow and move)
    const TC *init = init_in ? stage_in<TC>(ctx, BUF_INIT, init_in, kd * (size_t)p->n_init) : nullptr;
    const double *draws_dev = nullptr;
    int64_t n_draws = 0;
    if (!init) {
        // k-means++ draws: caller's flat stream, or splitmix64 per run.
        n_draws = p->draws ? p->n_draws : 1 + (k - 1) * kpp_trials_host(k);
        if (p->draws) draws_dev = stage_in<double>(ctx, BUF_DRAWS, p->draws, (size_t)n_draws);
    }
    int64_t draws_pos = 0;
    std::vector<double> hdraws;

    bool have = false;
    TC best_inertia = FMax<TC>::v();
    int64_t best_iter = 0;
    bool x_changed = true;
    // Mixed path on f32 X: after a run's first (full) update, the exact sums
    // are updated from the rows whose label changed. Decided once the first
    // preparation has shown X finite and inside the split's exponent range.
    bool inc_candidate = false, incremental = false;
    if constexpr (std::is_same<TX, float>::value && std::is_same<TC, double>::value)
        inc_candidate = p->precision != FK_PRECISION_PLAIN && incremental_shape_ok((const float *)x, (int)d);
    for (int64_t run = 0; run < p->n_init; run++) {
        if (init) {
            FK_CUDA(cudaMemcpyAsync(cb3[0], init + (size_t)run * kd, sizeof(TC) * kd, cudaMemcpyDeviceToDevice, s));
        } else {
            Timer t(timing, ctx, rep ? &rep->ms_init : nullptr);
            const double *dr;
            int64_t ndr;
            if (p->draws) {
                if (draws_pos >= n_draws) {
                    set_error("injected draw stream exhausted before run %lld", (long long)run);
                    fail(FK_ERR_INVALID_PARAMETER);
                }
                dr = draws_dev + draws_pos;
                ndr = n_draws - draws_pos;
            } else {
                uint64_t seed = (p->has_random_state ? p->random_state : 0) + (uint64_t)run;
                hdraws.resize((size_t)n_draws);
                host_draws(seed, n_draws, hdraws.data());
                double *dd = (double *)ctx.get(BUF_DRAWS, sizeof(double) * (size_t)n_draws);
                FK_CUDA(cudaMemcpyAsync(dd, hdraws.data(), sizeof(double) * (size_t)n_draws,
                                        cudaMemcpyHostToDevice, s));
                FK_CUDA(cudaStreamSynchronize(s));  // hdraws is reused next run
                dr = dd;
                ndr = n_draws;
            }
            int64_t used = 0;
            if constexpr (std::is_same<TX, TC>::value) {
                run_kmeanspp<TC>(ctx, x, n, (int)d, (int)k, dr, ndr, cb3[0], &used);
            } else {
                // k-means++ on the exactly widened matrix.
                TC *xw = (TC *)ctx.get(BUF_XC, sizeof(TC) * (size_t)n * d);
                launch_convert<TX, TC>(x, (int64_t)n * d, xw, s);
                run_kmeanspp<TC>(ctx, xw, n, (int)d, (int)k, dr, ndr, cb3[0], &used);
            }
            if (p->draws) draws_pos += used;
        }
        int64_t n_iter = 0;
        TC inertia = FMax<TC>::v();
        // Iteration it reads cb3[it % 3] and writes cb3[(it + 1) % 3] and
        // labels2[it & 1]; its scalars are copied to pinned host memory right
        // after it, and read once the next iteration has been queued, so the
        // GPU never waits for the host. A converged iteration's successor is
        // discarded (it touched neither the converged centres, nor their
        // input, nor the labels).
        // Mixed forms on f32 X: from the fourth iteration on, the main pass may be
        // the count pass (thresholds carried from the previous iteration). It
        // runs while the last iteration whose statistics are in (they are
        // read one iteration late) re-checked at most a quarter of the rows;
        // a count iteration that sent more than a tenth of the rows to the
        // second pass, or 0.2% to the exhaustive re-score, holds it off for
        // the next two iterations (the centres still move too much for the
        // carried bound).
        bool count_ok = false, calm = false;
        if constexpr (std::is_same<TX, float>::value && std::is_same<TC, double>::value)
            count_ok = p->precision == FK_PRECISION_MIXED_BF16 || p->precision == FK_PRECISION_MIXED_FP8;
        bool was_count[2] = {false, false};
        int64_t count_from = FK_COUNT_FROM;
        auto finish = [&](int64_t r) {
            FK_CUDA(cudaEventSynchronize(iter_done[r & 1]));
            const DevScalars &h = ctx.host_scalars[1 + (r & 1)];
            if (h.error_word) {
                set_error("a bounded device wait gave up (code %llu)", h.error_word);
                fail(FK_ERR_TIMEOUT);
            }
            calm = (int64_t)(h.flag_count + h.full_count) <= n / 4;
            if (was_count[r & 1] && ((int64_t)h.full_count > n / 10 || (int64_t)h.ex_count > n / 500))
                count_from = std::max(count_from, r + 3);
            accumulate_report(rep, h, n);
            inertia = (TC)h.inertia;
            n_iter = r + 1;
            return shift_from_bits<TC>(h.shift_bits) < (TC)p->tol;
        };
        bool stop = false;
        int64_t launched = 0;
        for (int64_t it = 0; it < p->max_iter && !stop; it++) {
            const int par = (int)(it & 1);
            // the first two iterations move many rows (a third of them is
            // common in the second): the full pass is cheaper there
            const int mode = !inc_candidate ? UPDATE_FULL
                             : (it < 2 || !incremental) ? UPDATE_FULL_STATE
                                                        : UPDATE_INCREMENTAL;
            const bool count = count_ok && calm && it >= count_from;
            was_count[par] = count;
            if (count && rep) rep->count_iterations++;
            // iteration it - 1 read cb3[(it + 2) % 3]; it is not overwritten before iteration it + 1
            auto iteration = [&] {
                lloyd_iteration<TX, TC>(ctx, x, n, (int)d, cb3[it % 3], (int)k, p->precision, cb3[(it + 1) % 3],
                                        labels2 + (size_t)par * n, sc, plan, x_changed, rep, timing, mode,
                                        labels2 + (size_t)(par ^ 1) * n, count ? cb3[(it + 2) % 3] : nullptr);
            };
            if (!timing && !x_changed && it >= 2) {
                // steady state: the memset, the iteration and the scalars' copy as one graph
                // (phase timers record events, so timed fits run without graphs)
                const uint64_t key[10] = {(uint64_t)(uintptr_t)x, (uint64_t)n, (uint64_t)d, (uint64_t)k,
                                          (uint64_t)p->precision, (uint64_t)(it % 6), (uint64_t)mode,
                                          (uint64_t)count, (uint64_t)(uintptr_t)sc, sizeof(TX) * 16 + sizeof(TC)};
                run_graphed(ctx, key, [&] {
                    FK_CUDA(cudaMemsetAsync(sc, 0, sizeof(DevScalars), s));
                    iteration();
                    FK_CUDA(cudaMemcpyAsync(&ctx.host_scalars[1 + par], sc, sizeof(DevScalars),
                                            cudaMemcpyDeviceToHost, s));
                });
                FK_CUDA(cudaEventRecord(iter_done[par], s));
                launched = it + 1;
                if (it > 0) stop = finish(it - 1);
                continue;
            }
            FK_CUDA(cudaMemsetAsync(sc, 0, sizeof(DevScalars), s));
            iteration();
            if (x_changed && inc_candidate) {
                // once per fit: X finite and the split's grids valid?
                MixedStats hs;
                FK_CUDA(cudaMemcpyAsync(&hs, ctx.get(BUF_CF32, sizeof(MixedStats)), sizeof(MixedStats),
                                        cudaMemcpyDeviceToHost, s));
                FK_CUDA(cudaStreamSynchronize(s));
                const int ea = hs.amax > 0.f ? std::ilogb(hs.amax) : -126;
                incremental = hs.nonfinite == 0.f && ea >= -90 && ea <= 100;
            }
            x_changed = false;
            FK_CUDA(cudaMemcpyAsync(&ctx.host_scalars[1 + par], sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, s));
            FK_CUDA(cudaEventRecord(iter_done[par], s));
            launched = it + 1;
            if (it > 0) stop = finish(it - 1);
        }
        if (!stop && launched > 0) finish(launched - 1);
        // the result of iteration n_iter - 1: centres in cb3[n_iter % 3]
        c = cb3[n_iter % 3];
        int32_t *labels = labels2 + (size_t)((n_iter > 0 ? n_iter - 1 : 0) & 1) * n;
        if (incremental && n_iter > 0) {
            // the incremental updates skip the per-iteration inertia: that of
            // the kept assignment, against its centres cb3[(n_iter - 1) % 3]
            if constexpr (std::is_same<TX, float>::value && std::is_same<TC, double>::value) {
                launch_row_inertia(ctx, x, n, (int)d, labels, cb3[(n_iter - 1) % 3], (int)k, sc);
                read_scalars(ctx, sc);
                inertia = (TC)ctx.host_scalars->inertia;
            }
        }
        if (rep) rep->iterations_total += n_iter;
        if (!have || inertia < best_inertia) {
            have = true;
            best_inertia = inertia;
            best_iter = n_iter;
            if (rep) rep->best_run = run;
            FK_CUDA(cudaMemcpyAsync(cbest, c, sizeof(TC) * kd, cudaMemcpyDeviceToDevice, s));
            FK_CUDA(cudaMemcpyAsync(lbest, labels, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToDevice, s));
        }
    }
    copy_out<TC>(ctx, centers_out, cbest, kd);
    if (is_device_ptr(labels_out)) {
        launch_labels_to_u64(lbest, n, labels_out, s);
    } else {
        uint64_t *l64 = (uint64_t *)ctx.get(BUF_OUT, sizeof(uint64_t) * (size_t)n);
        launch_labels_to_u64(lbest, n, l64, s);
        copy_out<uint64_t>(ctx, labels_out, l64, (size_t)n);
    }
    if (timing) {
        FK_CUDA(cudaEventRecord((*tev)[1], s));
        FK_CUDA(cudaEventSynchronize((*tev)[1]));
        float ms = 0.f;
        FK_CUDA(cudaEventElapsedTime(&ms, (*tev)[0], (*tev)[1]));
        rep->ms_total = ms;
    }
    FK_CUDA(cudaStreamSynchronize(s));
    flush_timers(ctx);
    *inertia_out = best_inertia;
    *n_iter_out = best_iter;
    return FK_OK;
}

// ----------------------------------------------------------------- step --
template <typename TX, typename TC>
fk_status step_impl(fk_ctx *ctxp, const TX *x_in, int64_t n, int64_t d, const TC *c_in, int64_t k, int32_t prec,
                    uint64_t *labels_out, TC *centers_out, TC *inertia_out, TC *shift_out, fk_fit_report *rep) {
    Ctx &ctx = *reinterpret_cast<Ctx *>(ctxp);
    if (k <= 0) {
        set_error("Invalid parameter `n_clusters`: must be at least 1");
        return FK_ERR_INVALID_PARAMETER;
    }
    if (n <= 0 || n < k) {
        set_error("Insufficient samples: need at least %lld, got %lld", (long long)k, (long long)n);
        return FK_ERR_INSUFFICIENT_SAMPLES;
    }
    if (!x_in || !c_in || !labels_out || !centers_out || !inertia_out || !shift_out) {
        set_error("required pointer is NULL");
        return FK_ERR_NULL_POINTER;
    }
    if (!precision_ok<TX, TC>(prec)) {
        precision_error(prec);
        return FK_ERR_UNSUPPORTED;
    }
    if (fk_status st = check_shape(n, d, k)) return st;
    ctx.bind();
    if (rep) {
        memset(rep, 0, sizeof(*rep));
        rep->precision_used = prec;
    }
    cudaStream_t s = ctx.stream;
    const size_t kd = (size_t)k * d;
    const TX *x = stage_in<TX>(ctx, BUF_X, x_in, (size_t)n * d);
    TC *c = (TC *)ctx.get(BUF_C0, sizeof(TC) * kd);
    TC *nc = (TC *)ctx.get(BUF_C1, sizeof(TC) * kd);
    FK_CUDA(cudaMemcpyAsync(c, c_in, sizeof(TC) * kd, cudaMemcpyDefault, s));
    int32_t *labels = (int32_t *)ctx.get(BUF_LABELS, sizeof(int32_t) * (size_t)n);
    DevScalars *sc = (DevScalars *)ctx.get(BUF_SCALARS, sizeof(DevScalars));
    FK_CUDA(cudaMemsetAsync(sc, 0, sizeof(DevScalars), s));
    SortPlan plan = make_sort_plan(n, (int)k);
    lloyd_iteration<TX, TC>(ctx, x, n, (int)d, c, (int)k, prec, nc, labels, sc, plan, true, rep, false);
    read_scalars(ctx, sc);
    accumulate_report(rep, *ctx.host_scalars, n);
    copy_out<TC>(ctx, centers_out, nc, kd);
    if (is_device_ptr(labels_out)) {
        launch_labels_to_u64(labels, n, labels_out, s);
    } else {
        uint64_t *l64 = (uint64_t *)ctx.get(BUF_OUT, sizeof(uint64_t) * (size_t)n);
        launch_labels_to_u64(labels, n, l64, s);
        copy_out<uint64_t>(ctx, labels_out, l64, (size_t)n);
    }
    FK_CUDA(cudaStreamSynchronize(s));
    *inertia_out = (TC)ctx.host_scalars->inertia;
    *shift_out = shift_from_bits<TC>(ctx.host_scalars->shift_bits);
    return FK_OK;
}

// -------------------------------------------------------------- predict --
template <typename TX, typename TC>
fk_status predict_impl(fk_ctx *ctxp, const TC *c_in, int64_t k, int64_t d_fit, const TX *x_in, int64_t n,
                       int64_t d, int32_t prec, uint64_t *labels_out) {
    Ctx &ctx = *reinterpret_cast<Ctx *>(ctxp);
    if (d != d_fit) {
        set_error("Shape mismatch in number of features must match fitted KMeans model: expected [%lld], got [%lld]",
                  (long long)d_fit, (long long)d);
        return FK_ERR_SHAPE_MISMATCH;
    }
    if (k <= 0 || n < 0) {
        set_error("Invalid parameter: k must be >= 1 and n >= 0");
        return FK_ERR_INVALID_PARAMETER;
    }
    if (n == 0) return FK_OK;
    if (!x_in || !c_in || !labels_out) {
        set_error("required pointer is NULL");
        return FK_ERR_NULL_POINTER;
    }
    if (!precision_ok<TX, TC>(prec)) {
        precision_error(prec);
        return FK_ERR_UNSUPPORTED;
    }
    if (fk_status st = check_shape(n, d, k)) return st;
    ctx.bind();
    cudaStream_t s = ctx.stream;
    const TX *x = stage_in<TX>(ctx, BUF_X, x_in, (size_t)n * d);
    const TC *c = stage_in<TC>(ctx, BUF_C0, c_in, (size_t)k * d);
    int32_t *labels = (int32_t *)ctx.get(BUF_LABELS, sizeof(int32_t) * (size_t)n);
    if (prec == FK_PRECISION_PLAIN) {
        if constexpr (std::is_same<TX, double>::value && std::is_same<TC, double>::value)
            launch_assign_f64_filtered(ctx, x, n, (int)d, c, (int)k, labels, nullptr, true);
        else
            launch_assign_direct<TX, TC>(x, n, (int)d, c, (int)k, labels, nullptr, s);
    } else {
        if constexpr (std::is_same<TX, float>::value && std::is_same<TC, double>::value) {
            DevScalars *sc = (DevScalars *)ctx.get(BUF_SCALARS, sizeof(DevScalars));
            FK_CUDA(cudaMemsetAsync(sc, 0, sizeof(DevScalars), s));
            run_assign_mixed(ctx, x, n, (int)d, c, (int)k, prec, labels, nullptr, sc, true);
        }
    }
    if (is_device_ptr(labels_out)) {
        launch_labels_to_u64(labels, n, labels_out, s);
    } else {
        uint64_t *l64 = (uint64_t *)ctx.get(BUF_OUT, sizeof(uint64_t) * (size_t)n);
        launch_labels_to_u64(labels, n, l64, s);
        copy_out<uint64_t>(ctx, labels_out, l64, (size_t)n);
    }
    FK_CUDA(cudaStreamSynchronize(s));
    return FK_OK;
}

template <typename T>
fk_status transform_impl(fk_ctx *ctxp, const T *c_in, int64_t k, int64_t d_fit, const T *x_in, int64_t n, int64_t d,
                         T *out) {
    Ctx &ctx = *reinterpret_cast<Ctx *>(ctxp);
    if (d != d_fit) {
        set_error("Shape mismatch in number of features must match fitted KMeans model: expected [%lld], got [%lld]",
                  (long long)d_fit, (long long)d);
        return FK_ERR_SHAPE_MISMATCH;
    }
    if (k <= 0 || n < 0) {
        set_error("Invalid parameter: k must be >= 1 and n >= 0");
        return FK_ERR_INVALID_PARAMETER;
    }
    if (n == 0) return FK_OK;
    if (!x_in || !c_in || !out) {
        set_error("required pointer is NULL");
        return FK_ERR_NULL_POINTER;
    }
    if (fk_status st = check_shape(n, d, k)) return st;
    ctx.bind();
    cudaStream_t s = ctx.stream;
    const T *x = stage_in<T>(ctx, BUF_X, x_in, (size_t)n * d);
    const T *c = stage_in<T>(ctx, BUF_C0, c_in, (size_t)k * d);
    T *o = is_device_ptr(out) ? out : (T *)ctx.get(BUF_OUT, sizeof(T) * (size_t)n * k);
    launch_transform_direct<T>(x, n, (int)d, c, (int)k, o, s);
    if (o != out) copy_out<T>(ctx, out, o, (size_t)n * k);
    FK_CUDA(cudaStreamSynchronize(s));
    return FK_OK;
}

template <typename T>
fk_status kpp_impl(fk_ctx *ctxp, const T *x_in, int64_t n, int64_t d, int64_t k, const double *draws, int64_t n_draws,
                   uint64_t seed, T *centers_out, int64_t *draws_used) {
    Ctx &ctx = *reinterpret_cast<Ctx *>(ctxp);
    if (k <= 0) {
        set_error("Invalid parameter `n_clusters`: must be at least 1");
        return FK_ERR_INVALID_PARAMETER;
    }
    if (n <= 0) {
        set_error("Insufficient samples: need at least 1, got 0");
        return FK_ERR_INSUFFICIENT_SAMPLES;
    }
    if (!x_in || !centers_out) {
        set_error("required pointer is NULL");
        return FK_ERR_NULL_POINTER;
    }
    if (draws && n_draws < 0) {
        set_error("Invalid parameter `n_draws`: negative");
        return FK_ERR_INVALID_PARAMETER;
    }
    if (fk_status st = check_shape(n, d, k)) return st;
    ctx.bind();
    cudaStream_t s = ctx.stream;
    const T *x = stage_in<T>(ctx, BUF_X, x_in, (size_t)n * d);
    std::vector<double> hd;
    const double *dr;
    if (draws) {
        dr = stage_in<double>(ctx, BUF_DRAWS, draws, (size_t)n_draws);
    } else {
        n_draws = 1 + (k - 1) * kpp_trials_host(k);
        hd.resize((size_t)n_draws);
        host_draws(seed, n_draws, hd.data());
        double *dd = (double *)ctx.get(BUF_DRAWS, sizeof(double) * (size_t)n_draws);
        FK_CUDA(cudaMemcpyAsync(dd, hd.data(), sizeof(double) * (size_t)n_draws, cudaMemcpyHostToDevice, s));
        dr = dd;
    }
    T *o = is_device_ptr(centers_out) ? centers_out : (T *)ctx.get(BUF_OUT, sizeof(T) * (size_t)k * d);
    int64_t used = 0;
    run_kmeanspp<T>(ctx, x, n, (int)d, (int)k, dr, n_draws, o, &used);
    if (o != centers_out) copy_out<T>(ctx, centers_out, o, (size_t)k * d);
    FK_CUDA(cudaStreamSynchronize(s));
    if (draws_used) *draws_used = used;
    return FK_OK;
}

// ----------------------------------------------------------- minibatch --
// The library's uniform stream from position pos of seed: every draw first
// advances the state by the golden gamma, so a position is one multiply.
struct UniformStream {
    uint64_t state;
    UniformStream(uint64_t seed, int64_t pos) : state(seed + (uint64_t)pos * 0x9E3779B97F4A7C15ULL) {}
    double next() { return (double)(splitmix64(&state) >> 11) * (1.0 / 9007199254740992.0); }
    // random_range(0..n) as min(floor(u n), n - 1)
    int64_t range(int64_t n) {
        const int64_t i = (int64_t)std::floor(next() * (double)n);
        return i < 0 ? 0 : (i >= n ? n - 1 : i);
    }
};

// min(count, n) picks of a Fisher-Yates pass over the pool 0..n, pick i
// swapping position i with i + random_range(0..n - i): random_init_mb
// (mini_batch_kmeans.rs:324-338) and sample_batch_indices (:451-472). A
// partial pass keeps only the displaced entries of the pool (a map), so a
// batch costs O(batch) whatever n; a full pass (count >= n) uses the pool.
template <typename I>
int64_t fisher_yates_picks(UniformStream &g, int64_t n, int64_t count, std::unordered_map<int64_t, int64_t> &moved,
                           std::vector<int64_t> &pool, I *out) {
    const int64_t m = count < n ? count : n;
    if (m == n) {
        pool.resize((size_t)n);
        for (int64_t i = 0; i < n; i++) pool[(size_t)i] = i;
        for (int64_t i = 0; i < n; i++) {
            const int64_t j = i + g.range(n - i);
            std::swap(pool[(size_t)i], pool[(size_t)j]);
            out[i] = (I)pool[(size_t)i];
        }
        return m;
    }
    moved.clear();
    auto at = [&](int64_t t) {
        auto it = moved.find(t);
        return it == moved.end() ? t : it->second;
    };
    for (int64_t i = 0; i < m; i++) {
        const int64_t j = i + g.range(n - i);
        const int64_t vi = at(i), vj = at(j);
        moved[i] = vj;
        moved[j] = vi;
        out[i] = (I)vj;
    }
    return m;
}

// MiniBatchKMeans::fit (mini_batch_kmeans.rs:492-591) on the GPU. Per run:
// the initial centres, then per iteration the batch rows gathered, their
// nearest centres (the direct-form assignment kernel), the in-order update
// and the max shift; the early stop reads the shift back only when tol > 0
// (a shift is never below a tol <= 0). The batch indices come from the host
// stream, uploaded a chunk of iterations at a time.
template <typename T>
fk_status minibatch_impl(fk_ctx *ctxp, const T *x_in, int64_t n, int64_t d, const fk_minibatch_params *p,
                         const T *init_in, T *centers_out, uint64_t *labels_out, T *inertia_out, int64_t *n_iter_out,
                         int64_t *best_run_out, fk_fit_report *rep) {
    Ctx &ctx = *reinterpret_cast<Ctx *>(ctxp);
    const int64_t k = p->n_clusters;
    // Validation order of mini_batch_kmeans.rs:495-526.
    if (k <= 0) {
        set_error("Invalid parameter `n_clusters`: must be at least 1");
        return FK_ERR_INVALID_PARAMETER;
    }
    if (p->batch_size <= 0) {
        set_error("Invalid parameter `batch_size`: must be at least 1");
        return FK_ERR_INVALID_PARAMETER;
    }
    if (p->n_init <= 0) {
        set_error("Invalid parameter `n_init`: must be at least 1");
        return FK_ERR_INVALID_PARAMETER;
    }
    if (n <= 0 || n < k) {
        set_error("Insufficient samples: need at least %lld, got %lld (MiniBatchKMeans requires at least "
                  "n_clusters samples)", (long long)k, (long long)(n < 0 ? 0 : n));
        return FK_ERR_INSUFFICIENT_SAMPLES;
    }
    if (p->max_iter < 0) {
        set_error("Invalid parameter `max_iter`: negative");
        return FK_ERR_INVALID_PARAMETER;
    }
    if (p->init != FK_MB_INIT_KMEANS_PLUS_PLUS && p->init != FK_MB_INIT_RANDOM) {
        set_error("Invalid parameter `init`: %d", p->init);
        return FK_ERR_INVALID_PARAMETER;
    }
    if (!x_in || !centers_out || !labels_out || !inertia_out || !n_iter_out) {
        set_error("required pointer is NULL");
        return FK_ERR_NULL_POINTER;
    }
    if (fk_status st = check_shape(n, d, k)) return st;
    ctx.bind();
    if (rep) {
        memset(rep, 0, sizeof(*rep));
        rep->precision_used = FK_PRECISION_PLAIN;
    }
    cudaStream_t s = ctx.stream;
    Events<2> tev;
    FK_CUDA(cudaEventRecord(tev[0], s));
    const size_t kd = (size_t)k * d;
    const int64_t m = std::min(p->batch_size, n);  // rows per batch
    const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(p->max_iter, ((int64_t)16 << 20) / m));
    const T *x = stage_in<T>(ctx, BUF_X, x_in, (size_t)n * d);
    const T *init = init_in ? stage_in<T>(ctx, BUF_INIT, init_in, kd * (size_t)p->n_init) : nullptr;
    T *c = (T *)ctx.get(BUF_C0, sizeof(T) * kd);
    T *old = (T *)ctx.get(BUF_MB_OLD, sizeof(T) * kd);
    T *cbest = (T *)ctx.get(BUF_CBEST, sizeof(T) * kd);
    long long *counts = (long long *)ctx.get(BUF_MB_COUNTS, sizeof(long long) * (size_t)k);
    int32_t *labels = (int32_t *)ctx.get(BUF_LABELS, sizeof(int32_t) * (size_t)n);
    int32_t *lbest = (int32_t *)ctx.get(BUF_LBEST, sizeof(int32_t) * (size_t)n);
    T *mind = (T *)ctx.get(BUF_MIND, sizeof(T) * (size_t)n);
    double *part = (double *)ctx.get(BUF_PARTIAL, sizeof(double) * (size_t)sum_fixed_partials(n));
    DevScalars *sc = (DevScalars *)ctx.get(BUF_SCALARS, sizeof(DevScalars));
    int32_t *didx = (int32_t *)ctx.get(BUF_MB_IDX, sizeof(int32_t) * (size_t)std::max(m * chunk, k));
    T *xb = (T *)ctx.get(BUF_MB_XB, sizeof(T) * (size_t)m * d);
    int32_t *blab = (int32_t *)ctx.get(BUF_MB_LAB, sizeof(int32_t) * (size_t)m);
    // a batch is too few rows to fill the GPU by row tiles: split the centres too
    const int splits = assign_splits<T>(m, (int)k, ctx.num_sms);
    T *part_v = splits > 1 ? (T *)ctx.get(BUF_MB_PARTV, sizeof(T) * (size_t)splits * m) : nullptr;
    int32_t *part_i = splits > 1 ? (int32_t *)ctx.get(BUF_MB_PARTI, sizeof(int32_t) * (size_t)splits * m) : nullptr;
    std::vector<int32_t> hidx;
    std::unordered_map<int64_t, int64_t> moved;
    std::vector<int64_t> pool;
    std::vector<double> hdraws;
    const std::vector<long long> ones((size_t)k, 1LL);  // per-centre counts start at 1 (:543)
    const uint64_t base = p->has_random_state ? p->random_state : 0;
    const T tol = (T)p->tol;
    bool have = false;
    T best_inertia = FMax<T>::v();
    int64_t best_iter = 0, best_run = 0;
    for (int64_t run = 0; run < p->n_init; run++) {
        const uint64_t seed = base + (uint64_t)run * 1000003ULL;
        int64_t pos = 0;  // stream position after the initial centres
        if (init) {
            FK_CUDA(cudaMemcpyAsync(c, init + (size_t)run * kd, sizeof(T) * kd, cudaMemcpyDeviceToDevice, s));
        } else if (p->init == FK_MB_INIT_RANDOM) {
            UniformStream g(seed, 0);
            hidx.resize((size_t)k);
            fisher_yates_picks(g, n, k, moved, pool, hidx.data());
            pos = k;
            FK_CUDA(cudaMemcpyAsync(didx, hidx.data(), sizeof(int32_t) * (size_t)k, cudaMemcpyHostToDevice, s));
            launch_gather_rows<T>(x, (int)d, didx, k, c, s);
            FK_CUDA(cudaStreamSynchronize(s));  // hidx is refilled below
        } else {
            const int64_t n_draws = 1 + (k - 1) * kpp_trials_host(k);
            hdraws.resize((size_t)n_draws);
            host_draws(seed, n_draws, hdraws.data());
            double *dd = (double *)ctx.get(BUF_DRAWS, sizeof(double) * (size_t)n_draws);
            FK_CUDA(cudaMemcpyAsync(dd, hdraws.data(), sizeof(double) * (size_t)n_draws, cudaMemcpyHostToDevice, s));
            run_kmeanspp<T>(ctx, x, n, (int)d, (int)k, dd, n_draws, c, &pos);  // synchronises
        }
        FK_CUDA(cudaMemcpyAsync(counts, ones.data(), sizeof(long long) * (size_t)k, cudaMemcpyHostToDevice, s));
        UniformStream g(seed, pos);
        int64_t n_iter = 0;
        bool stop = false;
        for (int64_t it0 = 0; it0 < p->max_iter && !stop; it0 += chunk) {
            const int64_t ci = std::min(chunk, p->max_iter - it0);
            FK_CUDA(cudaStreamSynchronize(s));  // the previous upload of hidx has completed
            hidx.resize((size_t)(ci * m));
            for (int64_t q = 0; q < ci; q++) fisher_yates_picks(g, n, p->batch_size, moved, pool, hidx.data() + q * m);
            FK_CUDA(cudaMemcpyAsync(didx, hidx.data(), sizeof(int32_t) * (size_t)(ci * m), cudaMemcpyHostToDevice, s));
            for (int64_t q = 0; q < ci; q++) {
                launch_gather_rows<T>(x, (int)d, didx + q * m, m, xb, s);
                launch_assign_direct_split<T, T>(xb, m, (int)d, c, (int)k, blab, nullptr, splits, part_v, part_i, s);
                launch_minibatch_update<T>(xb, blab, m, (int)d, (int)k, c, old, counts, &sc->shift_bits, s);
                n_iter += 1;
                if (tol > T(0)) {
                    FK_CUDA(cudaMemcpyAsync(&ctx.host_scalars->shift_bits, &sc->shift_bits, sizeof(unsigned long long),
                                            cudaMemcpyDeviceToHost, s));
                    FK_CUDA(cudaStreamSynchronize(s));
                    if (shift_from_bits<T>(ctx.host_scalars->shift_bits) < tol) {
                        stop = true;
                        break;
                    }
                }
            }
        }
        // assign_clusters_mb (:343-376) over every row: the run's labels and inertia
        FK_CUDA(cudaMemsetAsync(sc, 0, sizeof(DevScalars), s));
        if constexpr (std::is_same<T, double>::value)
            launch_assign_f64_filtered(ctx, x, n, (int)d, c, (int)k, labels, mind, true);
        else
            launch_assign_direct<T, T>(x, n, (int)d, c, (int)k, labels, mind, s);
        launch_sum_fixed<T>(mind, n, part, &sc->inertia, s);
        read_scalars(ctx, sc);
        const T inertia = (T)ctx.host_scalars->inertia;
        if (rep) rep->iterations_total += n_iter;
        if (!have || inertia < best_inertia) {
            have = true;
            best_inertia = inertia;
            best_iter = n_iter;
            best_run = run;
            FK_CUDA(cudaMemcpyAsync(cbest, c, sizeof(T) * kd, cudaMemcpyDeviceToDevice, s));
            FK_CUDA(cudaMemcpyAsync(lbest, labels, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToDevice, s));
        }
    }
    copy_out<T>(ctx, centers_out, cbest, kd);
    if (is_device_ptr(labels_out)) {
        launch_labels_to_u64(lbest, n, labels_out, s);
    } else {
        uint64_t *l64 = (uint64_t *)ctx.get(BUF_OUT, sizeof(uint64_t) * (size_t)n);
        launch_labels_to_u64(lbest, n, l64, s);
        copy_out<uint64_t>(ctx, labels_out, l64, (size_t)n);
    }
    FK_CUDA(cudaEventRecord(tev[1], s));
    FK_CUDA(cudaStreamSynchronize(s));
    if (rep) {
        float ms = 0.f;
        FK_CUDA(cudaEventElapsedTime(&ms, tev[0], tev[1]));
        rep->ms_total = ms;
        rep->best_run = best_run;
        rep->rows_assigned = n * p->n_init;
    }
    *inertia_out = best_inertia;
    *n_iter_out = best_iter;
    if (best_run_out) *best_run_out = best_run;
    return FK_OK;
}

// ------------------------------------------------------------ bisecting --
// BisectingKMeans::fit (bisecting_kmeans.rs:326-505). The clusters are
// segments of one row permutation on the device; the host keeps their list
// (segment, centre slot, SSE) in the reference's order and selects the next
// cluster as Rust's max_by_key / max_by do (the last of equal maxima). A
// split runs its n_init 2-means runs together: the two picked rows per run
// come from the host stream, then per iteration the assignment and changed
// flags, and the centre sums of the runs that changed; the best run
// (strictly lowest SSE) partitions the segment into the children (label 0
// first, each side in row order), whose SSEs are the row-order folds of
// their rows' distances.
struct BkCluster {
    int64_t lo, m;
    int slot;
    double sse;  // in F (exact for F = f32 too)
};

template <typename T>
fk_status bisecting_impl(fk_ctx *ctxp, const T *x_in, int64_t n, int64_t d, const fk_bisecting_params *p,
                         T *centers_out, int64_t *labels_out, T *inertia_out, int64_t *n_clusters_out) {
    Ctx &ctx = *reinterpret_cast<Ctx *>(ctxp);
    const int64_t k = p->n_clusters;
    // Validation order of bisecting_kmeans.rs:333-358.
    if (k <= 0) {
        set_error("Invalid parameter `n_clusters`: must be at least 1");
        return FK_ERR_INVALID_PARAMETER;
    }
    if (p->n_init <= 0) {
        set_error("Invalid parameter `n_init`: must be at least 1");
        return FK_ERR_INVALID_PARAMETER;
    }
    if (n <= 0 || n < k) {
        set_error("Insufficient samples: need at least %lld, got %lld (BisectingKMeans requires at least "
                  "n_clusters samples)", (long long)k, (long long)(n < 0 ? 0 : n));
        return FK_ERR_INSUFFICIENT_SAMPLES;
    }
    if (p->max_iter < 0) {
        set_error("Invalid parameter `max_iter`: negative");
        return FK_ERR_INVALID_PARAMETER;
    }
    if (p->strategy != FK_BISECT_LARGEST_CLUSTER && p->strategy != FK_BISECT_LARGEST_SSE) {
        set_error("Invalid parameter `bisecting_strategy`: %d", p->strategy);
        return FK_ERR_INVALID_PARAMETER;
    }
    if (!x_in || !centers_out || !labels_out || !inertia_out || !n_clusters_out) {
        set_error("required pointer is NULL");
        return FK_ERR_NULL_POINTER;
    }
    if (fk_status st = check_shape(n, d, k)) return st;
    if (d > BK_MAX_D || p->n_init > 1024) {
        set_error("BisectingKMeans on the GPU supports d <= %d and n_init <= 1024 (got d=%lld n_init=%lld)",
                  BK_MAX_D, (long long)d, (long long)p->n_init);
        return FK_ERR_UNSUPPORTED;
    }
    ctx.bind();
    cudaStream_t s = ctx.stream;
    const int runs = (int)p->n_init;
    const T *x = stage_in<T>(ctx, BUF_X, x_in, (size_t)n * d);
    int32_t *perm = (int32_t *)ctx.get(BUF_BK_PERM, sizeof(int32_t) * (size_t)n);
    uint8_t *lab = (uint8_t *)ctx.get(BUF_BK_LAB, (size_t)runs * n);
    T *cen = (T *)ctx.get(BUF_BK_CEN, sizeof(T) * 2 * (size_t)runs * d);
    T *dist = (T *)ctx.get(BUF_BK_DIST, sizeof(T) * (size_t)runs * n);
    int *flags = (int *)ctx.get(BUF_BK_FLAGS, sizeof(int) * 4 * (size_t)runs);
    int *changed = flags, *active = flags + runs, *picks = flags + 2 * runs;
    int32_t *scratch = (int32_t *)ctx.get(BUF_BK_SCRATCH, sizeof(int32_t) * bk_partition_scratch_ints(n));
    T *centres = (T *)ctx.get(BUF_BK_CENTRES, sizeof(T) * (size_t)(k + 1) * d);
    int64_t *seg = (int64_t *)ctx.get(BUF_BK_SEG, sizeof(int64_t) * (2 * (size_t)k + 2));
    int64_t *m0_dev = seg + 2 * k;
    T *fold = (T *)ctx.get(BUF_BK_FOLD, sizeof(T) * (size_t)std::max(runs, 2));
    // The reference's row-order sums (the 2-means centres and the SSEs) as
    // exact parallel folds (fk_fold.cu): chains [0, runs * 2 * d) are the
    // centre sums of the current segment (rows gathered into xseg), the next
    // runs + 2 the SSE folds.
    T *xseg = (T *)ctx.get(BUF_BK_XSEG, sizeof(T) * (size_t)n * d);
    const size_t nsum = (size_t)runs * 2 * d;
    FoldChain *dchains = (FoldChain *)ctx.get(BUF_BK_CHAINS, sizeof(FoldChain) * (nsum + runs + 2));
    T *fres = (T *)ctx.get(BUF_BK_FRES, sizeof(T) * (nsum + 8));
    long long *fcnt = (long long *)ctx.get(BUF_BK_FCNT, sizeof(long long) * (nsum + runs + 8));
    std::vector<FoldChain> hchains;
    auto upload_sum_chains = [&](const T *rows, int nr, bool gated) {
        hchains.assign((size_t)nr * 2 * d, FoldChain{});
        for (int r = 0; r < nr; r++)
            for (int side = 0; side < 2; side++)
                for (int64_t j = 0; j < d; j++)
                    hchains[((size_t)r * 2 + side) * d + j] =
                        FoldChain{rows + j, d, lab + (size_t)r * n, side, gated ? r : -1};
        FK_CUDA(cudaMemcpyAsync(dchains, hchains.data(), sizeof(FoldChain) * hchains.size(), cudaMemcpyHostToDevice,
                                s));
    };
    // folds of `cnt` distance arrays (base + c * stride, optionally masked by
    // label == c) into fold[0 .. cnt)
    auto sse_folds = [&](const T *base, int64_t stride, const uint8_t *mask, int cnt, int64_t m) {
        hchains.assign((size_t)cnt, FoldChain{});
        for (int c = 0; c < cnt; c++)
            hchains[(size_t)c] = FoldChain{base + (size_t)c * stride, 1, mask, mask ? c : 0, -1};
        FK_CUDA(cudaMemcpyAsync(dchains + nsum, hchains.data(), sizeof(FoldChain) * (size_t)cnt,
                                cudaMemcpyHostToDevice, s));
        run_exact_folds<T>(ctx, dchains + nsum, cnt, m, nullptr, fold, fcnt + nsum);
    };
    {
        std::vector<int32_t> iota((size_t)n);
        for (int64_t i = 0; i < n; i++) iota[(size_t)i] = (int32_t)i;
        FK_CUDA(cudaMemcpyAsync(perm, iota.data(), sizeof(int32_t) * (size_t)n, cudaMemcpyHostToDevice, s));
        FK_CUDA(cudaStreamSynchronize(s));
    }
    // compute_cluster_stats of every row (:192-222): the centre (sums / F::from(n)) and the SSE
    std::vector<T> hfold((size_t)std::max(runs, 2));
    FK_CUDA(cudaMemsetAsync(lab, 0, (size_t)n, s));
    upload_sum_chains(x, 1, false);  // every row, in row order (the permutation is the identity)
    run_exact_folds<T>(ctx, dchains, (int)(2 * d), n, nullptr, fres, fcnt);
    launch_bk_centres<T>(fres, fcnt, 1, (int)d, nullptr, true, n, cen, s);
    launch_bk_dist<T>(x, (int)d, perm, n, cen, lab, n, dist, n, 1, s);
    sse_folds(dist, n, nullptr, 1, n);
    FK_CUDA(cudaMemcpyAsync(centres, cen, sizeof(T) * (size_t)d, cudaMemcpyDeviceToDevice, s));
    FK_CUDA(cudaMemcpyAsync(hfold.data(), fold, sizeof(T), cudaMemcpyDeviceToHost, s));
    FK_CUDA(cudaStreamSynchronize(s));
    std::vector<BkCluster> cl;
    cl.push_back(BkCluster{0, n, 0, (double)hfold[0]});
    std::vector<int> free_slots;
    for (int64_t sl = k; sl >= 1; sl--) free_slots.push_back((int)sl);
    const uint64_t base = p->has_random_state ? p->random_state : 0;
    const int64_t max_splits = 4 * n + 4 * k + 16;
    uint64_t split_count = 0;
    std::vector<int> hpicks(2 * (size_t)runs), hact((size_t)runs), hch((size_t)runs);
    while ((int64_t)cl.size() < k) {
        if ((int64_t)split_count > max_splits) {
            set_error("the cluster selected for bisection cannot be separated (its rows are identical): the "
                      "reference does not terminate here");
            return FK_ERR_NUMERICAL_INSTABILITY;
        }
        int64_t t = -1;
        for (int64_t ci = 0; ci < (int64_t)cl.size(); ci++) {
            if (cl[(size_t)ci].m < 2) continue;
            if (t < 0) {
                t = ci;
                continue;
            }
            const BkCluster &a = cl[(size_t)t], &b = cl[(size_t)ci];
            const bool a_greater = p->strategy == FK_BISECT_LARGEST_CLUSTER ? a.m > b.m : (T)a.sse > (T)b.sse;
            if (!a_greater) t = ci;
        }
        if (t < 0) break;  // no cluster with two rows left
        const BkCluster target = cl[(size_t)t];
        const int64_t m = target.m;
        int32_t *segp = perm + target.lo;
        for (int r = 0; r < runs; r++) {
            UniformStream g(base + split_count * 1000ULL + (uint64_t)r, 0);
            const int64_t i0 = g.range(m);
            int64_t i1 = g.range(m);
            if (m > 1)
                while (i1 == i0) i1 = g.range(m);
            hpicks[2 * (size_t)r] = (int)i0;
            hpicks[2 * (size_t)r + 1] = (int)i1;
            hact[(size_t)r] = 1;
        }
        FK_CUDA(cudaMemcpyAsync(picks, hpicks.data(), sizeof(int) * 2 * (size_t)runs, cudaMemcpyHostToDevice, s));
        FK_CUDA(cudaMemcpyAsync(active, hact.data(), sizeof(int) * (size_t)runs, cudaMemcpyHostToDevice, s));
        launch_bk_pick<T>(x, (int)d, segp, picks, runs, cen, s);
        launch_gather_rows<T>(x, (int)d, segp, m, xseg, s);
        upload_sum_chains(xseg, runs, true);
        FK_CUDA(cudaMemset2DAsync(lab, (size_t)n, 0, (size_t)m, (size_t)runs, s));
        int nact = runs;
        for (int64_t it = 0; it < p->max_iter && nact > 0; it++) {
            FK_CUDA(cudaMemsetAsync(changed, 0, sizeof(int) * (size_t)runs, s));
            launch_bk_assign<T>(x, (int)d, segp, m, cen, lab, n, active, changed, runs, s);
            FK_CUDA(cudaMemcpyAsync(hch.data(), changed, sizeof(int) * (size_t)runs, cudaMemcpyDeviceToHost, s));
            FK_CUDA(cudaStreamSynchronize(s));
            for (int r = 0; r < runs; r++)
                if (hact[(size_t)r] && !hch[(size_t)r]) {
                    hact[(size_t)r] = 0;  // no label changed: this run is done (:263)
                    nact--;
                }
            if (nact == 0) break;
            FK_CUDA(cudaMemcpyAsync(active, hact.data(), sizeof(int) * (size_t)runs, cudaMemcpyHostToDevice, s));
            run_exact_folds<T>(ctx, dchains, (int)nsum, m, active, fres, fcnt);
            launch_bk_centres<T>(fres, fcnt, runs, (int)d, active, false, m, cen, s);
        }
        // each run's SSE against its final centres (:300-309)
        launch_bk_dist<T>(x, (int)d, segp, m, cen, lab, n, dist, n, runs, s);
        sse_folds(dist, n, nullptr, runs, m);
        FK_CUDA(cudaMemcpyAsync(hfold.data(), fold, sizeof(T) * (size_t)runs, cudaMemcpyDeviceToHost, s));
        FK_CUDA(cudaStreamSynchronize(s));
        int best = -1;
        T best_sse = FMax<T>::v();
        for (int r = 0; r < runs; r++)
            if (hfold[(size_t)r] < best_sse) {
                best_sse = hfold[(size_t)r];
                best = r;
            }
        split_count++;
        if (best < 0) {
            set_error("no 2-means run gave an SSE below F::MAX (non-finite rows)");
            return FK_ERR_NUMERICAL_INSTABILITY;
        }
        const uint8_t *blab = lab + (size_t)best * n;
        // the children's SSEs (:443-463), then their rows (:430-441)
        sse_folds(dist + (size_t)best * n, 0, blab, 2, m);
        launch_bk_partition(segp, blab, m, scratch, m0_dev, s);
        int64_t m0 = 0;
        FK_CUDA(cudaMemcpyAsync(hfold.data(), fold, sizeof(T) * 2, cudaMemcpyDeviceToHost, s));
        FK_CUDA(cudaMemcpyAsync(&m0, m0_dev, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        FK_CUDA(cudaStreamSynchronize(s));
        cl.erase(cl.begin() + t);
        free_slots.push_back(target.slot);
        const T *bc = cen + (size_t)best * 2 * d;
        if (m0 > 0) {
            const int sl = free_slots.back();
            free_slots.pop_back();
            FK_CUDA(cudaMemcpyAsync(centres + (size_t)sl * d, bc, sizeof(T) * (size_t)d, cudaMemcpyDeviceToDevice, s));
            cl.push_back(BkCluster{target.lo, m0, sl, (double)hfold[0]});
        }
        if (m - m0 > 0) {
            const int sl = free_slots.back();
            free_slots.pop_back();
            FK_CUDA(cudaMemcpyAsync(centres + (size_t)sl * d, bc + d, sizeof(T) * (size_t)d, cudaMemcpyDeviceToDevice,
                                    s));
            cl.push_back(BkCluster{target.lo + m0, m - m0, sl, (double)hfold[1]});
        }
    }
    // outputs: centres and labels in list order, the SSEs folded in F (:484-498)
    const int nc = (int)cl.size();
    std::vector<int64_t> hseg(2 * (size_t)nc);
    std::vector<int32_t> hslot((size_t)nc);
    T inertia = T(0);
    for (int ci = 0; ci < nc; ci++) {
        hseg[2 * (size_t)ci] = cl[(size_t)ci].lo;
        hseg[2 * (size_t)ci + 1] = cl[(size_t)ci].m;
        hslot[(size_t)ci] = cl[(size_t)ci].slot;
        inertia = inertia + (T)cl[(size_t)ci].sse;
    }
    FK_CUDA(cudaMemcpyAsync(seg, hseg.data(), sizeof(int64_t) * hseg.size(), cudaMemcpyHostToDevice, s));
    FK_CUDA(cudaMemcpyAsync(scratch, hslot.data(), sizeof(int32_t) * hslot.size(), cudaMemcpyHostToDevice, s));
    T *cout = (T *)ctx.get(BUF_OUT2, sizeof(T) * (size_t)nc * d + 16);
    launch_gather_rows<T>(centres, (int)d, scratch, nc, cout, s);
    copy_out<T>(ctx, centers_out, cout, (size_t)nc * d);
    int64_t *ldev = is_device_ptr(labels_out) ? labels_out : (int64_t *)ctx.get(BUF_BK_LABELS, sizeof(int64_t) * (size_t)n);
    launch_bk_labels(perm, seg, nc, ldev, s);
    if (ldev != labels_out) copy_out<int64_t>(ctx, labels_out, ldev, (size_t)n);
    FK_CUDA(cudaStreamSynchronize(s));
    *inertia_out = inertia;
    *n_clusters_out = nc;
    return FK_OK;
}

// Per-call state that points into a caller's report: timers not yet read
// and the contraction timer's target. Dropped before and after every call,
// so a call that failed half-way never writes into memory it no longer owns.
void drop_call_state(fk_ctx *ctxp) {
    Ctx &ctx = *reinterpret_cast<Ctx *>(ctxp);
    for (auto &p : ctx.pending) {
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    ctx.pending.clear();
    ctx.contract_acc = nullptr;
    ctx.count_acc = nullptr;
}

template <typename F>
fk_status guarded_body(fk_ctx *ctx, F &&f) {
    try {
        g_last_error.clear();
        return f();
    } catch (const Error &e) {
        return e.code;
    } catch (const std::bad_alloc &) {
        set_error("host allocation failed");
        return FK_ERR_OOM;
    } catch (...) {
        set_error("unexpected exception");
        return FK_ERR_CUDA;
    }
}

template <typename F>
fk_status guarded(fk_ctx *ctx, F &&f) {
    if (!ctx) {
        set_error("context is NULL");
        return FK_ERR_NULL_POINTER;
    }
    drop_call_state(ctx);
    const fk_status st = guarded_body(ctx, f);
    drop_call_state(ctx);
    return st;
}

}  // namespace
}  // namespace fk

using fk::guarded;

extern "C" {

fk_status fk_ctx_create(fk_ctx **out, int32_t device, void *cuda_stream) {
    if (!out) {
        fk::set_error("out is NULL");
        return FK_ERR_NULL_POINTER;
    }
    *out = nullptr;
    fk::Ctx *c = new (std::nothrow) fk::Ctx();
    if (!c) return FK_ERR_OOM;
    c->device = device;
    c->stream = (cudaStream_t)cuda_stream;
    *out = reinterpret_cast<fk_ctx *>(c);
    return FK_OK;
}

fk_status fk_ctx_destroy(fk_ctx *ctx) {
    if (!ctx) return FK_OK;
    fk::Ctx *c = reinterpret_cast<fk::Ctx *>(ctx);
    if (!c->initialized) {
        delete c;
        return FK_OK;
    }
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (int i = 0; i < fk::BUF_COUNT; i++)
        if (c->buf[i]) cudaFree(c->buf[i]);
    if (c->host_scalars) cudaFreeHost(c->host_scalars);
    if (c->mixed.ones) cudaFree(c->mixed.ones);
    if (c->mixed2.ones) cudaFree(c->mixed2.ones);
    if (c->mixedm.ones) cudaFree(c->mixedm.ones);
    if (c->mixedm2.ones) cudaFree(c->mixedm2.ones);
    if (c->mixedc.ones) cudaFree(c->mixedc.ones);
    for (auto &g : c->iter_graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return FK_OK;
}

const char *fk_last_error_message(void) { return fk::g_last_error.c_str(); }

const char *fk_version(void) { return "ferrokmeans-gb300 0.1.0 (sm_103a)"; }

uint64_t fk_debug_launch_count(void) { return __atomic_load_n(&fk::g_launch_count, __ATOMIC_RELAXED); }

void fk_kmeans_params_default(fk_kmeans_params *p, int64_t n_clusters) {
    if (!p) return;
    memset(p, 0, sizeof(*p));
    p->n_clusters = n_clusters;
    p->max_iter = 300;
    p->tol = 1e-4;
    p->n_init = 10;
    p->has_random_state = 0;
    p->precision = FK_PRECISION_PLAIN;
}

void fk_minibatch_params_default(fk_minibatch_params *p, int64_t n_clusters) {
    if (!p) return;
    memset(p, 0, sizeof(*p));
    p->n_clusters = n_clusters;  // MiniBatchKMeans::new, mini_batch_kmeans.rs:108-118
    p->batch_size = 1024;
    p->max_iter = 100;
    p->tol = 0.0;
    p->n_init = 3;
    p->has_random_state = 0;
    p->init = FK_MB_INIT_KMEANS_PLUS_PLUS;
}

fk_status fk_minibatch_fit_f64(fk_ctx *ctx, const double *x, int64_t n, int64_t d, const fk_minibatch_params *params,
                               const double *init, double *c_out, uint64_t *l_out, double *in_out, int64_t *it_out,
                               int64_t *best_out, fk_fit_report *rep) {
    if (!params) return FK_ERR_NULL_POINTER;
    return guarded(ctx, [&] {
        return fk::minibatch_impl<double>(ctx, x, n, d, params, init, c_out, l_out, in_out, it_out, best_out, rep);
    });
}

fk_status fk_minibatch_fit_f32(fk_ctx *ctx, const float *x, int64_t n, int64_t d, const fk_minibatch_params *params,
                               const float *init, float *c_out, uint64_t *l_out, float *in_out, int64_t *it_out,
                               int64_t *best_out, fk_fit_report *rep) {
    if (!params) return FK_ERR_NULL_POINTER;
    return guarded(ctx, [&] {
        return fk::minibatch_impl<float>(ctx, x, n, d, params, init, c_out, l_out, in_out, it_out, best_out, rep);
    });
}

void fk_bisecting_params_default(fk_bisecting_params *p, int64_t n_clusters) {
    if (!p) return;
    memset(p, 0, sizeof(*p));
    p->n_clusters = n_clusters;  // BisectingKMeans::new, bisecting_kmeans.rs:93-102
    p->max_iter = 300;
    p->n_init = 10;
    p->has_random_state = 0;
    p->strategy = FK_BISECT_LARGEST_CLUSTER;
}

fk_status fk_bisecting_fit_f64(fk_ctx *ctx, const double *x, int64_t n, int64_t d, const fk_bisecting_params *params,
                               double *c_out, int64_t *l_out, double *in_out, int64_t *nc_out) {
    if (!params) return FK_ERR_NULL_POINTER;
    return guarded(ctx, [&] { return fk::bisecting_impl<double>(ctx, x, n, d, params, c_out, l_out, in_out, nc_out); });
}

fk_status fk_bisecting_fit_f32(fk_ctx *ctx, const float *x, int64_t n, int64_t d, const fk_bisecting_params *params,
                               float *c_out, int64_t *l_out, float *in_out, int64_t *nc_out) {
    if (!params) return FK_ERR_NULL_POINTER;
    return guarded(ctx, [&] { return fk::bisecting_impl<float>(ctx, x, n, d, params, c_out, l_out, in_out, nc_out); });
}

fk_status fk_minibatch_batch_indices(uint64_t seed, int64_t pos, int64_t n, int64_t batch_size, int64_t iters,
                                     int64_t *out) {
    if (n <= 0 || batch_size <= 0 || iters < 0 || pos < 0) {
        fk::set_error("Invalid parameter: n and batch_size must be at least 1, iters and pos non-negative");
        return FK_ERR_INVALID_PARAMETER;
    }
    if (!out && iters > 0) return FK_ERR_NULL_POINTER;
    try {
        fk::UniformStream g(seed, pos);
        std::unordered_map<int64_t, int64_t> moved;
        std::vector<int64_t> pool;
        const int64_t m = std::min(batch_size, n);
        for (int64_t it = 0; it < iters; it++) fk::fisher_yates_picks(g, n, batch_size, moved, pool, out + it * m);
    } catch (const std::bad_alloc &) {
        fk::set_error("host allocation failed");
        return FK_ERR_OOM;
    }
    return FK_OK;
}

fk_status fk_draws_f64(uint64_t seed, int64_t count, double *out) {
    if (!out && count > 0) return FK_ERR_NULL_POINTER;
    fk::host_draws(seed, count, out);
    return FK_OK;
}

fk_status fk_kmeans_fit_f64(fk_ctx *ctx, const double *x, int64_t n, int64_t d, const fk_kmeans_params *params,
                            const double *init, double *c_out, uint64_t *l_out, double *in_out, int64_t *it_out,
                            fk_fit_report *rep) {
    if (!params) return FK_ERR_NULL_POINTER;
    return guarded(ctx, [&] { return fk::fit_impl<double, double>(ctx, x, n, d, params, init, c_out, l_out, in_out, it_out, rep); });
}

fk_status fk_kmeans_fit_f32(fk_ctx *ctx, const float *x, int64_t n, int64_t d, const fk_kmeans_params *params,
                            const float *init, float *c_out, uint64_t *l_out, float *in_out, int64_t *it_out,
                            fk_fit_report *rep) {
    if (!params) return FK_ERR_NULL_POINTER;
    return guarded(ctx, [&] { return fk::fit_impl<float, float>(ctx, x, n, d, params, init, c_out, l_out, in_out, it_out, rep); });
}

fk_status fk_kmeans_fit_f32x64(fk_ctx *ctx, const float *x, int64_t n, int64_t d, const fk_kmeans_params *params,
                               const double *init, double *c_out, uint64_t *l_out, double *in_out, int64_t *it_out,
                               fk_fit_report *rep) {
    if (!params) return FK_ERR_NULL_POINTER;
    return guarded(ctx, [&] { return fk::fit_impl<float, double>(ctx, x, n, d, params, init, c_out, l_out, in_out, it_out, rep); });
}

fk_status fk_lloyd_step_f64(fk_ctx *ctx, const double *x, int64_t n, int64_t d, const double *c, int64_t k,
                            int32_t prec, uint64_t *l, double *nc, double *in, double *sh, fk_fit_report *rep) {
    return guarded(ctx, [&] { return fk::step_impl<double, double>(ctx, x, n, d, c, k, prec, l, nc, in, sh, rep); });
}

fk_status fk_lloyd_step_f32(fk_ctx *ctx, const float *x, int64_t n, int64_t d, const float *c, int64_t k,
                            int32_t prec, uint64_t *l, float *nc, float *in, float *sh, fk_fit_report *rep) {
    return guarded(ctx, [&] { return fk::step_impl<float, float>(ctx, x, n, d, c, k, prec, l, nc, in, sh, rep); });
}

fk_status fk_lloyd_step_f32x64(fk_ctx *ctx, const float *x, int64_t n, int64_t d, const double *c, int64_t k,
                               int32_t prec, uint64_t *l, double *nc, double *in, double *sh, fk_fit_report *rep) {
    return guarded(ctx, [&] { return fk::step_impl<float, double>(ctx, x, n, d, c, k, prec, l, nc, in, sh, rep); });
}

fk_status fk_kmeans_predict_f64(fk_ctx *ctx, const double *c, int64_t k, int64_t d_fit, const double *x, int64_t n,
                                int64_t d, int32_t prec, uint64_t *l) {
    return guarded(ctx, [&] { return fk::predict_impl<double, double>(ctx, c, k, d_fit, x, n, d, prec, l); });
}

fk_status fk_kmeans_predict_f32(fk_ctx *ctx, const float *c, int64_t k, int64_t d_fit, const float *x, int64_t n,
                                int64_t d, int32_t prec, uint64_t *l) {
    return guarded(ctx, [&] { return fk::predict_impl<float, float>(ctx, c, k, d_fit, x, n, d, prec, l); });
}

fk_status fk_kmeans_predict_f32x64(fk_ctx *ctx, const double *c, int64_t k, int64_t d_fit, const float *x, int64_t n,
                                   int64_t d, int32_t prec, uint64_t *l) {
    return guarded(ctx, [&] { return fk::predict_impl<float, double>(ctx, c, k, d_fit, x, n, d, prec, l); });
}

fk_status fk_kmeans_transform_f64(fk_ctx *ctx, const double *c, int64_t k, int64_t d_fit, const double *x, int64_t n,
                                  int64_t d, double *out) {
    return guarded(ctx, [&] { return fk::transform_impl<double>(ctx, c, k, d_fit, x, n, d, out); });
}

fk_status fk_kmeans_transform_f32(fk_ctx *ctx, const float *c, int64_t k, int64_t d_fit, const float *x, int64_t n,
                                  int64_t d, float *out) {
    return guarded(ctx, [&] { return fk::transform_impl<float>(ctx, c, k, d_fit, x, n, d, out); });
}

fk_status fk_kmeans_plus_plus_f64(fk_ctx *ctx, const double *x, int64_t n, int64_t d, int64_t k, const double *draws,
                                  int64_t n_draws, uint64_t seed, double *out, int64_t *used) {
    return guarded(ctx, [&] { return fk::kpp_impl<double>(ctx, x, n, d, k, draws, n_draws, seed, out, used); });
}

fk_status fk_debug_measure_tc_peaks(fk_ctx *ctx, double *out) {
    return guarded(ctx, [&] {
        if (!out) {
            fk::set_error("required pointer is NULL");
            return FK_ERR_NULL_POINTER;
        }
        fk::Ctx &c = *reinterpret_cast<fk::Ctx *>(ctx);
        c.bind();
        fk::measure_tc_peaks(c, out);
        return FK_OK;
    });
}

fk_status fk_debug_measure_peaks(fk_ctx *ctx, double *out) {
    return guarded(ctx, [&] {
        fk::Ctx &c = *reinterpret_cast<fk::Ctx *>(ctx);
        c.bind();
        fk::measure_peaks(c, out);
        return FK_OK;
    });
}

fk_status fk_kmeans_fit_batched_f32(fk_ctx *ctx, fk_batch_problem *problems, int64_t n_problems, int32_t reduction,
                                    fk_batch_report *report) {
    return guarded(ctx, [&] {
        return fk::batched_fit_impl(*reinterpret_cast<fk::Ctx *>(ctx), problems, n_problems, reduction, report);
    });
}

fk_status fk_debug_tc_probe(fk_ctx *ctx, const float *x_dev, int64_t n, int64_t d, const double *c_dev, int64_t k,
                             int32_t precision, float *dump, void *xq, void *cq, uint16_t *aug, uint16_t *xaug,
                             void *top, int32_t *plan) {
    return guarded(ctx, [&] {
        fk::Ctx &c = *reinterpret_cast<fk::Ctx *>(ctx);
        c.bind();
        fk::debug_tc_probe(c, x_dev, n, (int)d, c_dev, (int)k, precision, dump, xq, cq, aug, xaug, (fk::Top2 *)top,
                           plan);
        return FK_OK;
    });
}

fk_status fk_debug_tc_plan(int64_t n, int64_t d, int64_t k, int32_t precision, int32_t topk, int32_t num_sms,
                           int64_t *out) {
    if (!out) return FK_ERR_NULL_POINTER;
    if ((precision != FK_PRECISION_MIXED_BF16 && precision != FK_PRECISION_MIXED_FP8) ||
        (topk != 1 && topk != 2 && topk != 3) ||
        n < 1 || d < 1 || k < 1 || d > (1 << 16) || k > (1 << 20)) {
        fk::set_error("fk_debug_tc_plan: unsupported arguments");
        return FK_ERR_INVALID_PARAMETER;
    }
    try {
        fk::g_last_error.clear();
        fk::MixedPlan mp;
        fk::plan_shape(mp, n, (int)d, (int)k, precision == FK_PRECISION_MIXED_FP8, topk, num_sms);
        const int64_t v[10] = {mp.d_pad, mp.kp, mp.parts, mp.k_pad, mp.nblocks, mp.xst, (int64_t)mp.smem,
                               mp.grid, mp.ctas_per_part, mp.tiles};
        for (int i = 0; i < 10; i++) out[i] = v[i];
        return FK_OK;
    } catch (const fk::Error &e) {
        return e.code;
    }
}

fk_status fk_kmeans_plus_plus_f32(fk_ctx *ctx, const float *x, int64_t n, int64_t d, int64_t k, const double *draws,
                                  int64_t n_draws, uint64_t seed, float *out, int64_t *used) {
    return guarded(ctx, [&] { return fk::kpp_impl<float>(ctx, x, n, d, k, draws, n_draws, seed, out, used); });
}

}  // extern "C"
