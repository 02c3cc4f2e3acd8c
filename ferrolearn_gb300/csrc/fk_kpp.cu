// fk_kpp.cu -- greedy k-means++ on the GPU (kmeans.rs:169-253).
//
// Per new centre, with no host round trip: fixed-order block sums of the D^2
// array, a single-block pass that forms the total, reads the next uniform
// draws and turns each into a threshold u * total (in F, as kmeans.rs:213-214),
// one block per trial that finds the first row whose running sum reaches the
// threshold (the sequential cumsum of kmeans.rs:215-223), a pass that forms
// min(D^2, d(x, candidate)) for every trial and its potential, and a choice of
// the strictly smallest potential (first trial wins ties, kmeans.rs:239-243).
// A non-positive total takes one uniform draw as a random row
// (kmeans.rs:202-206). Distances are the direct form with no FMA, identical
// to the reference; the sums are exact-order-independent fixed trees in f64,
// so a candidate can differ from a sequential fold only when a threshold
// falls within rounding of a running-sum boundary.
#include <cfloat>
#include <cmath>

#include "fk_internal.cuh"

namespace fk {
namespace {

template <typename T> __device__ __forceinline__ T kpp_sub(T a, T b);
template <> __device__ __forceinline__ float kpp_sub(float a, float b) { return __fsub_rn(a, b); }
template <> __device__ __forceinline__ double kpp_sub(double a, double b) { return __dsub_rn(a, b); }
template <typename T> __device__ __forceinline__ T kpp_mul(T a, T b);
template <> __device__ __forceinline__ float kpp_mul(float a, float b) { return __fmul_rn(a, b); }
template <> __device__ __forceinline__ double kpp_mul(double a, double b) { return __dmul_rn(a, b); }
template <typename T> __device__ __forceinline__ T kpp_add(T a, T b);
template <> __device__ __forceinline__ float kpp_add(float a, float b) { return __fadd_rn(a, b); }
template <> __device__ __forceinline__ double kpp_add(double a, double b) { return __dadd_rn(a, b); }

template <typename T>
__device__ __forceinline__ T sqeuc(const T *__restrict__ a, const T *__restrict__ b, int d) {
    T acc = T(0);
    for (int j = 0; j < d; j++) {
        T t = kpp_sub(a[j], b[j]);
        acc = kpp_add(acc, kpp_mul(t, t));
    }
    return acc;
}

constexpr int KPP_BLOCK = 4096;  // rows per partial sum
constexpr int KPP_THREADS = 256;
constexpr int MAX_TRIALS = 16;

struct KppState {
    long long cursor;             // uniform draws consumed so far
    int direct;                   // 1 = this centre was a uniform random row
    int best_trial;
    long long cand[MAX_TRIALS];   // candidate row per trial
    double thr[MAX_TRIALS];       // threshold per trial (value of F, widened)
    double total;
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// Fixed tree over the block: per-warp butterflies, then warp 0 folds.
__device__ double block_sum(double v, double *sh) {
    v = warp_sum(v);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (w == 0) {
        r = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
        r = warp_sum(r);
    }
    return r;
}

__device__ __forceinline__ long long draw_to_range(double u, long long n) {
    long long i = (long long)floor(u * (double)n);
    if (i < 0) i = 0;
    if (i >= n) i = n - 1;
    return i;
}

template <typename T>
__global__ void kpp_first_kernel(const T *__restrict__ x, long long n, int d, const double *__restrict__ draws,
                                 long long n_draws, KppState *st, T *__restrict__ centers) {
    // Single block: pick the first row, copy it.
    __shared__ long long first;
    if (threadIdx.x == 0) {
        double u = n_draws > 0 ? draws[0] : 0.0;
        first = draw_to_range(u, n);
        st->cursor = 1;
    }
    __syncthreads();
    for (int j = threadIdx.x; j < d; j += blockDim.x) centers[j] = x[first * d + j];
}

template <typename T>
__global__ void kpp_init_mind_kernel(const T *__restrict__ x, long long n, int d, const T *__restrict__ c0,
                                     T *__restrict__ mind) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) mind[i] = sqeuc(x + i * d, c0, d);
}

template <typename T>
__global__ void kpp_partial_kernel(const T *__restrict__ v, long long n, double *__restrict__ part) {
    __shared__ double sh[32];
    long long lo = (long long)blockIdx.x * KPP_BLOCK, hi = min(n, lo + KPP_BLOCK);
    double s = 0.0;
    for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) s += (double)v[i];
    double r = block_sum(s, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = r;
}

// Single block: total, thresholds, draw consumption, block prefix sums.
template <typename T>
__global__ void kpp_select_kernel(const double *__restrict__ part, long long nb, double *__restrict__ bpre,
                                  const double *__restrict__ draws, long long n_draws, int n_trials, long long n,
                                  KppState *st) {
    __shared__ double sh[33];
    __shared__ double carry;
    if (threadIdx.x == 0) carry = 0.0;
    __syncthreads();
    // Exclusive prefix of the partial sums (fixed order, chunk by chunk).
    for (long long b0 = 0; b0 < nb; b0 += blockDim.x) {
        long long i = b0 + threadIdx.x;
        double v = i < nb ? part[i] : 0.0;
        // inclusive warp scan
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        double inc = v;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            double t = __shfl_up_sync(0xffffffffu, inc, off);
            if (lane >= off) inc += t;
        }
        if (lane == 31) sh[w] = inc;
        __syncthreads();
        if (threadIdx.x == 0) {
            double run = 0.0;
            for (int q = 0; q < (int)(blockDim.x >> 5); q++) {
                double t = sh[q];
                sh[q] = run;
                run += t;
            }
            sh[32] = run;
        }
        __syncthreads();
        if (i < nb) bpre[i] = carry + sh[w] + inc - v;
        __syncthreads();
        if (threadIdx.x == 0) carry += sh[32];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        bpre[nb] = carry;
        T total = (T)carry;
        st->total = (double)total;
        long long cur = st->cursor;
        if (!(total > T(0))) {
            double u = cur < n_draws ? draws[cur] : 0.0;
            st->direct = 1;
            st->cand[0] = draw_to_range(u, n);
            cur += 1;
        } else {
            st->direct = 0;
            for (int t = 0; t < n_trials; t++) {
                double u = cur < n_draws ? draws[cur] : 0.0;
                T thr = (T)u * total;
                st->thr[t] = (double)thr;
                cur += 1;
            }
        }
        st->cursor = cur;
    }
}

// One block per trial: first row whose running sum reaches the threshold.
template <typename T>
__global__ void kpp_find_kernel(const T *__restrict__ mind, long long n, const double *__restrict__ bpre,
                                long long nb, KppState *st) {
    if (st->direct) return;
    const int t = blockIdx.x;
    __shared__ double sh[33];
    __shared__ long long found;
    __shared__ long long b_start;
    const double thr = st->thr[t];
    if (threadIdx.x == 0) {
        // first block whose inclusive prefix reaches thr (binary search)
        long long lo = 0, hi = nb - 1, ans = nb;
        while (lo <= hi) {
            long long mid = (lo + hi) >> 1;
            if (bpre[mid + 1] >= thr) { ans = mid; hi = mid - 1; } else lo = mid + 1;
        }
        b_start = ans;
        found = -1;
    }
    __syncthreads();
    for (long long b = b_start; b < nb; b++) {
        double run = bpre[b];
        long long lo = b * KPP_BLOCK, hi = min(n, lo + KPP_BLOCK);
        for (long long c0 = lo; c0 < hi; c0 += blockDim.x) {
            long long i = c0 + threadIdx.x;
            double v = i < hi ? (double)mind[i] : 0.0;
            const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
            double inc = v;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                double tt = __shfl_up_sync(0xffffffffu, inc, off);
                if (lane >= off) inc += tt;
            }
            if (lane == 31) sh[w] = inc;
            __syncthreads();
            if (threadIdx.x == 0) {
                double r2 = 0.0;
                for (int q = 0; q < (int)(blockDim.x >> 5); q++) {
                    double tt = sh[q];
                    sh[q] = r2;
                    r2 += tt;
                }
                sh[32] = r2;
            }
            __syncthreads();
            double cum = run + sh[w] + inc;
            bool hit = (i < hi) && (cum >= thr);
            unsigned m = __ballot_sync(0xffffffffu, hit);
            if (lane == 0 && m) atomicMin((unsigned long long *)&found, (unsigned long long)(c0 + w * 32 + __ffs(m) - 1));
            __syncthreads();
            if (found >= 0) break;
            run += sh[32];
            __syncthreads();
        }
        if (found >= 0) break;
    }
    if (threadIdx.x == 0) st->cand[t] = found >= 0 ? found : n - 1;
}

// New distances and per-block potential partials for every trial.
template <typename T>
__global__ void kpp_trial_kernel(const T *__restrict__ x, long long n, int d, const T *__restrict__ mind,
                                 int n_trials, const KppState *st, T *__restrict__ nd, double *__restrict__ pot,
                                 long long nb) {
    if (st->direct) return;
    __shared__ double sh[32];
    long long lo = (long long)blockIdx.x * KPP_BLOCK, hi = min(n, lo + KPP_BLOCK);
    for (int t = 0; t < n_trials; t++) {
        const T *cand = x + st->cand[t] * d;
        double s = 0.0;
        for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) {
            T v = sqeuc(x + i * d, cand, d);
            T m = mind[i];
            T r = v < m ? v : m;
            nd[(long long)t * n + i] = r;
            s += (double)r;
        }
        double r = block_sum(s, sh);
        if (threadIdx.x == 0) pot[(long long)t * nb + blockIdx.x] = r;
    }
}

template <typename T>
__global__ void kpp_choose_kernel(const T *__restrict__ x, int d, const double *__restrict__ pot, long long nb,
                                  int n_trials, KppState *st, T *__restrict__ center_out) {
    __shared__ double sh[32];
    __shared__ int best;
    if (!st->direct) {
        T best_p = T(0);
        int bt = -1;
        for (int t = 0; t < n_trials; t++) {
            double s = 0.0;
            for (long long b = threadIdx.x; b < nb; b += blockDim.x) s += pot[(long long)t * nb + b];
            double r = block_sum(s, sh);
            if (threadIdx.x == 0) {
                T p = (T)r;
                if (bt < 0 || p < best_p) { bt = t; best_p = p; }
            }
        }
        if (threadIdx.x == 0) { best = bt; st->best_trial = bt; }
    } else if (threadIdx.x == 0) {
        best = -1;
        st->best_trial = -1;
    }
    __syncthreads();
    long long row = st->cand[best < 0 ? 0 : best];
    for (int j = threadIdx.x; j < d; j += blockDim.x) center_out[j] = x[row * d + j];
}

template <typename T>
__global__ void kpp_commit_kernel(T *__restrict__ mind, const T *__restrict__ nd, long long n, const KppState *st) {
    if (st->direct) return;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) mind[i] = nd[(long long)st->best_trial * n + i];
}

}  // namespace

int kpp_trials(int k) {
    long long t = 2 + (long long)std::floor(std::log((double)k));
    if (t < 1) t = 1;
    return (int)t;
}

template <typename T>
void run_kmeanspp(Ctx &ctx, const T *x, int64_t n, int d, int k, const double *draws_dev, int64_t n_draws,
                  T *centers_out, int64_t *draws_used) {
    cudaStream_t s = ctx.stream;
    const int n_trials = kpp_trials(k);
    if (n_trials > MAX_TRIALS) {
        set_error("k-means++ with k=%d needs %d trials (max %d)", k, n_trials, MAX_TRIALS);
        fail(FK_ERR_UNSUPPORTED);
    }
    FK_CUDA(cudaMemsetAsync(centers_out, 0, sizeof(T) * (size_t)k * d, s));
    const long long nb = (n + KPP_BLOCK - 1) / KPP_BLOCK;
    auto *st = (KppState *)ctx.get(BUF_KPP0, sizeof(KppState));
    T *mind = (T *)ctx.get(BUF_KPP1, sizeof(T) * (size_t)n);
    T *nd = (T *)ctx.get(BUF_KPP2, sizeof(T) * (size_t)n * n_trials);
    double *part = (double *)ctx.get(BUF_KPP3, sizeof(double) * (size_t)(nb * (n_trials + 1) + nb + 1));
    double *pot = part + nb;
    double *bpre = pot + nb * n_trials;
    FK_CUDA(cudaMemsetAsync(st, 0, sizeof(KppState), s));

    kpp_first_kernel<T><<<1, 128, 0, s>>>(x, n, d, draws_dev, n_draws, st, centers_out);
    FK_LAUNCH_CHECK();
    if (k > 1) {
        kpp_init_mind_kernel<T><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(x, n, d, centers_out, mind);
        FK_LAUNCH_CHECK();
    }
    for (int c = 1; c < k; c++) {
        kpp_partial_kernel<T><<<(unsigned)nb, KPP_THREADS, 0, s>>>(mind, n, part);
        FK_LAUNCH_CHECK();
        kpp_select_kernel<T><<<1, 1024, 0, s>>>(part, nb, bpre, draws_dev, n_draws, n_trials, n, st);
        FK_LAUNCH_CHECK();
        kpp_find_kernel<T><<<n_trials, 1024, 0, s>>>(mind, n, bpre, nb, st);
        FK_LAUNCH_CHECK();
        kpp_trial_kernel<T><<<(unsigned)nb, KPP_THREADS, 0, s>>>(x, n, d, mind, n_trials, st, nd, pot, nb);
        FK_LAUNCH_CHECK();
        kpp_choose_kernel<T><<<1, 1024, 0, s>>>(x, d, pot, nb, n_trials, st, centers_out + (int64_t)c * d);
        FK_LAUNCH_CHECK();
        kpp_commit_kernel<T><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(mind, nd, n, st);
        FK_LAUNCH_CHECK();
    }
    if (draws_used) {
        long long cur = 0;
        FK_CUDA(cudaMemcpyAsync(&cur, &st->cursor, sizeof(cur), cudaMemcpyDeviceToHost, s));
        FK_CUDA(cudaStreamSynchronize(s));
        *draws_used = cur;
    }
}

template void run_kmeanspp<double>(Ctx &, const double *, int64_t, int, int, const double *, int64_t, double *,
                                   int64_t *);
template void run_kmeanspp<float>(Ctx &, const float *, int64_t, int, int, const double *, int64_t, float *,
                                  int64_t *);

}  // namespace fk
