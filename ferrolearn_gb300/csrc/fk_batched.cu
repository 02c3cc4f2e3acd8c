// fk_batched.cu -- many independent KMeans<f32> fits (uneven n, d, k) in one
// call: kmeans.rs:417-512 once per (problem, run), all runs at once.
//
// Layout in HBM: every problem's rows packed into one f32 buffer (16-byte
// aligned starts); per fit (problem p, run r) an n_p-long int32 scratch pair
// (labels | members, reused as the k-means++ D^2 and running-sum arrays) and
// two k x d centre buffers that alternate between iterations.
//
// Launches:
//   batch_kpp_kernel     one persistent launch; a CTA takes the next fit from
//                        a work queue (largest first) and runs greedy
//                        k-means++ for it exactly as kmeans.rs:169-253 in f32:
//                        the running sum is the reference's sequential fold
//                        (one lane, the values broadcast by shuffles), each
//                        trial's potential likewise, trials in parallel warps.
//   batch_assign_kernel  per Lloyd iteration, one persistent launch per
//                        (d, k) bucket over a queue of (fit, row range) items,
//                        largest fits first; the fit's centres in shared
//                        memory, rows in registers; direct-form f32 distances
//                        (no FMA), strict < from F::MAX. The tile shape (rows
//                        per thread x centres per pass) is the autotuner's
//                        choice for the bucket. Per item a fixed-tree f64
//                        inertia partial.
//   batch_update_kernel  per iteration, one persistent launch over the fits:
//                        counting sort of the labels (stable, eight warps over
//                        contiguous row ranges), then per (cluster, feature)
//                        either the row-order f32 sum exactly like
//                        recompute_centroids_into (kmeans.rs:358-401), or the
//                        exact sum (integer, order-free) rounded once to f64
//                        with the mean rounded once to f32; the empty cluster
//                        rule, sqrt of the max squared shift, the tol test,
//                        n_iter and the inertia (partials in item order).
// One iteration (counter reset + bucket launches + update) is captured once
// in a CUDA graph and replayed until every fit has converged or reached
// max_iter; converged fits are skipped inside the kernels.
#include <cfloat>
#include <cmath>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "fk_internal.cuh"

namespace fk {
namespace {

struct BFit {
    int64_t x_off;  // float offset of the problem's rows in the packed X
    int64_t s_off;  // offset of this fit's n-long scratch arrays
    int64_t c_off;  // float offset of this fit's two k x d centre buffers
    int32_t n, d, k, max_iter;
    float tol;
    int32_t first_item, n_items;
    int32_t trials, prob;
    uint64_t seed;
};

struct BState {
    double inertia;
    int32_t cur, n_iter, done, pad;
};

struct BItem {
    int32_t fit, lo, hi, pad;
};

constexpr int KPP_T = 256;
constexpr int KPP_TILE = 8192;  // floats of shared memory for a tile of rows (padded stride d + 1)
static_assert(KPP_TILE % 256 == 0, "tile prefetch assumes 256 threads");
constexpr int ASSIGN_T = 128;
constexpr int UPDATE_T = 256;
constexpr int NBUCKETS = 20;  // d in {8, 16, 32, 64, other} x k in {<=16, <=32, <=64, >64}
constexpr int NVARIANTS = 5;  // (rows per thread, centres per pass): (1,1) (2,1) (1,2) (2,2) (4,1)
constexpr int MAX_K = 1024, MAX_D = 256, MAX_KD = 32768;

__device__ __forceinline__ uint64_t dev_splitmix64(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
__device__ __forceinline__ double dev_uniform(uint64_t &s) {
    return (double)(dev_splitmix64(s) >> 11) * (1.0 / 9007199254740992.0);
}
__device__ __forceinline__ int dev_range(double u, int n) {
    long long i = (long long)floor(u * (double)n);
    if (i < 0) i = 0;
    if (i >= n) i = n - 1;
    return (int)i;
}

// squared_euclidean (kmeans.rs:159-163) in f32: left fold, no FMA.
__device__ __forceinline__ float sqeuc_f32(const float *__restrict__ a, const float *__restrict__ b, int d) {
    float acc = 0.f;
    for (int j = 0; j < d; j++) {
        const float t = __fsub_rn(a[j], b[j]);
        acc = __fadd_rn(acc, __fmul_rn(t, t));
    }
    return acc;
}

// ------------------------------------------------------------- k-means++ --
// First index i with cum[i] >= thr (cum is non-decreasing); n - 1 if none.
__device__ int first_reaching(const float *__restrict__ cum, int n, float thr) {
    int lo = 0, hi = n;  // answer in [lo, hi]
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (cum[mid] >= thr) hi = mid;
        else lo = mid + 1;
    }
    return lo < n ? lo : n - 1;
}

// Sequential f32 fold of v[0..n) by one warp (the reference's in-order
// sum): the warp stages 256 values at a time in its shared-memory slice
// (coalesced loads, one batch ahead), then every lane runs the same chain
// over broadcast reads; with cum, lane 0 also records each running value in
// the slice and the warp writes them out coalesced.
constexpr int FOLD_N = 256;

__device__ float warp_serial_fold(const float *__restrict__ v, int n, float *__restrict__ cum,
                                  float *__restrict__ stage, float *__restrict__ cbuf) {
    const int lane = threadIdx.x & 31;
    float run = 0.f;
    float cur[FOLD_N / 32], nxt[FOLD_N / 32];
#pragma unroll
    for (int b = 0; b < FOLD_N / 32; b++) cur[b] = b * 32 + lane < n ? v[b * 32 + lane] : 0.f;
    for (int base = 0; base < n; base += FOLD_N) {
#pragma unroll
        for (int b = 0; b < FOLD_N / 32; b++) {
            const int i = base + FOLD_N + b * 32 + lane;
            nxt[b] = i < n ? v[i] : 0.f;
        }
        __syncwarp();
#pragma unroll
        for (int b = 0; b < FOLD_N / 32; b++) stage[b * 32 + lane] = cur[b];
        __syncwarp();
        const int m = min(FOLD_N, n - base);
        if (m == FOLD_N) {
#pragma unroll 16
            for (int q = 0; q < FOLD_N / 4; q++) {
                const float4 f = reinterpret_cast<const float4 *>(stage)[q];
                run = __fadd_rn(run, f.x);
                if (cum && lane == 0) cbuf[4 * q] = run;
                run = __fadd_rn(run, f.y);
                if (cum && lane == 0) cbuf[4 * q + 1] = run;
                run = __fadd_rn(run, f.z);
                if (cum && lane == 0) cbuf[4 * q + 2] = run;
                run = __fadd_rn(run, f.w);
                if (cum && lane == 0) cbuf[4 * q + 3] = run;
            }
        } else {
            for (int e = 0; e < m; e++) {
                run = __fadd_rn(run, stage[e]);
                if (cum && lane == 0) cbuf[e] = run;
            }
        }
        if (cum) {
            __syncwarp();
#pragma unroll
            for (int b = 0; b < FOLD_N / 32; b++)
                if (b * 32 + lane < m) cum[base + b * 32 + lane] = cbuf[b * 32 + lane];
        }
#pragma unroll
        for (int b = 0; b < FOLD_N / 32; b++) cur[b] = nxt[b];
    }
    return run;
}

// Distances (direct form) of every row to ntr candidate rows (crow, ntr x d,
// shared memory) over tiles of rows staged in shared memory (coalesced loads,
// padded stride d + 1: conflict-free reads; the next tile is loaded into
// registers while the current one is scored); the (row, candidate) pairs of
// a tile are spread evenly over the threads. mode 0: mind[i] = d(x_i,
// crow[0]); mode 1: nd[t n + i] = min(d(x_i, crow[t]), mind[i]).
constexpr int KPP_PF = KPP_TILE / 256;  // prefetched floats per thread

__device__ void tile_distances(const float *__restrict__ x, int n, int d, const float *__restrict__ crow, int ntr,
                               int mode, float *__restrict__ mind, float *__restrict__ nd, float *__restrict__ tile) {
    const int tid = threadIdx.x;
    const int TR = KPP_TILE / (d + 1) < 256 ? KPP_TILE / (d + 1) : 256;  // rows per tile
    float pf[KPP_PF];
    auto fetch = [&](int i0) {
        const int cnt = min(TR, n - i0) * d;
#pragma unroll
        for (int u = 0; u < KPP_PF; u++) {
            const int e = tid + u * KPP_T;
            pf[u] = e < cnt ? x[(int64_t)i0 * d + e] : 0.f;
        }
    };
    if (n > 0) fetch(0);
    for (int i0 = 0; i0 < n; i0 += TR) {
        const int rows = min(TR, n - i0);
        __syncthreads();
#pragma unroll
        for (int u = 0; u < KPP_PF; u++) {
            const int e = tid + u * KPP_T;
            if (e < rows * d) {
                const int rr = e / d, j = e - rr * d;
                tile[rr * (d + 1) + j] = pf[u];
            }
        }
        __syncthreads();
        if (i0 + TR < n) fetch(i0 + TR);
        for (int pr = tid; pr < rows * ntr; pr += KPP_T) {
            const int r = pr % rows, t = pr / rows;
            const float *xr = tile + r * (d + 1);
            const float *cr = crow + t * d;
            float acc = 0.f;
            for (int j = 0; j < d; j++) {
                const float df = __fsub_rn(xr[j], cr[j]);
                acc = __fadd_rn(acc, __fmul_rn(df, df));
            }
            const int i = i0 + r;
            if (mode == 0) {
                mind[i] = acc;
            } else {
                const float mv = mind[i];
                nd[(int64_t)t * n + i] = acc < mv ? acc : mv;
            }
        }
    }
    __syncthreads();
}

// One CTA per fit. Per new centre: the running sum of D^2 (warp 0), the
// thresholds and candidates (thread 0), one pass over the rows computing
// min(d(x, candidate t), D^2) for every trial t into nd (the CTA's scratch),
// the trials' potentials (one warp each, sequential folds), the choice, and
// D^2 <- nd[best].
__global__ void __launch_bounds__(KPP_T) batch_kpp_kernel(const float *__restrict__ X, const BFit *__restrict__ fits,
                                                          const int *__restrict__ order, int nf, int *counter,
                                                          int *__restrict__ lab, int *__restrict__ mem,
                                                          float *__restrict__ C, float *__restrict__ nd_all,
                                                          int64_t nd_stride) {
    __shared__ int q_sh, idx_sh;
    __shared__ float total_sh;
    __shared__ int cand_sh[16];
    __shared__ float pot_sh[16], thr_sh[16];
    __shared__ float crow[8 * MAX_D];
    __shared__ float tile[KPP_TILE];
    __shared__ __align__(16) float fold_sm[KPP_T / 32][2 * FOLD_N];
    const int tid = threadIdx.x, warp = tid >> 5;
    float *stage = fold_sm[warp], *cbuf = fold_sm[warp] + FOLD_N;
    float *nd = nd_all + (int64_t)blockIdx.x * nd_stride;
    uint64_t rng = 0;  // thread 0 only
    while (true) {
        if (tid == 0) q_sh = atomicAdd(counter, 1);
        __syncthreads();
        const int q = q_sh;
        __syncthreads();
        if (q >= nf) break;
        const BFit F = fits[order[q]];
        const int n = F.n, d = F.d, k = F.k, trials = F.trials;
        const float *x = X + F.x_off;
        float *mind = reinterpret_cast<float *>(lab + F.s_off);
        float *cum = reinterpret_cast<float *>(mem + F.s_off);
        float *cen = C + F.c_off;  // buffer 0
        if (tid == 0) {
            rng = F.seed;
            idx_sh = dev_range(dev_uniform(rng), n);
        }
        __syncthreads();
        for (int j = tid; j < d; j += KPP_T) {
            const float v = x[(int64_t)idx_sh * d + j];
            cen[j] = v;
            crow[j] = v;
        }
        __syncthreads();
        if (k > 1) tile_distances(x, n, d, crow, 1, 0, mind, nullptr, tile);
        for (int c = 1; c < k; c++) {
            if (warp == 0) {
                const float total = warp_serial_fold(mind, n, cum, stage, cbuf);  // the reference's sequential f32 sum
                if ((tid & 31) == 0) total_sh = total;
            }
            __syncthreads();
            const float total = total_sh;
            if (total <= 0.f) {  // kmeans.rs:202-206: a uniform random row (NaN falls through)
                if (tid == 0) idx_sh = dev_range(dev_uniform(rng), n);
                __syncthreads();
                for (int j = tid; j < d; j += KPP_T) cen[(int64_t)c * d + j] = x[(int64_t)idx_sh * d + j];
                __syncthreads();
                continue;
            }
            if (tid == 0)  // the draws in order, one per trial (kmeans.rs:213-214)
                for (int t = 0; t < trials; t++) thr_sh[t] = __fmul_rn(__double2float_rn(dev_uniform(rng)), total);
            __syncthreads();
            if (tid < trials) cand_sh[tid] = first_reaching(cum, n, thr_sh[tid]);
            __syncthreads();
            for (int e = tid; e < trials * d; e += KPP_T) {
                const int t = e / d, j = e - t * d;
                crow[t * d + j] = x[(int64_t)cand_sh[t] * d + j];
            }
            __syncthreads();
            tile_distances(x, n, d, crow, trials, 1, mind, nd, tile);
            for (int t = warp; t < trials; t += KPP_T / 32) {
                const float pot = warp_serial_fold(nd + (int64_t)t * n, n, nullptr, stage, cbuf);
                if ((tid & 31) == 0) pot_sh[t] = pot;
            }
            __syncthreads();
            if (tid == 0) {  // strictly smallest potential, first trial on ties (kmeans.rs:239-243)
                int best = 0;
                float bp = pot_sh[0];
                for (int t = 1; t < trials; t++)
                    if (pot_sh[t] < bp) {
                        bp = pot_sh[t];
                        best = t;
                    }
                idx_sh = best;
            }
            __syncthreads();
            const int best = idx_sh;
            for (int j = tid; j < d; j += KPP_T) cen[(int64_t)c * d + j] = crow[best * d + j];
            for (int i = tid; i < n; i += KPP_T) mind[i] = nd[(int64_t)best * n + i];
            __syncthreads();
        }
    }
}

// ------------------------------------------------------------ assignment --
__device__ __forceinline__ double block_sum_f64(double v, double *sh) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0)
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) r += sh[q];
    return r;
}

// D > 0: rows of exactly D features in registers (TR per thread), CP centres
// per pass; D = 0: any d, one row and one centre at a time.
template <int D, int TR, int CP>
__global__ void __launch_bounds__(ASSIGN_T) batch_assign_kernel(const float *__restrict__ X,
                                                                const BFit *__restrict__ fits,
                                                                const BState *__restrict__ state,
                                                                const BItem *__restrict__ items, int nitems,
                                                                int *counter, const float *__restrict__ C,
                                                                int *__restrict__ lab, double *__restrict__ partial) {
    extern __shared__ float cs[];
    __shared__ int it_sh;
    __shared__ double red[ASSIGN_T / 32];
    const int tid = threadIdx.x;
    int loaded = -1;
    while (true) {
        if (tid == 0) it_sh = atomicAdd(counter, 1);
        __syncthreads();
        const int it = it_sh;
        __syncthreads();
        if (it >= nitems) break;
        const BItem I = items[it];
        const int f = I.fit;
        if (state[f].done) continue;
        const BFit F = fits[f];
        const int d = D > 0 ? D : F.d, k = F.k;
        if (f != loaded) {
            const float *src = C + F.c_off + (int64_t)state[f].cur * k * d;
            for (int e = tid; e < k * d; e += ASSIGN_T) cs[e] = src[e];
            __syncthreads();
            loaded = f;
        }
        const float *x = X + F.x_off;
        int *L = lab + F.s_off;
        double s = 0.0;
        if constexpr (D > 0) {
            for (int base = I.lo; base < I.hi; base += ASSIGN_T * TR) {
                float xr[TR][D];
                int rr[TR];
#pragma unroll
                for (int u = 0; u < TR; u++) {
                    rr[u] = base + tid + u * ASSIGN_T;
                    const bool ok = rr[u] < I.hi;
#pragma unroll
                    for (int j4 = 0; j4 < D / 4; j4++) {
                        const float4 v = ok ? reinterpret_cast<const float4 *>(x + (int64_t)rr[u] * D)[j4]
                                            : make_float4(0.f, 0.f, 0.f, 0.f);
                        xr[u][4 * j4] = v.x;
                        xr[u][4 * j4 + 1] = v.y;
                        xr[u][4 * j4 + 2] = v.z;
                        xr[u][4 * j4 + 3] = v.w;
                    }
                }
                float best[TR];
                int bi[TR];
#pragma unroll
                for (int u = 0; u < TR; u++) {
                    best[u] = FLT_MAX;
                    bi[u] = 0;
                }
                for (int c = 0; c < k; c += CP) {
                    float acc[TR][CP];
#pragma unroll
                    for (int u = 0; u < TR; u++)
#pragma unroll
                        for (int p = 0; p < CP; p++) acc[u][p] = 0.f;
#pragma unroll
                    for (int j = 0; j < D; j++) {
#pragma unroll
                        for (int p = 0; p < CP; p++) {
                            const float cv = c + p < k ? cs[(c + p) * D + j] : 0.f;
#pragma unroll
                            for (int u = 0; u < TR; u++) {
                                const float t = __fsub_rn(xr[u][j], cv);
                                acc[u][p] = __fadd_rn(acc[u][p], __fmul_rn(t, t));
                            }
                        }
                    }
#pragma unroll
                    for (int p = 0; p < CP; p++)
                        if (c + p < k)
#pragma unroll
                            for (int u = 0; u < TR; u++)
                                if (acc[u][p] < best[u]) {
                                    best[u] = acc[u][p];
                                    bi[u] = c + p;
                                }
                }
#pragma unroll
                for (int u = 0; u < TR; u++)
                    if (rr[u] < I.hi) {
                        L[rr[u]] = bi[u];
                        s += (double)best[u];
                    }
            }
        } else {
            for (int r = I.lo + tid; r < I.hi; r += ASSIGN_T) {
                const float *xr = x + (int64_t)r * d;
                float best = FLT_MAX;
                int bi = 0;
                for (int c = 0; c < k; c++) {
                    const float v = sqeuc_f32(xr, cs + c * d, d);
                    if (v < best) {
                        best = v;
                        bi = c;
                    }
                }
                L[r] = bi;
                s += (double)best;
            }
        }
        const double tot = block_sum_f64(s, red);
        if (tid == 0) partial[it] = tot;
        __syncthreads();
    }
}

// ---------------------------------------------------------------- update --
// Exact cluster sums for the f64 reduction: x = q1 2^(kb-23) + q2 2^(kb-46)
// + r2 with integer q1, q2 (the two-grid split: 2^ea <= max|x| < 2^(ea+1),
// kb = ea + 2, C1 = 1.5 2^kb, C2 = 1.5 2^(kb-23)); r2 is exact and zero
// unless |x| < 2^(ea-21), and then goes to a 128-bit fixed-point sum with F
// fraction bits (F = 124 - bitlen(n) - ea, so no sum can overflow; bits
// below 2^-F are truncated toward zero). Integer sums are order-free, so the
// result is the exact sum whatever the order, rounded once to f64.
__device__ __forceinline__ void add128u(uint64_t &lo, uint64_t &hi, uint64_t tlo, uint64_t thi) {
    asm("add.cc.u64 %0, %0, %2;\n\taddc.u64 %1, %1, %3;" : "+l"(lo), "+l"(hi) : "l"(tlo), "l"(thi));
}

__device__ __noinline__ void fixed_add_small(uint64_t &lo, uint64_t &hi, float x, int F) {
    const uint32_t b = __float_as_uint(x);
    const uint32_t ex = (b >> 23) & 0xFFu;
    if (ex == 0xFFu) return;
    const uint64_t m = (uint64_t)((b & 0x7FFFFFu) | (ex ? 0x800000u : 0u));
    const int s = (ex ? (int)ex : 1) - 150 + F;
    uint64_t tlo, thi;
    if (s >= 64) {
        tlo = 0;
        thi = m << (s - 64);
    } else if (s >= 0) {
        tlo = m << s;
        thi = s > 40 ? m >> (64 - s) : 0;
    } else {
        tlo = s > -32 ? m >> (-s) : 0;
        thi = 0;
    }
    if (b >> 31) {
        tlo = ~tlo;
        thi = ~thi;
        add128u(tlo, thi, 1ull, 0ull);
    }
    add128u(lo, hi, tlo, thi);
}

// Correctly rounded (nearest, ties to even) f64 value of the signed 128-bit
// fixed-point number (hi:lo) with F fraction bits.
__device__ double fixed128_to_double(uint64_t lo, uint64_t hi, int F) {
    const bool neg = (hi >> 63) != 0;
    if (neg) {
        lo = ~lo;
        hi = ~hi;
        add128u(lo, hi, 1ull, 0ull);
    }
    if (lo == 0 && hi == 0) return 0.0;
    const int msb = hi ? 127 - __clzll((long long)hi) : 63 - __clzll((long long)lo);
    double r;
    if (msb <= 52) {
        r = scalbn((double)lo, -F);
    } else {
        const int sh = msb - 52;  // 1 <= sh <= 75
        uint64_t mant, rem_hi, rem_lo, half_hi, half_lo;
        if (sh < 64) {
            mant = (lo >> sh) | (sh ? (hi << (64 - sh)) : 0);
            rem_lo = lo & ((1ull << sh) - 1ull);
            rem_hi = 0;
            half_lo = 1ull << (sh - 1);
            half_hi = 0;
        } else {
            mant = hi >> (sh - 64);
            rem_lo = lo;
            rem_hi = sh > 64 ? hi & ((1ull << (sh - 64)) - 1ull) : 0;
            half_lo = sh == 64 ? (1ull << 63) : 0;
            half_hi = sh > 64 ? (1ull << (sh - 65)) : 0;
        }
        const bool above = rem_hi > half_hi || (rem_hi == half_hi && rem_lo > half_lo);
        const bool tie = rem_hi == half_hi && rem_lo == half_lo;
        if (above || (tie && (mant & 1ull))) mant += 1;
        r = scalbn((double)mant, sh - F);
    }
    return neg ? -r : r;
}

__device__ __forceinline__ int bitlen64(long long v) { return 64 - __clzll(v > 0 ? v : 1); }

template <bool WIDE>
__global__ void __launch_bounds__(UPDATE_T) batch_update_kernel(const float *__restrict__ X,
                                                                const BFit *__restrict__ fits,
                                                                BState *__restrict__ state,
                                                                const int *__restrict__ order, int nf, int *counter,
                                                                float *__restrict__ C, const int *__restrict__ lab,
                                                                int *__restrict__ mem,
                                                                const double *__restrict__ partial, int *active,
                                                                const float *__restrict__ pamax) {
    constexpr int NW = UPDATE_T / 32;
    __shared__ int wrun[NW][MAX_K];
    __shared__ int hist[MAX_K], off[MAX_K];
    __shared__ int q_sh;
    __shared__ float red[NW];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned full = 0xffffffffu;
    while (true) {
        if (tid == 0) q_sh = atomicAdd(counter, 1);
        __syncthreads();
        const int q = q_sh;
        __syncthreads();
        if (q >= nf) break;
        const int f = order[q];
        if (state[f].done) continue;
        const BFit F = fits[f];
        const int n = F.n, d = F.d, k = F.k;
        const int *L = lab + F.s_off;
        int *M = mem + F.s_off;
        // counting sort, stable: warp w owns the contiguous rows [w R, (w+1) R)
        const int R = (n + NW - 1) / NW;
        const int rlo = min(n, warp * R), rhi = min(n, rlo + R);
        for (int e = tid; e < NW * k; e += UPDATE_T) wrun[e / k][e % k] = 0;
        __syncthreads();
        for (int i = rlo + lane; i < rhi; i += 32) atomicAdd(&wrun[warp][L[i]], 1);
        __syncthreads();
        for (int c = tid; c < k; c += UPDATE_T) {
            int t = 0;
            for (int w = 0; w < NW; w++) t += wrun[w][c];
            hist[c] = t;
        }
        __syncthreads();
        if (tid == 0) {
            int acc = 0;
            for (int c = 0; c < k; c++) {
                off[c] = acc;
                acc += hist[c];
            }
        }
        __syncthreads();
        for (int c = tid; c < k; c += UPDATE_T) {
            int start = off[c];
            for (int w = 0; w < NW; w++) {
                const int t = wrun[w][c];
                wrun[w][c] = start;
                start += t;
            }
        }
        __syncthreads();
        for (int base = rlo; base < rhi; base += 32) {
            const int i = base + lane;
            const int l = i < rhi ? L[i] : -1;
            const unsigned peers = __match_any_sync(full, l);
            const int leader = __ffs(peers) - 1;
            const int rank = __popc(peers & ((1u << lane) - 1u));
            int b = 0;
            if (lane == leader && l >= 0) {
                b = wrun[warp][l];
                wrun[warp][l] = b + __popc(peers);
            }
            b = __shfl_sync(full, b, leader);
            if (l >= 0) M[b + rank] = i;
        }
        __syncthreads();
        const int cur = state[f].cur;
        const float *oldc = C + F.c_off + (int64_t)cur * k * d;
        float *newc = C + F.c_off + (int64_t)(1 - cur) * k * d;
        const float *x = X + F.x_off;
        // exact-sum constants (f64 reduction)
        const float amax = WIDE ? pamax[F.prob] : 0.f;
        const int ea = amax > 0.f ? (int)((__float_as_uint(amax) >> 23) & 0xFFu) - 127 : -126;
        const bool grids = ea >= -90 && ea <= 100;
        const int kb = ea + 2;
        const int Fb = 124 - bitlen64(n) - ea;
        const float C1 = grids ? ldexpf(1.5f, kb) : 0.f, C2 = grids ? ldexpf(1.5f, kb - 23) : 0.f;
        const int b1 = __float_as_int(C1), b2 = __float_as_int(C2);
        for (int pr = tid; pr < k * d; pr += UPDATE_T) {
            const int c = pr / d, j = pr - c * d;
            const int cnt = hist[c], o = off[c];
            if (cnt == 0) {
                newc[pr] = oldc[pr];  // empty cluster keeps its centre
                continue;
            }
            // values of the cluster's rows in row order, loaded 8 ahead
            float cur8[8], nxt8[8];
#pragma unroll
            for (int u = 0; u < 8; u++) cur8[u] = u < cnt ? x[(int64_t)M[o + u] * d + j] : 0.f;
            if (WIDE) {
                long long a1 = 0, a2 = 0;
                uint64_t slo = 0, shi = 0;
                float probe = 0.f;
                for (int m = 0; m < cnt; m += 8) {
#pragma unroll
                    for (int u = 0; u < 8; u++) nxt8[u] = m + 8 + u < cnt ? x[(int64_t)M[o + m + 8 + u] * d + j] : 0.f;
#pragma unroll
                    for (int u = 0; u < 8; u++) {
                        const float xv = cur8[u];  // 0 past the end
                        probe = __fmaf_rn(xv, 0.f, probe);
                        if (grids) {
                            const float s1 = __fadd_rn(xv, C1);
                            a1 += __float_as_int(s1) - b1;
                            const float r = __fsub_rn(xv, __fsub_rn(s1, C1));
                            const float s2 = __fadd_rn(r, C2);
                            a2 += __float_as_int(s2) - b2;
                            const float r2 = __fsub_rn(r, __fsub_rn(s2, C2));
                            if (r2 != 0.f) fixed_add_small(slo, shi, r2, Fb);
                        } else {
                            fixed_add_small(slo, shi, xv, Fb);
                        }
                    }
#pragma unroll
                    for (int u = 0; u < 8; u++) cur8[u] = nxt8[u];
                }
                double sum;
                if (!(probe == 0.f)) {  // a non-finite value: IEEE f64 summation of the specials
                    uint32_t fl = 0u;
                    for (int m = 0; m < cnt; m++) {
                        const uint32_t bb = __float_as_uint(x[(int64_t)M[o + m] * d + j]);
                        if (((bb >> 23) & 0xFFu) == 0xFFu) fl |= (bb & 0x7FFFFFu) ? 1u : ((bb >> 31) ? 4u : 2u);
                    }
                    sum = ((fl & 1u) || (fl & 6u) == 6u) ? __longlong_as_double(0x7FF8000000000000LL)
                          : (fl & 2u) ? __longlong_as_double(0x7FF0000000000000LL)
                                      : __longlong_as_double((long long)0xFFF0000000000000ULL);
                } else {
                    if (grids) {
                        const __int128 v1 = (__int128)a1 << (kb - 23 + Fb);
                        const __int128 v2 = (__int128)a2 << (kb - 46 + Fb);
                        add128u(slo, shi, (uint64_t)v1, (uint64_t)((unsigned __int128)v1 >> 64));
                        add128u(slo, shi, (uint64_t)v2, (uint64_t)((unsigned __int128)v2 >> 64));
                    }
                    sum = fixed128_to_double(slo, shi, Fb);
                }
                newc[pr] = __double2float_rn(__ddiv_rn(sum, (double)cnt));
            } else {
                float acc = 0.f;
                for (int m = 0; m < cnt; m += 8) {
#pragma unroll
                    for (int u = 0; u < 8; u++) nxt8[u] = m + 8 + u < cnt ? x[(int64_t)M[o + m + 8 + u] * d + j] : 0.f;
#pragma unroll
                    for (int u = 0; u < 8; u++)
                        if (m + u < cnt) acc = __fadd_rn(acc, cur8[u]);
#pragma unroll
                    for (int u = 0; u < 8; u++) cur8[u] = nxt8[u];
                }
                newc[pr] = __fdiv_rn(acc, (float)cnt);  // counts as F are exact below 2^24
            }
        }
        __syncthreads();
        // sqrt of the largest squared shift (NaN shifts never raise it)
        float ms = 0.f;
        for (int c = tid; c < k; c += UPDATE_T) {
            const float sh = sqeuc_f32(newc + (int64_t)c * d, oldc + (int64_t)c * d, d);
            if (sh > ms) ms = sh;
        }
#pragma unroll
        for (int o2 = 16; o2 >= 1; o2 >>= 1) ms = fmaxf(ms, __shfl_xor_sync(full, ms, o2));
        if (lane == 0) red[warp] = ms;
        __syncthreads();
        if (tid == 0) {
            float m2 = 0.f;
            for (int w = 0; w < NW; w++) m2 = fmaxf(m2, red[w]);
            const float shift = __fsqrt_rn(m2);
            double in = 0.0;
            for (int it = 0; it < F.n_items; it++) in += partial[F.first_item + it];
            BState st = state[f];
            st.inertia = in;
            st.n_iter += 1;
            st.cur = 1 - cur;
            if (shift < F.tol || st.n_iter >= F.max_iter) {
                st.done = 1;
                atomicSub(active, 1);
            }
            state[f] = st;
        }
        __syncthreads();
    }
}

// max |x| over the finite values of each problem (the exact sums' scale)
__global__ void batch_amax_kernel(const float *__restrict__ X, const int64_t *__restrict__ xoff,
                                  const int64_t *__restrict__ xlen, int np, float *__restrict__ amax) {
    __shared__ float red[32];
    for (int p = blockIdx.x; p < np; p += gridDim.x) {
        const float *x = X + xoff[p];
        float m = 0.f;
        for (int64_t e = threadIdx.x; e < xlen[p]; e += blockDim.x) {
            const float a = fabsf(x[e]);
            if (a < INFINITY) m = fmaxf(m, a);
        }
#pragma unroll
        for (int o = 16; o >= 1; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
        __syncthreads();
        if (threadIdx.x == 0) {
            float r = 0.f;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) r = fmaxf(r, red[w]);
            amax[p] = r;
        }
        __syncthreads();
    }
}

__global__ void batch_labels_u64_kernel(const int *__restrict__ l, int n, uint64_t *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (uint64_t)l[i];
}

// --------------------------------------------------------------- host side --
int dbucket(int d) { return d == 8 ? 0 : d == 16 ? 1 : d == 32 ? 2 : d == 64 ? 3 : 4; }
int kbucket(int k) { return k <= 16 ? 0 : k <= 32 ? 1 : k <= 64 ? 2 : 3; }
int bucket_d(int b) { static const int v[5] = {8, 16, 32, 64, 0}; return v[b / 4]; }

using AssignFn = void (*)(const float *, const BFit *, const BState *, const BItem *, int, int *, const float *,
                          int *, double *);

template <int D>
AssignFn pick_variant(int v) {
    switch (v) {
        case 0: return batch_assign_kernel<D, 1, 1>;
        case 1: return batch_assign_kernel<D, 2, 1>;
        case 2: return batch_assign_kernel<D, 1, 2>;
        case 3: return batch_assign_kernel<D, 2, 2>;
        default: return batch_assign_kernel<D, (D <= 32 ? 4 : 2), 1>;
    }
}

AssignFn assign_fn(int bucket, int v) {
    switch (bucket_d(bucket)) {
        case 8: return pick_variant<8>(v);
        case 16: return pick_variant<16>(v);
        case 32: return pick_variant<32>(v);
        case 64: return v <= 2 ? pick_variant<64>(v) : pick_variant<64>(1);
        default: return batch_assign_kernel<0, 1, 1>;
    }
}

int n_variants(int bucket) {
    const int d = bucket_d(bucket);
    return d == 0 ? 1 : d == 64 ? 3 : NVARIANTS;
}

}  // namespace

fk_status batched_fit_impl(Ctx &ctx, fk_batch_problem *P, int64_t np, int reduction, fk_batch_report *rep) {
    if (np < 0 || (np > 0 && !P)) {
        set_error("problems is NULL or n_problems is negative");
        return FK_ERR_INVALID_PARAMETER;
    }
    if (reduction != FK_REDUCE_REFERENCE && reduction != FK_REDUCE_F64) {
        set_error("unknown reduction %d", reduction);
        return FK_ERR_INVALID_PARAMETER;
    }
    // Validation of every problem first, in the order of kmeans.rs:421-449.
    for (int64_t p = 0; p < np; p++) {
        const fk_batch_problem &q = P[p];
        if (q.n_clusters <= 0) {
            set_error("problem %lld: Invalid parameter `n_clusters`: must be at least 1", (long long)p);
            return FK_ERR_INVALID_PARAMETER;
        }
        if (q.n <= 0 || q.n < q.n_clusters) {
            set_error("problem %lld: Insufficient samples: need at least %lld, got %lld", (long long)p,
                      (long long)q.n_clusters, (long long)(q.n < 0 ? 0 : q.n));
            return FK_ERR_INSUFFICIENT_SAMPLES;
        }
        if (q.n_init <= 0) {
            set_error("problem %lld: Invalid parameter `n_init`: must be at least 1", (long long)p);
            return FK_ERR_INVALID_PARAMETER;
        }
        if (q.max_iter < 0 || q.d < 1) {
            set_error("problem %lld: Invalid parameter `max_iter`/`d`", (long long)p);
            return FK_ERR_INVALID_PARAMETER;
        }
        if (!q.x || !q.centers_out || !q.labels_out || !q.inertia_out || !q.n_iter_out) {
            set_error("problem %lld: required pointer is NULL", (long long)p);
            return FK_ERR_NULL_POINTER;
        }
        if (q.n_clusters > MAX_K || q.d > MAX_D || q.n_clusters * q.d > MAX_KD || q.n > INT32_MAX / 2 ||
            q.max_iter > INT32_MAX) {
            set_error("problem %lld: batched fits support k <= %d, d <= %d, k*d <= %d (got k=%lld d=%lld)",
                      (long long)p, MAX_K, MAX_D, MAX_KD, (long long)q.n_clusters, (long long)q.d);
            return FK_ERR_UNSUPPORTED;
        }
    }
    if (rep) {
        double *fi = rep->fit_inertia;
        int64_t *fn = rep->fit_n_iter;
        memset(rep, 0, sizeof(*rep));
        rep->fit_inertia = fi;
        rep->fit_n_iter = fn;
        for (int b = 0; b < NBUCKETS; b++) rep->bucket_variant[b] = -1;
    }
    if (np == 0) return FK_OK;
    ctx.bind();
    cudaStream_t s = ctx.stream;
    Events<6> ev;
    FK_CUDA(cudaEventRecord(ev[0], s));

    // ---- layout
    std::vector<int64_t> xoff(np);
    int64_t xtot = 0;
    for (int64_t p = 0; p < np; p++) {
        xoff[p] = xtot;
        xtot += (P[p].n * P[p].d + 3) / 4 * 4;  // 16-byte aligned starts
    }
    std::vector<BFit> fits;
    std::vector<int> fit_prob, fit_run;
    int64_t soff = 0, coff = 0;
    for (int64_t p = 0; p < np; p++) {
        const fk_batch_problem &q = P[p];
        for (int64_t r = 0; r < q.n_init; r++) {
            BFit F;
            memset(&F, 0, sizeof(F));
            F.x_off = xoff[p];
            F.s_off = soff;
            F.c_off = coff;
            F.n = (int32_t)q.n;
            F.d = (int32_t)q.d;
            F.k = (int32_t)q.n_clusters;
            F.max_iter = (int32_t)q.max_iter;
            F.tol = (float)q.tol;
            F.trials = kpp_trials_host(q.n_clusters);
            F.seed = q.random_state + (uint64_t)r;
            F.prob = (int32_t)p;
            fits.push_back(F);
            fit_prob.push_back((int)p);
            fit_run.push_back((int)r);
            soff += q.n;
            coff += 2 * q.n_clusters * q.d;
        }
    }
    const int nf = (int)fits.size();
    // work items: chunks of rows, grouped by (d, k) bucket, largest fits first
    auto cost = [&](int f) { return (double)fits[f].n * fits[f].k * fits[f].d; };
    std::vector<int> byc(nf);
    std::iota(byc.begin(), byc.end(), 0);
    std::stable_sort(byc.begin(), byc.end(), [&](int a, int b) { return cost(a) > cost(b); });
    std::vector<BItem> items;
    int bstart[NBUCKETS + 1] = {0};
    for (int b = 0; b < NBUCKETS; b++) {
        bstart[b] = (int)items.size();
        for (int f : byc) {
            BFit &F = fits[f];
            if (dbucket(F.d) * 4 + kbucket(F.k) != b) continue;
            const int ch = std::max(128, std::min(8192, (int)(4194304.0 / ((double)F.k * F.d * 3.0)) / 128 * 128));
            F.first_item = (int)items.size();
            for (int lo = 0; lo < F.n; lo += ch) items.push_back(BItem{f, lo, std::min(F.n, lo + ch), 0});
            F.n_items = (int)items.size() - F.first_item;
        }
    }
    bstart[NBUCKETS] = (int)items.size();
    std::vector<int> kpp_order;
    for (int f : byc)
        if (!P[fit_prob[f]].init) kpp_order.push_back(f);

    // ---- device buffers
    float *X = (float *)ctx.get(BUF_BX, sizeof(float) * (size_t)xtot + 16);
    BFit *dfits = (BFit *)ctx.get(BUF_BFITS, sizeof(BFit) * (size_t)nf);
    BState *dstate = (BState *)ctx.get(BUF_BSTATE, sizeof(BState) * (size_t)nf);
    BItem *ditems = (BItem *)ctx.get(BUF_BITEMS, sizeof(BItem) * items.size() + 16);
    double *dpart = (double *)ctx.get(BUF_BPART, sizeof(double) * items.size() + 16);
    int *dorder = (int *)ctx.get(BUF_BORDER, sizeof(int) * (size_t)(2 * nf) + 16);
    int *dctr = (int *)ctx.get(BUF_BCTR, sizeof(int) * 32);
    int *dlab = (int *)ctx.get(BUF_BLAB, sizeof(int) * (size_t)soff + 16);
    int *dmem = (int *)ctx.get(BUF_BMEM, sizeof(int) * (size_t)soff + 16);
    float *dC = (float *)ctx.get(BUF_BCEN, sizeof(float) * (size_t)coff + 16);
    int64_t *dxo = (int64_t *)ctx.get(BUF_BXOFF, sizeof(int64_t) * (size_t)(2 * np) + sizeof(float) * (size_t)np + 64);
    float *damax = (float *)(dxo + 2 * np);
    for (int64_t p = 0; p < np; p++)
        FK_CUDA(cudaMemcpyAsync(X + xoff[p], P[p].x, sizeof(float) * (size_t)(P[p].n * P[p].d), cudaMemcpyDefault,
                                s));
    FK_CUDA(cudaMemcpyAsync(dfits, fits.data(), sizeof(BFit) * (size_t)nf, cudaMemcpyHostToDevice, s));
    {
        std::vector<int64_t> xol(2 * np);
        for (int64_t p = 0; p < np; p++) {
            xol[p] = xoff[p];
            xol[np + p] = P[p].n * P[p].d;
        }
        FK_CUDA(cudaMemcpyAsync(dxo, xol.data(), sizeof(int64_t) * xol.size(), cudaMemcpyHostToDevice, s));
        FK_CUDA(cudaStreamSynchronize(s));  // xol is host stack memory
        batch_amax_kernel<<<(unsigned)std::min<int64_t>(np, ctx.num_sms * 4), 256, 0, s>>>(X, dxo, dxo + np, (int)np,
                                                                                        damax);
        FK_LAUNCH_CHECK();
    }
    if (!items.empty())
        FK_CUDA(cudaMemcpyAsync(ditems, items.data(), sizeof(BItem) * items.size(), cudaMemcpyHostToDevice, s));
    std::vector<int> orders(byc);
    orders.insert(orders.end(), kpp_order.begin(), kpp_order.end());
    FK_CUDA(cudaMemcpyAsync(dorder, orders.data(), sizeof(int) * orders.size(), cudaMemcpyHostToDevice, s));
    std::vector<BState> st0(nf);
    int active = 0;
    for (int f = 0; f < nf; f++) {
        st0[f].inertia = (double)FLT_MAX;
        st0[f].cur = 0;
        st0[f].n_iter = 0;
        st0[f].done = fits[f].max_iter == 0 ? 1 : 0;
        st0[f].pad = 0;
        active += st0[f].done ? 0 : 1;
    }
    FK_CUDA(cudaMemcpyAsync(dstate, st0.data(), sizeof(BState) * (size_t)nf, cudaMemcpyHostToDevice, s));
    FK_CUDA(cudaMemsetAsync(dlab, 0, sizeof(int) * (size_t)soff, s));
    FK_CUDA(cudaMemsetAsync(dctr, 0, sizeof(int) * 32, s));
    FK_CUDA(cudaMemcpyAsync(dctr + 31, &active, sizeof(int), cudaMemcpyHostToDevice, s));
    for (int f = 0; f < nf; f++) {
        const fk_batch_problem &q = P[fit_prob[f]];
        if (q.init) {
            const int64_t run = fit_run[f];
            FK_CUDA(cudaMemcpyAsync(dC + fits[f].c_off, q.init + run * q.n_clusters * q.d,
                                    sizeof(float) * (size_t)(q.n_clusters * q.d), cudaMemcpyDefault, s));
        }
    }
    FK_CUDA(cudaEventRecord(ev[1], s));

    // ---- k-means++ (one persistent launch)
    if (!kpp_order.empty()) {
        const int grid = std::min((int)kpp_order.size(), ctx.num_sms * 2);
        int64_t nmax_kpp = 1;
        for (int f : kpp_order) nmax_kpp = std::max<int64_t>(nmax_kpp, fits[f].n);
        const int64_t nd_stride = 8 * nmax_kpp;  // trials <= 8 (k <= 1024)
        float *nd = (float *)ctx.get(BUF_BND, sizeof(float) * (size_t)(nd_stride * grid));
        batch_kpp_kernel<<<grid, KPP_T, 0, s>>>(X, dfits, dorder + nf, (int)kpp_order.size(), dctr + 30, dlab, dmem,
                                                dC, nd, nd_stride);
        FK_LAUNCH_CHECK();
        // k-means++ used the label arrays as scratch: fits that run no
        // iteration report all-zero labels (kmeans.rs:459-466)
        for (int f = 0; f < nf; f++)
            if (fits[f].max_iter == 0)
                FK_CUDA(cudaMemsetAsync(dlab + fits[f].s_off, 0, sizeof(int) * (size_t)fits[f].n, s));
    }
    FK_CUDA(cudaEventRecord(ev[2], s));

    // ---- autotuner: time every variant of each new (d, k) bucket on its items
    int bmaxkd[NBUCKETS] = {0};
    for (const BFit &F : fits) {
        const int b = dbucket(F.d) * 4 + kbucket(F.k);
        bmaxkd[b] = std::max(bmaxkd[b], F.k * F.d);
    }
    int64_t tuned = 0;
    for (int b = 0; b < NBUCKETS; b++) {
        const int cnt = bstart[b + 1] - bstart[b];
        if (cnt == 0) continue;
        const size_t smem = sizeof(float) * (size_t)bmaxkd[b];
        for (int v = 0; v < n_variants(b); v++)
            FK_CUDA(cudaFuncSetAttribute((const void *)assign_fn(b, v), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)std::max<size_t>(smem, 1)));
        if (ctx.batch_variant[b] >= 0) continue;
        const int grid = std::min(cnt, ctx.num_sms * 8);
        float bestms = 1e30f;
        int bestv = 0;
        for (int v = 0; v < n_variants(b); v++) {
            FK_CUDA(cudaMemsetAsync(dctr + b, 0, sizeof(int), s));
            FK_CUDA(cudaEventRecord(ev[4], s));
            assign_fn(b, v)<<<grid, ASSIGN_T, smem, s>>>(X, dfits, dstate, ditems + bstart[b], cnt, dctr + b, dC,
                                                          dlab, dpart + bstart[b]);
            FK_LAUNCH_CHECK();
            FK_CUDA(cudaEventRecord(ev[5], s));
            FK_CUDA(cudaEventSynchronize(ev[5]));
            float ms = 0.f;
            FK_CUDA(cudaEventElapsedTime(&ms, ev[4], ev[5]));
            if (ms < bestms) {
                bestms = ms;
                bestv = v;
            }
        }
        ctx.batch_variant[b] = bestv;
        tuned++;
    }
    FK_CUDA(cudaEventRecord(ev[3], s));

    // ---- Lloyd iterations: one captured iteration, replayed
    auto one_iteration = [&]() {
        FK_CUDA(cudaMemsetAsync(dctr, 0, sizeof(int) * 21, s));
        for (int b = 0; b < NBUCKETS; b++) {
            const int cnt = bstart[b + 1] - bstart[b];
            if (cnt == 0) continue;
            const int grid = std::min(cnt, ctx.num_sms * 8);
            assign_fn(b, ctx.batch_variant[b])<<<grid, ASSIGN_T, sizeof(float) * (size_t)bmaxkd[b], s>>>(
                X, dfits, dstate, ditems + bstart[b], cnt, dctr + b, dC, dlab, dpart + bstart[b]);
        }
        const int ug = std::min(nf, ctx.num_sms * 4);
        if (reduction == FK_REDUCE_F64)
            batch_update_kernel<true><<<ug, UPDATE_T, 0, s>>>(X, dfits, dstate, dorder, nf, dctr + 20, dC, dlab,
                                                              dmem, dpart, dctr + 31, damax);
        else
            batch_update_kernel<false><<<ug, UPDATE_T, 0, s>>>(X, dfits, dstate, dorder, nf, dctr + 20, dC, dlab,
                                                               dmem, dpart, dctr + 31, damax);
    };
    int max_iter = 0;
    for (const BFit &F : fits) max_iter = std::max(max_iter, F.max_iter);
    int64_t replays = 0;
    if (active > 0) {
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        FK_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        try {
            one_iteration();
        } catch (...) {
            // end the capture so that the caller's stream stays usable
            cudaGraph_t partial = nullptr;
            (void)cudaStreamEndCapture(s, &partial);
            if (partial) cudaGraphDestroy(partial);
            (void)cudaGetLastError();
            throw;
        }
        cudaError_t ce = cudaStreamEndCapture(s, &graph);
        if (ce != cudaSuccess) {
            set_error("graph capture failed: %s", cudaGetErrorString(ce));
            fail(FK_ERR_CUDA);
        }
        ce = cudaGraphInstantiate(&exec, graph, 0);
        if (ce != cudaSuccess) {
            cudaGraphDestroy(graph);
            set_error("graph instantiation failed: %s", cudaGetErrorString(ce));
            fail(FK_ERR_CUDA);
        }
        int left = active;
        const int group = 4;  // replays between checks of the active count
        while (left > 0 && replays < max_iter) {
            const int g = (int)std::min<int64_t>(group, max_iter - replays);
            for (int r = 0; r < g; r++) {
                ce = cudaGraphLaunch(exec, s);
                if (ce != cudaSuccess) break;
                replays++;
            }
            if (ce == cudaSuccess) ce = cudaMemcpyAsync(&left, dctr + 31, sizeof(int), cudaMemcpyDeviceToHost, s);
            if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
            if (ce != cudaSuccess) break;
        }
        cudaGraphExecDestroy(exec);
        cudaGraphDestroy(graph);
        if (ce != cudaSuccess) {
            set_error("batched Lloyd iterations failed: %s", cudaGetErrorString(ce));
            fail(FK_ERR_CUDA);
        }
    }
    FK_CUDA(cudaEventRecord(ev[4], s));

    // ---- best run per problem (strictly lowest inertia, first run on ties), outputs
    std::vector<BState> st(nf);
    FK_CUDA(cudaMemcpyAsync(st.data(), dstate, sizeof(BState) * (size_t)nf, cudaMemcpyDeviceToHost, s));
    FK_CUDA(cudaStreamSynchronize(s));
    int64_t nmax = 1;
    for (int64_t p = 0; p < np; p++) nmax = std::max(nmax, P[p].n);
    uint64_t *l64 = (uint64_t *)ctx.get(BUF_OUT, sizeof(uint64_t) * (size_t)nmax);
    int64_t iters = 0;
    for (int f = 0; f < nf; f++) iters += st[f].n_iter;
    int f0 = 0;
    for (int64_t p = 0; p < np; p++) {
        const fk_batch_problem &q = P[p];
        int best = -1;
        float bi = 0.f;
        for (int64_t r = 0; r < q.n_init; r++) {
            const float in = (float)st[f0 + r].inertia;
            if (best < 0 || in < bi) {
                best = (int)r;
                bi = in;
            }
        }
        const int f = f0 + best;
        const BFit &F = fits[f];
        FK_CUDA(cudaMemcpyAsync(q.centers_out, dC + F.c_off + (int64_t)st[f].cur * F.k * F.d,
                                sizeof(float) * (size_t)(F.k * F.d), cudaMemcpyDefault, s));
        batch_labels_u64_kernel<<<(F.n + 255) / 256, 256, 0, s>>>(dlab + F.s_off, F.n, l64);
        FK_LAUNCH_CHECK();
        FK_CUDA(cudaMemcpyAsync(q.labels_out, l64, sizeof(uint64_t) * (size_t)F.n, cudaMemcpyDefault, s));
        FK_CUDA(cudaStreamSynchronize(s));  // l64 is reused by the next problem
        *q.inertia_out = bi;
        *q.n_iter_out = st[f].n_iter;
        if (q.best_run_out) *q.best_run_out = best;
        f0 += (int)q.n_init;
    }
    FK_CUDA(cudaEventRecord(ev[5], s));
    FK_CUDA(cudaEventSynchronize(ev[5]));
    if (rep) {
        rep->fits = nf;
        rep->iterations_total = iters;
        rep->graph_launches = replays;
        rep->tuned_buckets = tuned;
        for (int b = 0; b < NBUCKETS; b++)
            rep->bucket_variant[b] = bstart[b + 1] > bstart[b] ? ctx.batch_variant[b] : -1;
        float ms = 0.f;
        FK_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
        rep->ms_upload = ms;
        FK_CUDA(cudaEventElapsedTime(&ms, ev[1], ev[2]));
        rep->ms_init = ms;
        FK_CUDA(cudaEventElapsedTime(&ms, ev[2], ev[3]));
        rep->ms_tune = ms;
        FK_CUDA(cudaEventElapsedTime(&ms, ev[3], ev[4]));
        rep->ms_lloyd = ms;
        FK_CUDA(cudaEventElapsedTime(&ms, ev[4], ev[5]));
        rep->ms_download = ms;
        FK_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[5]));
        rep->ms_total = ms;
        for (int f = 0; f < nf; f++) {
            if (rep->fit_inertia) rep->fit_inertia[f] = st[f].inertia;
            if (rep->fit_n_iter) rep->fit_n_iter[f] = st[f].n_iter;
        }
    }
    return FK_OK;
}

}  // namespace fk
