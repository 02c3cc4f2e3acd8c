// fk_assign.cu -- direct-form assignment, transform and fixed-order sums.
//
// The direct form is sum_j (x_j - c_j)^2 folded left to right from zero with
// no fused multiply-add: exactly squared_euclidean (kmeans.rs:159-163). Every
// floating-point step below uses the _rn intrinsics, which the compiler never
// contracts, and this file is also built with -fmad=false. The argmin keeps
// the lowest index among equal distances and only accepts distances strictly
// below F::MAX, which is nearest_center's strict `<` from F::max_value()
// (kmeans.rs:295-309) for any visiting order.
#include <algorithm>
#include <cfloat>

#include "fk_internal.cuh"

namespace fk {
namespace {

template <typename T> struct Arith;
template <> struct Arith<float> {
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float maxv() { return FLT_MAX; }
    static __device__ __forceinline__ float root(float v) { return __fsqrt_rn(v); }
};
template <> struct Arith<double> {
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double maxv() { return DBL_MAX; }
    static __device__ __forceinline__ double root(double v) { return __dsqrt_rn(v); }
};

// Per-thread output tile: 8 x 8 in f32 (16 shared-memory loads per 192
// operations), 4 x 4 in f64 (its registers; the f64 direct form waits on the
// FP64 pipe, not on loads). 16 x 16 threads a block.
// The transform (every distance stored) keeps 4 x 4 in both: its stores, not
// its loads, set its pace.
template <typename TC, bool WRITE_ALL = false> struct Tile { static constexpr int TM = 8, TN = 8; };
template <bool WRITE_ALL> struct Tile<double, WRITE_ALL> { static constexpr int TM = 4, TN = 4; };
template <> struct Tile<float, true> { static constexpr int TM = 4, TN = 4; };
constexpr int DJ = 16;   // feature chunk staged in shared memory

constexpr int NT = 256;  // threads per block (16 x 16)

// Lexicographic (distance, index) order: a strictly better candidate has a
// smaller distance, or the same distance and a lower centre index.
template <typename T>
__device__ __forceinline__ bool better(T dv, int di, T bv, int bi) {
    return dv < bv || (dv == bv && di < bi);
}

// Centres [y * c_per, min(k, (y + 1) * c_per)) of split y = blockIdx.y
// against row tiles (blockIdx.x); with part_v set, each split writes
// each row's best (distance,
// index) of its range to part_v / part_i[blockIdx.y * n + row] (index
// INT32_MAX: none below F::MAX) for assign_combine_kernel, else the labels
// and minimum distances directly.
template <typename TX, typename TC, bool WRITE_ALL>
__global__ void __launch_bounds__(NT)
assign_direct_kernel(const TX *__restrict__ x, int64_t n, int d, const TC *__restrict__ c, int k,
                     int32_t *__restrict__ labels, TC *__restrict__ mind, TC *__restrict__ out, int c_per,
                     TC *__restrict__ part_v, int32_t *__restrict__ part_i) {
    constexpr int TM = Tile<TC, WRITE_ALL>::TM, TN = Tile<TC, WRITE_ALL>::TN;
    constexpr int BM = 16 * TM, BN = 16 * TN;  // rows and centres of a block tile
    static_assert(BM == BN, "the staging loop fills both tiles with one index");
    const int c_begin = (int)blockIdx.y * c_per;
    const int c_end = min(k, c_begin + c_per);
    using A = Arith<TC>;
    __shared__ __align__(16) TC xs[DJ][BM];
    __shared__ __align__(16) TC cs[DJ][BN];

    const int tid = threadIdx.x;
    const int tx = tid & 15;  // centre group
    const int ty = tid >> 4;  // row group
    const int64_t row0 = (int64_t)blockIdx.x * BM;

    TC best_v[TM];
    int best_i[TM];
#pragma unroll
    for (int a = 0; a < TM; a++) { best_v[a] = A::maxv(); best_i[a] = INT32_MAX; }

    for (int ct = c_begin; ct < c_end; ct += BN) {
        TC acc[TM][TN];
#pragma unroll
        for (int a = 0; a < TM; a++)
#pragma unroll
            for (int b = 0; b < TN; b++) acc[a][b] = TC(0);

        for (int j0 = 0; j0 < d; j0 += DJ) {
#pragma unroll
            for (int e = 0; e < (BM * DJ) / NT; e++) {
                int idx = tid + e * NT;
                int r = idx / DJ, jj = idx % DJ;
                int64_t gr = row0 + r;
                int gj = j0 + jj;
                xs[jj][r] = (gr < n && gj < d) ? (TC)x[gr * d + gj] : TC(0);
                int gc = ct + r;
                cs[jj][r] = (gc < c_end && gj < d) ? c[(int64_t)gc * d + gj] : TC(0);
            }
            __syncthreads();
            const int jn = min(DJ, d - j0);
            for (int jj = 0; jj < jn; jj++) {
                TC xv[TM], cv[TN];
#pragma unroll
                for (int a = 0; a < TM; a++) xv[a] = xs[jj][ty * TM + a];
#pragma unroll
                for (int b = 0; b < TN; b++) cv[b] = cs[jj][tx * TN + b];
#pragma unroll
                for (int a = 0; a < TM; a++)
#pragma unroll
                    for (int b = 0; b < TN; b++) {
                        TC t = A::sub(xv[a], cv[b]);
                        acc[a][b] = A::add(acc[a][b], A::mul(t, t));
                    }
            }
            __syncthreads();
        }

#pragma unroll
        for (int a = 0; a < TM; a++) {
            int64_t gr = row0 + ty * TM + a;
#pragma unroll
            for (int b = 0; b < TN; b++) {
                int gc = ct + tx * TN + b;
                if (gc < c_end) {
                    TC v = acc[a][b];
                    if (WRITE_ALL) {
                        if (gr < n) out[gr * k + gc] = A::root(v);
                    } else if (v < A::maxv() && better(v, gc, best_v[a], best_i[a])) {
                        best_v[a] = v;
                        best_i[a] = gc;
                    }
                }
            }
        }
    }
    if constexpr (!WRITE_ALL) {
        // Reduce over the 16 centre groups that share these rows (same half-warp).
#pragma unroll
        for (int a = 0; a < TM; a++) {
            TC v = best_v[a];
            int i = best_i[a];
#pragma unroll
            for (int off = 8; off >= 1; off >>= 1) {
                TC ov = __shfl_xor_sync(0xffffffffu, v, off);
                int oi = __shfl_xor_sync(0xffffffffu, i, off);
                if (better(ov, oi, v, i)) { v = ov; i = oi; }
            }
            int64_t gr = row0 + ty * TM + a;
            if (tx == 0 && gr < n) {
                if (part_v) {
                    part_v[(int64_t)blockIdx.y * n + gr] = v;
                    part_i[(int64_t)blockIdx.y * n + gr] = i;
                    continue;
                }
                if (i == INT32_MAX) { i = 0; v = A::maxv(); }  // nothing below F::MAX
                labels[gr] = i;
                if (mind) mind[gr] = v;
            }
        }
    }
}

// The splits' bests of each row in split order, lexicographic (distance,
// index): the lowest index among equal minima, as one pass over every centre.
template <typename TC>
__global__ void assign_combine_kernel(const TC *__restrict__ part_v, const int32_t *__restrict__ part_i, int splits,
                                      int64_t n, int32_t *__restrict__ labels, TC *__restrict__ mind) {
    using A = Arith<TC>;
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    TC v = A::maxv();
    int i = INT32_MAX;
    for (int q = 0; q < splits; q++) {
        const TC pv = part_v[(int64_t)q * n + r];
        const int pi = part_i[(int64_t)q * n + r];
        if (pi != INT32_MAX && better(pv, pi, v, i)) {
            v = pv;
            i = pi;
        }
    }
    if (i == INT32_MAX) { i = 0; v = A::maxv(); }
    labels[r] = i;
    if (mind) mind[r] = v;
}

// ---------------------------------------------------------- fixed sums --
constexpr int SUM_THREADS = 256;

__device__ __forceinline__ double block_sum_fixed(double v, double *sh) {
    // Fixed tree: warp butterfly, then the first warp folds the warp sums.
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (w == 0) {
        r = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) r += __shfl_xor_sync(0xffffffffu, r, off);
    }
    return r;
}

template <typename T>
__global__ void sum_partial_kernel(const T *__restrict__ v, int64_t n, int64_t per,
                                   double *__restrict__ partial) {
    __shared__ double sh[32];
    int64_t lo = (int64_t)blockIdx.x * per;
    int64_t hi = min(n, lo + per);
    double s = 0.0;
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) s += (double)v[i];
    double r = block_sum_fixed(s, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = r;
}

__global__ void sum_final_kernel(const double *__restrict__ partial, int64_t m, double *out) {
    __shared__ double sh[32];
    double s = 0.0;
    for (int64_t i = threadIdx.x; i < m; i += blockDim.x) s += partial[i];
    double r = block_sum_fixed(s, sh);
    if (threadIdx.x == 0) *out = r;
}

__global__ void labels_u64_kernel(const int32_t *__restrict__ l, int64_t n, uint64_t *__restrict__ o) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) o[i] = (uint64_t)(uint32_t)l[i];
}

template <typename TS, typename TD>
__global__ void convert_kernel(const TS *__restrict__ s, int64_t count, TD *__restrict__ d) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) d[i] = (TD)s[i];
}

}  // namespace

template <typename TX, typename TC>
void launch_assign_direct(const TX *x, int64_t n, int d, const TC *c, int k, int32_t *labels,
                          TC *mind, cudaStream_t s) {
    if (n == 0) return;
    constexpr int BM = 16 * Tile<TC>::TM;
    dim3 grid((unsigned)((n + BM - 1) / BM));
    assign_direct_kernel<TX, TC, false><<<grid, NT, 0, s>>>(x, n, d, c, k, labels, mind, nullptr, k, nullptr,
                                                            nullptr);
    FK_LAUNCH_CHECK();
}

template <typename TC>
int assign_splits(int64_t n, int k, int num_sms) {
    constexpr int BM = 16 * Tile<TC>::TM, BN = 16 * Tile<TC>::TN;
    const int64_t tiles = (n + BM - 1) / BM;
    const int64_t want = (2 * (int64_t)num_sms + tiles - 1) / tiles;  // about two CTAs per SM
    const int64_t most = (k + BN - 1) / BN;
    return (int)std::max<int64_t>(1, std::min(want, most));
}

template <typename TX, typename TC>
void launch_assign_direct_split(const TX *x, int64_t n, int d, const TC *c, int k, int32_t *labels, TC *mind,
                                int splits, TC *part_v, int32_t *part_i, cudaStream_t s) {
    if (n == 0) return;
    if (splits <= 1) {
        launch_assign_direct<TX, TC>(x, n, d, c, k, labels, mind, s);
        return;
    }
    // split q takes whole centre tiles [q * per, (q + 1) * per)
    constexpr int BM = 16 * Tile<TC>::TM, BN = 16 * Tile<TC>::TN;
    const int tiles_k = (k + BN - 1) / BN;
    const int per = (tiles_k + splits - 1) / splits * BN;
    const int used = (k + per - 1) / per;
    dim3 grid((unsigned)((n + BM - 1) / BM), (unsigned)used);
    assign_direct_kernel<TX, TC, false><<<grid, NT, 0, s>>>(x, n, d, c, k, nullptr, nullptr, nullptr, per, part_v,
                                                            part_i);
    FK_LAUNCH_CHECK();
    assign_combine_kernel<TC><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(part_v, part_i, used, n, labels, mind);
    FK_LAUNCH_CHECK();
}

template <typename T>
void launch_transform_direct(const T *x, int64_t n, int d, const T *c, int k, T *out,
                             cudaStream_t s) {
    if (n == 0) return;
    constexpr int BM = 16 * Tile<T, true>::TM;
    dim3 grid((unsigned)((n + BM - 1) / BM));
    assign_direct_kernel<T, T, true><<<grid, NT, 0, s>>>(x, n, d, c, k, nullptr, nullptr, out, k, nullptr, nullptr);
    FK_LAUNCH_CHECK();
}

// The partial count depends on n only, so the summation tree (and hence the
// rounded result) is the same on every run and every GPU.
int64_t sum_fixed_partials(int64_t n) {
    int64_t g = (n + 4095) / 4096;
    if (g < 1) g = 1;
    if (g > 1024) g = 1024;
    return g;
}

template <typename T>
void launch_sum_fixed(const T *v, int64_t n, double *partial, double *out, cudaStream_t s) {
    int64_t g = sum_fixed_partials(n);
    int64_t per = (n + g - 1) / g;
    sum_partial_kernel<T><<<(unsigned)g, SUM_THREADS, 0, s>>>(v, n, per, partial);
    FK_LAUNCH_CHECK();
    sum_final_kernel<<<1, 1024, 0, s>>>(partial, g, out);
    FK_LAUNCH_CHECK();
}

void launch_labels_to_u64(const int32_t *l, int64_t n, uint64_t *out, cudaStream_t s) {
    if (n == 0) return;
    labels_u64_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(l, n, out);
    FK_LAUNCH_CHECK();
}

template <typename TS, typename TD>
void launch_convert(const TS *src, int64_t count, TD *dst, cudaStream_t s) {
    if (count == 0) return;
    convert_kernel<TS, TD><<<(unsigned)((count + 255) / 256), 256, 0, s>>>(src, count, dst);
    FK_LAUNCH_CHECK();
}

template int assign_splits<float>(int64_t, int, int);
template int assign_splits<double>(int64_t, int, int);
template void launch_assign_direct<double, double>(const double *, int64_t, int, const double *, int,
                                                   int32_t *, double *, cudaStream_t);
template void launch_assign_direct<float, float>(const float *, int64_t, int, const float *, int,
                                                 int32_t *, float *, cudaStream_t);
template void launch_assign_direct<float, double>(const float *, int64_t, int, const double *, int,
                                                  int32_t *, double *, cudaStream_t);
template void launch_assign_direct_split<double, double>(const double *, int64_t, int, const double *, int,
                                                         int32_t *, double *, int, double *, int32_t *, cudaStream_t);
template void launch_assign_direct_split<float, float>(const float *, int64_t, int, const float *, int, int32_t *,
                                                       float *, int, float *, int32_t *, cudaStream_t);
template void launch_transform_direct<double>(const double *, int64_t, int, const double *, int,
                                              double *, cudaStream_t);
template void launch_transform_direct<float>(const float *, int64_t, int, const float *, int, float *,
                                             cudaStream_t);
template void launch_sum_fixed<double>(const double *, int64_t, double *, double *, cudaStream_t);
template void launch_sum_fixed<float>(const float *, int64_t, double *, double *, cudaStream_t);
template void launch_convert<float, double>(const float *, int64_t, double *, cudaStream_t);
template void launch_convert<double, float>(const double *, int64_t, float *, cudaStream_t);

}  // namespace fk
