// fk_update.cu -- centroid update: stable counting sort by cluster, then one
// sequential row-order sum per (cluster, feature) -- the exact summation order
// of recompute_centroids_into (kmeans.rs:370-375) -- so the new centres are
// bit-identical to the reference's for F = f32 and F = f64. Then divide, keep
// the old centre of an empty cluster (kmeans.rs:378-386) and take the max
// squared shift (kmeans.rs:389-400).
//
// Sort: rows are cut into segments of seg_len rows; one warp per segment
// counts labels (shared-memory histogram), an exclusive scan over the
// (cluster-major, segment-minor) count matrix gives every (cluster, segment)
// its output offset, and a second pass scatters row indices in row order
// (warp match + prefix popcount keeps equal labels in lane order). The
// result: members[] lists each cluster's rows in increasing row index.
//
// The mixed precisions (f32 X, f64 centres) sum exactly instead: integer
// sums on two grids plus 128-bit fixed-point remainders, rounded once to f64
// (centroid_fixed_part4_kernel). Those sums can be kept and updated from the
// rows whose label changed (label_diff / moved_scatter / exact_delta4 /
// exact_means), which a fit does after its first two iterations; it then
// computes the inertia of the assignment it keeps once, from the rows
// (row_inertia4_kernel).
#include <algorithm>

#include <type_traits>

#include "fk_internal.cuh"

namespace fk {
namespace {

// --------------------------------------------------------------- scan --
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

// Exclusive scan of one value per thread across the block; returns the
// prefix, and the block total in *total.
__device__ __forceinline__ int block_excl_scan(int v, int *sh, int *total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int incl = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += t;
    }
    if (lane == 31) sh[w] = incl;
    __syncthreads();
    if (w == 0) {
        int nw = blockDim.x >> 5;
        int s = lane < nw ? sh[lane] : 0;
        int si = s;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, si, off);
            if (lane >= off) si += t;
        }
        if (lane < nw) sh[lane] = si - s;  // exclusive warp offsets
        if (lane == nw - 1) sh[32] = si;
    }
    __syncthreads();
    int r = sh[w] + incl - v;
    *total = sh[32];
    __syncthreads();
    return r;
}

__global__ void scan_reduce_kernel(const int32_t *__restrict__ a, int64_t m, int32_t *__restrict__ bsum) {
    __shared__ int sh[33];
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
    int s = 0;
#pragma unroll
    for (int e = 0; e < SCAN_ITEMS; e++)
        if (base + e < m) s += a[base + e];
    int total;
    block_excl_scan(s, sh, &total);
    if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

__global__ void scan_top_kernel(int32_t *__restrict__ bsum, int64_t nb) {
    __shared__ int sh[33];
    int carry = 0;
    for (int64_t b0 = 0; b0 < nb; b0 += SCAN_THREADS) {
        int64_t i = b0 + threadIdx.x;
        int v = i < nb ? bsum[i] : 0;
        int total;
        int ex = block_excl_scan(v, sh, &total);
        if (i < nb) bsum[i] = carry + ex;
        carry += total;
    }
}

__global__ void scan_down_kernel(int32_t *__restrict__ a, int64_t m, const int32_t *__restrict__ bsum) {
    __shared__ int sh[33];
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
    int v[SCAN_ITEMS];
    int s = 0;
#pragma unroll
    for (int e = 0; e < SCAN_ITEMS; e++) {
        v[e] = base + e < m ? a[base + e] : 0;
        s += v[e];
    }
    int total;
    int ex = block_excl_scan(s, sh, &total) + bsum[blockIdx.x];
#pragma unroll
    for (int e = 0; e < SCAN_ITEMS; e++) {
        if (base + e < m) a[base + e] = ex;
        ex += v[e];
    }
}

// --------------------------------------------------------- segment sort --
__global__ void seg_hist_kernel(const int32_t *__restrict__ labels, int64_t n, int k, int64_t seg_len,
                                int64_t nseg, int32_t *__restrict__ hist) {
    extern __shared__ int cnt[];
    const int lane = threadIdx.x;
    const int64_t s = blockIdx.x;
    for (int c = lane; c < k; c += 32) cnt[c] = 0;
    __syncwarp();
    int64_t lo = s * seg_len, hi = min(n, lo + seg_len);
    for (int64_t i = lo + lane; i < hi; i += 32) atomicAdd(&cnt[labels[i]], 1);
    __syncwarp();
    for (int c = lane; c < k; c += 32) hist[(int64_t)c * nseg + s] = cnt[c];
}

__global__ void seg_scatter_kernel(const int32_t *__restrict__ labels, int64_t n, int k, int64_t seg_len,
                                   int64_t nseg, const int32_t *__restrict__ offs,
                                   int32_t *__restrict__ members) {
    extern __shared__ int cnt[];
    const int lane = threadIdx.x;
    const int64_t s = blockIdx.x;
    for (int c = lane; c < k; c += 32) cnt[c] = offs[(int64_t)c * nseg + s];
    __syncwarp();
    const unsigned lt = (1u << lane) - 1u;
    int64_t lo = s * seg_len, hi = min(n, lo + seg_len);
    for (int64_t base = lo; base < hi; base += 32) {
        int64_t i = base + lane;
        bool active = i < hi;
        unsigned act = __ballot_sync(0xffffffffu, active);
        int rank = 0, l = 0;
        unsigned peers = 0;
        if (active) {
            l = labels[i];
            peers = __match_any_sync(act, l);
            rank = __popc(peers & lt);
            members[cnt[l] + rank] = (int32_t)i;
        }
        __syncwarp();
        if (active && rank == 0) cnt[l] += __popc(peers);
        __syncwarp();
    }
}

// ------------------------------------------------------- centroid sums --
template <typename T> struct UArith;
template <> struct UArith<float> {
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
};
template <> struct UArith<double> {
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
};

constexpr int UPD_R = 32;  // member rows loaded per batch

// One block per (cluster, feature slab); thread j keeps the running sum of
// feature j over the cluster's rows in row order. With INERTIA, thread j also
// accumulates (x_ij - c_j)^2 against the old centre in compensated f32
// (Kahan), for the mixed precisions' inertia.
template <typename TX, typename TC, bool INERTIA>
__global__ void centroid_sum_kernel(const TX *__restrict__ x, int d, int k, int64_t n,
                                    const int32_t *__restrict__ members,
                                    const int32_t *__restrict__ offs, int64_t nseg,
                                    const TC *__restrict__ old_c, TC *__restrict__ new_c,
                                    double *__restrict__ inertia_part) {
    using A = UArith<TC>;
    __shared__ int32_t sidx[UPD_R];
    const int c = blockIdx.x;
    const int j = blockIdx.y * blockDim.x + threadIdx.x;
    const int64_t start = offs[(int64_t)c * nseg];
    const int64_t end = (c + 1 < k) ? (int64_t)offs[(int64_t)(c + 1) * nseg] : n;
    TC s = TC(0);
    float isum = 0.f, icomp = 0.f;
    const float cj = (INERTIA && j < d) ? (float)old_c[(int64_t)c * d + j] : 0.f;
    for (int64_t base = start; base < end; base += UPD_R) {
        const int cnt = (int)min((int64_t)UPD_R, end - base);
        __syncthreads();
        if (threadIdx.x < UPD_R && threadIdx.x < cnt) sidx[threadIdx.x] = members[base + threadIdx.x];
        __syncthreads();
        if (j < d) {
            TX v[UPD_R];
#pragma unroll
            for (int r = 0; r < UPD_R; r++) v[r] = r < cnt ? x[(int64_t)sidx[r] * d + j] : TX(0);
#pragma unroll
            for (int r = 0; r < UPD_R; r++)
                if (r < cnt) s = A::add(s, (TC)v[r]);
            if (INERTIA) {
#pragma unroll
                for (int r = 0; r < UPD_R; r++) {
                    if (r < cnt) {
                        float df = __fsub_rn((float)v[r], cj);
                        float y = __fsub_rn(__fmul_rn(df, df), icomp);
                        float t = __fadd_rn(isum, y);
                        icomp = __fsub_rn(__fsub_rn(t, isum), y);
                        isum = t;
                    }
                }
            }
        }
    }
    if (j < d) {
        const int64_t cntc = end - start;
        new_c[(int64_t)c * d + j] = cntc > 0 ? A::div(s, (TC)cntc) : old_c[(int64_t)c * d + j];
        if (INERTIA) inertia_part[(int64_t)c * d + j] = (double)isum - (double)icomp;
    }
}

// Plain update (KMeans<f32> and KMeans<f64>): the same row-order chain in F
// per (cluster, feature), but fed from shared memory. A block takes one
// cluster and a slab of 32 features; all its threads load a page of member
// rows (two rows a thread for f32, one for f64; the slab's features
// contiguous, 16-byte loads when the rows allow) while warp 0 adds the
// previous page from shared memory, one lane per feature. One warp loading
// for itself keeps a few dozen rows in flight and a long chain waits on
// memory; here the block's loads set the pace and the chain runs at the
// dependent-add rate. Rows are padded to 33 values in shared memory so that
// neither the row-wise stores nor the column-wise reads conflict in a bank.
constexpr int CH_THREADS = 256;
constexpr int CH_SW = 32;  // features per block
constexpr int CH_PITCH = CH_SW + 1;
template <typename T> struct ChainPage { static constexpr int rows = 512; };  // two rows a thread
template <> struct ChainPage<double> { static constexpr int rows = 256; };    // one: the registers
template <typename T>
size_t chain_smem_bytes() { return sizeof(T) * (size_t)ChainPage<T>::rows * CH_PITCH; }

template <typename T>
__global__ void __launch_bounds__(CH_THREADS)
    centroid_chain_kernel(const T *__restrict__ x, int d, int k, int64_t n, const int32_t *__restrict__ members,
                          const int32_t *__restrict__ offs, int64_t nseg, const T *__restrict__ old_c,
                          T *__restrict__ new_c) {
    using A = UArith<T>;
    constexpr int PAGE = ChainPage<T>::rows;
    constexpr int RPT = PAGE / CH_THREADS;      // rows a thread
    constexpr int VW = 16 / (int)sizeof(T);     // values per 16-byte load
    extern __shared__ __align__(16) unsigned char ch_raw[];
    T *ch_page = reinterpret_cast<T *>(ch_raw);
    const int c = blockIdx.x;
    const int j0 = blockIdx.y * CH_SW;
    const int sw = min(CH_SW, d - j0);
    const int lane = threadIdx.x & 31;
    const int64_t start = offs[(int64_t)c * nseg];
    const int64_t end = (c + 1 < k) ? (int64_t)offs[(int64_t)(c + 1) * nseg] : n;
    // j0 is a multiple of 32: the slab starts on a 16-byte boundary when the rows do
    const bool vec = sw == CH_SW && (d % VW) == 0 && (((uintptr_t)x) & 15u) == 0;
    T v[RPT][CH_SW];
    auto load_page = [&](int64_t base) {
#pragma unroll
        for (int h = 0; h < RPT; h++) {
            const int64_t r = base + threadIdx.x + h * CH_THREADS;
            if (r < end) {
                const T *row = x + (int64_t)members[r] * d + j0;
                if (vec) {
#pragma unroll
                    for (int q = 0; q < CH_SW / VW; q++) {
                        const uint4 u = reinterpret_cast<const uint4 *>(row)[q];
                        const T *e = reinterpret_cast<const T *>(&u);
#pragma unroll
                        for (int t = 0; t < VW; t++) v[h][VW * q + t] = e[t];
                    }
                } else {
#pragma unroll
                    for (int f = 0; f < CH_SW; f++) v[h][f] = f < sw ? row[f] : T(0);
                }
            }
        }
    };
    T s = T(0);
    int64_t base = start;
    if (base < end) load_page(base);
    while (base < end) {
        const int cnt = (int)min((int64_t)PAGE, end - base);
        __syncthreads();  // the previous page has been added
#pragma unroll
        for (int h = 0; h < RPT; h++) {
            const int r = threadIdx.x + h * CH_THREADS;
            if (r < cnt) {
#pragma unroll
                for (int f = 0; f < CH_SW; f++) ch_page[r * CH_PITCH + f] = v[h][f];
            }
        }
        __syncthreads();
        const int64_t next = base + PAGE;
        if (next < end) load_page(next);  // in flight while warp 0 adds this page
        if (threadIdx.x < 32 && lane < sw) {
            const T *col = ch_page + lane;
#pragma unroll 8
            for (int r = 0; r < cnt; r++) s = A::add(s, col[r * CH_PITCH]);
        }
        base = next;
    }
    if (threadIdx.x < 32 && lane < sw) {
        const int64_t cntc = end - start;
        const int64_t o = (int64_t)c * d + j0 + lane;
        new_c[o] = cntc > 0 ? A::div(s, (T)cntc) : old_c[o];
    }
}

// ----------------------------------------------- exact fixed-point sums --
// Mixed precisions (X stored f32, centres f64): every f32 value is an
// integer multiple of 2^-149, so the cluster sums can be formed EXACTLY in
// 128-bit fixed point with F fraction bits, F chosen from n and max |x| so no
// partial sum can overflow (values below 2^-F, far under any centroid's
// precision, are truncated). The exact sum is rounded once to f64 and then
// divided by the count like kmeans.rs:381; the result is the correctly
// rounded mean of the exact sum -- it equals the reference's sequential f64
// sum whenever that sum is exact (the usual case for f32 inputs) and differs
// by at most a few ulp otherwise. Integer addition is associative, so the
// rows are processed in any order without changing the result.
struct FixedAcc {
    uint64_t plo, phi;  // sum of the positive values
    uint64_t nlo, nhi;  // sum of the magnitudes of the negative values
    uint32_t flags;     // 1 = NaN seen, 2 = +inf seen, 4 = -inf seen
};

__device__ __forceinline__ void add128(uint64_t &lo, uint64_t &hi, uint64_t tlo, uint64_t thi) {
    asm("add.cc.u64 %0, %0, %2;\n\taddc.u64 %1, %1, %3;" : "+l"(lo), "+l"(hi) : "l"(tlo), "l"(thi));
}

__device__ __forceinline__ void fixed_add(FixedAcc &a, float x, int F) {
    const uint32_t b = __float_as_uint(x);
    const uint32_t ex = (b >> 23) & 0xFFu;
    if (ex == 0xFFu) {
        a.flags |= (b & 0x7FFFFFu) ? 1u : ((b >> 31) ? 4u : 2u);
        return;
    }
    const uint64_t m = (uint64_t)((b & 0x7FFFFFu) | (ex ? 0x800000u : 0u));
    const int s = (ex ? (int)ex : 1) - 150 + F;  // x = m * 2^(s - F); m < 2^24, s <= 101
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
    if (b >> 31)
        add128(a.nlo, a.nhi, tlo, thi);
    else
        add128(a.plo, a.phi, tlo, thi);
}

// Correctly rounded (to nearest, ties to even) f64 value of a signed 128-bit
// fixed-point number with F fraction bits.
__device__ double fixed_to_double(unsigned __int128 a, int F) {
    const bool neg = (a >> 127) != 0;
    unsigned __int128 u = neg ? (unsigned __int128)0 - a : a;
    if (u == 0) return 0.0;
    const uint64_t hi = (uint64_t)(u >> 64), lo = (uint64_t)u;
    const int msb = hi ? 127 - __clzll((long long)hi) : 63 - __clzll((long long)lo);
    double r;
    if (msb <= 52) {
        r = (double)(uint64_t)u;  // exact
        r = scalbn(r, -F);
    } else {
        int sh = msb - 52;
        uint64_t mant = (uint64_t)(u >> sh);
        const unsigned __int128 rem = u - ((unsigned __int128)mant << sh);
        const unsigned __int128 half = (unsigned __int128)1 << (sh - 1);
        if (rem > half || (rem == half && (mant & 1ull))) mant += 1;
        r = scalbn((double)mant, sh - F);  // mant <= 2^53 is exact in f64
    }
    return neg ? -r : r;
}

constexpr int FIX_R = 64;       // member rows whose indices are staged per batch
constexpr int FIX_SPLIT = 16;   // at most this many blocks per cluster (gridDim.y; the sums are order-free)
constexpr int FIX_U = 8;        // rows loaded ahead per thread

struct alignas(16) FixedPart {
    unsigned long long lo, hi;  // signed 128-bit partial sum (two's complement)
    double inert;               // partial inertia (compensated f32 sums, folded in f64)
    uint32_t flags, pad;
};

// Signed 128-bit fixed-point accumulation of one finite value (non-finite
// values are skipped: the caller detects them separately).
__device__ __noinline__ void fixed_add_signed(uint64_t &lo, uint64_t &hi, float x, int F) {
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
    if (b >> 31) {  // two's complement of the 128-bit magnitude
        tlo = ~tlo;
        thi = ~thi;
        add128(tlo, thi, 1ull, 0ull);
    }
    add128(lo, hi, tlo, thi);
}

__device__ __forceinline__ int fixed_bits(const float *amax_ptr, int64_t n) {
    // fraction bits: n * max|x| * 2^F < 2^126, so no partial sum can overflow
    const float amax = *amax_ptr;
    const int ea = amax > 0.f ? (int)((__float_as_uint(amax) >> 23) & 0xFFu) - 127 : -126;
    const int ln = 64 - __clzll((long long)(n > 0 ? n : 1));
    return 124 - ln - ea;
}

// Block (cluster c, part y) sums feature j over its share of the cluster's
// rows exactly, and the compensated-f32 inertia partial against the old centre.
__global__ void centroid_fixed_part_kernel(const float *__restrict__ x, int d, int k, int64_t n,
                                           const int32_t *__restrict__ members, const int32_t *__restrict__ offs,
                                           int64_t nseg, const double *__restrict__ old_c,
                                           const float *__restrict__ amax_ptr, FixedPart *__restrict__ parts) {
    __shared__ int32_t sidx[FIX_R];
    const int c = blockIdx.x, y = blockIdx.y;
    const int j = blockIdx.z * blockDim.x + threadIdx.x;
    const int64_t cstart = offs[(int64_t)c * nseg];
    const int64_t cend = (c + 1 < k) ? (int64_t)offs[(int64_t)(c + 1) * nseg] : n;
    const int64_t share = (cend - cstart + gridDim.y - 1) / gridDim.y;
    const int64_t start = cstart + (int64_t)y * share;
    const int64_t end = min(cend, start + share);
    const int F = fixed_bits(amax_ptr, n);
    FixedAcc a{0, 0, 0, 0, 0u};
    float isum = 0.f, icomp = 0.f;
    const float cj = j < d ? (float)old_c[(int64_t)c * d + j] : 0.f;
    for (int64_t base = start; base < end; base += FIX_R) {
        const int cnt = (int)min((int64_t)FIX_R, end - base);
        __syncthreads();
        for (int t = threadIdx.x; t < cnt; t += blockDim.x) sidx[t] = members[base + t];
        __syncthreads();
        if (j < d) {
            for (int r0 = 0; r0 < cnt; r0 += FIX_U) {
                float v[FIX_U];
#pragma unroll
                for (int u = 0; u < FIX_U; u++) v[u] = r0 + u < cnt ? x[(int64_t)sidx[r0 + u] * d + j] : 0.f;
#pragma unroll
                for (int u = 0; u < FIX_U; u++) {
                    if (r0 + u < cnt) {
                        fixed_add(a, v[u], F);
                        const float df = __fsub_rn(v[u], cj);
                        const float yy = __fsub_rn(__fmul_rn(df, df), icomp);
                        const float tt = __fadd_rn(isum, yy);
                        icomp = __fsub_rn(__fsub_rn(tt, isum), yy);
                        isum = tt;
                    }
                }
            }
        }
    }
    if (j < d) {
        unsigned long long lo = a.plo, hi = a.phi;
        asm("sub.cc.u64 %0, %0, %2;\n\tsubc.u64 %1, %1, %3;" : "+l"(lo), "+l"(hi) : "l"(a.nlo), "l"(a.nhi));
        parts[((int64_t)c * gridDim.y + y) * d + j] = FixedPart{lo, hi, (double)isum - (double)icomp, a.flags, 0u};
    }
}

// Vectorised form for d % 4 == 0 (16-byte aligned X): thread (g, sl) owns the
// four features of float4 slot sl and the rows g, g + G, ... of the block's
// share (G = 256 / (d / 4) row groups), four rows in flight; the groups'
// exact sums are then added in shared memory (integer adds: order-free) and
// their inertia partials folded in group order (deterministic).
//
// Exact split on two grids instead of per-element shifts: with 2^ea <= max|x|
// < 2^(ea+1), kb = ea + 2 and C1 = 1.5 * 2^kb, every finite |x| < 2^kb / 2, so
// x + C1 stays in [2^kb, 2^(kb+1)] and its bit pattern minus that of C1 is
// the integer q1 = round(x / 2^(kb-23)) (|q1| <= 2^22); r = x - ((x + C1) - C1)
// is exact with |r| <= 2^(kb-24), and the same step on C2 = 1.5 * 2^(kb-23)
// gives q2 (unit 2^(kb-46)) and an exact remainder r2, which is zero unless
// |x| < 2^(ea-21); the rare non-zero r2 goes through fixed_add. So
// x = q1 2^(kb-23) + q2 2^(kb-46) + r2 exactly, and the sums of q1, q2 are
// integers. Non-finite values are detected with x * 0 (NaN for inf and NaN)
// and their flags recomputed from the rows. The inertia term sums (x - c)^2
// of four rows in f32 and adds that to a compensated (Kahan) f32 sum.
constexpr int FIX4_THREADS = 256;
constexpr int FIX4_U = 4;      // rows per thread and step
constexpr int FIX4_IDX = 1024; // member indices staged per chunk
constexpr int TAIL_CAP = 512;  // remainders listed per block before falling back to a rescan

struct FixRed {
    uint64_t lo[4], hi[4];
    double inert[4];
    uint32_t flags[4];
};

// signed 128-bit v = a * 2^sh (sh >= 0) added to (lo, hi)
__device__ __forceinline__ void add_shifted(uint64_t &lo, uint64_t &hi, long long a, int sh) {
    const __int128 v = (__int128)a << sh;
    add128(lo, hi, (uint64_t)v, (uint64_t)((unsigned __int128)v >> 64));
}

__global__ void __launch_bounds__(FIX4_THREADS, 3) centroid_fixed_part4_kernel(
    const float *__restrict__ x, int d, int k, int64_t n, const int32_t *__restrict__ members,
    const int32_t *__restrict__ offs, int64_t nseg, const double *__restrict__ old_c,
    const float *__restrict__ amax_ptr, FixedPart *__restrict__ parts) {
    __shared__ FixRed red[FIX4_THREADS];
    __shared__ int32_t sidx[FIX4_IDX];
    __shared__ float tail_v[TAIL_CAP];
    __shared__ int tail_f[TAIL_CAP];
    __shared__ int tail_n;
    const int S = d >> 2;
    const int G = FIX4_THREADS / S;
    const int g = (int)threadIdx.x / S, sl = (int)threadIdx.x % S;
    const bool active = g < G;
    const int c = blockIdx.x, y = blockIdx.y;
    const int64_t cstart = offs[(int64_t)c * nseg];
    const int64_t cend = (c + 1 < k) ? (int64_t)offs[(int64_t)(c + 1) * nseg] : n;
    const int64_t share = (cend - cstart + gridDim.y - 1) / gridDim.y;
    const int64_t start = cstart + (int64_t)y * share;
    const int64_t end = min(cend, start + share);
    const int F = fixed_bits(amax_ptr, n);
    const float amax = *amax_ptr;
    const int ea = amax > 0.f ? (int)((__float_as_uint(amax) >> 23) & 0xFFu) - 127 : -126;
    // grids of the split; outside this exponent range every value takes the exact slow path
    const bool grids = ea >= -90 && ea <= 100;
    const int kb = ea + 2;
    const float C1 = grids ? ldexpf(1.5f, kb) : 0.f, C2 = grids ? ldexpf(1.5f, kb - 23) : 0.f;
    const int b1 = __float_as_int(C1), b2 = __float_as_int(C2);
    long long acc1[4], acc2[4];
    uint64_t slo[4], shi[4];
    if (threadIdx.x == 0) tail_n = 0;
    float isum[4], icomp[4], cj[4], probe[4];
#pragma unroll
    for (int f = 0; f < 4; f++) {
        acc1[f] = acc2[f] = 0;
        slo[f] = shi[f] = 0;
        isum[f] = icomp[f] = probe[f] = 0.f;
        cj[f] = active ? (float)old_c[(int64_t)c * d + 4 * sl + f] : 0.f;
    }
    // the block's member indices are staged in shared memory; the row loads of
    // the next step are issued before the current step is processed
    for (int64_t cb = start; cb < end; cb += FIX4_IDX) {
        const int cnt = (int)min((int64_t)FIX4_IDX, end - cb);
        __syncthreads();
        for (int t = threadIdx.x; t < cnt; t += FIX4_THREADS) sidx[t] = members[cb + t];
        __syncthreads();
        if (!active) continue;
        float4 cur[FIX4_U], nxt[FIX4_U];
#pragma unroll
        for (int u = 0; u < FIX4_U; u++) {
            const int r = g + u * G;
            cur[u] = r < cnt ? reinterpret_cast<const float4 *>(x + (int64_t)sidx[r] * d)[sl]
                             : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        for (int r0 = g; r0 < cnt; r0 += G * FIX4_U) {
#pragma unroll
            for (int u = 0; u < FIX4_U; u++) {
                const int r = r0 + (u + FIX4_U) * G;
                nxt[u] = r < cnt ? reinterpret_cast<const float4 *>(x + (int64_t)sidx[r] * d)[sl]
                                 : make_float4(0.f, 0.f, 0.f, 0.f);
            }
            float pf[4] = {0.f, 0.f, 0.f, 0.f};
            uint32_t q1s[4] = {0u, 0u, 0u, 0u}, q2s[4] = {0u, 0u, 0u, 0u};  // wrap harmlessly without grids
#pragma unroll
            for (int u = 0; u < FIX4_U; u++) {
                const bool valid = r0 + u * G < cnt;
                const float e[4] = {cur[u].x, cur[u].y, cur[u].z, cur[u].w};
#pragma unroll
                for (int f = 0; f < 4; f++) {
                    const float xv = e[f];  // rows past the end read as 0
                    probe[f] = __fmaf_rn(xv, 0.f, probe[f]);
                    const float s1 = __fadd_rn(xv, C1);
                    q1s[f] += __float_as_uint(s1) - (uint32_t)b1;
                    const float r = __fsub_rn(xv, __fsub_rn(s1, C1));
                    const float s2 = __fadd_rn(r, C2);
                    q2s[f] += __float_as_uint(s2) - (uint32_t)b2;
                    const float r2 = __fsub_rn(r, __fsub_rn(s2, C2));
                    if (r2 != 0.f) {  // rare: |x| < 2^(ea-21); kept for the exact path below
                        const int slot = atomicAdd(&tail_n, 1);
                        if (slot < TAIL_CAP) {
                            tail_v[slot] = r2;
                            tail_f[slot] = 4 * sl + f;
                        }
                    }
                    const float df = __fsub_rn(xv, cj[f]);
                    pf[f] = valid ? __fmaf_rn(df, df, pf[f]) : pf[f];
                }
            }
#pragma unroll
            for (int f = 0; f < 4; f++) {
                acc1[f] += (int32_t)q1s[f];
                acc2[f] += (int32_t)q2s[f];
                const float yy = __fsub_rn(pf[f], icomp[f]);
                const float tt = __fadd_rn(isum[f], yy);
                icomp[f] = __fsub_rn(__fsub_rn(tt, isum[f]), yy);
                isum[f] = tt;
            }
#pragma unroll
            for (int u = 0; u < FIX4_U; u++) cur[u] = nxt[u];
        }
    }
    // rare remainders (|x| < 2^(ea-21)) go through the exact 128-bit path:
    // from the block's list, or -- when the list overflowed or the grids do
    // not apply -- by scoring this thread's rows again
    __syncthreads();
    const int tn = tail_n;
    if (g == 0 && active && tn <= TAIL_CAP) {
        for (int e = 0; e < tn; e++) {
            const int fe = tail_f[e];
            if ((fe >> 2) != sl) continue;
#pragma unroll
            for (int f = 0; f < 4; f++)
                if ((fe & 3) == f) fixed_add_signed(slo[f], shi[f], tail_v[e], F);
        }
    }
    if (active && (tn > TAIL_CAP || !grids)) {
        for (int64_t cb = start; cb < end; cb += FIX4_IDX) {
            const int cnt = (int)min((int64_t)FIX4_IDX, end - cb);
            for (int r = g; r < cnt; r += G) {
                const float4 v = reinterpret_cast<const float4 *>(x + (int64_t)members[cb + r] * d)[sl];
                const float e[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                for (int f = 0; f < 4; f++) {
                    float rem = e[f];
                    if (grids) {
                        const float s1 = __fadd_rn(e[f], C1);
                        const float rr = __fsub_rn(e[f], __fsub_rn(s1, C1));
                        const float s2 = __fadd_rn(rr, C2);
                        rem = __fsub_rn(rr, __fsub_rn(s2, C2));
                    }
                    if (rem != 0.f) fixed_add_signed(slo[f], shi[f], rem, F);
                }
            }
        }
    }
    FixRed mine;
#pragma unroll
    for (int f = 0; f < 4; f++) {
        uint64_t lo = slo[f], hi = shi[f];
        if (grids) {
            add_shifted(lo, hi, acc1[f], kb - 23 + F);  // kb - 23 + F = 103 - log2 n >= 72
            add_shifted(lo, hi, acc2[f], kb - 46 + F);
        }
        uint32_t fl = 0u;
        if (active && !(probe[f] == 0.f)) {
            // a non-finite value in this thread's rows: recompute its flags
            for (int64_t r = start + g; r < end; r += G) {
                const float xv = x[(int64_t)members[r] * d + 4 * sl + f];
                const uint32_t bb = __float_as_uint(xv);
                if (((bb >> 23) & 0xFFu) == 0xFFu) fl |= (bb & 0x7FFFFFu) ? 1u : ((bb >> 31) ? 4u : 2u);
            }
        }
        mine.lo[f] = lo;
        mine.hi[f] = hi;
        mine.inert[f] = (double)isum[f] - (double)icomp[f];
        mine.flags[f] = fl;
    }
    red[threadIdx.x] = mine;
    __syncthreads();
    if (g == 0) {
        FixRed t = red[sl];
        for (int gg = 1; gg < G; gg++) {
            const FixRed &o = red[gg * S + sl];
#pragma unroll
            for (int f = 0; f < 4; f++) {
                add128(t.lo[f], t.hi[f], o.lo[f], o.hi[f]);
                t.inert[f] += o.inert[f];
                t.flags[f] |= o.flags[f];
            }
        }
#pragma unroll
        for (int f = 0; f < 4; f++)
            parts[((int64_t)c * gridDim.y + y) * d + 4 * sl + f] =
                FixedPart{t.lo[f], t.hi[f], t.inert[f], t.flags[f], 0u};
    }
}

// Per (cluster, feature): exact sum of the parts, rounded once to f64, then
// divided by the count (empty cluster: keep the old centre); the inertia
// partials folded in a fixed order.
__global__ void centroid_fixed_combine_kernel(int d, int k, int splits, int64_t n, const int32_t *__restrict__ offs,
                                              int64_t nseg,
                                              const double *__restrict__ old_c, double *__restrict__ new_c,
                                              const float *__restrict__ amax_ptr, const FixedPart *__restrict__ parts,
                                              double *__restrict__ inertia_part, ExactState *__restrict__ state,
                                              long long *__restrict__ counts) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)k * d) return;
    const int c = (int)(idx / d), j = (int)(idx % d);
    const int64_t cstart = offs[(int64_t)c * nseg];
    const int64_t cend = (c + 1 < k) ? (int64_t)offs[(int64_t)(c + 1) * nseg] : n;
    const int F = fixed_bits(amax_ptr, n);
    unsigned long long lo = 0, hi = 0;
    uint32_t fl = 0;
    double inert = 0.0;
    for (int y = 0; y < splits; y++) {
        const FixedPart q = parts[((int64_t)c * splits + y) * d + j];
        asm("add.cc.u64 %0, %0, %2;\n\taddc.u64 %1, %1, %3;" : "+l"(lo), "+l"(hi) : "l"(q.lo), "l"(q.hi));
        fl |= q.flags;
        inert += q.inert;
    }
    const int64_t cntc = cend - cstart;
    double mean;
    if (cntc == 0) {
        mean = old_c[idx];
    } else {
        double sum;
        if ((fl & 1u) || (fl & 6u) == 6u) sum = __longlong_as_double(0x7FF8000000000000LL);
        else if (fl & 2u) sum = __longlong_as_double(0x7FF0000000000000LL);
        else if (fl & 4u) sum = __longlong_as_double((long long)0xFFF0000000000000ULL);
        else sum = fixed_to_double(((unsigned __int128)hi << 64) | lo, F);
        mean = __ddiv_rn(sum, (double)cntc);
    }
    new_c[idx] = mean;
    inertia_part[idx] = inert;
    if (state) {  // the exact sums and counts that later iterations update incrementally
        state[idx] = ExactState{lo, hi};
        if (j == 0) counts[c] = cntc;
    }
}

// squared_euclidean(new, old) per cluster, folded over j; max over clusters as
// raw bits (non-negative IEEE values order like unsigned integers). NaN
// shifts are skipped, as `shift > max_shift` is false for NaN.
template <typename TC> struct ShiftBits;
template <> struct ShiftBits<double> {
    static __device__ __forceinline__ unsigned long long bits(double v) {
        return (unsigned long long)__double_as_longlong(v);
    }
};
template <> struct ShiftBits<float> {
    static __device__ __forceinline__ unsigned long long bits(float v) {
        return (unsigned long long)(unsigned)__float_as_uint(v);
    }
};

// One warp per cluster: the lanes form the squares (x - y)^2 of the features
// in parallel (coalesced loads) into shared memory, then one lane adds them
// in feature order -- the same left fold as the one-thread form below.
constexpr int SHIFT_THREADS = 256;

template <typename TC>
__global__ void __launch_bounds__(SHIFT_THREADS)
    max_shift_warp_kernel(const TC *__restrict__ new_c, const TC *__restrict__ old_c, int k, int d,
                          unsigned long long *shift_bits) {
    using A = UArith<TC>;
    extern __shared__ unsigned char shift_smem[];
    TC *sq = reinterpret_cast<TC *>(shift_smem) + (size_t)(threadIdx.x >> 5) * d;
    const int lane = threadIdx.x & 31;
    const int c = blockIdx.x * (SHIFT_THREADS / 32) + (threadIdx.x >> 5);
    if (c >= k) return;  // warp-uniform; no block barrier below
    for (int j = lane; j < d; j += 32) {
        const TC t = A::sub(new_c[(int64_t)c * d + j], old_c[(int64_t)c * d + j]);
        sq[j] = A::mul(t, t);
    }
    __syncwarp();
    if (lane == 0) {
        TC acc = TC(0);
        for (int j = 0; j < d; j++) acc = A::add(acc, sq[j]);
        if (acc > TC(0)) atomicMax(shift_bits, ShiftBits<TC>::bits(acc));
    }
}


template <typename TC>
__global__ void max_shift_kernel(const TC *__restrict__ new_c, const TC *__restrict__ old_c, int k, int d,
                                 unsigned long long *shift_bits) {
    using A = UArith<TC>;
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= k) return;
    TC acc = TC(0);
    for (int j = 0; j < d; j++) {
        TC t = A::sub(new_c[(int64_t)c * d + j], old_c[(int64_t)c * d + j]);
        acc = A::add(acc, A::mul(t, t));
    }
    if (acc > TC(0)) atomicMax(shift_bits, ShiftBits<TC>::bits(acc));
}

template <typename TC>
void launch_max_shift(const TC *new_c, const TC *old_c, int k, int d, unsigned long long *shift_bits, cudaStream_t s) {
    const size_t smem = sizeof(TC) * (size_t)d * (SHIFT_THREADS / 32);
    if (smem <= 48 * 1024) {
        max_shift_warp_kernel<TC><<<(k + SHIFT_THREADS / 32 - 1) / (SHIFT_THREADS / 32), SHIFT_THREADS, smem, s>>>(
            new_c, old_c, k, d, shift_bits);
    } else {
        max_shift_kernel<TC><<<(k + 127) / 128, 128, 0, s>>>(new_c, old_c, k, d, shift_bits);
    }
    FK_LAUNCH_CHECK();
}

// ------------------------------------------------ incremental exact sums --
// The mixed path's cluster sums are exact integers (the two-grid split plus
// the 128-bit fixed-point remainders, see centroid_fixed_part4_kernel), so
// once they are known for one assignment, the sums of the next one follow
// from the rows whose label changed: each such row is taken out of its old
// cluster and added to its new one with the same integer decomposition. The
// result is bit for bit the sum the full pass would form. Used only when X is
// finite and the two grids apply (the full pass handles the rest).

constexpr int DIFF_THREADS = 512;
constexpr int DIFF_ROWS = 4;  // rows per thread (16-byte loads of both label arrays)

// Rows whose label differs between two assignments, appended as (row, old,
// new) with one atomic per block; hist counts the entries per cluster (one
// for the old cluster, one for the new). Thread t of a block takes the rows
// 4 t .. 4 t + 3 of the block's 2048.
__global__ void __launch_bounds__(DIFF_THREADS)
    label_diff_kernel(const int32_t *__restrict__ prev, const int32_t *__restrict__ cur, int64_t n,
                      int4 *__restrict__ moved, unsigned long long *moved_count, int32_t *__restrict__ hist) {
    __shared__ unsigned int wcnt[DIFF_THREADS / 32];
    __shared__ unsigned long long base;
    const int64_t i0 = ((int64_t)blockIdx.x * DIFF_THREADS + threadIdx.x) * DIFF_ROWS;
    int o[DIFF_ROWS] = {0, 0, 0, 0}, nw[DIFF_ROWS] = {0, 0, 0, 0};
    const bool vec = (((uintptr_t)prev | (uintptr_t)cur) & 15u) == 0;  // i0 % 4 == 0: aligned pieces
    if (vec && i0 + DIFF_ROWS <= n) {
        const int4 a = *reinterpret_cast<const int4 *>(prev + i0), b = *reinterpret_cast<const int4 *>(cur + i0);
        o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
        nw[0] = b.x; nw[1] = b.y; nw[2] = b.z; nw[3] = b.w;
    } else {
        for (int r = 0; r < DIFF_ROWS; r++)
            if (i0 + r < n) {
                o[r] = prev[i0 + r];
                nw[r] = cur[i0 + r];
            }
    }
    unsigned mine = 0;
#pragma unroll
    for (int r = 0; r < DIFF_ROWS; r++) mine += (i0 + r < n && o[r] != nw[r]) ? 1u : 0u;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned incl = mine;  // inclusive prefix over the warp
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const unsigned v = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += v;
    }
    if (lane == 31) wcnt[w] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned t = 0;
        for (int q = 0; q < DIFF_THREADS / 32; q++) {
            const unsigned v = wcnt[q];
            wcnt[q] = t;
            t += v;
        }
        base = t ? atomicAdd(moved_count, (unsigned long long)t) : 0ull;
    }
    __syncthreads();
    if (mine) {
        unsigned long long slot = base + wcnt[w] + (incl - mine);
#pragma unroll
        for (int r = 0; r < DIFF_ROWS; r++) {
            if (i0 + r < n && o[r] != nw[r]) {
                moved[slot++] = make_int4((int)(i0 + r), o[r], nw[r], 0);
                atomicAdd(&hist[nw[r]], 1);
                atomicAdd(&hist[o[r]], 1);
            }
        }
    }
}

// Entries grouped by cluster (order inside a cluster is free: the sums are
// integers): row << 1 into the new cluster, row << 1 | 1 out of the old one.
__global__ void moved_scatter_kernel(const int4 *__restrict__ moved, const unsigned long long *moved_count,
                                     int32_t *__restrict__ cursor, uint32_t *__restrict__ ent) {
    const unsigned long long cnt = *moved_count;
    for (unsigned long long q = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; q < cnt;
         q += (unsigned long long)gridDim.x * blockDim.x) {
        const int4 e = moved[q];
        const int pin = atomicAdd(&cursor[e.z], 1);
        ent[pin] = (uint32_t)e.x << 1;
        const int pout = atomicAdd(&cursor[e.y], 1);
        ent[pout] = ((uint32_t)e.x << 1) | 1u;
    }
}

// One block per cluster: the signed exact sum of its entries (the same
// decomposition as centroid_fixed_part4_kernel, d % 4 == 0), added to the
// cluster's state, and the change of its count.
__global__ void __launch_bounds__(FIX4_THREADS, 3) exact_delta4_kernel(
    const float *__restrict__ x, int d, int k, int64_t n, const int32_t *__restrict__ eoff,
    const unsigned long long *moved_count, const uint32_t *__restrict__ ent, const float *__restrict__ amax_ptr,
    ExactState *__restrict__ state, long long *__restrict__ counts) {
    __shared__ FixRed red[FIX4_THREADS];
    __shared__ uint32_t sent[FIX4_IDX];
    __shared__ float tail_v[TAIL_CAP];
    __shared__ int tail_f[TAIL_CAP];
    __shared__ int tail_n, cdelta;
    const int c = blockIdx.x;
    const int64_t total = 2 * (int64_t)*moved_count;
    const int64_t start = eoff[c];
    const int64_t end = c + 1 < k ? (int64_t)eoff[c + 1] : total;
    if (start >= end) return;  // block-uniform
    const int S = d >> 2;
    const int G = FIX4_THREADS / S;
    const int g = (int)threadIdx.x / S, sl = (int)threadIdx.x % S;
    const bool active = g < G;
    const int F = fixed_bits(amax_ptr, n);
    const float amax = *amax_ptr;
    const int ea = amax > 0.f ? (int)((__float_as_uint(amax) >> 23) & 0xFFu) - 127 : -126;
    const int kb = ea + 2;  // the caller guarantees -90 <= ea <= 100
    const float C1 = ldexpf(1.5f, kb), C2 = ldexpf(1.5f, kb - 23);
    const int b1 = __float_as_int(C1), b2 = __float_as_int(C2);
    long long acc1[4] = {0, 0, 0, 0}, acc2[4] = {0, 0, 0, 0};
    int my_delta = 0;
    if (threadIdx.x == 0) {
        tail_n = 0;
        cdelta = 0;
    }
    for (int64_t cb = start; cb < end; cb += FIX4_IDX) {
        const int cnt = (int)min((int64_t)FIX4_IDX, end - cb);
        __syncthreads();
        for (int t = threadIdx.x; t < cnt; t += FIX4_THREADS) sent[t] = ent[cb + t];
        __syncthreads();
        if (!active) continue;
        uint32_t e_nxt = g < cnt ? sent[g] : 0u;
        float4 v_nxt = g < cnt ? reinterpret_cast<const float4 *>(x + (int64_t)(e_nxt >> 1) * d)[sl]
                               : make_float4(0.f, 0.f, 0.f, 0.f);
        for (int r = g; r < cnt; r += G) {
            const uint32_t e = e_nxt;
            const float4 v = v_nxt;
            if (r + G < cnt) {  // the next row of this thread loads while this one is split
                e_nxt = sent[r + G];
                v_nxt = reinterpret_cast<const float4 *>(x + (int64_t)(e_nxt >> 1) * d)[sl];
            }
            const bool neg = (e & 1u) != 0u;
            if (sl == 0) my_delta += neg ? -1 : 1;
            const float ev[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int f = 0; f < 4; f++) {
                const float s1 = __fadd_rn(ev[f], C1);
                const int q1 = (int)(__float_as_uint(s1) - (uint32_t)b1);
                const float rr = __fsub_rn(ev[f], __fsub_rn(s1, C1));
                const float s2 = __fadd_rn(rr, C2);
                const int q2 = (int)(__float_as_uint(s2) - (uint32_t)b2);
                const float r2 = __fsub_rn(rr, __fsub_rn(s2, C2));
                acc1[f] += neg ? -q1 : q1;
                acc2[f] += neg ? -q2 : q2;
                if (r2 != 0.f) {
                    const int slot = atomicAdd(&tail_n, 1);
                    if (slot < TAIL_CAP) {
                        tail_v[slot] = neg ? -r2 : r2;
                        tail_f[slot] = 4 * sl + f;
                    }
                }
            }
        }
    }
    __syncthreads();
    const int tn = tail_n;
    uint64_t slo[4] = {0, 0, 0, 0}, shi[4] = {0, 0, 0, 0};
    if (g == 0 && active && tn <= TAIL_CAP) {
        for (int e = 0; e < tn; e++) {
            const int fe = tail_f[e];
            if ((fe >> 2) != sl) continue;
#pragma unroll
            for (int f = 0; f < 4; f++)
                if ((fe & 3) == f) fixed_add_signed(slo[f], shi[f], tail_v[e], F);
        }
    }
    if (active && tn > TAIL_CAP) {  // the list overflowed: this thread's remainders again
        for (int64_t q = start + g; q < end; q += G) {
            const uint32_t e = ent[q];
            const bool neg = (e & 1u) != 0u;
            const float4 v = reinterpret_cast<const float4 *>(x + (int64_t)(e >> 1) * d)[sl];
            const float ev[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int f = 0; f < 4; f++) {
                const float s1 = __fadd_rn(ev[f], C1);
                const float rr = __fsub_rn(ev[f], __fsub_rn(s1, C1));
                const float s2 = __fadd_rn(rr, C2);
                const float r2 = __fsub_rn(rr, __fsub_rn(s2, C2));
                if (r2 != 0.f) fixed_add_signed(slo[f], shi[f], neg ? -r2 : r2, F);
            }
        }
    }
    FixRed mine;
#pragma unroll
    for (int f = 0; f < 4; f++) {
        uint64_t lo = slo[f], hi = shi[f];
        add_shifted(lo, hi, acc1[f], kb - 23 + F);
        add_shifted(lo, hi, acc2[f], kb - 46 + F);
        mine.lo[f] = lo;
        mine.hi[f] = hi;
        mine.inert[f] = 0.0;
        mine.flags[f] = 0u;
    }
    red[threadIdx.x] = mine;
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) my_delta += __shfl_xor_sync(0xffffffffu, my_delta, off);
    if ((threadIdx.x & 31) == 0 && my_delta != 0) atomicAdd(&cdelta, my_delta);
    __syncthreads();
    if (g == 0 && active) {
        FixRed t = red[sl];
        for (int gg = 1; gg < G; gg++) {
            const FixRed &o = red[gg * S + sl];
#pragma unroll
            for (int f = 0; f < 4; f++) add128(t.lo[f], t.hi[f], o.lo[f], o.hi[f]);
        }
#pragma unroll
        for (int f = 0; f < 4; f++) {
            ExactState &st = state[(int64_t)c * d + 4 * sl + f];
            uint64_t lo = st.lo, hi = st.hi;
            add128(lo, hi, t.lo[f], t.hi[f]);
            st = ExactState{lo, hi};
        }
    }
    if (threadIdx.x == 0) counts[c] += cdelta;
}

// Means from the exact state: the sum rounded once to f64, divided by the
// count (an empty cluster keeps its centre), as centroid_fixed_combine_kernel.
__global__ void exact_means_kernel(int d, int k, int64_t n, const ExactState *__restrict__ state,
                                   const long long *__restrict__ counts, const float *__restrict__ amax_ptr,
                                   const double *__restrict__ old_c, double *__restrict__ new_c) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)k * d) return;
    const long long cnt = counts[idx / d];
    if (cnt <= 0) {
        new_c[idx] = old_c[idx];
        return;
    }
    const ExactState st = state[idx];
    const double sum = fixed_to_double(((unsigned __int128)st.hi << 64) | st.lo, fixed_bits(amax_ptr, n));
    new_c[idx] = __ddiv_rn(sum, (double)cnt);
}

// ------------------------------------------------------- row inertia --
// sum_i ||x_i - c_{l_i}||^2 for one assignment: the centres split into f32
// hi + lo parts (x - c = (x - hi) - lo to about 2^-23 relative), each lane's
// squares over all its rows summed with compensation (Kahan) in f32, then the
// lanes in f64; the warps' sums folded in a fixed order per block (a fixed
// grid makes the result deterministic).
constexpr int RI_THREADS = 256;

__global__ void split_centres_kernel(const double *__restrict__ c, int64_t kd, float *__restrict__ hi,
                                     float *__restrict__ lo) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kd) return;
    const double v = c[i];
    const float h = __double2float_rn(v);
    hi[i] = h;
    lo[i] = __double2float_rn(__dsub_rn(v, (double)h));
}

// The same sum for d % 4 == 0 and d <= 256 (every mixed-path shape with f32
// X): lane l owns the 16-byte pieces l and l + 32 of a row; the next row's
// label and features load while this row is summed, and its centre pieces
// right after.
__global__ void __launch_bounds__(RI_THREADS)
    row_inertia4_kernel(const float *__restrict__ x, int64_t n, int d, const int32_t *__restrict__ labels,
                        const float *__restrict__ chi, const float *__restrict__ clo, double *__restrict__ block_part) {
    __shared__ double wsum[RI_THREADS / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t nw = (int64_t)gridDim.x * (RI_THREADS / 32);
    const int d4 = d >> 2;
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    auto load_x = [&](int64_t r, float4 (&v)[2]) {
#pragma unroll
        for (int i = 0; i < 2; i++) {
            const int q = lane + 32 * i;
            v[i] = (r < n && q < d4) ? reinterpret_cast<const float4 *>(x + r * d)[q] : z4;
        }
    };
    auto load_c = [&](int64_t r, int lab, float4 (&h)[2], float4 (&l)[2]) {
#pragma unroll
        for (int i = 0; i < 2; i++) {
            const int q = lane + 32 * i;
            const bool ok = r < n && q < d4;
            h[i] = ok ? reinterpret_cast<const float4 *>(chi + (int64_t)lab * d)[q] : z4;
            l[i] = ok ? reinterpret_cast<const float4 *>(clo + (int64_t)lab * d)[q] : z4;
        }
    };
    float s = 0.f, comp = 0.f;  // this lane's compensated sum over all its rows
    int64_t r = (int64_t)blockIdx.x * (RI_THREADS / 32) + w;
    float4 xa[2], ha[2], la[2];
    load_x(r, xa);
    load_c(r, r < n ? labels[r] : 0, ha, la);
    for (; r < n; r += nw) {
        const int64_t rn = r + nw;
        const int lbn = rn < n ? labels[rn] : 0;
        float4 xb[2], hb[2], lb[2];
        load_x(rn, xb);
#pragma unroll
        for (int i = 0; i < 2; i++) {
            const float xs[4] = {xa[i].x, xa[i].y, xa[i].z, xa[i].w};
            const float hs[4] = {ha[i].x, ha[i].y, ha[i].z, ha[i].w};
            const float ls[4] = {la[i].x, la[i].y, la[i].z, la[i].w};
#pragma unroll
            for (int e = 0; e < 4; e++) {  // padding pieces are zero on both sides
                const float t = __fsub_rn(__fsub_rn(xs[e], hs[e]), ls[e]);
                const float y = __fsub_rn(__fmul_rn(t, t), comp);
                const float u = __fadd_rn(s, y);
                comp = __fsub_rn(__fsub_rn(u, s), y);
                s = u;
            }
        }
        load_c(rn, lbn, hb, lb);
#pragma unroll
        for (int i = 0; i < 2; i++) {
            xa[i] = xb[i];
            ha[i] = hb[i];
            la[i] = lb[i];
        }
    }
    // FP64 is slow on this part: lanes fold into f64 once, not per row
    double acc = (double)s - (double)comp;
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    if (lane == 0) wsum[w] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int q = 0; q < RI_THREADS / 32; q++) t += wsum[q];
        block_part[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(RI_THREADS)
    row_inertia_kernel(const float *__restrict__ x, int64_t n, int d, const int32_t *__restrict__ labels,
                       const float *__restrict__ chi, const float *__restrict__ clo, double *__restrict__ block_part) {
    __shared__ double wsum[RI_THREADS / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t nw = (int64_t)gridDim.x * (RI_THREADS / 32);
    float s = 0.f, comp = 0.f;  // this lane's compensated sum over all its rows
    for (int64_t r = (int64_t)blockIdx.x * (RI_THREADS / 32) + w; r < n; r += nw) {
        const int64_t cl = labels[r];
        const float *xr = x + r * d, *ch = chi + cl * d, *cl2 = clo + cl * d;
        for (int j = lane; j < d; j += 32) {
            const float t = __fsub_rn(__fsub_rn(xr[j], ch[j]), cl2[j]);
            const float y = __fsub_rn(__fmul_rn(t, t), comp);
            const float u = __fadd_rn(s, y);
            comp = __fsub_rn(__fsub_rn(u, s), y);
            s = u;
        }
    }
    double acc = (double)s - (double)comp;
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    if (lane == 0) wsum[w] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int q = 0; q < RI_THREADS / 32; q++) t += wsum[q];
        block_part[blockIdx.x] = t;
    }
}

void launch_scan(int32_t *a, int64_t m, int32_t *tmp, cudaStream_t s) {
    int64_t nb = (m + SCAN_TILE - 1) / SCAN_TILE;
    scan_reduce_kernel<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(a, m, tmp);
    FK_LAUNCH_CHECK();
    scan_top_kernel<<<1, SCAN_THREADS, 0, s>>>(tmp, nb);
    FK_LAUNCH_CHECK();
    scan_down_kernel<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(a, m, tmp);
    FK_LAUNCH_CHECK();
}

// ------------------------------------------------------ mini-batch --
// MiniBatchKMeans: the batch's rows gathered into a contiguous block (the
// assignment kernel then reads them like any matrix).
template <typename T>
__global__ void gather_rows_kernel(const T *__restrict__ x, int d, const int32_t *__restrict__ idx, int64_t m,
                                   T *__restrict__ out) {
    const int64_t total = m * d;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = e / d;
        out[e] = x[(int64_t)idx[r] * d + (e - r * d)];
    }
}

// update_centers_mini_batch (mini_batch_kmeans.rs:410-447): one block per
// centre. Every thread walks the whole batch in order (the labels staged in
// shared memory, so the test is uniform across the block) and owns fixed
// features, so each feature of the centre receives c += (1 / count)(x - c)
// for the centre's rows in batch order: count is the centre's running count
// (starting at 1 before the first batch), 1 / count correctly rounded, no
// fused multiply-add. old receives the centre before the batch.
constexpr int MB_THREADS = 128;
constexpr int MB_LABELS = 2048;

template <typename T>
__global__ void __launch_bounds__(MB_THREADS)
    minibatch_update_kernel(const T *__restrict__ xb, const int32_t *__restrict__ labels, int64_t m, int d,
                            T *__restrict__ centres, T *__restrict__ old, long long *__restrict__ counts) {
    using A = UArith<T>;
    __shared__ int32_t lab[MB_LABELS];
    const int c = blockIdx.x;
    T *row = centres + (int64_t)c * d;
    for (int j = threadIdx.x; j < d; j += MB_THREADS) old[(int64_t)c * d + j] = row[j];
    long long cnt = counts[c];
    for (int64_t b0 = 0; b0 < m; b0 += MB_LABELS) {
        const int len = (int)(m - b0 < MB_LABELS ? m - b0 : MB_LABELS);
        __syncthreads();  // the previous chunk's labels are no longer read
        for (int i = threadIdx.x; i < len; i += MB_THREADS) lab[i] = labels[b0 + i];
        __syncthreads();
        for (int i = 0; i < len; i++) {
            if (lab[i] != c) continue;
            cnt += 1;
            const T lr = A::div(T(1), (T)cnt);
            const T *xr = xb + (b0 + i) * d;
            for (int j = threadIdx.x; j < d; j += MB_THREADS) {
                const T cj = row[j];
                row[j] = A::add(cj, A::mul(lr, A::sub(xr[j], cj)));
            }
        }
    }
    if (threadIdx.x == 0) counts[c] = cnt;
}

// ------------------------------------------------------- bisecting --
// BisectingKMeans (bisecting_kmeans.rs): a cluster is a segment of a row
// permutation; the n_init 2-means runs of one split proceed together
// (blockIdx.y or blockIdx.x = run), each with its labels (uint8, stride
// lab_stride), two centres (2 x d, run-major) and a changed flag.

// Each run's centres from its two picked positions of the segment.
template <typename T>
__global__ void bk_pick_kernel(const T *__restrict__ x, int d, const int32_t *__restrict__ perm,
                               const int32_t *__restrict__ picks, T *__restrict__ cen) {
    const int run = blockIdx.x;
    T *c = cen + (int64_t)run * 2 * d;
    const int64_t r0 = perm[picks[2 * run]], r1 = perm[picks[2 * run + 1]];
    for (int j = threadIdx.x; j < d; j += blockDim.x) {
        c[j] = x[r0 * d + j];
        c[d + j] = x[r1 * d + j];
    }
}

// run_2means' assignment (:245-262): label 0 when d0 <= d1 (direct forms),
// else 1; any change sets the run's flag. Runs that stopped are skipped.
template <typename T>
__global__ void bk_assign_kernel(const T *__restrict__ x, int d, const int32_t *__restrict__ perm, int64_t m,
                                 const T *__restrict__ cen, uint8_t *__restrict__ lab, int64_t lab_stride,
                                 const int *__restrict__ active, int *__restrict__ changed) {
    using A = UArith<T>;
    const int run = blockIdx.y;
    if (!active[run]) return;  // uniform over the block
    const T *c0 = cen + (int64_t)run * 2 * d;
    const T *c1 = c0 + d;
    uint8_t *l = lab + (int64_t)run * lab_stride;
    int any = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const T *row = x + (int64_t)perm[i] * d;
        T d0 = T(0), d1 = T(0);
        for (int j = 0; j < d; j++) {
            const T v = row[j];
            const T t0 = A::sub(v, c0[j]);
            d0 = A::add(d0, A::mul(t0, t0));
            const T t1 = A::sub(v, c1[j]);
            d1 = A::add(d1, A::mul(t1, t1));
        }
        const uint8_t nl = d0 <= d1 ? 0 : 1;
        if (nl != l[i]) {
            l[i] = nl;
            any = 1;
        }
    }
    if (__syncthreads_or(any) && threadIdx.x == 0) changed[run] = 1;
}

// Each row's direct-form distance to its run's centre of its label.
template <typename T>
__global__ void bk_dist_kernel(const T *__restrict__ x, int d, const int32_t *__restrict__ perm, int64_t m,
                               const T *__restrict__ cen, const uint8_t *__restrict__ lab, int64_t lab_stride,
                               T *__restrict__ dist, int64_t dist_stride) {
    using A = UArith<T>;
    const int run = blockIdx.y;
    const T *c = cen + (int64_t)run * 2 * d;
    const uint8_t *l = lab + (int64_t)run * lab_stride;
    T *o = dist + (int64_t)run * dist_stride;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const T *row = x + (int64_t)perm[i] * d;
        const T *cc = l[i] ? c + d : c;
        T acc = T(0);
        for (int j = 0; j < d; j++) {
            const T t = A::sub(row[j], cc[j]);
            acc = A::add(acc, A::mul(t, t));
        }
        o[i] = acc;
    }
}

// Stable partition of a segment by labels (label 0 first, each side in row
// order): pos holds the exclusive scan of (label == 0).
__global__ void bk_flag_kernel(const uint8_t *__restrict__ lab, int64_t m, int32_t *__restrict__ flag) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        flag[i] = lab[i] == 0 ? 1 : 0;
}

__global__ void bk_zeros_kernel(const int32_t *__restrict__ pos, const uint8_t *__restrict__ lab, int64_t m,
                                int64_t *__restrict__ m0) {
    *m0 = (int64_t)pos[m - 1] + (lab[m - 1] == 0 ? 1 : 0);
}

__global__ void bk_scatter_kernel(const int32_t *__restrict__ seg, const uint8_t *__restrict__ lab,
                                  const int32_t *__restrict__ pos, int64_t m, const int64_t *__restrict__ m0,
                                  int32_t *__restrict__ out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        out[lab[i] == 0 ? (int64_t)pos[i] : *m0 + (i - (int64_t)pos[i])] = seg[i];
}

// run_2means' centre update (:264-298) and compute_cluster_stats' centre
// (:192-211) from the exact folds of chain (run * 2 + side) * d + feature:
// sum / count with the count as the reference forms it -- the fold of
// F::one() per row, exact up to 2^(MB+1) where it stops growing, or F::from(m)
// for the whole segment -- an empty side keeping its centre.
template <typename T>
__global__ void bk_centres_kernel(const T *__restrict__ sums, const long long *__restrict__ counts, int runs, int d,
                                  const int *__restrict__ active, int whole, int64_t m, T *__restrict__ cen) {
    using A = UArith<T>;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= runs * 2 * d) return;
    const int r = c / (2 * d);
    if (active && !active[r]) return;
    const long long cap = sizeof(T) == 4 ? (1LL << 24) : (1LL << 53);
    const long long cnt = counts[c];
    const T cf = whole ? (T)m : (T)(cnt < cap ? cnt : cap);
    if (cf > T(0)) cen[c] = A::div(sums[c], cf);
}

// Final labels: cluster ci (block ci) owns the rows of its segment.
__global__ void bk_labels_kernel(const int32_t *__restrict__ perm, const int64_t *__restrict__ seg,
                                 int64_t *__restrict__ labels) {
    const int64_t lo = seg[2 * blockIdx.x], m = seg[2 * blockIdx.x + 1];
    for (int64_t i = threadIdx.x; i < m; i += blockDim.x) labels[perm[lo + i]] = blockIdx.x;
}

}  // namespace

template <typename T>
void launch_gather_rows(const T *x, int d, const int32_t *idx, int64_t m, T *out, cudaStream_t s) {
    const int64_t total = m * (int64_t)d;
    if (total <= 0) return;
    const unsigned grid = (unsigned)std::min<int64_t>((total + 255) / 256, 4096);
    gather_rows_kernel<T><<<grid, 256, 0, s>>>(x, d, idx, m, out);
    FK_LAUNCH_CHECK();
}

template <typename T>
void launch_minibatch_update(const T *xb, const int32_t *labels, int64_t m, int d, int k, T *centres, T *old,
                             long long *counts, unsigned long long *shift_bits, cudaStream_t s) {
    FK_CUDA(cudaMemsetAsync(shift_bits, 0, sizeof(unsigned long long), s));
    minibatch_update_kernel<T><<<(unsigned)k, MB_THREADS, 0, s>>>(xb, labels, m, d, centres, old, counts);
    FK_LAUNCH_CHECK();
    launch_max_shift<T>(centres, old, k, d, shift_bits, s);
}

int bk_chunk_rows(int d, size_t elem) {
    const size_t per = (size_t)d * elem + 1;
    const size_t rows = (40 * 1024) / per;
    return (int)std::max<size_t>(1, std::min<size_t>(64, rows));
}

template <typename T>
void launch_bk_pick(const T *x, int d, const int32_t *perm, const int32_t *picks, int runs, T *cen, cudaStream_t s) {
    bk_pick_kernel<T><<<(unsigned)runs, 128, 0, s>>>(x, d, perm, picks, cen);
    FK_LAUNCH_CHECK();
}

template <typename T>
void launch_bk_assign(const T *x, int d, const int32_t *perm, int64_t m, const T *cen, uint8_t *lab,
                      int64_t lab_stride, const int *active, int *changed, int runs, cudaStream_t s) {
    const unsigned gx = (unsigned)std::max<int64_t>(1, std::min<int64_t>((m + 255) / 256, 1024));
    bk_assign_kernel<T><<<dim3(gx, (unsigned)runs), 256, 0, s>>>(x, d, perm, m, cen, lab, lab_stride, active, changed);
    FK_LAUNCH_CHECK();
}


template <typename T>
void launch_bk_dist(const T *x, int d, const int32_t *perm, int64_t m, const T *cen, const uint8_t *lab,
                    int64_t lab_stride, T *dist, int64_t dist_stride, int runs, cudaStream_t s) {
    const unsigned gx = (unsigned)std::max<int64_t>(1, std::min<int64_t>((m + 255) / 256, 1024));
    bk_dist_kernel<T><<<dim3(gx, (unsigned)runs), 256, 0, s>>>(x, d, perm, m, cen, lab, lab_stride, dist,
                                                               dist_stride);
    FK_LAUNCH_CHECK();
}


template <typename T>
void launch_bk_centres(const T *sums, const long long *counts, int runs, int d, const int *active, bool whole,
                       int64_t m, T *cen, cudaStream_t s) {
    const int total = runs * 2 * d;
    bk_centres_kernel<T><<<(total + 255) / 256, 256, 0, s>>>(sums, counts, runs, d, active, whole ? 1 : 0, m, cen);
    FK_LAUNCH_CHECK();
}
template void launch_bk_centres<double>(const double *, const long long *, int, int, const int *, bool, int64_t,
                                        double *, cudaStream_t);
template void launch_bk_centres<float>(const float *, const long long *, int, int, const int *, bool, int64_t, float *,
                                       cudaStream_t);

size_t bk_partition_scratch_ints(int64_t m) { return 2 * (size_t)m + (size_t)((m + SCAN_TILE - 1) / SCAN_TILE + 1); }

// The segment reordered in place: its label-0 rows first, each side in row
// order (*m0 receives their count). scratch: bk_partition_scratch_ints(m).
void launch_bk_partition(int32_t *seg, const uint8_t *lab, int64_t m, int32_t *scratch, int64_t *m0,
                         cudaStream_t s) {
    if (m <= 0) return;
    int32_t *pos = scratch;      // m: exclusive scan of (label == 0)
    int32_t *out = scratch + m;  // m: the reordered segment
    int32_t *tmp = out + m;      // the scan's block sums
    const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((m + 255) / 256, 4096));
    bk_flag_kernel<<<g, 256, 0, s>>>(lab, m, pos);
    FK_LAUNCH_CHECK();
    launch_scan(pos, m, tmp, s);
    bk_zeros_kernel<<<1, 1, 0, s>>>(pos, lab, m, m0);
    FK_LAUNCH_CHECK();
    bk_scatter_kernel<<<g, 256, 0, s>>>(seg, lab, pos, m, m0, out);
    FK_LAUNCH_CHECK();
    FK_CUDA(cudaMemcpyAsync(seg, out, sizeof(int32_t) * (size_t)m, cudaMemcpyDeviceToDevice, s));
}

void launch_bk_labels(const int32_t *perm, const int64_t *seg, int nclusters, int64_t *labels, cudaStream_t s) {
    if (nclusters <= 0) return;
    bk_labels_kernel<<<(unsigned)nclusters, 256, 0, s>>>(perm, seg, labels);
    FK_LAUNCH_CHECK();
}

template void launch_bk_pick<double>(const double *, int, const int32_t *, const int32_t *, int, double *,
                                     cudaStream_t);
template void launch_bk_pick<float>(const float *, int, const int32_t *, const int32_t *, int, float *, cudaStream_t);
template void launch_bk_assign<double>(const double *, int, const int32_t *, int64_t, const double *, uint8_t *,
                                       int64_t, const int *, int *, int, cudaStream_t);
template void launch_bk_assign<float>(const float *, int, const int32_t *, int64_t, const float *, uint8_t *, int64_t,
                                      const int *, int *, int, cudaStream_t);
template void launch_bk_dist<double>(const double *, int, const int32_t *, int64_t, const double *, const uint8_t *,
                                     int64_t, double *, int64_t, int, cudaStream_t);
template void launch_bk_dist<float>(const float *, int, const int32_t *, int64_t, const float *, const uint8_t *,
                                    int64_t, float *, int64_t, int, cudaStream_t);

template void launch_gather_rows<double>(const double *, int, const int32_t *, int64_t, double *, cudaStream_t);
template void launch_gather_rows<float>(const float *, int, const int32_t *, int64_t, float *, cudaStream_t);
template void launch_minibatch_update<double>(const double *, const int32_t *, int64_t, int, int, double *, double *,
                                              long long *, unsigned long long *, cudaStream_t);
template void launch_minibatch_update<float>(const float *, const int32_t *, int64_t, int, int, float *, float *,
                                             long long *, unsigned long long *, cudaStream_t);

SortPlan make_sort_plan(int64_t n, int k) {
    SortPlan p;
    p.n = n;
    p.k = k;
    int64_t L = 4 * (int64_t)k;
    if (L < 1024) L = 1024;
    // Keep k * nseg (the count matrix) within 64M entries.
    while ((int64_t)k * ((n + L - 1) / L) > (int64_t)64 << 20) L *= 2;
    L = (L + 31) / 32 * 32;
    p.seg_len = L;
    p.nseg = n > 0 ? (n + L - 1) / L : 1;
    int64_t m = (int64_t)k * p.nseg;
    p.scan_tmp_bytes = sizeof(int32_t) * (size_t)((m + SCAN_TILE - 1) / SCAN_TILE + 1);
    return p;
}

static void set_smem_attr(const void *fn, size_t bytes) {
    if (bytes > 48 * 1024) FK_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
}

void launch_sort_by_cluster(const SortPlan &p, const int32_t *labels, int32_t *seg_hist, int32_t *scan_tmp,
                            int32_t *members, cudaStream_t s) {
    if (p.n == 0) return;
    size_t smem = sizeof(int) * (size_t)p.k;
    set_smem_attr((const void *)seg_hist_kernel, smem);
    set_smem_attr((const void *)seg_scatter_kernel, smem);
    seg_hist_kernel<<<(unsigned)p.nseg, 32, smem, s>>>(labels, p.n, p.k, p.seg_len, p.nseg, seg_hist);
    FK_LAUNCH_CHECK();
    launch_scan(seg_hist, (int64_t)p.k * p.nseg, scan_tmp, s);
    seg_scatter_kernel<<<(unsigned)p.nseg, 32, smem, s>>>(labels, p.n, p.k, p.seg_len, p.nseg, seg_hist, members);
    FK_LAUNCH_CHECK();
}

template <typename TX, typename TC>
void launch_update_centroids(const SortPlan &p, const TX *x, int d, const int32_t *members,
                             const int32_t *seg_hist, const TC *old_c, TC *new_c, DevScalars *scalars,
                             cudaStream_t s, double *inertia_part) {
    FK_CUDA(cudaMemsetAsync(&scalars->shift_bits, 0, sizeof(unsigned long long), s));
    if (d == 0 || p.k == 0) return;
    if constexpr (std::is_same<TX, TC>::value) {
        if (!inertia_part) {
            const size_t smem = chain_smem_bytes<TC>();
            FK_CUDA(cudaFuncSetAttribute((const void *)centroid_chain_kernel<TC>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            dim3 g((unsigned)p.k, (unsigned)((d + CH_SW - 1) / CH_SW));
            centroid_chain_kernel<TC><<<g, CH_THREADS, smem, s>>>(x, d, p.k, p.n, members, seg_hist, p.nseg, old_c,
                                                                 new_c);
            FK_LAUNCH_CHECK();
            launch_max_shift<TC>(new_c, old_c, p.k, d, &scalars->shift_bits, s);
            return;
        }
    }
    int threads = d >= 256 ? 256 : (d + 31) / 32 * 32;
    dim3 grid((unsigned)p.k, (unsigned)((d + threads - 1) / threads));
    if (inertia_part)
        centroid_sum_kernel<TX, TC, true><<<grid, threads, 0, s>>>(x, d, p.k, p.n, members, seg_hist, p.nseg, old_c,
                                                                   new_c, inertia_part);
    else
        centroid_sum_kernel<TX, TC, false><<<grid, threads, 0, s>>>(x, d, p.k, p.n, members, seg_hist, p.nseg, old_c,
                                                                    new_c, nullptr);
    FK_LAUNCH_CHECK();
    launch_max_shift<TC>(new_c, old_c, p.k, d, &scalars->shift_bits, s);
}

size_t update_exact_scratch_bytes(int k, int d) { return sizeof(FixedPart) * (size_t)k * FIX_SPLIT * d; }

void launch_update_centroids_exact(const SortPlan &p, const float *x, int d, const int32_t *members,
                                   const int32_t *seg_hist, const double *old_c, double *new_c, DevScalars *scalars,
                                   const float *amax, double *inertia_part, void *scratch, cudaStream_t s,
                                   ExactState *state, long long *counts) {
    FixedPart *parts = (FixedPart *)scratch;
    FK_CUDA(cudaMemsetAsync(&scalars->shift_bits, 0, sizeof(unsigned long long), s));
    if (d == 0 || p.k == 0) return;
    // blocks per cluster: about 1024 rows each, at most FIX_SPLIT
    const int splits = (int)std::max<int64_t>(1, std::min<int64_t>(FIX_SPLIT, (p.n / p.k + 1023) / 1024));
    if (d % 4 == 0 && d / 4 <= FIX4_THREADS && ((uintptr_t)x & 15u) == 0) {
        dim3 grid((unsigned)p.k, (unsigned)splits);
        centroid_fixed_part4_kernel<<<grid, FIX4_THREADS, 0, s>>>(x, d, p.k, p.n, members, seg_hist, p.nseg, old_c,
                                                                  amax, parts);
    } else {
        int threads = d >= 256 ? 256 : (d + 31) / 32 * 32;
        dim3 grid((unsigned)p.k, (unsigned)splits, (unsigned)((d + threads - 1) / threads));
        centroid_fixed_part_kernel<<<grid, threads, 0, s>>>(x, d, p.k, p.n, members, seg_hist, p.nseg, old_c, amax,
                                                            parts);
    }
    FK_LAUNCH_CHECK();
    const int64_t kd = (int64_t)p.k * d;
    centroid_fixed_combine_kernel<<<(unsigned)((kd + 255) / 256), 256, 0, s>>>(
        d, p.k, splits, p.n, seg_hist, p.nseg, old_c, new_c, amax, parts, inertia_part, state, counts);
    FK_LAUNCH_CHECK();
    launch_max_shift<double>(new_c, old_c, p.k, d, &scalars->shift_bits, s);
}

bool incremental_shape_ok(const float *x, int d) {
    return d > 0 && d % 4 == 0 && d / 4 <= FIX4_THREADS && ((uintptr_t)x & 15u) == 0;
}

void launch_update_centroids_incremental(Ctx &ctx, const float *x, int64_t n, int d, int k,
                                         const int32_t *prev_labels, const int32_t *labels, const double *old_c,
                                         double *new_c, DevScalars *scalars, const float *amax, ExactState *state,
                                         long long *counts) {
    cudaStream_t s = ctx.stream;
    FK_CUDA(cudaMemsetAsync(&scalars->shift_bits, 0, sizeof(unsigned long long), s));
    if (n == 0 || k == 0 || d == 0) return;
    int4 *moved = (int4 *)ctx.get(BUF_MOVED, sizeof(int4) * (size_t)n);
    uint32_t *ent = (uint32_t *)ctx.get(BUF_MOVED_ENT, sizeof(uint32_t) * 2 * (size_t)n);
    // [0, k): per-cluster entry counts, scanned in place into offsets; then
    // the scatter cursors; then the moved-row counter
    const size_t kb = ((size_t)k * sizeof(int32_t) + 255) / 256 * 256;
    char *ws = (char *)ctx.get(BUF_MOVED_HIST, 2 * kb + 256);
    int32_t *hist = (int32_t *)ws, *cursor = (int32_t *)(ws + kb);
    unsigned long long *moved_count = (unsigned long long *)(ws + 2 * kb);
    const int64_t nb = (k + SCAN_TILE - 1) / SCAN_TILE;
    int32_t *tmp = (int32_t *)ctx.get(BUF_MOVED_TMP, sizeof(int32_t) * (size_t)(nb + 1));
    FK_CUDA(cudaMemsetAsync(ws, 0, 2 * kb + 256, s));
    label_diff_kernel<<<(unsigned)((n + DIFF_THREADS * DIFF_ROWS - 1) / (DIFF_THREADS * DIFF_ROWS)), DIFF_THREADS, 0,
                        s>>>(
        prev_labels, labels, n, moved, moved_count, hist);
    FK_LAUNCH_CHECK();
    launch_scan(hist, k, tmp, s);
    FK_CUDA(cudaMemcpyAsync(cursor, hist, sizeof(int32_t) * (size_t)k, cudaMemcpyDeviceToDevice, s));
    moved_scatter_kernel<<<(unsigned)(ctx.num_sms * 8), 256, 0, s>>>(moved, moved_count, cursor, ent);
    FK_LAUNCH_CHECK();
    exact_delta4_kernel<<<(unsigned)k, FIX4_THREADS, 0, s>>>(x, d, k, n, hist, moved_count, ent, amax, state,
                                                             counts);
    FK_LAUNCH_CHECK();
    const int64_t kd = (int64_t)k * d;
    exact_means_kernel<<<(unsigned)((kd + 255) / 256), 256, 0, s>>>(d, k, n, state, counts, amax, old_c, new_c);
    FK_LAUNCH_CHECK();
    launch_max_shift<double>(new_c, old_c, k, d, &scalars->shift_bits, s);
    // for the report: how many rows this update moved, and that it was incremental
    FK_CUDA(cudaMemcpyAsync(&scalars->moved_rows, moved_count, sizeof(unsigned long long), cudaMemcpyDeviceToDevice,
                            s));
    FK_CUDA(cudaMemsetAsync(&scalars->incremental, 1, 1, s));
}

void launch_row_inertia(Ctx &ctx, const float *x, int64_t n, int d, const int32_t *labels, const double *c, int k,
                        DevScalars *scalars) {
    cudaStream_t s = ctx.stream;
    const int64_t kd = (int64_t)k * d;
    const int64_t kd4 = (kd + 3) / 4 * 4;  // the lo half starts 16-byte aligned
    float *split = (float *)ctx.get(BUF_CSPLIT, sizeof(float) * 2 * (size_t)kd4 + 64);
    split_centres_kernel<<<(unsigned)((kd + 255) / 256), 256, 0, s>>>(c, kd, split, split + kd4);
    FK_LAUNCH_CHECK();
    const int blocks = ctx.num_sms * 8;
    double *part = (double *)ctx.get(BUF_RINERT, sizeof(double) * (size_t)blocks);
    if (d % 4 == 0 && d <= 256 && ((uintptr_t)x & 15u) == 0)
        row_inertia4_kernel<<<(unsigned)blocks, RI_THREADS, 0, s>>>(x, n, d, labels, split, split + kd4, part);
    else
        row_inertia_kernel<<<(unsigned)blocks, RI_THREADS, 0, s>>>(x, n, d, labels, split, split + kd4, part);
    FK_LAUNCH_CHECK();
    launch_mixed_inertia(ctx, part, blocks, scalars);
}

template void launch_update_centroids<double, double>(const SortPlan &, const double *, int, const int32_t *,
                                                      const int32_t *, const double *, double *, DevScalars *,
                                                      cudaStream_t, double *);
template void launch_update_centroids<float, float>(const SortPlan &, const float *, int, const int32_t *,
                                                    const int32_t *, const float *, float *, DevScalars *,
                                                    cudaStream_t, double *);
template void launch_update_centroids<float, double>(const SortPlan &, const float *, int, const int32_t *,
                                                     const int32_t *, const double *, double *, DevScalars *,
                                                     cudaStream_t, double *);

}  // namespace fk
