// fk_mixed.cu -- mixed-precision assignment with an exact FP64 re-check.
//
// The approximate pass scores every (row, centre) pair as
//     T_c = xh . ch + a_c,   a_c = BIG - ||c'||^2 / 2,
// where x' = x - mu and c' = c - mu are centred by the column mean mu, xh and
// ch are their BF16 roundings (or E4M3 values times power-of-two scales:
// per row for X, one per launch for the centres), and BIG is a per-iteration
// constant that makes every T_c positive. Maximising T_c minimises
// ||x - c||^2. The contraction runs on the tensor cores (fk_tc.cu); a_c
// enters as three extra BF16 columns multiplied by a constant column of ones
// (by the row's scale for FP8), so the epilogue only ranks values.
//
// Per row, with the pass's best and second-best values v1 >= v2, the error
// bound (in T units)
//     E = ex * Cn + xn * Ec + ACC * (xn * Chn + BIG) + REPR * BIG
// (ex = ||x' - xh||, xn = ||xh||, Cn = max ||c'||, Ec = max ||c' - ch||,
// Chn = max ||ch||; ACC and REPR generous multiples of 2^-22 covering the FP32
// accumulation and the three-term BF16 split of a_c), the key-grid quantum q
// and the FP64 oracle's own rounding delta give the threshold
// thr = 2E + q + delta (evaluated in f32 with upward rounding). If
// v1 - v2 > thr no other centre can win in the FP64 direct form, so the label
// is final. Otherwise, if the best value outside the top two is also below
// v1 - thr, only the top two are re-scored exactly; else the row goes through
// a second tensor-core pass. After a BF16 main pass it recomputes the row's
// scores from the same operands and marks every centre scoring above
// v1 - 2 thr (a superset of the centres that can still win); 1 to 32 marked
// centres are re-scored, more or none send the row to the exhaustive
// re-score. After an FP8 main pass it runs in BF16 (its own operands, made
// from the row's f32 values, and its own bound -- 16x tighter than the FP8
// one): a count pass against the row's floor, then the mask pass with the
// threshold its exact best score gives (rows with more than 32 such centres,
// or a non-finite score, are re-scored against every centre, one CTA per
// row).
// Every re-score ends
// in the direct-form sum (x_j - c_j)^2 in FP64 with no FMA and the lowest
// index on ties, i.e. exactly kmeans.rs:159-163 / 295-309, so the labels
// equal the FP64 oracle's in every case.
#include <cfloat>
#include <cmath>
#include <cuda_bf16.h>
#include <cuda_fp8.h>

#include <algorithm>
#include <cstddef>
#include <type_traits>
#include <vector>

#include "fk_internal.cuh"

namespace fk {
namespace {

constexpr double ACC_REL_PER_K = 0.0000002384185791015625;  // 2^-22 per accumulated column
constexpr float REPR_REL_F = 0.0000002384185791015625f;     // 2^-22 (exact)

__device__ __forceinline__ void atomic_max_pos(float *addr, float v) {
    // non-negative floats order like their bit patterns
    if (v >= 0.f) atomicMax((unsigned int *)addr, __float_as_uint(v));
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// ----------------------------------------------------------- row prep --
// Column means (mu only centres the data, so any finite value is valid:
// partial sums in f32, non-finite entries skipped, the final fold in f64).
template <typename TX>
__global__ void col_mean_partial_kernel(const TX *__restrict__ x, int64_t n, int d, int64_t rows_per,
                                        int64_t stride, double *__restrict__ part) {
    int j = threadIdx.x + blockIdx.y * blockDim.x;
    if (j >= d) return;
    int64_t lo = (int64_t)blockIdx.x * rows_per, hi = lo + rows_per;
    float s = 0.f;
    for (int64_t t = lo; t < hi; t++) {
        const int64_t i = t * stride;
        if (i >= n) break;
        float v = (float)x[i * d + j];
        if (isfinite(v)) s += v;
    }
    part[(int64_t)blockIdx.x * d + j] = (double)s;
}

__global__ void col_mean_final_kernel(const double *__restrict__ part, int nparts, int64_t rows, int d,
                                      double *__restrict__ mu, float *__restrict__ mu32) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= d) return;
    double s = 0.0;
    for (int p = 0; p < nparts; p++) s += part[(int64_t)p * d + j];
    float m = (float)(s / (double)rows);
    if (!isfinite(m)) m = 0.f;
    mu32[j] = m;
    mu[j] = (double)m;  // the centring is by the f32 value, for rows and centres alike
}

// FP8: max |x - mu| over the same strided sample, the anchor of every scale
// of the launch (the centres' t and the range of the per-row scales).
template <typename TX>
__global__ void sample_tmax_kernel(const TX *__restrict__ x, int64_t n, int d, int64_t stride, int64_t rows,
                                   const float *__restrict__ mu32, MixedStats *stats) {
    float m = 0.f;
    const int64_t total = rows * (int64_t)d;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = (e / d) * stride;
        const int j = (int)(e % d);
        if (i < n) {
            const float t = fabsf(__fsub_rn((float)x[i * d + j], mu32[j]));
            if (t < INFINITY) m = fmaxf(m, t);
        }
    }
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
    if ((threadIdx.x & 31) == 0 && m > 0.f) atomicMax((unsigned int *)&stats->tmax, __float_as_uint(m));
}

// Exponent of the FP8 centre scale t = 2^sh_t: max |t| / t in [128, 256).
__device__ __forceinline__ int fp8_scale_exp(float tmax) {
    int sh = 0;
    if (tmax > 0.f && tmax < INFINITY) sh = ilogbf(tmax) - 7;
    return sh < -120 ? -120 : (sh > 120 ? 120 : sh);
}
constexpr int FP8_ROW_BELOW = 40;  // per-row scales stay within [2^(sh_t-40), 2^(sh_t+60)]
constexpr int FP8_ROW_ABOVE = 60;

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

__device__ __forceinline__ float half_warp_sum_f(float v) {
#pragma unroll
    for (int off = 8; off >= 1; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// This lane's part of the FP32 direct-form squared distance between x and c
// (f32 rows of d features) when `group` lanes share one distance: lane g of
// the group takes the features g, g + group, ... in 16-byte pieces when d is
// a multiple of 4 and both rows start 16-byte aligned, else one at a time. The
// parts are summed by the caller; any summation order stays within the
// (d + 4) 2^-23 d32 term of bound32.
__device__ __forceinline__ float sq_partial(const float *__restrict__ x, const float *__restrict__ c, int d, int g,
                                            int group) {
    float acc = 0.f;
    if ((d & 3) == 0 && (((uintptr_t)x | (uintptr_t)c) & 15u) == 0) {  // 16-byte pieces need 16-byte rows
        const float4 *x4 = reinterpret_cast<const float4 *>(x), *c4 = reinterpret_cast<const float4 *>(c);
#pragma unroll 4
        for (int f = g; f < (d >> 2); f += group) {  // unrolled: the loads of four pieces are in flight at once
            const float4 xv = x4[f], cv = c4[f];
            float t = xv.x - cv.x;
            acc = fmaf(t, t, acc);
            t = xv.y - cv.y;
            acc = fmaf(t, t, acc);
            t = xv.z - cv.z;
            acc = fmaf(t, t, acc);
            t = xv.w - cv.w;
            acc = fmaf(t, t, acc);
        }
    } else {
        for (int f = g; f < d; f += group) {
            const float t = x[f] - c[f];
            acc = fmaf(t, t, acc);
        }
    }
    return acc;
}

// One warp per row: BF16 copy of x - mu (row stride d_pad, zero padded) and
// the row's bound ingredients {||xh||, ||x' - xh||, ||x||}, all computed in
// f32 and then inflated to upper bounds: t = fl(x - mu) differs from x - mu
// by at most 2^-24 |t|, xh = bf16(t) and t - xh is exact, so
// ||x' - xh|| <= ||t - xh|| + 2^-24 ||t||; each sum of squares is scaled by
// (1 + (d + 64) 2^-23) to cover its own rounding before the rounded-up root.
// Also records max |x| (for the fixed-point centroid sums) and max ||xh||.
// FP8 rows: t = fl(x - mu) is scaled by a power of two s = 2^sh chosen per
// row so that max |t| / s lies in [128, 256) (inside E4M3's +-448), each t / s
// (exact) is rounded to E4M3 (saturating), and the dequantised value s * q
// stands where the BF16 value stands above; rowinfo.w = 2^-sh and the row's
// augmentation row is [2^-sh, 2^-sh, 2^-sh, 0, ...] (BF16, exact), so the
// tensor cores see every score of the row divided by s (and by the centres'
// scale t). sh is kept within [sh_t - 40, sh_t + 60] (and [-120, 120]) so
// that every scaled score stays a normal float.
// With a list (second pass), output slot s holds row list[s], s < *count.
template <typename TX, bool FP8>
__global__ void prep_rows_kernel(const TX *__restrict__ x, int64_t n, int d, int d_pad,
                                 const float *__restrict__ mu32, void *__restrict__ xq_out,
                                 __nv_bfloat16 *__restrict__ xaug, float4 *__restrict__ rowinfo, MixedStats *stats,
                                 const int32_t *__restrict__ list = nullptr,
                                 const unsigned long long *count = nullptr) {
    __shared__ float sh_xn[32], sh_am[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
    const int64_t slots = list ? (int64_t)*count : n;
    float xn_hi = 0.f, am_hi = 0.f, nonfin = 0.f;
    for (int64_t slot = (int64_t)blockIdx.x * (blockDim.x >> 5) + w; slot < slots; slot += nwarps) {
        const int64_t row = list ? (int64_t)list[slot] : slot;
        float xn2 = 0.f, ex2 = 0.f, tn2 = 0.f, xo2 = 0.f, amax = 0.f, tmax = 0.f;  // tmax: FP8 only
        float scale = 1.f, inv = 1.f;
        if (FP8) {
            for (int j = lane; j < d; j += 32) {
                const float tv = fabsf(__fsub_rn((float)x[row * d + j], mu32[j]));
                if (tv < INFINITY) tmax = fmaxf(tmax, tv);
            }
#pragma unroll
            for (int off = 16; off >= 1; off >>= 1) tmax = fmaxf(tmax, __shfl_xor_sync(0xffffffffu, tmax, off));
            const int sh_t = fp8_scale_exp(stats->tmax);
            int sh = tmax > 0.f ? fp8_scale_exp(tmax) : sh_t;
            sh = max(min(sh, sh_t + FP8_ROW_ABOVE), sh_t - FP8_ROW_BELOW);
            sh = max(min(sh, 120), -120);
            scale = ldexpf(1.f, sh);
            inv = ldexpf(1.f, -sh);
            tmax = 0.f;
        }
        for (int j = lane; j < d_pad; j += 32) {
            float hv = 0.f;
            if (j < d) {
                const float xv = (float)x[row * d + j];
                const float t = __fsub_rn(xv, mu32[j]);
                if (FP8) {
                    const __nv_fp8_e4m3 q8(__fmul_rn(t, inv));
                    ((unsigned char *)xq_out)[slot * d_pad + j] = q8.__x;
                    hv = __fmul_rn((float)q8, scale);
                } else {
                    const __nv_bfloat16 h = __float2bfloat16_rn(t);
                    ((__nv_bfloat16 *)xq_out)[slot * d_pad + j] = h;
                    hv = __bfloat162float(h);
                }
                const float e = __fsub_rn(t, hv);
                xn2 = __fmaf_rn(hv, hv, xn2);
                ex2 = __fmaf_rn(e, e, ex2);
                tn2 = __fmaf_rn(t, t, tn2);
                xo2 = __fmaf_rn(xv, xv, xo2);
                if (fabsf(xv) < INFINITY) amax = fmaxf(amax, fabsf(xv));  // finite values only
            } else if (FP8) {
                ((unsigned char *)xq_out)[slot * d_pad + j] = 0;
            } else {
                ((__nv_bfloat16 *)xq_out)[slot * d_pad + j] = __float2bfloat16_rn(0.f);
            }
        }
        xn2 = warp_sum_f(xn2);
        ex2 = warp_sum_f(ex2);
        tn2 = warp_sum_f(tn2);
        xo2 = warp_sum_f(xo2);
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, off));
        const float up = 1.0f + (float)(d + 64) * 1.1920929e-07f;
        float xn = __fsqrt_ru(__fmul_ru(xn2, up));
        float ex = __fadd_ru(__fsqrt_ru(__fmul_ru(ex2, up)), __fmul_ru(__fsqrt_ru(__fmul_ru(tn2, up)), 5.9604645e-08f));
        float xo = __fsqrt_ru(__fmul_ru(xo2, up));
        if (lane == 0) rowinfo[slot] = make_float4(xn, ex, xo, inv);
        if (FP8 && lane < 16)
            xaug[slot * 16 + lane] = lane < 3 ? __float2bfloat16_rn(inv) : __float2bfloat16_rn(0.f);
        if (xn < INFINITY) xn_hi = fmaxf(xn_hi, xn);  // NaN / inf rows are re-scored in full
        if (!(xo < INFINITY)) nonfin = 1.f;
        am_hi = fmaxf(am_hi, amax);
    }
    if (lane == 0) {
        sh_xn[w] = xn_hi;
        sh_am[w] = am_hi;
    }
    if (nonfin != 0.f) stats->nonfinite = 1.f;  // benign race: every writer stores 1
    __syncthreads();
    if (threadIdx.x == 0) {
        float a = 0.f, b = 0.f;
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) {
            a = fmaxf(a, sh_xn[q]);
            b = fmaxf(b, sh_am[q]);
        }
        atomic_max_pos(&stats->xn_max, a);
        atomic_max_pos(&stats->amax, b);
    }
}

// The same outputs as prep_rows_kernel for f32 rows with d a multiple of 4
// and d_pad <= 16 LPR: LPR lanes per row (32 / LPR rows a warp), lane l of a
// row owning its 4-feature pieces l, l + LPR, l + 2 LPR, l + 3 LPR, loaded
// with 16-byte loads, the warp's next rows in flight while these are
// processed; the reductions run over the row's LPR lanes. The norms are
// summed in another order than in prep_rows_kernel, which the upward
// inflation by (d + 64) 2^-23 covers.
template <int LPR>
__device__ __forceinline__ float group_sum_f(float v) {
#pragma unroll
    for (int off = LPR / 2; off >= 1; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

template <int LPR>
__device__ __forceinline__ float group_max_f(float v) {
#pragma unroll
    for (int off = LPR / 2; off >= 1; off >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, off));
    return v;
}

template <bool FP8, int LPR>
__global__ void prep_rows4_kernel(const float *__restrict__ x, int64_t n, int d, int d_pad,
                                  const float *__restrict__ mu32, void *__restrict__ xq_out,
                                  __nv_bfloat16 *__restrict__ xaug, float4 *__restrict__ rowinfo, MixedStats *stats,
                                  const int32_t *__restrict__ list, const unsigned long long *count) {
    constexpr int RPW = 32 / LPR;  // rows a warp
    constexpr int NPL = 4;         // 4-feature pieces a lane
    __shared__ float sh_xn[32], sh_am[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int sl = lane % LPR, g = lane / LPR;
    const int64_t stride = (int64_t)gridDim.x * (blockDim.x >> 5) * RPW;
    const int64_t slots = list ? (int64_t)*count : n;
    const int d4 = d >> 2, dp4 = d_pad >> 2;
    const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 m4[NPL];
#pragma unroll
    for (int i = 0; i < NPL; i++) {
        const int q = sl + LPR * i;
        m4[i] = q < d4 ? reinterpret_cast<const float4 *>(mu32)[q] : zero4;
    }
    auto load_row = [&](int64_t sl0, float4 (&v)[NPL]) {
        const int64_t slot = sl0 + g;
        const bool ok = slot < slots;
        const int64_t row = !ok ? 0 : list ? (int64_t)list[slot] : slot;
        const float4 *r4 = reinterpret_cast<const float4 *>(x + row * d);
#pragma unroll
        for (int i = 0; i < NPL; i++) {
            const int q = sl + LPR * i;
            v[i] = ok && q < d4 ? r4[q] : zero4;
        }
    };
    float xn_hi = 0.f, am_hi = 0.f, nonfin = 0.f;
    int64_t base = ((int64_t)blockIdx.x * (blockDim.x >> 5) + w) * RPW;  // warp-uniform
    float4 cur[NPL];
#pragma unroll
    for (int i = 0; i < NPL; i++) cur[i] = zero4;
    if (base < slots) load_row(base, cur);
    for (; base < slots; base += stride) {
        float4 nxt[NPL];
#pragma unroll
        for (int i = 0; i < NPL; i++) nxt[i] = zero4;
        if (base + stride < slots) load_row(base + stride, nxt);
        const int64_t slot = base + g;
        const bool ok = slot < slots;  // every lane stays for the shuffles
        float xn2 = 0.f, ex2 = 0.f, tn2 = 0.f, xo2 = 0.f, amax = 0.f;
        float scale = 1.f, inv = 1.f;
        if (FP8) {
            float tmax = 0.f;
#pragma unroll
            for (int i = 0; i < NPL; i++) {
                if (sl + LPR * i >= d4) continue;
                const float xs[4] = {cur[i].x, cur[i].y, cur[i].z, cur[i].w};
                const float ms[4] = {m4[i].x, m4[i].y, m4[i].z, m4[i].w};
#pragma unroll
                for (int c = 0; c < 4; c++) {
                    const float tv = fabsf(__fsub_rn(xs[c], ms[c]));
                    if (tv < INFINITY) tmax = fmaxf(tmax, tv);
                }
            }
            tmax = group_max_f<LPR>(tmax);
            const int sh_t = fp8_scale_exp(stats->tmax);
            int sh = tmax > 0.f ? fp8_scale_exp(tmax) : sh_t;
            sh = max(min(sh, sh_t + FP8_ROW_ABOVE), sh_t - FP8_ROW_BELOW);
            sh = max(min(sh, 120), -120);
            scale = ldexpf(1.f, sh);
            inv = ldexpf(1.f, -sh);
        }
#pragma unroll
        for (int i = 0; i < NPL; i++) {
            const int q = sl + LPR * i;
            if (q >= dp4) continue;
            if (q < d4) {
                const float xs[4] = {cur[i].x, cur[i].y, cur[i].z, cur[i].w};
                const float ms[4] = {m4[i].x, m4[i].y, m4[i].z, m4[i].w};
                uint32_t packed[2] = {0u, 0u};
#pragma unroll
                for (int c = 0; c < 4; c++) {
                    const float xv = xs[c];
                    const float t = __fsub_rn(xv, ms[c]);
                    float hv;
                    if (FP8) {
                        const __nv_fp8_e4m3 q8(__fmul_rn(t, inv));
                        packed[0] |= (uint32_t)q8.__x << (8 * c);
                        hv = __fmul_rn((float)q8, scale);
                    } else {
                        const __nv_bfloat16 h = __float2bfloat16_rn(t);
                        packed[c >> 1] |= (uint32_t)__bfloat16_as_ushort(h) << (16 * (c & 1));
                        hv = __bfloat162float(h);
                    }
                    const float e = __fsub_rn(t, hv);
                    xn2 = __fmaf_rn(hv, hv, xn2);
                    ex2 = __fmaf_rn(e, e, ex2);
                    tn2 = __fmaf_rn(t, t, tn2);
                    xo2 = __fmaf_rn(xv, xv, xo2);
                    if (fabsf(xv) < INFINITY) amax = fmaxf(amax, fabsf(xv));  // finite values only
                }
                if (ok) {
                    if (FP8)
                        reinterpret_cast<uint32_t *>(xq_out)[slot * dp4 + q] = packed[0];
                    else
                        reinterpret_cast<uint2 *>(xq_out)[slot * dp4 + q] = make_uint2(packed[0], packed[1]);
                }
            } else if (ok) {
                if (FP8)
                    reinterpret_cast<uint32_t *>(xq_out)[slot * dp4 + q] = 0u;
                else
                    reinterpret_cast<uint2 *>(xq_out)[slot * dp4 + q] = make_uint2(0u, 0u);
            }
        }
        xn2 = group_sum_f<LPR>(xn2);
        ex2 = group_sum_f<LPR>(ex2);
        tn2 = group_sum_f<LPR>(tn2);
        xo2 = group_sum_f<LPR>(xo2);
        amax = group_max_f<LPR>(amax);
        const float up = 1.0f + (float)(d + 64) * 1.1920929e-07f;
        const float xn = __fsqrt_ru(__fmul_ru(xn2, up));
        const float ex =
            __fadd_ru(__fsqrt_ru(__fmul_ru(ex2, up)), __fmul_ru(__fsqrt_ru(__fmul_ru(tn2, up)), 5.9604645e-08f));
        const float xo = __fsqrt_ru(__fmul_ru(xo2, up));
        if (ok) {
            if (sl == 0) rowinfo[slot] = make_float4(xn, ex, xo, inv);
            if (FP8) {
#pragma unroll
                for (int j = sl; j < 16; j += LPR)
                    xaug[slot * 16 + j] = j < 3 ? __float2bfloat16_rn(inv) : __float2bfloat16_rn(0.f);
            }
            if (xn < INFINITY) xn_hi = fmaxf(xn_hi, xn);  // NaN / inf rows are re-scored in full
            if (!(xo < INFINITY)) nonfin = 1.f;
            am_hi = fmaxf(am_hi, amax);
        }
#pragma unroll
        for (int i = 0; i < NPL; i++) cur[i] = nxt[i];
    }
    // the warp's maxima (every lane holds its rows' values)
    xn_hi = group_max_f<32>(xn_hi);
    am_hi = group_max_f<32>(am_hi);
    if (lane == 0) {
        sh_xn[w] = xn_hi;
        sh_am[w] = am_hi;
    }
    if (nonfin != 0.f) stats->nonfinite = 1.f;  // benign race: every writer stores 1
    __syncthreads();
    if (threadIdx.x == 0) {
        float a = 0.f, b = 0.f;
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) {
            a = fmaxf(a, sh_xn[q]);
            b = fmaxf(b, sh_am[q]);
        }
        atomic_max_pos(&stats->xn_max, a);
        atomic_max_pos(&stats->amax, b);
    }
}

// Row preparation launch: the 16-byte kernel where it applies.
template <typename TX, bool FP8>
void launch_prep_rows(Ctx &ctx, const TX *x, int64_t n, int d, int d_pad, const float *mu32, void *xq,
                      __nv_bfloat16 *xaug, float4 *rowinfo, MixedStats *stats, const int32_t *list = nullptr,
                      const unsigned long long *count = nullptr) {
    const int64_t pblocks = std::min<int64_t>((n + 7) / 8, (int64_t)ctx.num_sms * 16);
    if (std::is_same<TX, float>::value && (d & 3) == 0 && d_pad <= 256 && ((uintptr_t)x & 15u) == 0) {
        // 8 lanes a row up to 128 features (4 rows a warp), else 16 (2 rows a warp)
        if (d_pad <= 128)
            prep_rows4_kernel<FP8, 8><<<(unsigned)std::min<int64_t>((n + 31) / 32, (int64_t)ctx.num_sms * 16), 256,
                                        0, ctx.stream>>>((const float *)x, n, d, d_pad, mu32, xq, xaug, rowinfo,
                                                         stats, list, count);
        else
            prep_rows4_kernel<FP8, 16><<<(unsigned)std::min<int64_t>((n + 15) / 16, (int64_t)ctx.num_sms * 16),
                                         256, 0, ctx.stream>>>((const float *)x, n, d, d_pad, mu32, xq, xaug, rowinfo,
                                                               stats, list, count);
    } else {
        prep_rows_kernel<TX, FP8><<<(unsigned)pblocks, 256, 0, ctx.stream>>>(x, n, d, d_pad, mu32, xq, xaug,
                                                                             rowinfo, stats, list, count);
    }
    FK_LAUNCH_CHECK();
}

// -------------------------------------------------------- centre prep --
// One warp per (padded) centre row: BF16 copy of c - mu, and the maxima of
// ||c'||, ||c' - ch||, ||ch||, ||c'||^2 / 2, ||c|| over the real centres.
// FP8 centres: one power-of-two scale t for all centres, from the data's range
// (centres are means of rows, so they stay inside it; a centre outside would
// saturate, which the exact error ||c' - ch|| below accounts for).
template <bool FP8>
__global__ void prep_centres_kernel(const double *__restrict__ c, int k, int k_pad, int d, int d_pad,
                                    const double *__restrict__ mu, void *__restrict__ cq_out,
                                    double *__restrict__ half_norm, float *__restrict__ c32,
                                    float *__restrict__ ec32, float *__restrict__ c32t, MixedStats *stats) {
    const int lane = threadIdx.x & 31;
    const int q = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (q >= k_pad) return;
    float tsc = 1.f, tinv = 1.f;
    if (FP8) {
        const int sh = fp8_scale_exp(stats->tmax);
        tsc = ldexpf(1.f, sh);
        tinv = ldexpf(1.f, -sh);
        if (q == 0 && lane == 0) {
            stats->tscale = tsc;
            stats->inv_t = tinv;
        }
    } else if (q == 0 && lane == 0) {
        stats->tscale = 1.f;
        stats->inv_t = 1.f;
    }
    double cn2 = 0.0, ec2 = 0.0, ch2 = 0.0, co2 = 0.0, e32 = 0.0;
    for (int j = lane; j < d_pad; j += 32) {
        __nv_bfloat16 h = __float2bfloat16_rn(0.f);
        unsigned char h8 = 0;
        if (q < k && j < d) {
            double cv = c[(int64_t)q * d + j];
            double cc = cv - mu[j];
            double hv;
            if (FP8) {
                const __nv_fp8_e4m3 q8((float)(cc * (double)tinv));
                h8 = q8.__x;
                hv = (double)(float)q8 * (double)tsc;
            } else {
                h = __float2bfloat16_rn((float)cc);
                hv = (double)__bfloat162float(h);
            }
            cn2 += cc * cc;
            ec2 += (cc - hv) * (cc - hv);
            ch2 += hv * hv;
            co2 += cv * cv;
            float f = (float)cv;
            if (c32) {
                c32[(int64_t)q * d + j] = f;
                c32t[(int64_t)j * k + q] = f;
            }
            e32 += (cv - (double)f) * (cv - (double)f);
        }
        if (FP8)
            ((unsigned char *)cq_out)[(int64_t)q * d_pad + j] = h8;
        else
            ((__nv_bfloat16 *)cq_out)[(int64_t)q * d_pad + j] = h;
    }
    cn2 = warp_sum_d(cn2);
    ec2 = warp_sum_d(ec2);
    ch2 = warp_sum_d(ch2);
    co2 = warp_sum_d(co2);
    e32 = warp_sum_d(e32);
    if (lane == 0 && q < k) {
        const double up = 1.0 + 1e-12;
        if (ec32) ec32[q] = __double2float_ru(sqrt(e32) * up);
        half_norm[q] = 0.5 * cn2;
        atomic_max_pos(&stats->cn_max, __double2float_ru(sqrt(cn2) * up));
        atomic_max_pos(&stats->ec_max, __double2float_ru(sqrt(ec2) * up));
        atomic_max_pos(&stats->ch_max, __double2float_ru(sqrt(ch2) * up));
        atomic_max_pos(&stats->h_max, __double2float_ru(0.5 * cn2 * up));
        atomic_max_pos(&stats->co_max, __double2float_ru(sqrt(co2) * up));
    }
}

// a_c = BIG - ||c'||^2/2 split into three BF16 terms (columns 0..2 of the
// 16-column augmentation row); padded centres get a_c = 0, so they score 0.
// BIG = 1.5 * 2^E with 2^E >= 2.02 (max||xh|| max||ch|| + max||c'||^2/2) + 256,
// so every real score T = xh.ch + a_c lies in [2^E, 2^(E+1)) with room to
// spare: all scores of a launch share one exponent, which lets the epilogue
// round them to a common grid and insert the column code exactly.
__global__ void prep_aug_kernel(const double *__restrict__ half_norm, int k, int k_pad, bool fp8,
                                __nv_bfloat16 *__restrict__ caug, MixedStats *stats) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= k_pad) return;
    const double span = (double)stats->xn_max * (double)stats->ch_max + (double)stats->h_max;
    const double tsc = (double)stats->tscale;  // FP8: 256 t^2 is the floor of 2^E in the centres' units
    const double le = ceil(log2(2.02 * span + 256.0 * tsc * tsc));
    const int e = le < 200.0 ? (int)le : 200;  // NaN / inf span: 200, then BIG = inf below
    double big = 1.5 * ldexp(1.0, e);
    // The accumulators hold T r, r = 1 (BF16) or 2^-(sh_row + sh_t) (FP8); keys
    // need T r + 3 * 2^(e+6) r to stay finite and 2^(e-23) r to stay normal.
    // Outside that range BIG is infinite and every row is re-scored exactly.
    int rmax_exp = 0, rmin_exp = 0;
    if (fp8) {
        const int sh_t = ilogbf(stats->tscale);
        rmax_exp = -(max(sh_t - FP8_ROW_BELOW, -120) + sh_t);
        rmin_exp = -(min(sh_t + FP8_ROW_ABOVE, 120) + sh_t);
    }
    if (e + 9 + rmax_exp > 126 || e - 23 + rmin_exp < -126) big = INFINITY;
    // BIG, cgrid and ulp are kept in score units as f32: they must be normal
    if (e + 9 > 126 || e - 23 < -126) big = INFINITY;
    if (q == 0) {
        stats->big = (float)big;
        stats->cgrid = (float)(3.0 * ldexp(1.0, e + 6));
        stats->ulp = (float)ldexp(1.0, e - 23);
    }
    __nv_bfloat16 t[16];
#pragma unroll
    for (int j = 0; j < 16; j++) t[j] = __float2bfloat16_rn(0.f);
    if (q < k) {
        double a = (big - half_norm[q]) * (double)stats->inv_t;  // FP8: in units of the centres' scale
        __nv_bfloat16 a1 = __float2bfloat16_rn((float)a);
        double r1 = a - (double)__bfloat162float(a1);
        __nv_bfloat16 a2 = __float2bfloat16_rn((float)r1);
        double r2 = r1 - (double)__bfloat162float(a2);
        __nv_bfloat16 a3 = __float2bfloat16_rn((float)r2);
        t[0] = a1;
        t[1] = a2;
        t[2] = a3;
    }
#pragma unroll
    for (int j = 0; j < 16; j++) caug[(int64_t)q * 16 + j] = t[j];
}

// --------------------------------------------------------------- finalize --
// E, the row's bound on |T - S| between a tensor-core score T and the exact
// score S of the same centre (score units; see the file header). Every step
// rounds upward, so the result bounds the exact expression.
__device__ __forceinline__ float row_error(const float4 ri, const MixedStats *stats, float acc_rel) {
    const float xn = ri.x, ex = ri.y;
    const float cn = stats->cn_max, ec = stats->ec_max, ch = stats->ch_max, big = stats->big;
    return __fadd_ru(__fadd_ru(__fmul_ru(ex, cn), __fmul_ru(xn, ec)),
                     __fadd_ru(__fmul_ru(acc_rel, __fadd_ru(__fmul_ru(xn, ch), big)), __fmul_ru(REPR_REL_F, big)));
}

// Half the FP64 oracle's rounding bound on two direct-form distances: a
// centre whose exact score is below another's by more than this cannot win
// in the oracle.
__device__ __forceinline__ float row_slack64(const float4 ri, const MixedStats *stats, float mu_norm, int d) {
    const float xn = ri.x, ex = ri.y, xo = ri.z;
    const float xo_b = fminf(xo, __fadd_ru(__fadd_ru(xn, ex), mu_norm));  // ||x||: both bounds are valid
    const float sx = __fadd_ru(xo_b, stats->co_max);
    const float delta = __fmul_ru(__fmul_ru(__fmul_ru((float)(d + 4), 1.1102230246251565e-16f), sx), sx);
    return __fmul_ru(0.5f, delta);
}

// Threshold on a score margin above which no other centre can win in the
// FP64 direct form (see the file header): 2E + key quantum + FP64 rounding.
__device__ __forceinline__ float row_threshold(const float4 ri, const MixedStats *stats, float acc_rel, float mu_norm,
                                               int d, float v1) {
    const float e = row_error(ri, stats, acc_rel);
    // keys: each score rounded to a multiple of 128 ulp (error <= 64 ulp) plus a
    // column code below 128 ulp, so a key is within 192 ulp of its score
    const float q = 384.f * stats->ulp;
    float thr = __fadd_ru(__fmul_ru(__fadd_ru(__fadd_ru(__fmul_ru(2.f, e), q), row_slack64(ri, stats, mu_norm, d)),
                                    1.0000012f),
                          1e-30f);
    if (!(v1 >= stats->big * 0.6f)) thr = INFINITY;  // not a real score (NaN row, all slices padded)
    return thr;
}

// Lower bound, BIG removed, of the exact score S(c) - BIG of whichever centre
// c the oracle gives the row, from a pass whose best value is v1 (a key, or
// a raw score with key_slack 0): the winner's exact score is within the
// FP64 slack of the best exact score, which is at least v1 - key_slack - E.
// The next iteration's count pass starts from it.
__device__ __forceinline__ float row_floor(float v1, float key_slack, const float4 ri, const MixedStats *stats,
                                           float acc_rel, float mu_norm, int d) {
    float f = __fsub_rd(v1, key_slack);
    f = __fsub_rd(f, row_error(ri, stats, acc_rel));
    f = __fsub_rd(f, row_slack64(ri, stats, mu_norm, d));
    return __fsub_rd(f, stats->big);
}

// Merge of two slice records: (v1 >= v2, i1, i2) with u3 bounding the rest,
// and the same for the other slice.
__device__ __forceinline__ void merge_top2(float &v1, int &i1, float &v2, int &i2, float &u3, float w1, int j1,
                                           float w2, int j2, float wu) {
    if (w1 > v1) {
        if (v1 > w2) {
            u3 = fmaxf(u3, fmaxf(v2, w2));
            v2 = v1;
            i2 = i1;
        } else {
            u3 = fmaxf(u3, fmaxf(v1, wu));
            v2 = w2;
            i2 = j2;
        }
        v1 = w1;
        i1 = j1;
    } else if (w1 > v2) {
        u3 = fmaxf(u3, fmaxf(v2, w2));
        v2 = w1;
        i2 = j1;
    } else {
        u3 = fmaxf(u3, w1);
    }
}

// Warp-aggregated list append: the lanes of the calling (converged) group
// with pred set get consecutive slots from one atomic.
__device__ __forceinline__ unsigned long long warp_reserve(unsigned long long *counter, bool pred) {
    const unsigned mask = __activemask();
    const unsigned want = __ballot_sync(mask, pred);
    const int lane = threadIdx.x & 31;
    unsigned long long base = 0;
    if (want) {
        const int leader = __ffs(want) - 1;
        if (lane == leader) base = atomicAdd(counter, (unsigned long long)__popc(want));
        base = __shfl_sync(mask, base, leader);
    }
    return base + (unsigned long long)__popc(want & ((1u << lane) - 1u));
}

constexpr int FINALIZE_THREADS = 512;

// A row's class after the main pass: 0 decided (the kernel wrote the label),
// 1 a pair (a, b) for the exact re-score, 2 the second pass with threshold
// th; -1 no row.
struct RowClass {
    int cls, a, b;
    float th;
};

// Persistent finalize loop: each block takes chunks of FINALIZE_THREADS rows
// (grid-stride), with the next chunk's records (load) in flight while this
// chunk is classified (classify). A chunk's pair and full entries get
// consecutive list slots after a block scan of the warps' ballots and one
// atomic per list, which thread 0 issues for chunk i and whose results are
// only read while chunk i + 1 is handled: the entries of chunk i are written
// one iteration late, so no chunk waits on an atomic's round trip.
template <typename Load, typename Classify>
__device__ __forceinline__ void finalize_rows(int64_t n, Load load, Classify classify, int4 *__restrict__ pair_list,
                                              int32_t *__restrict__ full_list, float *__restrict__ full_thresh,
                                              DevScalars *sc) {
    __shared__ unsigned wa[2][FINALIZE_THREADS / 32], wb[2][FINALIZE_THREADS / 32];
    __shared__ unsigned long long base_a, base_b;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned below = (1u << lane) - 1u;
    const int64_t chunks = (n + FINALIZE_THREADS - 1) / FINALIZE_THREADS;
    int64_t ch = blockIdx.x;
    decltype(load(int64_t(0))) cur{}, nxt{};
    if (ch < chunks && ch * FINALIZE_THREADS + threadIdx.x < n) cur = load(ch * FINALIZE_THREADS + threadIdx.x);
    // the previous chunk's entry of this thread, its warp's ballots, and
    // (thread 0) the atomics' pending results
    RowClass pc{-1, -1, -1, 0.f};
    int64_t pi = -1;
    unsigned pba = 0u, pbb = 0u;
    unsigned long long pend_a = 0ull, pend_b = 0ull;
    int buf = 0;
    bool have_prev = false;
    auto write_prev = [&](int pbuf) {
        if (pc.cls == 1) pair_list[base_a + wa[pbuf][w] + (unsigned)__popc(pba & below)] = make_int4((int)pi, pc.a, pc.b, 0);
        if (pc.cls == 2) {
            const unsigned long long q = base_b + wb[pbuf][w] + (unsigned)__popc(pbb & below);
            full_list[q] = (int32_t)pi;
            if (full_thresh) full_thresh[q] = pc.th;
        }
    };
    for (; ch < chunks; ch += gridDim.x) {
        const int64_t nrow = (ch + gridDim.x) * FINALIZE_THREADS + threadIdx.x;
        if (ch + gridDim.x < chunks && nrow < n) nxt = load(nrow);
        const int64_t i = ch * FINALIZE_THREADS + threadIdx.x;
        RowClass c{-1, -1, -1, 0.f};
        if (i < n) c = classify(i, cur);
        const unsigned ba = __ballot_sync(0xffffffffu, c.cls == 1), bb = __ballot_sync(0xffffffffu, c.cls == 2);
        if (lane == 0) {
            wa[buf][w] = (unsigned)__popc(ba);
            wb[buf][w] = (unsigned)__popc(bb);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            // the previous chunk's bases (its atomics have had a whole chunk to return)
            base_a = pend_a;
            base_b = pend_b;
            unsigned ta = 0, tb = 0;
            for (int q = 0; q < FINALIZE_THREADS / 32; q++) {
                const unsigned xa = wa[buf][q], xb = wb[buf][q];
                wa[buf][q] = ta;
                wb[buf][q] = tb;
                ta += xa;
                tb += xb;
            }
            pend_a = ta ? atomicAdd(&sc->flag_count, (unsigned long long)ta) : 0ull;
            pend_b = tb ? atomicAdd(&sc->full_count, (unsigned long long)tb) : 0ull;
        }
        __syncthreads();
        if (have_prev) write_prev(buf ^ 1);
        pc = c;
        pi = i;
        pba = ba;
        pbb = bb;
        have_prev = true;
        buf ^= 1;
        cur = nxt;
        __syncthreads();  // base_a, base_b and this buffer's offsets are rewritten next
    }
    if (have_prev) {
        if (threadIdx.x == 0) {
            base_a = pend_a;
            base_b = pend_b;
        }
        __syncthreads();
        write_prev(buf ^ 1);
    }
}

__global__ void __launch_bounds__(FINALIZE_THREADS, 2)
    finalize_kernel(const SliceTop2 *__restrict__ parts, int nparts, int kp, int64_t n, int k, int d,
                    const float4 *__restrict__ rowinfo, const MixedStats *stats, float acc_rel, float mu_norm,
                    int32_t *__restrict__ labels, int4 *__restrict__ pair_list, int32_t *__restrict__ full_list,
                    float *__restrict__ full_thresh, float *__restrict__ floor_out, DevScalars *sc) {
    struct Rec {
        float4 ri;
        SliceTop2 t, o1;
    };
    auto load = [&](int64_t i) {
        Rec r;
        r.ri = rowinfo[i];
        r.t = parts[i];
        r.o1 = nparts > 1 ? parts[(int64_t)n + i] : r.t;
        return r;
    };
    auto classify = [&](int64_t i, const Rec &rec) {
        RowClass c{-1, -1, -1, -INFINITY};
        const float4 ri = rec.ri;
        const SliceTop2 t = rec.t, o1 = rec.o1;
        float v1 = t.v1, v2 = t.v2, u3 = t.u3;
        int i1 = slice_index(t.ids & 0xFFFFu, 0);
        int i2 = slice_index(t.ids >> 16, 0);
        if (nparts > 1)
            merge_top2(v1, i1, v2, i2, u3, o1.v1, slice_index(o1.ids & 0xFFFFu, kp), o1.v2,
                       slice_index(o1.ids >> 16, kp), o1.u3);
        for (int p = 2; p < nparts; p++) {
            const SliceTop2 o = parts[(int64_t)p * n + i];
            merge_top2(v1, i1, v2, i2, u3, o.v1, slice_index(o.ids & 0xFFFFu, p * kp), o.v2,
                       slice_index(o.ids >> 16, p * kp), o.u3);
        }
        {  // FP8 rows are scored in units of 1/(s_i t): back to score units (exact powers of two)
            const float unit = stats->tscale / ri.w;
            v1 *= unit;
            v2 *= unit;
            u3 *= unit;
        }
        const float thr = row_threshold(ri, stats, acc_rel, mu_norm, d, v1);
        if (floor_out) floor_out[i] = row_floor(v1, 192.f * stats->ulp, ri, stats, acc_rel, mu_norm, d);
        const float m12 = __fsub_rd(v1, v2);  // lower bounds of the margins
        const float m13 = __fsub_rd(v1, u3);
        c.a = i1;
        c.b = i2;
        if (i1 >= 0 && i1 < k && m12 > thr) {
            c.cls = 0;
            labels[i] = i1;
        } else if (i1 >= 0 && i1 < k && i2 >= 0 && i2 < k && i1 != i2 && m13 > thr) {
            c.cls = 1;
        } else {
            c.cls = 2;
            // Mask pass threshold (BF16 main pass, whose scores the mask pass
            // recomputes from the same operands): any centre that can still
            // win scores at least v1 - 2 thr there. The best centre c* has
            // T'(c*) >= T'(i1) >= T(i1) - 2E >= v1 - 192 ulp - 2E, and a
            // centre is needed only within thr of T'(c*); thr >= 2E + 384
            // ulp covers both. Thresholds below 2^(E-2) (or NaN) become
            // -inf: every centre is then a candidate.
            const float t2 = __fsub_rd(v1, __fmul_ru(2.f, thr));
            c.th = t2 >= stats->ulp * 2097152.f ? t2 : -INFINITY;
        }
        return c;
    };
    finalize_rows(n, load, classify, pair_list, full_list, full_thresh, sc);
}

// ------------------------------------------------------------ count pass --
// From the fourth iteration of a fit on, the main pass can skip the top-2
// ranking: a row's best score this iteration is bounded below from the
// previous one, so a threshold th below which no centre can win is known
// before the pass, which then only counts the centres at or above it (the
// mask pass's exact marks) and keeps the row's largest score. One marked
// centre is the label; two are a pair for the exact re-score; more (or
// none) go to the second pass with the same threshold.
//
// The bound: with c the centre the oracle gave the row in the previous
// iteration and F the row floor of that iteration (S_prev(c) - BIG_prev >=
// F), the exact scores move by S(c) - S_prev(c) = x'.(c - c_prev) - (h(c) -
// h_prev(c)) + (BIG - BIG_prev), h = ||c'||^2 / 2, so the best score T_max
// of this pass satisfies T_max >= T(c) >= S(c) - E >= F + BIG - ||x'|| D_c -
// |dh_c| - E =: L, with D_c = ||c - c_prev|| and ||x'|| <= ||xh|| + ||x' -
// xh||. A centre that can win in the oracle has S >= S(winner) - slack >=
// S(c) - slack >= L + E - slack, so its score here is at least L - slack >=
// L - thr =: th.

// Per centre, upper bounds of ||c - c_prev|| and of |h(c) - h_prev(c)|: one
// warp per centre, FP64 sums of squares inflated by (d + 8) 2^-52 for their
// roundings, then rounded up to f32.
__global__ void centre_shift_kernel(const double *__restrict__ c, const double *__restrict__ cprev,
                                    const double *__restrict__ mu, int k, int d, float2 *__restrict__ shift) {
    const int lane = threadIdx.x & 31;
    const int q = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (q >= k) return;  // warp-uniform
    double dd = 0.0, hn = 0.0, ho = 0.0;
    for (int j = lane; j < d; j += 32) {
        const double a = c[(int64_t)q * d + j], b = cprev[(int64_t)q * d + j], m = mu[j];
        const double t = a - b, u = a - m, v = b - m;
        dd += t * t;
        hn += u * u;
        ho += v * v;
    }
    dd = warp_sum_d(dd);
    hn = warp_sum_d(hn);
    ho = warp_sum_d(ho);
    if (lane == 0) {
        const double rel = (double)(d + 8) * 2.220446049250313e-16;
        const double dist = __dsqrt_ru(__dmul_ru(dd, 1.0 + rel));
        const double dh = __dadd_ru(__dmul_ru(0.5, fabs(hn - ho)), __dmul_ru(0.5 * rel, __dadd_ru(hn, ho)));
        const bool ok = dist < 1e30 && dh < 1e30;  // NaN or huge: no usable bound
        shift[q] = make_float2(ok ? __double2float_ru(dist) : INFINITY, ok ? __double2float_ru(dh) : INFINITY);
    }
}

// th for every row (score units, directed rounding), or -inf where no usable
// bound exists (then every centre is marked and the row is re-scored in full).
__global__ void count_thresh_kernel(int64_t n, int k, int d, const float *__restrict__ floor_prev,
                                    const int32_t *__restrict__ labels_prev, const float4 *__restrict__ rowinfo,
                                    const float2 *__restrict__ shift, const MixedStats *stats, float acc_rel,
                                    float mu_norm, float *__restrict__ th_out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int l = labels_prev[i];
    const float4 ri = rowinfo[i];
    float th = -INFINITY;
    if (l >= 0 && l < k) {
        const float2 sh = shift[l];
        const float xnorm = __fadd_ru(ri.x, ri.y);
        float lb = __fadd_rd(floor_prev[i], stats->big);
        lb = __fsub_rd(lb, __fmul_ru(xnorm, sh.x));
        lb = __fsub_rd(lb, sh.y);
        lb = __fsub_rd(lb, row_error(ri, stats, acc_rel));
        const float t = __fsub_rd(lb, row_threshold(ri, stats, acc_rel, mu_norm, d, stats->big));
        // the marks are exact 0 / 1 only for thresholds of at least 2^(E-2)
        th = t >= stats->ulp * 2097152.f ? t : -INFINITY;
    }
    th_out[i] = th;
}

// Centre of bit b of mask word w of slice base `base` (the mask pass's layout).
__device__ __forceinline__ int count_column(int base, int w, int b) {
    return base + 32 * w + (b < 16 ? 2 * (15 - b) : 2 * (31 - b) + 1);
}

// Merges the slices' count records of each row and classifies it: one marked
// centre is the label, two go to the pair re-score, more or none to the
// second pass with the row's threshold. Also the row floor for the next
// iteration (the largest score is a raw accumulator: no key slack).
__global__ void __launch_bounds__(FINALIZE_THREADS, 2)  // two blocks an SM: 64 registers a thread
    finalize_count_kernel(const SliceCount *__restrict__ parts, int nparts, int kp, int64_t n, int k, int d,
                          const float4 *__restrict__ rowinfo, const MixedStats *stats, float acc_rel, float mu_norm,
                          const float *__restrict__ thresh, int32_t *__restrict__ labels,
                          int4 *__restrict__ pair_list, int32_t *__restrict__ full_list,
                          float *__restrict__ full_thresh, float *__restrict__ floor_out, DevScalars *sc) {
    struct Rec {
        float4 ri;
        SliceCount o0, o1;
        float th;
    };
    auto load = [&](int64_t i) {
        Rec r;
        r.ri = rowinfo[i];
        r.o0 = parts[i];
        r.o1 = nparts > 1 ? parts[(int64_t)n + i] : r.o0;
        r.th = thresh[i];
        return r;
    };
    auto classify = [&](int64_t i, const Rec &rec) {
        RowClass c{-1, -1, -1, 0.f};
        float vmax = 0.f;
        uint32_t cnt = 0, w1 = 0, w2 = 0;
        int b1 = 0, b2 = 0;  // the words' first centre
        for (int p = 0; p < nparts; p++) {
            const SliceCount o = p == 0 ? rec.o0 : p == 1 ? rec.o1 : parts[(int64_t)p * n + i];
            vmax = fmaxf(vmax, o.vmax);
            cnt += o.meta & 0xFFFFu;
            const int wi[2] = {(int)((o.meta >> 16) & 0xFFu), (int)(o.meta >> 24)};
            const uint32_t ow[2] = {o.w1, o.w2};
#pragma unroll
            for (int u = 0; u < 2; u++) {
                if (!ow[u]) continue;
                if (!w1) {
                    w1 = ow[u];
                    b1 = p * kp + 32 * wi[u];
                } else if (!w2) {
                    w2 = ow[u];
                    b2 = p * kp + 32 * wi[u];
                }
            }
        }
        const float4 ri = rec.ri;
        vmax *= stats->tscale / ri.w;  // FP8: back to score units (a power of two; 1 for BF16)
        floor_out[i] = row_floor(vmax, 0.f, ri, stats, acc_rel, mu_norm, d);
        int a = -1, b = -1;
        if (cnt == 1 && w1) {
            a = count_column(b1, 0, __ffs(w1) - 1);
        } else if (cnt == 2 && w1) {
            a = count_column(b1, 0, __ffs(w1) - 1);
            const uint32_t rest = w1 & (w1 - 1u);
            b = rest ? count_column(b1, 0, __ffs(rest) - 1) : (w2 ? count_column(b2, 0, __ffs(w2) - 1) : -1);
        }
        c.a = a;
        c.b = b;
        if (cnt == 1 && a >= 0 && a < k) {
            c.cls = 0;
            labels[i] = a;
        } else if (cnt == 2 && a >= 0 && a < k && b >= 0 && b < k && a != b) {
            c.cls = 1;
        } else {
            c.cls = 2;
            // the second pass's threshold: the carried one, or tighter, from
            // this pass's exact best score -- a centre that can win scores at
            // least vmax - 2E - FP64 slack >= vmax - thr in any pass with
            // error bound E (a wide carried window would send the row to the
            // exhaustive re-score)
            const float t2 = __fsub_rd(vmax, row_threshold(ri, stats, acc_rel, mu_norm, d, stats->big));
            c.th = fmaxf(rec.th, t2 >= stats->ulp * 2097152.f ? t2 : -INFINITY);
        }
        return c;
    };
    finalize_rows(n, load, classify, pair_list, full_list, full_thresh, sc);
}

// ------------------------------------------------------------ re-checks --
// A row and at most eight candidate centres (second-pass rows, and the rows
// whose candidates are left to FP64).
struct alignas(16) Oct {
    int row, m;
    int ids[8];
    int pad0, pad1;
};

// Queues a row for the FP64 decision among its m candidates (lane 0 of the
// calling warp appends; any lane may pass the ids).
__device__ __forceinline__ void queue_f64(Oct *__restrict__ items, DevScalars *sc, int row, int m,
                                          const int (&ids)[8]) {
    if ((threadIdx.x & 31) == 0) {
        const unsigned long long slot = atomicAdd(&sc->f64_count, 1ULL);
        Oct o;
        o.row = row;
        o.m = m;
#pragma unroll
        for (int j = 0; j < 8; j++) o.ids[j] = ids[j];
        o.pad0 = o.pad1 = 0;
        items[slot] = o;
    }
}

// FP64 direct form in the oracle's order (x widened exactly, one running
// sum over increasing j). Kept register-light: it runs inside kernels whose
// FP32 paths need the occupancy.
template <typename TX>
__device__ __forceinline__ double sqeuc64(const TX *__restrict__ x, const double *__restrict__ c, int d) {
    double acc = 0.0;
#pragma unroll 4
    for (int j = 0; j < d; j++) {
        double t = __dsub_rn((double)x[j], c[j]);
        acc = __dadd_rn(acc, __dmul_rn(t, t));
    }
    return acc;
}

__device__ __forceinline__ bool near_tie(double a, double b) {
    double lo = a < b ? a : b;
    return fabs(a - b) <= 1e-12 * lo;
}

// a certainly below b (false for any NaN or infinity)
__device__ __forceinline__ bool below(float da, float ea, float db, float eb) {
    return __fadd_ru(da, ea) < __fsub_rd(db, eb);
}

// One warp per listed row (coalesced over the features): FP32 distances to
// the two candidates decide the row when their bounded intervals do not
// overlap; otherwise lanes 0 and 1 score the two exactly in FP64 (direct
// form, strict < over increasing index).
template <typename TX>
__global__ void pair_rescore_kernel(const TX *__restrict__ x, int d, const double *__restrict__ c,
                                    const float *__restrict__ c32, const float *__restrict__ ec32,
                                    const int4 *__restrict__ list, DevScalars *sc, int32_t *__restrict__ labels,
                                    Oct *__restrict__ f64_items) {
    const unsigned long long cnt = sc->flag_count;
    const int lane = threadIdx.x & 31;
    const unsigned long long wid = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned long long nw = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
    for (unsigned long long s = wid; s < cnt; s += nw) {
        const int4 e = list[s];
        const TX *row = x + (int64_t)e.x * d;
        const int a = e.y < e.z ? e.y : e.z, b = e.y < e.z ? e.z : e.y;
        if constexpr (std::is_same<TX, float>::value) {
            // lanes 0-15 score centre a, lanes 16-31 centre b, 16-byte loads
            const int hl = lane & 15;
            const float *cc = c32 + (int64_t)(lane < 16 ? a : b) * d;
            const float acc = half_warp_sum_f(sq_partial(row, cc, d, hl, 16));
            const float sa = __shfl_sync(0xffffffffu, acc, 0), sb = __shfl_sync(0xffffffffu, acc, 16);
            const float ea = bound32(sa, ec32[a], d), eb = bound32(sb, ec32[b], d);
            if (below(sa, ea, sb, eb)) {
                if (lane == 0) labels[e.x] = a;
                continue;
            }
            if (below(sb, eb, sa, ea)) {
                if (lane == 0) labels[e.x] = b;
                continue;
            }
        }
        const int ids[8] = {a, b, 0, 0, 0, 0, 0, 0};
        queue_f64(f64_items, sc, e.x, 2, ids);
    }
}

// pair_rescore_kernel for f32 rows with d % 4 == 0 and d <= 128: the same
// decisions, software-pipelined -- the list entry two rows ahead and the
// feature and centre pieces (and the centres' rounding errors) one row ahead
// load while this row is decided.
// Lanes 0-15 hold centre a, lanes 16-31 centre b, 16-byte pieces hl, hl + 16.
__global__ void __launch_bounds__(256)
    pair_rescore4_kernel(const float *__restrict__ x, int d, const double *__restrict__ c,
                         const float *__restrict__ c32, const float *__restrict__ ec32,
                         const int4 *__restrict__ list, DevScalars *sc, int32_t *__restrict__ labels,
                         Oct *__restrict__ f64_items) {
    const unsigned long long cnt = sc->flag_count;
    const int lane = threadIdx.x & 31, hl = lane & 15;
    const unsigned long long nw = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
    const int d4 = d >> 2;
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    auto entry = [&](unsigned long long q) { return q < cnt ? list[q] : make_int4(-1, 0, 0, 0); };
    // this lane's pieces of the row and of its centre (a for lanes 0-15, b for
    // 16-31), and that centre's rounding error
    auto pieces = [&](const int4 &e, float4 (&xv)[2], float4 (&cv)[2], float &ec) {
        const int a = min(e.y, e.z), b = max(e.y, e.z);
#pragma unroll
        for (int i = 0; i < 2; i++) {
            const int q = hl + 16 * i;
            const bool ok = e.x >= 0 && q < d4;
            xv[i] = ok ? reinterpret_cast<const float4 *>(x + (int64_t)e.x * d)[q] : z4;
            cv[i] = ok ? reinterpret_cast<const float4 *>(c32 + (int64_t)(lane < 16 ? a : b) * d)[q] : z4;
        }
        ec = e.x >= 0 ? ec32[lane < 16 ? a : b] : 0.f;
    };
    unsigned long long s = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int4 e0 = entry(s), e1 = entry(s + nw);
    float4 xa[2], ca[2];
    float eca;
    pieces(e0, xa, ca, eca);
    for (; s < cnt; s += nw) {
        const int4 e2 = entry(s + 2 * nw);
        float4 xb[2], cb[2];
        float ecb;
        pieces(e1, xb, cb, ecb);
        float acc = 0.f;  // padding pieces are zero on both sides
#pragma unroll
        for (int i = 0; i < 2; i++) {
            float t = xa[i].x - ca[i].x;
            acc = fmaf(t, t, acc);
            t = xa[i].y - ca[i].y;
            acc = fmaf(t, t, acc);
            t = xa[i].z - ca[i].z;
            acc = fmaf(t, t, acc);
            t = xa[i].w - ca[i].w;
            acc = fmaf(t, t, acc);
        }
        acc = half_warp_sum_f(acc);
        const float sa = __shfl_sync(0xffffffffu, acc, 0), sb = __shfl_sync(0xffffffffu, acc, 16);
        const int a = min(e0.y, e0.z), b = max(e0.y, e0.z);
        const float ea = bound32(sa, __shfl_sync(0xffffffffu, eca, 0), d),
                    eb = bound32(sb, __shfl_sync(0xffffffffu, eca, 16), d);
        if (below(sa, ea, sb, eb)) {
            if (lane == 0) labels[e0.x] = a;
        } else if (below(sb, eb, sa, ea)) {
            if (lane == 0) labels[e0.x] = b;
        } else {
            const int ids[8] = {a, b, 0, 0, 0, 0, 0, 0};
            queue_f64(f64_items, sc, e0.x, 2, ids);
        }
        e0 = e1;
        e1 = e2;
        eca = ecb;
#pragma unroll
        for (int i = 0; i < 2; i++) {
            xa[i] = xb[i];
            ca[i] = cb[i];
        }
    }
}

// One CTA per listed row, f32 rows: the row in shared memory, FP32 distances
// to every centre (threads over centres, four centres per thread at a time,
// reading the transposed f32 centres: coalesced and L2-resident), kept in
// shared memory for chunks of EX_CHUNK centres; the smallest upper bound UB
// over all centres; then FP64 (direct form) for every centre whose lower
// bound reaches UB or whose FP32 value is not finite, lowest index on ties.
constexpr int EX_CHUNK = 8192;
constexpr int EX_THREADS = 256;

__device__ __forceinline__ void ex_chunk_dists(const float *__restrict__ xs, int d, const float *__restrict__ c32t,
                                               int k, int c0, int c1, float *__restrict__ dist) {
    for (int q0 = c0 + (int)threadIdx.x; q0 < c1; q0 += 4 * EX_THREADS) {
        float a[4] = {0.f, 0.f, 0.f, 0.f};
        for (int j = 0; j < d; j++) {
            const float xv = xs[j];
            const float *ct = c32t + (int64_t)j * k;
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int q = q0 + u * EX_THREADS;
                if (q < c1) {
                    const float t = xv - ct[q];
                    a[u] = fmaf(t, t, a[u]);
                }
            }
        }
#pragma unroll
        for (int u = 0; u < 4; u++)
            if (q0 + u * EX_THREADS < c1) dist[q0 + u * EX_THREADS - c0] = a[u];
    }
}

__global__ void __launch_bounds__(EX_THREADS) exhaustive_rescore_kernel(
    const float *__restrict__ x, int d, const double *__restrict__ c, const float *__restrict__ c32t,
    const float *__restrict__ ec32, int k, const int32_t *__restrict__ list, const unsigned long long *count_ptr,
    DevScalars *sc, int32_t *__restrict__ labels) {
    extern __shared__ float ex_smem[];
    const int d_al = (d + 3) & ~3;
    float *xs = ex_smem;
    float *dist = ex_smem + d_al;
    __shared__ float red_f[EX_THREADS / 32];
    __shared__ double red_b1[EX_THREADS / 32], red_b2[EX_THREADS / 32];
    __shared__ int red_i[EX_THREADS / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned long long cnt = *count_ptr;
    const int nchunks = (k + EX_CHUNK - 1) / EX_CHUNK;
    for (unsigned long long s = blockIdx.x; s < cnt; s += gridDim.x) {
        const int64_t r = list[s];
        const float *row = x + r * d;
        for (int j = threadIdx.x; j < d; j += EX_THREADS) xs[j] = row[j];
        __syncthreads();
        // pass 1: smallest upper bound over all centres (each thread reads back
        // only the distances it wrote itself)
        float ub = INFINITY;
        for (int ch = 0; ch < nchunks; ch++) {
            const int c0 = ch * EX_CHUNK, c1 = min(k, c0 + EX_CHUNK);
            ex_chunk_dists(xs, d, c32t, k, c0, c1, dist);
            for (int q = c0 + (int)threadIdx.x; q < c1; q += EX_THREADS) {
                const float dv = dist[q - c0];
                const float hi = __fadd_ru(dv, bound32(dv, ec32[q], d));
                if (hi < ub) ub = hi;  // NaN never lowers the bound
            }
        }
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) ub = fminf(ub, __shfl_xor_sync(0xffffffffu, ub, off));
        if (lane == 0) red_f[w] = ub;
        __syncthreads();
        ub = red_f[0];
#pragma unroll
        for (int q = 1; q < EX_THREADS / 32; q++) ub = fminf(ub, red_f[q]);
        // pass 2: FP64 on the survivors, in increasing centre order per thread
        double b1 = DBL_MAX, b2 = DBL_MAX;
        int i1 = INT32_MAX;
        for (int ch = 0; ch < nchunks; ch++) {
            const int c0 = ch * EX_CHUNK, c1 = min(k, c0 + EX_CHUNK);
            if (nchunks > 1) ex_chunk_dists(xs, d, c32t, k, c0, c1, dist);
            for (int q = c0 + (int)threadIdx.x; q < c1; q += EX_THREADS) {
                const float dv = dist[q - c0];
                if (!(__fsub_rd(dv, bound32(dv, ec32[q], d)) > ub)) {
                    const double v = sqeuc64(xs, c + (int64_t)q * d, d);
                    if (v < b1) {
                        b2 = b1;
                        b1 = v;
                        i1 = q;
                    } else if (v < b2) {
                        b2 = v;
                    }
                }
            }
        }
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) {
            const double o1 = __shfl_xor_sync(0xffffffffu, b1, off);
            const double o2 = __shfl_xor_sync(0xffffffffu, b2, off);
            const int oi = __shfl_xor_sync(0xffffffffu, i1, off);
            if (o1 < b1 || (o1 == b1 && oi < i1)) {
                b2 = fmin(b1, o2);
                b1 = o1;
                i1 = oi;
            } else {
                b2 = fmin(b2, o1);
            }
        }
        if (lane == 0) {
            red_b1[w] = b1;
            red_b2[w] = b2;
            red_i[w] = i1;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            b1 = red_b1[0];
            b2 = red_b2[0];
            i1 = red_i[0];
            for (int q = 1; q < EX_THREADS / 32; q++) {
                const double o1 = red_b1[q], o2 = red_b2[q];
                const int oi = red_i[q];
                if (o1 < b1 || (o1 == b1 && oi < i1)) {
                    b2 = fmin(b1, o2);
                    b1 = o1;
                    i1 = oi;
                } else {
                    b2 = fmin(b2, o1);
                }
            }
            labels[r] = i1 == INT32_MAX ? 0 : i1;
            atomicAdd(&sc->recheck_rows, 1ULL);
            atomicAdd(&sc->full_rows, 1ULL);
            if (i1 != INT32_MAX && b2 < DBL_MAX && near_tie(b1, b2)) atomicAdd(&sc->near_tie_rows, 1ULL);
        }
        __syncthreads();  // xs, dist and the reduction slots are reused by the next row
    }
}

size_t exhaustive_smem_bytes(int d, int k) {
    return sizeof(float) * ((size_t)((d + 3) & ~3) + (size_t)std::min(k, EX_CHUNK));
}

// ------------------------------------------------------- second pass --
// Rows whose third-best score was inside the bound are scored again by the
// tensor cores in BF16 with candidate-marking epilogues (second_pass below):
// slot s of a second-pass list holds row list[s]; after an FP8 main pass its
// row data (rowinfo2) and statistics (stats2) are its own.

// Mask pass rows (BF16 main pass): slot s of the list holds row list[s] and
// its candidate mask, wpr words with bit per centre (mask_chunk's layout:
// word w, bit b < 16 is centre 32 w + 2 (15 - b), bit b >= 16 is centre
// 32 w + 2 (31 - b) + 1). One warp per row: the candidates below k are
// collected (a warp scan of the words' bit counts places them); with 1 to 32 of
// them, FP32 distances with rigorous bounds (four lanes per candidate,
// eight at a time), then the candidates whose lower bound reaches the
// smallest upper bound decide: one is the label, up to eight go to FP64,
// more (or none, or more than 32 candidates) to the exhaustive re-score.
constexpr int MASK_CANDS = 32;
constexpr int MASK_WARPS = 8;

__device__ __forceinline__ int mask_column(int w, int b) {
    return 32 * w + (b < 16 ? 2 * (15 - b) : 2 * (31 - b) + 1);
}

// FP32 distances from one row to candidates cand[0..m) (m <= 32): candidate j's
// distance ends in lane j. FAST (16-byte rows, d <= 256): the row's 16-byte
// pieces are in registers (lane l: pieces l and l + 32), and four candidates
// are scored at a time, each a warp sum, so their loads are in flight
// together. Otherwise four lanes per candidate, eight candidates at a time.
template <bool FAST>
__device__ __forceinline__ float cand_dists(const float *__restrict__ xrow, const float4 (&xv)[2],
                                            const float *__restrict__ c32, const int *cand, int m, int d) {
    const int lane = threadIdx.x & 31;
    float my = 0.f;
    if constexpr (FAST) {
        const int d4 = d >> 2;
        for (int j0 = 0; j0 < m; j0 += 4) {  // m is warp-uniform
            float acc[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                acc[u] = 0.f;
                if (j0 + u < m) {
                    const float4 *cr = reinterpret_cast<const float4 *>(c32 + (int64_t)cand[j0 + u] * d);
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        const int q = lane + 32 * h;
                        if (q < d4) {
                            const float4 cv = cr[q];
                            float t = xv[h].x - cv.x;
                            acc[u] = fmaf(t, t, acc[u]);
                            t = xv[h].y - cv.y;
                            acc[u] = fmaf(t, t, acc[u]);
                            t = xv[h].z - cv.z;
                            acc[u] = fmaf(t, t, acc[u]);
                            t = xv[h].w - cv.w;
                            acc[u] = fmaf(t, t, acc[u]);
                        }
                    }
                }
            }
#pragma unroll
            for (int off = 16; off >= 1; off >>= 1)
#pragma unroll
                for (int u = 0; u < 4; u++) acc[u] += __shfl_xor_sync(0xffffffffu, acc[u], off);
#pragma unroll
            for (int u = 0; u < 4; u++)
                if (lane == j0 + u) my = acc[u];
        }
    } else {
        for (int r0 = 0; r0 < m; r0 += 8) {
            const int cj = r0 + (lane >> 2);
            float acc = 0.f;
            if (cj < m) acc = sq_partial(xrow, c32 + (int64_t)cand[cj] * d, d, lane & 3, 4);
            acc += __shfl_xor_sync(0xffffffffu, acc, 2);
            acc += __shfl_xor_sync(0xffffffffu, acc, 1);
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const float v = __shfl_sync(0xffffffffu, acc, 4 * j);
                if (lane == r0 + j) my = v;
            }
        }
    }
    return my;
}

template <bool FAST>
__global__ void __launch_bounds__(MASK_WARPS * 32)
    mask_rescore_kernel(const float *__restrict__ x, int d, const float *__restrict__ c32,
                        const float *__restrict__ ec32, int k, const uint32_t *__restrict__ masks, int wpr,
                        const int32_t *__restrict__ list, const unsigned long long *count, DevScalars *sc,
                        int32_t *__restrict__ labels, Oct *__restrict__ f64_items, int32_t *__restrict__ ex_list) {
    __shared__ int cand_sm[MASK_WARPS][MASK_CANDS];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int *cand = cand_sm[wid];
    const unsigned long long cnt = *count;
    const unsigned long long nw = (unsigned long long)gridDim.x * MASK_WARPS;
    unsigned long long s = (unsigned long long)blockIdx.x * MASK_WARPS + wid;
    unsigned long long decided = 0;  // rows this warp decided among its candidates (lane 0)
    // the next row's list entry and first 32 mask words load while this row
    // is decided
    int row_next = 0;
    uint32_t word_next = 0u;
    if (s < cnt) {
        row_next = list[s];
        word_next = lane < wpr ? masks[(int64_t)s * wpr + lane] : 0u;
    }
    for (; s < cnt; s += nw) {
        const int row = row_next;
        const uint32_t first = word_next;
        if (s + nw < cnt) {
            row_next = list[s + nw];
            word_next = lane < wpr ? masks[(int64_t)(s + nw) * wpr + lane] : 0u;
        }
        const float *xrow = x + (int64_t)row * d;
        float4 xv[2] = {make_float4(0.f, 0.f, 0.f, 0.f), make_float4(0.f, 0.f, 0.f, 0.f)};
        if constexpr (FAST) {  // the row's pieces load while the mask is decoded
#pragma unroll
            for (int h = 0; h < 2; h++)
                if (lane + 32 * h < (d >> 2)) xv[h] = reinterpret_cast<const float4 *>(xrow)[lane + 32 * h];
        }
        const uint32_t *mw = masks + (int64_t)s * wpr;
        int m = 0;  // candidates so far (warp-uniform)
        for (int w0 = 0; w0 < wpr; w0 += 32) {
            const int w = w0 + lane;
            uint32_t word = w0 == 0 ? first : (w < wpr ? mw[w] : 0u);
            if (32 * w + 32 > k) {  // centres at or above k are padding
                uint32_t keep = 0u;
                for (int b = 0; b < 32; b++)
                    if (mask_column(w, b) < k) keep |= 1u << b;
                word &= keep;
            }
            const int c = __popc(word);
            int incl = c;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, incl, off);
                if (lane >= off) incl += t;
            }
            const int total = __shfl_sync(0xffffffffu, incl, 31);
            if (m + total <= MASK_CANDS) {
                // this lane's candidates (one step per set bit; any order)
                int pos = m + incl - c;
                for (uint32_t rest = word; rest; rest &= rest - 1u) cand[pos++] = mask_column(w, __ffs(rest) - 1);
            }
            m += total;
        }
        __syncwarp();
        bool to_ex = m == 0 || m > MASK_CANDS;
        if (!to_ex) {
            const bool is_cand = lane < m;
            const int my_id = is_cand ? cand[lane] : INT32_MAX;
            const float my_ec = is_cand ? ec32[my_id] : 0.f;  // in flight during the distances
            const float my_dist = cand_dists<FAST>(xrow, xv, c32, cand, m, d);
            const float my_err = is_cand ? bound32(my_dist, my_ec, d) : 0.f;
            float ub = is_cand ? __fadd_ru(my_dist, my_err) : INFINITY;
#pragma unroll
            for (int off = 16; off >= 1; off >>= 1) ub = fminf(ub, __shfl_xor_sync(0xffffffffu, ub, off));
            const unsigned surv = __ballot_sync(0xffffffffu, is_cand && !(__fsub_rd(my_dist, my_err) > ub));
            const int nsurv = __popc(surv);
            if (nsurv == 1) {
                const int only = __shfl_sync(0xffffffffu, my_id, __ffs(surv) - 1);
                if (lane == 0) {
                    labels[row] = only;
                    decided++;
                }
            } else {
                // the survivors (all candidates if no FP32 value was finite)
                const unsigned take = nsurv == 0 ? __ballot_sync(0xffffffffu, is_cand) : surv;
                if (__popc(take) <= 8) {
                    int ids[8];
                    int mm = 0;
                    unsigned rest = take;
#pragma unroll
                    for (int j = 0; j < 8; j++) {  // take is warp-uniform, so every lane shuffles
                        const int v = __shfl_sync(0xffffffffu, my_id, rest ? __ffs(rest) - 1 : 0);
                        ids[j] = rest ? v : 0;
                        if (rest) {
                            rest &= rest - 1u;
                            mm++;
                        }
                    }
                    queue_f64(f64_items, sc, row, mm, ids);
                    if (lane == 0) decided++;
                } else {
                    to_ex = true;
                }
            }
        }
        if (to_ex && lane == 0) ex_list[atomicAdd(&sc->ex_count, 1ULL)] = row;
        __syncwarp();  // cand is reused by the next row
    }
    // one add per warp: a per-row atomic on the shared counter serialises in L2
    if (lane == 0 && decided) atomicAdd(&sc->quad_count, decided);
}

// FP8 second pass, slot s = row list[s] of the main pass's full list. The
// BF16 count pass there runs against th[s] = F + BIG2 - slack - E2: the
// oracle's winner w has S(w) - BIG >= F (the row floor of the FP8 pass), so
// its BF16 score is at least F + BIG2 - E2 -- it is always marked, and one
// mark is the label.
__global__ void second_thresh_kernel(const int32_t *__restrict__ list, const unsigned long long *count,
                                     const float *__restrict__ floors, const float4 *__restrict__ rowinfo2,
                                     const MixedStats *st2, float acc_rel2, float mu_norm, int d,
                                     float *__restrict__ th) {
    const unsigned long long cnt = *count;
    for (unsigned long long s = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; s < cnt;
         s += (unsigned long long)gridDim.x * blockDim.x) {
        const float4 ri = rowinfo2[s];
        float t = __fadd_rd(floors[list[s]], st2->big);
        t = __fsub_rd(t, row_slack64(ri, st2, mu_norm, d));
        t = __fsub_rd(t, row_error(ri, st2, acc_rel2));
        th[s] = t >= st2->ulp * 2097152.f ? t : -INFINITY;
    }
}

// After that count pass: one mark is the label; none (a NaN row) the
// exhaustive re-score; more go to the mask pass with max(th, vmax - thr),
// vmax the pass's exact best score (the winner scores at least vmax - 2 E2 -
// FP64 slack there). list3 / slot3 hold the row and its slot here.
__global__ void second_finalize_kernel(const SliceCount *__restrict__ parts, int nparts, int kp, int64_t cap, int k,
                                       int d, const int32_t *__restrict__ list, const unsigned long long *count,
                                       const float4 *__restrict__ rowinfo2, const MixedStats *st2, float acc_rel2,
                                       float mu_norm, const float *__restrict__ th, int32_t *__restrict__ labels,
                                       int32_t *__restrict__ ex_list, int32_t *__restrict__ list3,
                                       int32_t *__restrict__ slot3, float *__restrict__ th3, DevScalars *sc) {
    const unsigned long long cnt = *count;
    for (unsigned long long s = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; s < cnt;
         s += (unsigned long long)gridDim.x * blockDim.x) {
        float vmax = 0.f;
        uint32_t marks = 0, w1 = 0;
        int b1 = 0;
        for (int p = 0; p < nparts; p++) {
            const SliceCount o = parts[(int64_t)p * cap + s];
            vmax = fmaxf(vmax, o.vmax);
            marks += o.meta & 0xFFFFu;
            if (!w1 && o.w1) {
                w1 = o.w1;
                b1 = p * kp + 32 * (int)((o.meta >> 16) & 0xFFu);
            }
        }
        const int row = list[s];
        const int a = (marks == 1 && w1) ? count_column(b1, 0, __ffs(w1) - 1) : -1;
        const bool decided = marks == 1 && a >= 0 && a < k;
        const bool to_ex = !decided && marks == 0;
        const bool to_mask = !decided && !to_ex;
        if (decided) labels[row] = a;
        const unsigned long long es = warp_reserve(&sc->ex_count, to_ex);
        const unsigned long long ms = warp_reserve(&sc->mask_count, to_mask);
        if (to_ex) ex_list[es] = row;
        if (to_mask) {
            const float4 ri = rowinfo2[s];
            const float t2 = __fsub_rd(vmax, row_threshold(ri, st2, acc_rel2, mu_norm, d, st2->big));
            list3[ms] = row;
            slot3[ms] = (int32_t)s;
            th3[ms] = fmaxf(th[s], t2 >= st2->ulp * 2097152.f ? t2 : -INFINITY);
        }
    }
}

// BF16 rows of the main pass's operand copied for the listed rows (slot s =
// row list[s]), 16 bytes per thread.
__global__ void gather_xq_rows_kernel(const uint4 *__restrict__ xq, int pieces, const int32_t *__restrict__ list,
                                      const unsigned long long *count, uint4 *__restrict__ out) {
    const unsigned long long total = *count * (unsigned long long)pieces;
    for (unsigned long long e = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned long long s = e / (unsigned)pieces;
        const int q = (int)(e - s * (unsigned)pieces);
        out[e] = xq[(int64_t)list[s] * pieces + q];
    }
}

// The FP64 decisions: one warp per queued row stages the widened row and its
// candidate centres (rows padded by one double) in shared memory, then lane
// j < m sums candidate j in the oracle's order (sqeuc64's arithmetic from
// shared memory, so the dependent FP64 additions are the only wait); the
// lowest distance below F::MAX wins, the lowest index on ties, else label 0,
// exactly as nearest_center.
constexpr int F64_WARPS = 4;
size_t f64_smem_bytes(int d) { return sizeof(double) * (size_t)F64_WARPS * ((size_t)d + 8 * ((size_t)d + 1)); }

template <typename TX>
__global__ void __launch_bounds__(F64_WARPS * 32)
    f64_decide_kernel(const TX *__restrict__ x, int d, const double *__restrict__ c, const Oct *__restrict__ items,
                      DevScalars *sc, int32_t *__restrict__ labels) {
    extern __shared__ double f64_smem[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    double *xs = f64_smem + (size_t)w * ((size_t)d + 8 * ((size_t)d + 1)), *cs = xs + d;
    const unsigned long long cnt = sc->f64_count;
    const unsigned long long nw = (unsigned long long)gridDim.x * F64_WARPS;
    for (unsigned long long q = (unsigned long long)blockIdx.x * F64_WARPS + w; q < cnt; q += nw) {
        const Oct it = items[q];
        for (int j = lane; j < d; j += 32) xs[j] = (double)x[(int64_t)it.row * d + j];
        int my_id = INT32_MAX;
#pragma unroll
        for (int t = 0; t < 8; t++)
            if (t < it.m && t == lane) my_id = it.ids[t];
        // the candidates' rows as one flat index space, so every load of the
        // staging is independent of the others
        const int md = it.m * d;
        for (int e = lane; e < md; e += 32) {
            const int t = e / d, j = e - t * d;
            int id = it.ids[0];
#pragma unroll
            for (int u = 1; u < 8; u++)
                if (u == t) id = it.ids[u];
            cs[(size_t)t * (d + 1) + j] = c[(int64_t)id * d + j];
        }
        __syncwarp();
        double v = DBL_MAX;
        int id = INT32_MAX;
        if (lane < it.m) {
            const double *cr = cs + (size_t)lane * (d + 1);
            double acc = 0.0;
#pragma unroll 8
            for (int j = 0; j < d; j++) {  // unrolled: the loads and squares run ahead of the add chain
                const double t = __dsub_rn(xs[j], cr[j]);
                acc = __dadd_rn(acc, __dmul_rn(t, t));
            }
            if (acc < DBL_MAX) {  // not below F::MAX (or NaN): never chosen
                v = acc;
                id = my_id;
            }
        }
        double b2 = DBL_MAX;
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) {
            const double ov = __shfl_xor_sync(0xffffffffu, v, off);
            const int oi = __shfl_xor_sync(0xffffffffu, id, off);
            const double ob2 = __shfl_xor_sync(0xffffffffu, b2, off);
            if (ov < v || (ov == v && oi < id)) {
                b2 = fmin(v, ob2);
                v = ov;
                id = oi;
            } else {
                b2 = fmin(b2, ov);
            }
        }
        if (lane == 0) {
            labels[it.row] = id == INT32_MAX ? 0 : id;
            atomicAdd(&sc->recheck_rows, 1ULL);
            if (id != INT32_MAX && b2 < DBL_MAX && near_tie(v, b2)) atomicAdd(&sc->near_tie_rows, 1ULL);
        }
        __syncwarp();  // the staging area is reused for the next row
    }
}

template <typename TX>
void launch_f64_decide(Ctx &ctx, const TX *x, int d, const double *c, const Oct *items, DevScalars *sc,
                       int32_t *labels) {
    const size_t smem = f64_smem_bytes(d);
    FK_CUDA(cudaFuncSetAttribute((const void *)f64_decide_kernel<TX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem));
    f64_decide_kernel<TX><<<ctx.num_sms * 2, F64_WARPS * 32, smem, ctx.stream>>>(x, d, c, items, sc, labels);
    FK_LAUNCH_CHECK();
}

// ---------------------------------------------------- mixed inertia --
// Two-level fixed-order sum of the per-(cluster, feature) partials: block b
// folds its contiguous range (four interleaved chains per thread, then a
// tree), then one block folds the block sums in order. Deterministic.
constexpr int INERTIA_BLOCKS = 256;
__global__ void inertia_partial_kernel(const double *__restrict__ part, int64_t m, double *__restrict__ out) {
    __shared__ double sh[32];
    const int64_t per = (m + gridDim.x - 1) / gridDim.x;
    const int64_t lo = (int64_t)blockIdx.x * per, hi = min(m, lo + per);
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    int64_t i = lo + threadIdx.x;
    for (; i + 3 * (int64_t)blockDim.x < hi; i += 4 * (int64_t)blockDim.x) {
        a0 += part[i];
        a1 += part[i + blockDim.x];
        a2 += part[i + 2 * blockDim.x];
        a3 += part[i + 3 * blockDim.x];
    }
    for (; i < hi; i += blockDim.x) a0 += part[i];
    double s = (a0 + a1) + (a2 + a3);
    s = warp_sum_d(s);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) sh[w] = s;
    __syncthreads();
    if (w == 0) {
        double r = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
        r = warp_sum_d(r);
        if (lane == 0) out[blockIdx.x] = r;
    }
}

__global__ void inertia_final_kernel(const double *__restrict__ part, int64_t m, double *out) {
    __shared__ double sh[32];
    double s = 0.0;
    for (int64_t i = threadIdx.x; i < m; i += blockDim.x) s += part[i];
    s = warp_sum_d(s);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) sh[w] = s;
    __syncthreads();
    if (w == 0) {
        double r = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
        r = warp_sum_d(r);
        if (lane == 0) *out = r;
    }
}

}  // namespace

// ------------------------------------------------------------- host side --
namespace {

// Device buffers of one mixed assignment.
struct MixedBufs {
    MixedStats *stats;
    double *mu;
    float *mu32;
    void *xq;               // BF16 or E4M3 rows, n x d_pad
    __nv_bfloat16 *xaug;    // FP8: per-row augmentation rows, n x 16
    float4 *rowinfo;
    void *cq;               // BF16 or E4M3 centres, k_pad x d_pad
    __nv_bfloat16 *caug;    // k_pad x 16
    double *half_norm;
    float *c32, *ec32, *c32t;
};

// Plans the launch and prepares the rows (when X changed) and the centres.
template <typename TX>
MixedBufs prepare_mixed(Ctx &ctx, const TX *x, int64_t n, int d, const double *c, int k, bool fp8, bool x_changed) {
    cudaStream_t s = ctx.stream;
    MixedPlan &mp = ctx.mixed;
    const bool replan = x_changed || mp.n != n || mp.d != d || mp.k != k || mp.x != (const void *)x || mp.fp8 != fp8;
    if (replan) plan_tc(ctx, mp, n, d, k, fp8, 2);
    mp.x = (const void *)x;
    const size_t es = fp8 ? 1 : 2;
    MixedBufs B;
    B.stats = (MixedStats *)ctx.get(BUF_CF32, sizeof(MixedStats));
    B.mu = (double *)ctx.get(BUF_COUNTS, sizeof(double) * 2 * (size_t)d + sizeof(float) * (size_t)d + 64);
    B.mu32 = (float *)(B.mu + 2 * d);
    B.xq = ctx.get(BUF_XB, es * (size_t)n * mp.d_pad);
    B.xaug = fp8 ? (__nv_bfloat16 *)ctx.get(BUF_XAUG, sizeof(__nv_bfloat16) * 16 * (size_t)n) : nullptr;
    B.rowinfo = (float4 *)ctx.get(BUF_XNORM, sizeof(float4) * (size_t)n);
    if (replan) {
        FK_CUDA(cudaMemsetAsync(B.stats, 0, sizeof(MixedStats), s));
        // the centring vector only needs to be finite: a strided sample of at
        // most 65536 rows is enough
        const int64_t stride = n > 65536 ? n / 65536 : 1;
        const int64_t rows = (n + stride - 1) / stride;
        const int64_t rows_per = 64;
        const int nparts = (int)((rows + rows_per - 1) / rows_per);
        double *part = (double *)ctx.get(BUF_PARTIAL, sizeof(double) * (size_t)nparts * d);
        dim3 g1(nparts, (d + 127) / 128);
        col_mean_partial_kernel<TX><<<g1, 128, 0, s>>>(x, n, d, rows_per, stride, part);
        FK_LAUNCH_CHECK();
        col_mean_final_kernel<<<(d + 127) / 128, 128, 0, s>>>(part, nparts, rows, d, B.mu, B.mu32);
        FK_LAUNCH_CHECK();
        if (fp8) {
            sample_tmax_kernel<TX><<<ctx.num_sms * 2, 256, 0, s>>>(x, n, d, stride, rows, B.mu32, B.stats);
            FK_LAUNCH_CHECK();
        }
        if (fp8)
            launch_prep_rows<TX, true>(ctx, x, n, d, mp.d_pad, B.mu32, B.xq, B.xaug, B.rowinfo, B.stats);
        else
            launch_prep_rows<TX, false>(ctx, x, n, d, mp.d_pad, B.mu32, B.xq, nullptr, B.rowinfo, B.stats);
        // ||mu|| for the bound on ||x|| (host side, tiny)
        std::vector<double> hmu(d);
        FK_CUDA(cudaMemcpyAsync(hmu.data(), B.mu, sizeof(double) * d, cudaMemcpyDeviceToHost, s));
        FK_CUDA(cudaStreamSynchronize(s));
        double m2 = 0.0;
        for (double v : hmu) m2 += v * v;
        mp.mu_norm = std::sqrt(m2) * (1.0 + 1e-12);
    } else {
        // centre statistics are per iteration; the row maxima stay
        FK_CUDA(cudaMemsetAsync((char *)B.stats + offsetof(MixedStats, cn_max), 0,
                                sizeof(MixedStats) - offsetof(MixedStats, cn_max), s));
    }
    B.cq = ctx.get(BUF_CB, es * (size_t)mp.k_pad * mp.d_pad);
    B.caug = (__nv_bfloat16 *)ctx.get(BUF_CAUX, sizeof(__nv_bfloat16) * (size_t)mp.k_pad * 16 + 8192);
    B.half_norm = (double *)ctx.get(BUF_MIND, sizeof(double) * (size_t)mp.k_pad);
    B.c32 = (float *)ctx.get(BUF_CF32C, sizeof(float) * (2 * (size_t)k * d + (size_t)k) + 64);
    B.ec32 = B.c32 + (size_t)k * d;
    B.c32t = B.ec32 + k;
    if (fp8)
        prep_centres_kernel<true><<<(mp.k_pad + 7) / 8, 256, 0, s>>>(c, k, mp.k_pad, d, mp.d_pad, B.mu, B.cq,
                                                                     B.half_norm, B.c32, B.ec32, B.c32t, B.stats);
    else
        prep_centres_kernel<false><<<(mp.k_pad + 7) / 8, 256, 0, s>>>(c, k, mp.k_pad, d, mp.d_pad, B.mu, B.cq,
                                                                      B.half_norm, B.c32, B.ec32, B.c32t, B.stats);
    FK_LAUNCH_CHECK();
    prep_aug_kernel<<<(mp.k_pad + 255) / 256, 256, 0, s>>>(B.half_norm, k, mp.k_pad, fp8, B.caug, B.stats);
    FK_LAUNCH_CHECK();
    return B;
}

// Blocks of `threads` threads that fit on one SM at once (the grid of a
// latency-bound grid-stride kernel: every warp resident, no second wave).
int resident_blocks(const void *fn, int threads) {
    int b = 0;
    FK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, fn, threads, 0));
    return b > 0 ? b : 1;
}

// FP8: r = 2^-sh_row * 2^-sh_t, the factor between a row's scores and its
// accumulators (exact: a product of powers of two in range).
__global__ void rowscale_kernel(const float4 *__restrict__ rowinfo, int64_t n, const MixedStats *stats,
                                float *__restrict__ rowscale) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) rowscale[i] = rowinfo[i].w * stats->inv_t;
}

// ||mu|| as an f32 upper bound.
float mu_norm_up(double v) {
    const float f = (float)v;
    return (double)f >= v ? f : std::nextafter(f, INFINITY);
}

// Second pass over the rows listed in full (count sc->full_count). After a
// BF16 main pass: the rows' BF16 operands gathered from the main pass's
// copy, a tensor pass that marks every centre scoring above the row's
// threshold, then the re-score of at most 32 candidates, or of every centre.
// After an FP8 main pass: BF16 operands made from the rows' f32 values, a
// BF16 count pass against thresholds from the rows' floors, the mask pass
// over the rows it leaves open, then the same re-score.
void second_pass(Ctx &ctx, const float *x, int64_t n, int d, const double *c, int k, const MixedBufs &B,
                 double mu_norm, const int32_t *full, const float *full_thresh, int32_t *labels, DevScalars *sc,
                 Oct *f64_items) {
    cudaStream_t s = ctx.stream;
    const int grid = ctx.num_sms * 4;
    int32_t *ex = (int32_t *)ctx.get(BUF_EX, sizeof(int32_t) * (size_t)n);
    if (!ctx.mixed.fp8) {
        // BF16 main pass: the same operands again for the listed rows, with
        // candidate masks against the thresholds the finalize left.
        const MixedPlan &mp = ctx.mixed;
        MixedPlan &mm = ctx.mixedm;
        if (mm.n != n || mm.d != d || mm.k != k || mm.kp != mp.kp) plan_tc(ctx, mm, n, d, k, false, 1, mp.kp);
        if (mm.k_pad != mp.k_pad || mm.d_pad != mp.d_pad) {
            set_error("mask pass plan (k_pad %d, d_pad %d) differs from the main pass (%d, %d)", mm.k_pad, mm.d_pad,
                      mp.k_pad, mp.d_pad);
            fail(FK_ERR_CUDA);
        }
        void *xb2 = ctx.get(BUF_XB2, sizeof(__nv_bfloat16) * (size_t)n * mm.d_pad);
        const int wpr = mm.k_pad / 32;
        uint32_t *masks = (uint32_t *)ctx.get(BUF_MASKS, sizeof(uint32_t) * (size_t)n * wpr);
        const int pieces = mm.d_pad * 2 / 16;
        gather_xq_rows_kernel<<<ctx.num_sms * 8, 256, 0, s>>>((const uint4 *)B.xq, pieces, full, &sc->full_count,
                                                              (uint4 *)xb2);
        FK_LAUNCH_CHECK();
        launch_tc_assign(ctx, mm, xb2, B.cq, B.caug, nullptr, sc, B.stats, nullptr, &sc->full_count,
                         nullptr, nullptr, masks, full_thresh);
        // latency-bound (a few dependent loads per row): as many warps as the SMs hold
        if (d % 4 == 0 && d <= 256 && (((uintptr_t)x | (uintptr_t)B.c32) & 15u) == 0) {
            static const int mask_blocks = resident_blocks((const void *)mask_rescore_kernel<true>, MASK_WARPS * 32);
            mask_rescore_kernel<true><<<ctx.num_sms * mask_blocks, MASK_WARPS * 32, 0, s>>>(
                x, d, B.c32, B.ec32, k, masks, wpr, full, &sc->full_count, sc, labels, f64_items, ex);
        } else {
            static const int mask_blocks = resident_blocks((const void *)mask_rescore_kernel<false>, MASK_WARPS * 32);
            mask_rescore_kernel<false><<<ctx.num_sms * mask_blocks, MASK_WARPS * 32, 0, s>>>(
                x, d, B.c32, B.ec32, k, masks, wpr, full, &sc->full_count, sc, labels, f64_items, ex);
        }
        FK_LAUNCH_CHECK();
        exhaustive_rescore_kernel<<<ctx.num_sms * 2, EX_THREADS, exhaustive_smem_bytes(d, k), s>>>(
            x, d, c, B.c32t, B.ec32, k, ex, &sc->ex_count, sc, labels);
        FK_LAUNCH_CHECK();
        return;
    }
    // FP8 main pass: BF16 operands made from the listed rows' f32 values
    // (their own statistics, a bound 16x tighter), a BF16 count pass against
    // thresholds from the rows' floors, then the mask pass over the rows it
    // leaves open and the re-score of at most 32 candidates
    MixedPlan &m2 = ctx.mixed2;
    if (m2.n != n || m2.d != d || m2.k != k || m2.topk != 3) plan_tc(ctx, m2, n, d, k, false, 3);
    MixedPlan &mm = ctx.mixedm2;
    if (mm.n != n || mm.d != d || mm.k != k || mm.kp != m2.kp) plan_tc(ctx, mm, n, d, k, false, 1, m2.kp);
    if (mm.k_pad != m2.k_pad || mm.d_pad != m2.d_pad) {
        set_error("second mask pass plan (k_pad %d, d_pad %d) differs from its count pass (%d, %d)", mm.k_pad,
                  mm.d_pad, m2.k_pad, m2.d_pad);
        fail(FK_ERR_CUDA);
    }
    MixedStats *st2 = (MixedStats *)ctx.get(BUF_STATS2, sizeof(MixedStats));
    void *xb2 = ctx.get(BUF_XB2, sizeof(__nv_bfloat16) * (size_t)n * m2.d_pad);
    float4 *ri2 = (float4 *)ctx.get(BUF_ROWINFO2, sizeof(float4) * (size_t)n);
    void *cb2 = ctx.get(BUF_CB2, sizeof(__nv_bfloat16) * (size_t)m2.k_pad * m2.d_pad);
    __nv_bfloat16 *caug2 = (__nv_bfloat16 *)ctx.get(BUF_CAUG2, sizeof(__nv_bfloat16) * (size_t)m2.k_pad * 16 + 8192);
    double *hn2 = (double *)ctx.get(BUF_HALF2, sizeof(double) * (size_t)m2.k_pad);
    float *th2 = (float *)ctx.get(BUF_TH2, sizeof(float) * (size_t)n);
    SliceCount *cnt2 = (SliceCount *)ctx.get(BUF_CNT2, sizeof(SliceCount) * (size_t)n * m2.parts);
    int32_t *list3 = (int32_t *)ctx.get(BUF_LIST3, sizeof(int32_t) * (size_t)n);
    int32_t *slot3 = (int32_t *)ctx.get(BUF_SLOT3, sizeof(int32_t) * (size_t)n);
    float *th3 = (float *)ctx.get(BUF_TH3, sizeof(float) * (size_t)n);
    void *xb3 = ctx.get(BUF_XB3, sizeof(__nv_bfloat16) * (size_t)n * m2.d_pad);
    const int wpr = mm.k_pad / 32;
    uint32_t *masks = (uint32_t *)ctx.get(BUF_MASKS, sizeof(uint32_t) * (size_t)n * wpr);
    const float *floors = (const float *)ctx.get(BUF_FLOORS, sizeof(float) * (size_t)n);
    const float acc_rel2 = (float)((double)((size_t)m2.d_pad + 32) * ACC_REL_PER_K);  // exact: integer * 2^-22
    const float mun = mu_norm_up(mu_norm);
    FK_CUDA(cudaMemsetAsync(st2, 0, sizeof(MixedStats), s));
    launch_prep_rows<float, false>(ctx, x, n, d, m2.d_pad, B.mu32, xb2, nullptr, ri2, st2, full, &sc->full_count);
    prep_centres_kernel<false><<<(m2.k_pad + 7) / 8, 256, 0, s>>>(c, k, m2.k_pad, d, m2.d_pad, B.mu, cb2, hn2,
                                                                  nullptr, nullptr, nullptr, st2);
    FK_LAUNCH_CHECK();
    prep_aug_kernel<<<(m2.k_pad + 255) / 256, 256, 0, s>>>(hn2, k, m2.k_pad, false, caug2, st2);
    FK_LAUNCH_CHECK();
    second_thresh_kernel<<<grid, 256, 0, s>>>(full, &sc->full_count, floors, ri2, st2, acc_rel2, mun, d, th2);
    FK_LAUNCH_CHECK();
    launch_tc_assign(ctx, m2, xb2, cb2, caug2, nullptr, sc, st2, nullptr, &sc->full_count, nullptr, nullptr,
                     nullptr, th2, cnt2);
    second_finalize_kernel<<<grid, 256, 0, s>>>(cnt2, m2.parts, m2.kp, n, k, d, full, &sc->full_count, ri2, st2,
                                                acc_rel2, mun, th2, labels, ex, list3, slot3, th3, sc);
    FK_LAUNCH_CHECK();
    const int pieces = m2.d_pad * 2 / 16;
    gather_xq_rows_kernel<<<ctx.num_sms * 8, 256, 0, s>>>((const uint4 *)xb2, pieces, slot3, &sc->mask_count,
                                                          (uint4 *)xb3);
    FK_LAUNCH_CHECK();
    launch_tc_assign(ctx, mm, xb3, cb2, caug2, nullptr, sc, st2, nullptr, &sc->mask_count, nullptr,
                     nullptr, masks, th3);
    if (d % 4 == 0 && d <= 256 && (((uintptr_t)x | (uintptr_t)B.c32) & 15u) == 0) {
        static const int mask_blocks = resident_blocks((const void *)mask_rescore_kernel<true>, MASK_WARPS * 32);
        mask_rescore_kernel<true><<<ctx.num_sms * mask_blocks, MASK_WARPS * 32, 0, s>>>(
            x, d, B.c32, B.ec32, k, masks, wpr, list3, &sc->mask_count, sc, labels, f64_items, ex);
    } else {
        static const int mask_blocks = resident_blocks((const void *)mask_rescore_kernel<false>, MASK_WARPS * 32);
        mask_rescore_kernel<false><<<ctx.num_sms * mask_blocks, MASK_WARPS * 32, 0, s>>>(
            x, d, B.c32, B.ec32, k, masks, wpr, list3, &sc->mask_count, sc, labels, f64_items, ex);
    }
    FK_LAUNCH_CHECK();
    exhaustive_rescore_kernel<<<ctx.num_sms * 2, EX_THREADS, exhaustive_smem_bytes(d, k), s>>>(
        x, d, c, B.c32t, B.ec32, k, ex, &sc->ex_count, sc, labels);
    FK_LAUNCH_CHECK();
}

}  // namespace

template <typename TX>
void run_assign_mixed(Ctx &ctx, const TX *x, int64_t n, int d, const double *c, int k, int precision,
                      int32_t *labels, double *, DevScalars *sc, bool x_changed, const double *c_prev,
                      const int32_t *labels_prev) {
    cudaStream_t s = ctx.stream;
    MixedPlan &mp = ctx.mixed;
    if (precision != FK_PRECISION_MIXED_BF16 && precision != FK_PRECISION_MIXED_FP8) {
        set_error("precision %d is not built", precision);
        fail(FK_ERR_UNSUPPORTED);
    }
    static_assert(std::is_same<TX, float>::value, "the mixed forms read X stored as f32 (the f32x64 entry points)");
    const bool fp8 = precision == FK_PRECISION_MIXED_FP8;
    if (d < 1 || d > 256) {
        set_error("the tensor-core path supports 1 <= d <= 256 (got %d)", d);
        fail(FK_ERR_UNSUPPORTED);
    }
    MixedBufs B = prepare_mixed<TX>(ctx, x, n, d, c, k, fp8, x_changed);
    float *rowscale = nullptr;
    if (fp8) {
        rowscale = (float *)ctx.get(BUF_ROWSCALE, sizeof(float) * (size_t)n);
        rowscale_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(B.rowinfo, n, B.stats, rowscale);
        FK_LAUNCH_CHECK();
    }

    int4 *pairs = (int4 *)ctx.get(BUF_FLAGS, sizeof(int4) * (size_t)n);
    int32_t *full = (int32_t *)ctx.get(BUF_FULL, sizeof(int32_t) * (size_t)n);
    float *full_thresh = fp8 ? nullptr : (float *)ctx.get(BUF_THRESH, sizeof(float) * (size_t)n);
    // every pass leaves each row's floor for a count pass in the next iteration
    float *floors = (float *)ctx.get(BUF_FLOORS, sizeof(float) * (size_t)n);
    const float acc_rel = (float)((double)((size_t)mp.d_pad + 32) * ACC_REL_PER_K);  // exact: integer * 2^-22
    const float mun = mu_norm_up(mp.mu_norm);
    static const int fin_top2 = resident_blocks((const void *)finalize_kernel, FINALIZE_THREADS);
    static const int fin_count = resident_blocks((const void *)finalize_count_kernel, FINALIZE_THREADS);
    const int64_t fin_chunks = (n + FINALIZE_THREADS - 1) / FINALIZE_THREADS;
    if (c_prev && labels_prev) {
        // count pass, against thresholds carried from the previous iteration
        MixedPlan &mc = ctx.mixedc;
        if (mc.n != n || mc.d != d || mc.k != k || mc.kp != mp.kp || mc.fp8 != fp8)
            plan_tc(ctx, mc, n, d, k, fp8, 3, mp.kp);
        if (mc.k_pad != mp.k_pad || mc.d_pad != mp.d_pad) {
            set_error("count pass plan (k_pad %d, d_pad %d) differs from the main pass (%d, %d)", mc.k_pad, mc.d_pad,
                      mp.k_pad, mp.d_pad);
            fail(FK_ERR_CUDA);
        }
        float2 *shift = (float2 *)ctx.get(BUF_SHIFT, sizeof(float2) * (size_t)k);
        centre_shift_kernel<<<(unsigned)(((int64_t)k * 32 + 255) / 256), 256, 0, s>>>(c, c_prev, B.mu, k, d, shift);
        FK_LAUNCH_CHECK();
        float *th = (float *)ctx.get(BUF_THMAIN, sizeof(float) * (size_t)n);
        count_thresh_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, k, d, floors, labels_prev, B.rowinfo,
                                                                      shift, B.stats, acc_rel, mun, th);
        FK_LAUNCH_CHECK();
        SliceCount *cnt = (SliceCount *)ctx.get(BUF_TOP2, sizeof(SliceCount) * (size_t)n * mc.parts);
        {
            Timer t(ctx.contract_acc != nullptr, ctx, ctx.contract_acc);
            Timer tc(ctx.count_acc != nullptr, ctx, ctx.count_acc);
            launch_tc_assign(ctx, mc, B.xq, B.cq, B.caug, nullptr, sc, B.stats, nullptr, nullptr, B.xaug,
                             rowscale, nullptr, th, cnt);
        }
        finalize_count_kernel<<<(unsigned)std::min<int64_t>(fin_chunks, (int64_t)ctx.num_sms * fin_count),
                                FINALIZE_THREADS, 0, s>>>(cnt, mc.parts, mc.kp, n, k, d, B.rowinfo,
                                                                      B.stats, acc_rel, mun, th, labels, pairs, full,
                                                                      full_thresh, floors, sc);
        FK_LAUNCH_CHECK();
    } else {
        SliceTop2 *top = (SliceTop2 *)ctx.get(BUF_TOP2, sizeof(SliceTop2) * (size_t)n * mp.parts);
        {
            Timer t(ctx.contract_acc != nullptr, ctx, ctx.contract_acc);
            launch_tc_assign(ctx, mp, B.xq, B.cq, B.caug, top, sc, B.stats, nullptr, nullptr, B.xaug,
                             rowscale);
        }
        finalize_kernel<<<(unsigned)std::min<int64_t>(fin_chunks, (int64_t)ctx.num_sms * fin_top2), FINALIZE_THREADS,
                          0, s>>>(top, mp.parts, mp.kp, n, k, d, B.rowinfo, B.stats,
                                                                acc_rel, mun, labels, pairs, full, full_thresh,
                                                                floors, sc);
        FK_LAUNCH_CHECK();
    }
    const int grid = ctx.num_sms * 4;
    Oct *f64_items = (Oct *)ctx.get(BUF_F64ITEMS, sizeof(Oct) * (size_t)n);
    if (std::is_same<TX, float>::value && d % 4 == 0 && d <= 128 && ((uintptr_t)x & 15u) == 0) {
        static const int pair_blocks = resident_blocks((const void *)pair_rescore4_kernel, 256);
        pair_rescore4_kernel<<<ctx.num_sms * pair_blocks, 256, 0, s>>>((const float *)x, d, c, B.c32, B.ec32, pairs,
                                                                       sc, labels, f64_items);
    } else
        pair_rescore_kernel<TX><<<grid, 256, 0, s>>>(x, d, c, B.c32, B.ec32, pairs, sc, labels, f64_items);
    FK_LAUNCH_CHECK();
    second_pass(ctx, x, n, d, c, k, B, mp.mu_norm, full, full_thresh, labels, sc, f64_items);
    launch_f64_decide<TX>(ctx, x, d, c, f64_items, sc, labels);
}

void launch_mixed_inertia(Ctx &ctx, const double *part, int64_t m, DevScalars *sc) {
    double *blocks = (double *)ctx.get(BUF_INERTIA2, sizeof(double) * INERTIA_BLOCKS);
    inertia_partial_kernel<<<INERTIA_BLOCKS, 256, 0, ctx.stream>>>(part, m, blocks);
    FK_LAUNCH_CHECK();
    inertia_final_kernel<<<1, 256, 0, ctx.stream>>>(blocks, INERTIA_BLOCKS, &sc->inertia);
    FK_LAUNCH_CHECK();
}

template void run_assign_mixed<float>(Ctx &, const float *, int64_t, int, const double *, int, int, int32_t *,
                                      double *, DevScalars *, bool, const double *, const int32_t *);

// Diagnostics for the tests: one tensor-core pass over x (f32, on the device)
// against c (f64), returning the raw accumulators of CTA 0's first tile and
// the quantised operands they were computed from.
void debug_tc_probe(Ctx &ctx, const float *x, int64_t n, int d, const double *c, int k, int precision,
                    float *dump_out, void *xq_out, void *cq_out, uint16_t *aug_out, uint16_t *xaug_out,
                    Top2 *top_out, int *plan_out) {
    cudaStream_t s = ctx.stream;
    MixedPlan &mp = ctx.mixed;
    const bool fp8 = precision == FK_PRECISION_MIXED_FP8;
    DevScalars *sc = (DevScalars *)ctx.get(BUF_SCALARS, sizeof(DevScalars));
    FK_CUDA(cudaMemsetAsync(sc, 0, sizeof(DevScalars), s));
    MixedBufs B = prepare_mixed<float>(ctx, x, n, d, c, k, fp8, true);
    mp.x = nullptr;
    float *rowscale = nullptr;
    if (fp8) {
        rowscale = (float *)ctx.get(BUF_ROWSCALE, sizeof(float) * (size_t)n);
        rowscale_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(B.rowinfo, n, B.stats, rowscale);
        FK_LAUNCH_CHECK();
    }
    SliceTop2 *top = (SliceTop2 *)ctx.get(BUF_TOP2, sizeof(SliceTop2) * (size_t)n * mp.parts);
    float *dump = (float *)ctx.get(BUF_OUT, sizeof(float) * 128 * (size_t)mp.kp);
    FK_CUDA(cudaMemsetAsync(dump, 0, sizeof(float) * 128 * (size_t)mp.kp, s));
    launch_tc_assign(ctx, mp, B.xq, B.cq, B.caug, top, sc, B.stats, dump, nullptr, B.xaug, rowscale);
    const size_t es = fp8 ? 1 : 2;
    FK_CUDA(cudaMemcpyAsync(dump_out, dump, sizeof(float) * 128 * (size_t)mp.kp, cudaMemcpyDeviceToHost, s));
    const int64_t rows = n < 128 ? n : 128;
    FK_CUDA(cudaMemcpyAsync(xq_out, B.xq, es * (size_t)rows * mp.d_pad, cudaMemcpyDeviceToHost, s));
    FK_CUDA(cudaMemcpyAsync(cq_out, B.cq, es * (size_t)mp.k_pad * mp.d_pad, cudaMemcpyDeviceToHost, s));
    FK_CUDA(cudaMemcpyAsync(aug_out, B.caug, sizeof(uint16_t) * (size_t)mp.k_pad * 16, cudaMemcpyDeviceToHost, s));
    if (fp8)
        FK_CUDA(cudaMemcpyAsync(xaug_out, B.xaug, sizeof(uint16_t) * 16 * (size_t)rows, cudaMemcpyDeviceToHost, s));
    std::vector<SliceTop2> recs((size_t)n * mp.parts);
    FK_CUDA(cudaMemcpyAsync(recs.data(), top, sizeof(SliceTop2) * recs.size(), cudaMemcpyDeviceToHost, s));
    FK_CUDA(cudaMemcpyAsync(ctx.host_scalars, sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, s));
    FK_CUDA(cudaStreamSynchronize(s));
    for (size_t e = 0; e < recs.size(); e++) {  // the records with absolute centre indices
        const int base = (int)(e / (size_t)n) * mp.kp;
        const SliceTop2 &r = recs[e];
        top_out[e] = Top2{r.v1, r.v2, r.u3, 0.f, slice_index(r.ids & 0xFFFFu, base), slice_index(r.ids >> 16, base),
                          0, 0};
    }
    plan_out[0] = mp.d_pad;
    plan_out[1] = mp.kp;
    plan_out[2] = mp.parts;
    plan_out[3] = mp.k_pad;
    plan_out[4] = mp.grid;
    plan_out[5] = (int)ctx.host_scalars->error_word;
}

}  // namespace fk
