// fk_mixed.cu -- mixed-precision assignment with an exact FP64 re-check.
//
// The approximate pass scores every (row, centre) pair as
//     T_c = xh . ch + a_c,   a_c = BIG - ||c'||^2 / 2,
// where x' = x - mu and c' = c - mu are centred by the column mean mu, xh and
// ch are their BF16 roundings, and BIG is a per-iteration constant that makes
// every T_c positive. Maximising T_c minimises ||x - c||^2. The contraction
// runs on the tensor cores (fk_tc.cu); a_c enters as three extra BF16 columns
// multiplied by a constant column of ones, so the epilogue only ranks values.
//
// Per row, with the pass's best and second-best values v1 >= v2, the error
// bound (in T units)
//     E = ex * Cn + xn * Ec + ACC * (xn * Chn + BIG) + REPR * BIG
// (ex = ||x' - xh||, xn = ||xh||, Cn = max ||c'||, Ec = max ||c' - ch||,
// Chn = max ||ch||; ACC and REPR generous multiples of 2^-22 covering the FP32
// accumulation and the three-term BF16 split of a_c), the key-truncation
// quantum q and the FP64 oracle's own rounding delta give the threshold
// thr = 2E + q + delta. If v1 - v2 > thr no other centre can win in the FP64
// direct form, so the label is final. Otherwise, if the best value outside the
// top two is also below v1 - thr, only the top two are re-scored exactly;
// else the row goes through a second tensor-core pass that keeps the best four
// scores, and only the centres inside the bound among those four are
// re-scored (rows with more than four such centres, or a non-finite score,
// are re-scored against every centre). Every re-score is the
// direct-form sum (x_j - c_j)^2 in FP64 with no FMA and the lowest index on
// ties, i.e. exactly kmeans.rs:159-163 / 295-309, so the labels equal the
// FP64 oracle's in every case.
#include <cfloat>
#include <cmath>
#include <cuda_bf16.h>

#include <algorithm>
#include <cstddef>
#include <type_traits>
#include <vector>

#include "fk_internal.cuh"

namespace fk {
namespace {

constexpr double ACC_REL_PER_K = 0.0000002384185791015625;  // 2^-22 per accumulated column
constexpr double REPR_REL = 0.0000002384185791015625;       // 2^-22

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

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// One warp per row: BF16 copy of x - mu (row stride d_pad, zero padded) and
// the row's bound ingredients {||xh||, ||x' - xh||, ||x||}, all computed in
// f32 and then inflated to upper bounds: t = fl(x - mu) differs from x - mu
// by at most 2^-24 |t|, xh = bf16(t) and t - xh is exact, so
// ||x' - xh|| <= ||t - xh|| + 2^-24 ||t||; each sum of squares is scaled by
// (1 + (d + 64) 2^-23) to cover its own rounding before the rounded-up root.
// Also records max |x| (for the fixed-point centroid sums) and max ||xh||.
template <typename TX>
__global__ void prep_rows_kernel(const TX *__restrict__ x, int64_t n, int d, int d_pad,
                                 const float *__restrict__ mu32, __nv_bfloat16 *__restrict__ xb,
                                 float4 *__restrict__ rowinfo, MixedStats *stats) {
    __shared__ float sh_xn[32], sh_am[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
    float xn_hi = 0.f, am_hi = 0.f;
    for (int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + w; row < n; row += nwarps) {
        float xn2 = 0.f, ex2 = 0.f, tn2 = 0.f, xo2 = 0.f, amax = 0.f;
        for (int j = lane; j < d_pad; j += 32) {
            __nv_bfloat16 h = __float2bfloat16_rn(0.f);
            if (j < d) {
                float xv = (float)x[row * d + j];
                float t = __fsub_rn(xv, mu32[j]);
                h = __float2bfloat16_rn(t);
                float hv = __bfloat162float(h);
                float e = __fsub_rn(t, hv);
                xn2 = __fmaf_rn(hv, hv, xn2);
                ex2 = __fmaf_rn(e, e, ex2);
                tn2 = __fmaf_rn(t, t, tn2);
                xo2 = __fmaf_rn(xv, xv, xo2);
                amax = fmaxf(amax, fabsf(xv));
            }
            xb[row * d_pad + j] = h;
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
        if (lane == 0) rowinfo[row] = make_float4(xn, ex, xo, 0.f);
        if (xn < INFINITY) xn_hi = fmaxf(xn_hi, xn);  // NaN / inf rows are re-scored in full
        if (amax < INFINITY) am_hi = fmaxf(am_hi, amax);
    }
    if (lane == 0) {
        sh_xn[w] = xn_hi;
        sh_am[w] = am_hi;
    }
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

// -------------------------------------------------------- centre prep --
// One warp per (padded) centre row: BF16 copy of c - mu, and the maxima of
// ||c'||, ||c' - ch||, ||ch||, ||c'||^2 / 2, ||c|| over the real centres.
__global__ void prep_centres_kernel(const double *__restrict__ c, int k, int k_pad, int d, int d_pad,
                                    const double *__restrict__ mu, __nv_bfloat16 *__restrict__ cb,
                                    double *__restrict__ half_norm, float *__restrict__ c32,
                                    float *__restrict__ ec32, float *__restrict__ c32t, MixedStats *stats) {
    const int lane = threadIdx.x & 31;
    const int q = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (q >= k_pad) return;
    double cn2 = 0.0, ec2 = 0.0, ch2 = 0.0, co2 = 0.0, e32 = 0.0;
    for (int j = lane; j < d_pad; j += 32) {
        __nv_bfloat16 h = __float2bfloat16_rn(0.f);
        if (q < k && j < d) {
            double cv = c[(int64_t)q * d + j];
            double cc = cv - mu[j];
            h = __float2bfloat16_rn((float)cc);
            double hv = (double)__bfloat162float(h);
            cn2 += cc * cc;
            ec2 += (cc - hv) * (cc - hv);
            ch2 += hv * hv;
            co2 += cv * cv;
            float f = (float)cv;
            c32[(int64_t)q * d + j] = f;
            c32t[(int64_t)j * k + q] = f;
            e32 += (cv - (double)f) * (cv - (double)f);
        }
        cb[(int64_t)q * d_pad + j] = h;
    }
    cn2 = warp_sum_d(cn2);
    ec2 = warp_sum_d(ec2);
    ch2 = warp_sum_d(ch2);
    co2 = warp_sum_d(co2);
    e32 = warp_sum_d(e32);
    if (lane == 0 && q < k) {
        const double up = 1.0 + 1e-12;
        ec32[q] = __double2float_ru(sqrt(e32) * up);
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
__global__ void prep_aug_kernel(const double *__restrict__ half_norm, int k, int k_pad,
                                __nv_bfloat16 *__restrict__ caug, MixedStats *stats) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= k_pad) return;
    const double span = (double)stats->xn_max * (double)stats->ch_max + (double)stats->h_max;
    const int e = (int)ceil(log2(2.02 * span + 256.0));
    const double big = 1.5 * ldexp(1.0, e);
    if (q == 0) {
        stats->big = (float)big;
        stats->cgrid = (float)(3.0 * ldexp(1.0, e + 6));
        stats->ulp = (float)ldexp(1.0, e - 23);
    }
    __nv_bfloat16 t[16];
#pragma unroll
    for (int j = 0; j < 16; j++) t[j] = __float2bfloat16_rn(0.f);
    if (q < k) {
        double a = big - half_norm[q];
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
// Threshold on a score margin above which no other centre can win in the
// FP64 direct form (see the file header): 2E + key quantum + FP64 rounding.
__device__ __forceinline__ double row_threshold(const float4 ri, const MixedStats *stats, double acc_rel, double mu_norm,
                                                int d, float v1) {
    const double xn = ri.x, ex = ri.y, xo = ri.z;
    const double cn = stats->cn_max, ec = stats->ec_max, ch = stats->ch_max, big = stats->big;
    const double co = stats->co_max;
    double e = ex * cn + xn * ec + acc_rel * (xn * ch + big) + REPR_REL * big;
    // keys: each score rounded to a multiple of 128 ulp (error <= 64 ulp) plus a
    // column code below 128 ulp, so a key is within 192 ulp of its score
    double q = 384.0 * (double)stats->ulp;
    double xo_b = xo > xn + ex + mu_norm ? xo : xn + ex + mu_norm;  // ||x|| (both bounds are valid)
    double delta = (double)(d + 4) * 1.1102230246251565e-16 * (xo_b + co) * (xo_b + co);  // FP64 rounding, D units
    double thr = (2.0 * e + q + 0.5 * delta) * (1.0 + 1e-6) + 1e-30;
    if (!(v1 >= stats->big * 0.6f)) thr = INFINITY;  // not a real score (NaN row, all slices padded)
    return thr;
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

__global__ void finalize_kernel(const Top2 *__restrict__ parts, int nparts, int64_t n, int k, int d,
                                const float4 *__restrict__ rowinfo, const MixedStats *stats, double acc_rel,
                                double mu_norm, int32_t *__restrict__ labels, int4 *__restrict__ pair_list,
                                int32_t *__restrict__ full_list, DevScalars *sc) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Top2 t = parts[i];
    float v1 = t.v1, v2 = t.v2, u3 = t.u3;
    int i1 = t.i1, i2 = t.i2;
    for (int p = 1; p < nparts; p++) {
        Top2 o = parts[(int64_t)p * n + i];
        merge_top2(v1, i1, v2, i2, u3, o.v1, o.i1, o.v2, o.i2, o.u3);
    }
    const double thr = row_threshold(rowinfo[i], stats, acc_rel, mu_norm, d, v1);
    double m12 = (double)v1 - (double)v2;
    if (i1 >= 0 && i1 < k && m12 > thr) {
        labels[i] = i1;
        return;
    }
    double m13 = (double)v1 - (double)u3;
    if (i1 >= 0 && i1 < k && i2 >= 0 && i2 < k && i1 != i2 && m13 > thr) {
        unsigned long long slot = atomicAdd(&sc->flag_count, 1ULL);
        pair_list[slot] = make_int4((int)i, i1, i2, 0);
    } else {
        unsigned long long slot = atomicAdd(&sc->full_count, 1ULL);
        full_list[slot] = (int32_t)i;
    }
}

// ------------------------------------------------------------ re-checks --
template <typename TX>
__device__ __forceinline__ double sqeuc64(const TX *__restrict__ x, const double *__restrict__ c, int d) {
    double acc = 0.0;
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

// FP32 direct form with a rigorous bound of its distance from the exact
// real distance: (d+3) 2^-23 d32 for the roundings of the differences, the
// squares and the running sum, plus the effect of the centre's rounding to
// f32 (ec = ||c - c32||), plus the FP64 oracle's own rounding.
__device__ __forceinline__ float sqeuc32(const float *__restrict__ x, const float *__restrict__ c, int d) {
    float acc = 0.f;
    for (int j = 0; j < d; j++) {
        float t = x[j] - c[j];
        acc = fmaf(t, t, acc);
    }
    return acc;
}

// Upper bound, in f32 with upward rounding, of |d32 - D| + |D64 - D| where D
// is the exact real distance and D64 the oracle's FP64 direct form:
// ((d+4) 2^-23 d32 + 2 sqrt(d32) ec + 3 ec^2) * 1.01.
__device__ __forceinline__ float bound32(float d32, float ec, int d) {
    const float dd = d32 > 0.f ? d32 : 0.f;
    float e = __fmul_ru((float)(d + 4) * 1.1920929e-07f, dd);
    e = __fadd_ru(e, __fmul_ru(__fmul_ru(2.0f, __fsqrt_ru(dd)), ec));
    e = __fadd_ru(e, __fmul_ru(3.0f, __fmul_ru(ec, ec)));
    return __fadd_ru(__fmul_ru(e, 1.01f), 1e-30f);
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
                                    const int4 *__restrict__ list, DevScalars *sc, int32_t *__restrict__ labels) {
    const unsigned long long cnt = sc->flag_count;
    const int lane = threadIdx.x & 31;
    const unsigned long long wid = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned long long nw = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
    for (unsigned long long s = wid; s < cnt; s += nw) {
        const int4 e = list[s];
        const TX *row = x + (int64_t)e.x * d;
        const int a = e.y < e.z ? e.y : e.z, b = e.y < e.z ? e.z : e.y;
        if constexpr (std::is_same<TX, float>::value) {
            const float *ca = c32 + (int64_t)a * d, *cb = c32 + (int64_t)b * d;
            float sa = 0.f, sb = 0.f;
            for (int j = lane; j < d; j += 32) {
                const float xv = row[j];
                const float ta = xv - ca[j], tb = xv - cb[j];
                sa = fmaf(ta, ta, sa);
                sb = fmaf(tb, tb, sb);
            }
            sa = warp_sum_f(sa);
            sb = warp_sum_f(sb);
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
        double dv = 0.0;
        if (lane < 2) dv = sqeuc64(row, c + (int64_t)(lane == 0 ? a : b) * d, d);
        const double da = __shfl_sync(0xffffffffu, dv, 0), db = __shfl_sync(0xffffffffu, dv, 1);
        if (lane == 0) {
            int best = 0;
            double bd = DBL_MAX;
            if (da < bd) { bd = da; best = a; }
            if (db < bd) { bd = db; best = b; }
            labels[e.x] = best;
            atomicAdd(&sc->recheck_rows, 1ULL);
            if (near_tie(da, db)) atomicAdd(&sc->near_tie_rows, 1ULL);
        }
    }
}

// One warp per listed row: FP32 distances to every centre give an upper
// bound UB of the minimum; only centres whose lower bound reaches UB (or
// whose FP32 value is not finite) are scored exactly in FP64, and the lowest
// index wins among equal FP64 distances below F::MAX, exactly as
// nearest_center.
template <typename TX>
__global__ void full_rescore_kernel(const TX *__restrict__ x, int d, const double *__restrict__ c,
                                    const float *__restrict__ c32, const float *__restrict__ ec32, int k,
                                    const int32_t *__restrict__ list, const unsigned long long *count_ptr,
                                    DevScalars *sc, int32_t *__restrict__ labels) {
    const unsigned long long cnt = *count_ptr;
    const int lane = threadIdx.x & 31;
    const unsigned long long wid = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned long long nw = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
    for (unsigned long long s = wid; s < cnt; s += nw) {
        const int64_t r = list[s];
        const TX *row = x + r * d;
        float ub = INFINITY;
        if constexpr (std::is_same<TX, float>::value) {
            for (int q = lane; q < k; q += 32) {
                float v = sqeuc32(row, c32 + (int64_t)q * d, d);
                float hi = __fadd_ru(v, bound32(v, ec32[q], d));
                if (hi < ub) ub = hi;  // NaN never lowers the bound
            }
#pragma unroll
            for (int off = 16; off >= 1; off >>= 1) ub = fminf(ub, __shfl_xor_sync(0xffffffffu, ub, off));
        }
        double b1 = DBL_MAX, b2 = DBL_MAX;
        int i1 = INT32_MAX;
        for (int q = lane; q < k; q += 32) {
            if constexpr (std::is_same<TX, float>::value) {
                float v = sqeuc32(row, c32 + (int64_t)q * d, d);
                if (__fsub_rd(v, bound32(v, ec32[q], d)) > ub) continue;  // certainly above the minimum
            }
            double v = sqeuc64(row, c + (int64_t)q * d, d);
            if (v < b1) { b2 = b1; b1 = v; i1 = q; }
            else if (v < b2) { b2 = v; }
        }
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) {
            double o1 = __shfl_xor_sync(0xffffffffu, b1, off);
            double o2 = __shfl_xor_sync(0xffffffffu, b2, off);
            int oi = __shfl_xor_sync(0xffffffffu, i1, off);
            if (o1 < b1 || (o1 == b1 && oi < i1)) {
                b2 = fmin(b1, o2);
                b1 = o1;
                i1 = oi;
            } else {
                b2 = fmin(b2, o1);
            }
        }
        if (lane == 0) {
            labels[r] = i1 == INT32_MAX ? 0 : i1;
            atomicAdd(&sc->recheck_rows, 1ULL);
            atomicAdd(&sc->full_rows, 1ULL);
            if (i1 != INT32_MAX && b2 < DBL_MAX && near_tie(b1, b2)) atomicAdd(&sc->near_tie_rows, 1ULL);
        }
    }
}

// One warp per listed row, f32 rows: FP32 distances to every centre, lanes
// over centres reading the transposed f32 centres (coalesced), 32 distances
// per lane in registers per batch of 1024 centres; the smallest upper bound
// UB over all centres, then FP64 (direct form, one lane per centre) for every
// centre whose lower bound reaches UB or whose FP32 value is not finite.
__global__ void exhaustive_rescore_kernel(const float *__restrict__ x, int d, const double *__restrict__ c,
                                          const float *__restrict__ c32t, const float *__restrict__ ec32, int k,
                                          const int32_t *__restrict__ list, const unsigned long long *count_ptr,
                                          DevScalars *sc, int32_t *__restrict__ labels) {
    const unsigned long long cnt = *count_ptr;
    const int lane = threadIdx.x & 31;
    const unsigned long long wid = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned long long nw = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
    for (unsigned long long s = wid; s < cnt; s += nw) {
        const int64_t r = list[s];
        const float *row = x + r * d;
        // pass 1: smallest upper bound over all centres
        float ub = INFINITY;
        float acc[32];
        for (int c0 = 0; c0 < k; c0 += 1024) {
#pragma unroll
            for (int u = 0; u < 32; u++) acc[u] = 0.f;
            for (int j = 0; j < d; j++) {
                const float xv = row[j];
                const float *ct = c32t + (int64_t)j * k;
#pragma unroll
                for (int u = 0; u < 32; u++) {
                    const int q = c0 + u * 32 + lane;
                    if (q < k) {
                        const float t = xv - ct[q];
                        acc[u] = fmaf(t, t, acc[u]);
                    }
                }
            }
#pragma unroll
            for (int u = 0; u < 32; u++) {
                const int q = c0 + u * 32 + lane;
                if (q < k) {
                    const float hi = __fadd_ru(acc[u], bound32(acc[u], ec32[q], d));
                    if (hi < ub) ub = hi;  // NaN never lowers the bound
                }
            }
        }
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) ub = fminf(ub, __shfl_xor_sync(0xffffffffu, ub, off));
        // pass 2: FP64 on the survivors (the distances of the first batch are
        // still in registers when k <= 1024; larger k recomputes them)
        double b1 = DBL_MAX, b2 = DBL_MAX;
        int i1 = INT32_MAX;
        for (int c0 = 0; c0 < k; c0 += 1024) {
            if (c0 > 0 || k > 1024) {
#pragma unroll
                for (int u = 0; u < 32; u++) acc[u] = 0.f;
                for (int j = 0; j < d; j++) {
                    const float xv = row[j];
                    const float *ct = c32t + (int64_t)j * k;
#pragma unroll
                    for (int u = 0; u < 32; u++) {
                        const int q = c0 + u * 32 + lane;
                        if (q < k) {
                            const float t = xv - ct[q];
                            acc[u] = fmaf(t, t, acc[u]);
                        }
                    }
                }
            }
            uint32_t cand = 0;
#pragma unroll
            for (int u = 0; u < 32; u++) {
                const int q = c0 + u * 32 + lane;
                if (q < k && !(__fsub_rd(acc[u], bound32(acc[u], ec32[q], d)) > ub)) cand |= 1u << u;
            }
            while (cand) {  // increasing centre index within this lane
                const int u = __ffs(cand) - 1;
                cand &= cand - 1;
                const int q = c0 + u * 32 + lane;
                const double v = sqeuc64(row, c + (int64_t)q * d, d);
                if (v < b1) { b2 = b1; b1 = v; i1 = q; }
                else if (v < b2) { b2 = v; }
            }
        }
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) {
            double o1 = __shfl_xor_sync(0xffffffffu, b1, off);
            double o2 = __shfl_xor_sync(0xffffffffu, b2, off);
            int oi = __shfl_xor_sync(0xffffffffu, i1, off);
            if (o1 < b1 || (o1 == b1 && oi < i1)) {
                b2 = fmin(b1, o2);
                b1 = o1;
                i1 = oi;
            } else {
                b2 = fmin(b2, o1);
            }
        }
        if (lane == 0) {
            labels[r] = i1 == INT32_MAX ? 0 : i1;
            atomicAdd(&sc->recheck_rows, 1ULL);
            if (i1 != INT32_MAX && b2 < DBL_MAX && near_tie(b1, b2)) atomicAdd(&sc->near_tie_rows, 1ULL);
        }
    }
}

// ------------------------------------------------------- second pass --
// Rows whose third-best BF16 score was inside the bound are gathered and
// scored again by the tensor cores with a top-4 epilogue; then only the (at
// most four) centres inside the bound are re-scored.
__global__ void gather_rows_kernel(const uint4 *__restrict__ xb, int row_vecs, const int32_t *__restrict__ list,
                                   const unsigned long long *count_ptr, uint4 *__restrict__ xb2) {
    const unsigned long long cnt = *count_ptr;
    const int lane = threadIdx.x & 31;
    const unsigned long long wid = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned long long nw = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
    for (unsigned long long s = wid; s < cnt; s += nw) {
        const int64_t r = list[s];
        for (int v = lane; v < row_vecs; v += 32) xb2[(int64_t)s * row_vecs + v] = xb[r * row_vecs + v];
    }
}

struct Quad {
    int row, m, i0, i1, i2, i3, pad0, pad1;
};

__device__ __forceinline__ uint32_t ins4u(uint32_t (&R)[4], int (&I)[4], uint32_t w, int j) {
#pragma unroll
    for (int p = 0; p < 4; p++) {
        if (w > R[p]) {
            const uint32_t tw = R[p];
            const int tj = I[p];
            R[p] = w;
            I[p] = j;
            w = tw;
            j = tj;
        }
    }
    return w;
}

__global__ void finalize4_kernel(const Top4 *__restrict__ parts, int nparts, int64_t cap, int k, int d,
                                 const int32_t *__restrict__ list, const float4 *__restrict__ rowinfo,
                                 const MixedStats *stats, double acc_rel, double mu_norm, int32_t *__restrict__ labels,
                                 Quad *__restrict__ quads, int32_t *__restrict__ ex_list, DevScalars *sc) {
    const unsigned long long cnt = sc->full_count;
    for (unsigned long long s = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; s < cnt;
         s += (unsigned long long)gridDim.x * blockDim.x) {
        uint32_t R[4], U;
        int I[4];
        {
            const Top4 t = parts[s];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                R[j] = __float_as_uint(t.v[j]);
                I[j] = t.i[j];
            }
            U = __float_as_uint(t.u5);
        }
        for (int p = 1; p < nparts; p++) {
            const Top4 o = parts[(int64_t)p * cap + s];
            U = max(U, __float_as_uint(o.u5));
#pragma unroll
            for (int j = 0; j < 4; j++) U = max(U, ins4u(R, I, __float_as_uint(o.v[j]), o.i[j]));
        }
        const int32_t row = list[s];
        const float v1 = __uint_as_float(R[0]);
        const double thr = row_threshold(rowinfo[row], stats, acc_rel, mu_norm, d, v1);
        const bool rest_out = (double)v1 - (double)__uint_as_float(U) > thr;
        int m = 0;
        bool valid = true;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            if ((double)v1 - (double)__uint_as_float(R[j]) <= thr) {
                m++;
                if (I[j] < 0 || I[j] >= k) valid = false;
            }
        }
        if (!rest_out || !valid || m == 0) {
            unsigned long long slot = atomicAdd(&sc->ex_count, 1ULL);
            ex_list[slot] = row;
        } else if (m == 1) {
            labels[row] = I[0];
        } else {
            unsigned long long slot = atomicAdd(&sc->quad_count, 1ULL);
            quads[slot] = Quad{row, m, I[0], I[1], I[2], I[3], 0, 0};
        }
    }
}

// One warp per row with at most four candidates: FP32 distances (lanes over
// the features) with rigorous bounds; the candidates whose lower bound
// reaches the smallest upper bound are scored exactly in FP64 (one lane
// each, direct form), lowest index on ties.
__global__ void quad_rescore_kernel(const float *__restrict__ x, int d, const double *__restrict__ c,
                                    const float *__restrict__ c32, const float *__restrict__ ec32,
                                    const Quad *__restrict__ quads, DevScalars *sc, int32_t *__restrict__ labels) {
    const unsigned long long cnt = sc->quad_count;
    const int lane = threadIdx.x & 31;
    const unsigned long long wid = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned long long nw = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
    for (unsigned long long s = wid; s < cnt; s += nw) {
        const Quad qd = quads[s];
        const int ids[4] = {qd.i0, qd.i1, qd.i2, qd.i3};
        const float *row = x + (int64_t)qd.row * d;
        float dist[4], err[4];
        float ub = INFINITY;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            float acc = 0.f;
            if (j < qd.m) {
                const float *cc = c32 + (int64_t)ids[j] * d;
                for (int f = lane; f < d; f += 32) {
                    const float t = row[f] - cc[f];
                    acc = fmaf(t, t, acc);
                }
            }
            acc = warp_sum_f(acc);
            dist[j] = acc;
            err[j] = j < qd.m ? bound32(acc, ec32[ids[j]], d) : 0.f;
            if (j < qd.m) ub = fminf(ub, __fadd_ru(acc, err[j]));
        }
        int nsurv = 0, only = -1;
#pragma unroll
        for (int j = 0; j < 4; j++)
            if (j < qd.m && !(__fsub_rd(dist[j], err[j]) > ub)) {
                nsurv++;
                only = ids[j];
            }
        if (nsurv == 1) {
            if (lane == 0) labels[qd.row] = only;
            continue;
        }
        // FP64 on the survivors (or on all candidates if some FP32 value was not finite)
        double v = DBL_MAX;
        int id = INT32_MAX;
        if (lane < qd.m) {
            const bool surv = nsurv == 0 || !(__fsub_rd(dist[lane], err[lane]) > ub);
            if (surv) {
                id = ids[lane];
                v = sqeuc64(row, c + (int64_t)id * d, d);
                if (!(v < DBL_MAX)) id = INT32_MAX;  // not below F::MAX: never chosen
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
            labels[qd.row] = id == INT32_MAX ? 0 : id;
            atomicAdd(&sc->recheck_rows, 1ULL);
            if (id != INT32_MAX && b2 < DBL_MAX && near_tie(v, b2)) atomicAdd(&sc->near_tie_rows, 1ULL);
        }
    }
}

// ---------------------------------------------------- mixed inertia --
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

// ---------------------------------------------------------------- driver --
template <typename TX>
void run_assign_mixed(Ctx &ctx, const TX *x, int64_t n, int d, const double *c, int k, int precision,
                      int32_t *labels, double *, DevScalars *sc, bool x_changed) {
    cudaStream_t s = ctx.stream;
    MixedPlan &mp = ctx.mixed;
    if (precision != FK_PRECISION_MIXED_BF16) {
        set_error("precision %d is not built", precision);
        fail(FK_ERR_UNSUPPORTED);
    }
    if (d < 1 || d > 256) {
        set_error("the BF16 tensor-core path supports 1 <= d <= 256 (got %d)", d);
        fail(FK_ERR_UNSUPPORTED);
    }
    const bool replan = x_changed || mp.n != n || mp.d != d || mp.k != k || mp.x != (const void *)x;
    if (replan) plan_tc(ctx, mp, n, d, k);
    mp.x = (const void *)x;
    auto *stats = (MixedStats *)ctx.get(BUF_CF32, sizeof(MixedStats));
    double *mu = (double *)ctx.get(BUF_COUNTS, sizeof(double) * 2 * (size_t)d + sizeof(float) * (size_t)d + 64);
    float *mu32 = (float *)(mu + 2 * d);
    __nv_bfloat16 *xb = (__nv_bfloat16 *)ctx.get(BUF_XB, sizeof(__nv_bfloat16) * (size_t)n * mp.d_pad);
    float4 *rowinfo = (float4 *)ctx.get(BUF_XNORM, sizeof(float4) * (size_t)n);
    if (replan) {
        FK_CUDA(cudaMemsetAsync(stats, 0, sizeof(MixedStats), s));
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
        col_mean_final_kernel<<<(d + 127) / 128, 128, 0, s>>>(part, nparts, rows, d, mu, mu32);
        FK_LAUNCH_CHECK();
        const int64_t pblocks = std::min<int64_t>((n + 7) / 8, (int64_t)ctx.num_sms * 16);
        prep_rows_kernel<TX><<<(unsigned)pblocks, 256, 0, s>>>(x, n, d, mp.d_pad, mu32, xb, rowinfo, stats);
        FK_LAUNCH_CHECK();
        // ||mu|| for the bound on ||x|| (host side, tiny)
        std::vector<double> hmu(d);
        FK_CUDA(cudaMemcpyAsync(hmu.data(), mu, sizeof(double) * d, cudaMemcpyDeviceToHost, s));
        FK_CUDA(cudaStreamSynchronize(s));
        double m2 = 0.0;
        for (double v : hmu) m2 += v * v;
        mp.mu_norm = std::sqrt(m2) * (1.0 + 1e-12);
    } else {
        // centre statistics are per iteration; the row maximum stays
        FK_CUDA(cudaMemsetAsync((char *)stats + offsetof(MixedStats, cn_max), 0,
                                sizeof(MixedStats) - offsetof(MixedStats, cn_max), s));
    }
    __nv_bfloat16 *cb = (__nv_bfloat16 *)ctx.get(BUF_CB, sizeof(__nv_bfloat16) * (size_t)mp.k_pad * mp.d_pad);
    __nv_bfloat16 *caug = (__nv_bfloat16 *)ctx.get(BUF_CAUX, sizeof(__nv_bfloat16) * (size_t)mp.k_pad * 16 + 8192);
    double *half_norm = (double *)ctx.get(BUF_MIND, sizeof(double) * (size_t)mp.k_pad);
    float *c32 = (float *)ctx.get(BUF_CF32C, sizeof(float) * (2 * (size_t)k * d + (size_t)k) + 64);
    float *ec32 = c32 + (size_t)k * d;
    float *c32t = ec32 + k;
    prep_centres_kernel<<<(mp.k_pad + 7) / 8, 256, 0, s>>>(c, k, mp.k_pad, d, mp.d_pad, mu, cb, half_norm, c32, ec32,
                                                           c32t, stats);
    FK_LAUNCH_CHECK();
    prep_aug_kernel<<<(mp.k_pad + 255) / 256, 256, 0, s>>>(half_norm, k, mp.k_pad, caug, stats);
    FK_LAUNCH_CHECK();

    Top2 *top = (Top2 *)ctx.get(BUF_TOP2, sizeof(Top2) * (size_t)n * mp.parts);
    {
        Timer t(ctx.contract_acc != nullptr, ctx, ctx.contract_acc);
        launch_tc_assign(ctx, mp, xb, cb, caug, top, sc, stats);
    }

    int4 *pairs = (int4 *)ctx.get(BUF_FLAGS, sizeof(int4) * (size_t)n);
    int32_t *full = (int32_t *)ctx.get(BUF_FULL, sizeof(int32_t) * (size_t)n);
    const double acc_rel = (double)(mp.d_pad + 32) * ACC_REL_PER_K;
    finalize_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(top, mp.parts, n, k, d, rowinfo, stats, acc_rel,
                                                               mp.mu_norm, labels, pairs, full, sc);
    FK_LAUNCH_CHECK();
    const int grid = ctx.num_sms * 4;
    pair_rescore_kernel<TX><<<grid, 256, 0, s>>>(x, d, c, c32, ec32, pairs, sc, labels);
    FK_LAUNCH_CHECK();
    if constexpr (std::is_same<TX, float>::value) {
        // second tensor pass over the rows whose third score was inside the bound
        __nv_bfloat16 *xb2 = (__nv_bfloat16 *)ctx.get(BUF_XB2, sizeof(__nv_bfloat16) * (size_t)n * mp.d_pad);
        Top4 *top4 = (Top4 *)ctx.get(BUF_TOP4, sizeof(Top4) * (size_t)n * mp.parts);
        Quad *quads = (Quad *)ctx.get(BUF_QUAD, sizeof(Quad) * (size_t)n);
        int32_t *ex = (int32_t *)ctx.get(BUF_EX, sizeof(int32_t) * (size_t)n);
        gather_rows_kernel<<<grid, 256, 0, s>>>((const uint4 *)xb, mp.d_pad * 2 / 16, full, &sc->full_count,
                                                (uint4 *)xb2);
        FK_LAUNCH_CHECK();
        launch_tc_assign(ctx, mp, xb2, cb, caug, nullptr, sc, stats, nullptr, top4, &sc->full_count);
        finalize4_kernel<<<grid, 256, 0, s>>>(top4, mp.parts, n, k, d, full, rowinfo, stats, acc_rel, mp.mu_norm,
                                              labels, quads, ex, sc);
        FK_LAUNCH_CHECK();
        quad_rescore_kernel<<<grid, 256, 0, s>>>(x, d, c, c32, ec32, quads, sc, labels);
        FK_LAUNCH_CHECK();
        exhaustive_rescore_kernel<<<grid, 256, 0, s>>>(x, d, c, c32t, ec32, k, ex, &sc->ex_count, sc, labels);
    } else {
        full_rescore_kernel<TX><<<grid, 256, 0, s>>>(x, d, c, c32, ec32, k, full, &sc->full_count, sc, labels);
    }
    FK_LAUNCH_CHECK();
}

void launch_mixed_inertia(Ctx &ctx, const double *part, int64_t m, DevScalars *sc) {
    inertia_final_kernel<<<1, 1024, 0, ctx.stream>>>(part, m, &sc->inertia);
    FK_LAUNCH_CHECK();
}

template void run_assign_mixed<float>(Ctx &, const float *, int64_t, int, const double *, int, int, int32_t *,
                                      double *, DevScalars *, bool);

// Diagnostics for the tests: one tensor-core pass over x (f32, on the device)
// against c (f64), returning the raw accumulators of CTA 0's first tile and
// the BF16 operands they were computed from.
void debug_tc_probe(Ctx &ctx, const float *x, int64_t n, int d, const double *c, int k, float *dump_out,
                    uint16_t *xb_out, uint16_t *cb_out, uint16_t *aug_out, Top2 *top_out, int *plan_out) {
    cudaStream_t s = ctx.stream;
    MixedPlan &mp = ctx.mixed;
    plan_tc(ctx, mp, n, d, k);
    mp.x = nullptr;
    DevScalars *sc = (DevScalars *)ctx.get(BUF_SCALARS, sizeof(DevScalars));
    FK_CUDA(cudaMemsetAsync(sc, 0, sizeof(DevScalars), s));
    auto *stats = (MixedStats *)ctx.get(BUF_CF32, sizeof(MixedStats));
    FK_CUDA(cudaMemsetAsync(stats, 0, sizeof(MixedStats), s));
    double *mu = (double *)ctx.get(BUF_COUNTS, sizeof(double) * 2 * (size_t)d + sizeof(float) * (size_t)d + 64);
    float *mu32 = (float *)(mu + 2 * d);
    __nv_bfloat16 *xb = (__nv_bfloat16 *)ctx.get(BUF_XB, sizeof(__nv_bfloat16) * (size_t)n * mp.d_pad);
    float4 *rowinfo = (float4 *)ctx.get(BUF_XNORM, sizeof(float4) * (size_t)n);
    const int64_t rows_per = 4096;
    const int nparts = (int)((n + rows_per - 1) / rows_per);
    double *part = (double *)ctx.get(BUF_PARTIAL, sizeof(double) * (size_t)nparts * d);
    col_mean_partial_kernel<float><<<dim3(nparts, (d + 127) / 128), 128, 0, s>>>(x, n, d, rows_per, 1, part);
    FK_LAUNCH_CHECK();
    col_mean_final_kernel<<<(d + 127) / 128, 128, 0, s>>>(part, nparts, n, d, mu, mu32);
    FK_LAUNCH_CHECK();
    prep_rows_kernel<float><<<(unsigned)((n + 7) / 8), 256, 0, s>>>(x, n, d, mp.d_pad, mu32, xb, rowinfo, stats);
    FK_LAUNCH_CHECK();
    __nv_bfloat16 *cb = (__nv_bfloat16 *)ctx.get(BUF_CB, sizeof(__nv_bfloat16) * (size_t)mp.k_pad * mp.d_pad);
    __nv_bfloat16 *caug = (__nv_bfloat16 *)ctx.get(BUF_CAUX, sizeof(__nv_bfloat16) * (size_t)mp.k_pad * 16 + 8192);
    double *half_norm = (double *)ctx.get(BUF_MIND, sizeof(double) * (size_t)mp.k_pad);
    float *c32 = (float *)ctx.get(BUF_CF32C, sizeof(float) * (2 * (size_t)k * d + (size_t)k) + 64);
    prep_centres_kernel<<<(mp.k_pad + 7) / 8, 256, 0, s>>>(c, k, mp.k_pad, d, mp.d_pad, mu, cb, half_norm, c32,
                                                           c32 + (size_t)k * d, c32 + (size_t)k * d + k, stats);
    FK_LAUNCH_CHECK();
    prep_aug_kernel<<<(mp.k_pad + 255) / 256, 256, 0, s>>>(half_norm, k, mp.k_pad, caug, stats);
    FK_LAUNCH_CHECK();
    Top2 *top = (Top2 *)ctx.get(BUF_TOP2, sizeof(Top2) * (size_t)n * mp.parts);
    float *dump = (float *)ctx.get(BUF_OUT, sizeof(float) * 128 * (size_t)mp.kp);
    FK_CUDA(cudaMemsetAsync(dump, 0, sizeof(float) * 128 * (size_t)mp.kp, s));
    launch_tc_assign(ctx, mp, xb, cb, caug, top, sc, stats, dump);
    FK_CUDA(cudaMemcpyAsync(dump_out, dump, sizeof(float) * 128 * (size_t)mp.kp, cudaMemcpyDeviceToHost, s));
    const int64_t rows = n < 128 ? n : 128;
    FK_CUDA(cudaMemcpyAsync(xb_out, xb, sizeof(uint16_t) * (size_t)rows * mp.d_pad, cudaMemcpyDeviceToHost, s));
    FK_CUDA(cudaMemcpyAsync(cb_out, cb, sizeof(uint16_t) * (size_t)mp.k_pad * mp.d_pad, cudaMemcpyDeviceToHost, s));
    FK_CUDA(cudaMemcpyAsync(aug_out, caug, sizeof(uint16_t) * (size_t)mp.k_pad * 16, cudaMemcpyDeviceToHost, s));
    FK_CUDA(cudaMemcpyAsync(top_out, top, sizeof(Top2) * (size_t)n * mp.parts, cudaMemcpyDeviceToHost, s));
    FK_CUDA(cudaMemcpyAsync(ctx.host_scalars, sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, s));
    FK_CUDA(cudaStreamSynchronize(s));
    plan_out[0] = mp.d_pad;
    plan_out[1] = mp.kp;
    plan_out[2] = mp.parts;
    plan_out[3] = mp.k_pad;
    plan_out[4] = mp.grid;
    plan_out[5] = (int)ctx.host_scalars->error_word;
}
template void run_assign_mixed<double>(Ctx &, const double *, int64_t, int, const double *, int, int, int32_t *,
                                       double *, DevScalars *, bool);

}  // namespace fk
