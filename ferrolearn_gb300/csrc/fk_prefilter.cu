// fk_prefilter.cu -- the plain f64 assignment through an exact FP32 prefilter.
//
// KMeans<f64>'s nearest_center (kmeans.rs:295-309) compares FP64 direct-form
// distances (squared_euclidean, :159-163), and FP64 runs at a small fraction
// of the FP32 rate on this part. The labels and distances here are still the
// FP64 ones, bit for bit:
//
//   1. X and the centres get f32 copies and, per row, an upper bound of the
//      norm of their rounding error, e = ||x - x32|| (rounded up).
//   2. A tiled FP32 pass forms each row's direct-form distances to every
//      centre from the f32 copies (t = x - c, acc = fma(t, t, acc)) and the
//      interval [d32 - b, d32 + b] with b = bound32(d32, e_x + e_c, d), which
//      holds the exact distance and the oracle's FP64 value. Per row it keeps
//      the centre a with the smallest upper bound and the smallest lower
//      bound L over every other centre. L > UB(a) proves that every other
//      centre's FP64 distance exceeds a's: a is nearest_center's result (no
//      tie is possible). Any NaN or infinite interval leaves the row open.
//   3. Decided rows: the FP64 direct form to the label, in the reference's
//      order, for the inertia.
//   4. Open rows (near ties, non-finite values, values beyond the f32 range):
//      the FP64 direct form to every centre, strict < from F::MAX, lowest
//      index on ties -- the plain kernel's rule.
#include <cfloat>

#include "fk_internal.cuh"

namespace fk {
namespace {

constexpr int PBM = 128;  // rows per block tile
constexpr int PBN = 128;  // centres per block tile
constexpr int PDJ = 16;   // feature chunk staged in shared memory
constexpr int PTM = 8;    // rows per thread
constexpr int PTN = 8;    // centres per thread
constexpr int PNT = 256;  // threads per block (16 x 16)

// |v - f| for f = v rounded to f32, as an f32 rounded up. For v in the f32
// normal range the error is exact integer arithmetic on v's bits: with E the
// exponent and r the 29 mantissa bits below f32's precision, |v - f| =
// min(r, 2^29 - r) 2^(E - 52) (rounding up into the next binade included).
// Zeros, f32 subnormals, overflow and NaN take two directed FP64
// subtractions (NaN stays NaN, overflow gives inf).
__device__ __forceinline__ float round_err(double v, float f) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const int E = (int)((b >> 52) & 0x7FFull) - 1023;
    if (E >= -126 && E <= 127 && fabsf(f) <= FLT_MAX) {
        const unsigned long long low = b & ((1ull << 29) - 1ull);
        const unsigned long long q = low < (1ull << 28) ? low : (1ull << 29) - low;  // <= 2^28
        const float qs = __fmul_rn(__ull2float_ru(q), 1.862645149230957e-09f);       // q (up) 2^-29: exact
        const int pe = E - 23;                                                         // >= -149
        const float p2 = pe >= -126 ? __int_as_float((pe + 127) << 23) : __int_as_float(1 << (pe + 149));
        return __fmul_ru(qs, p2);
    }
    const double fd = (double)f;
    const double hi = fabs(__dsub_ru(v, fd)), lo = fabs(__dsub_rd(v, fd));
    return __double2float_ru(hi > lo ? hi : lo);
}

// f32 copies of f64 rows (one warp per row) and an upper bound of the norm
// of each row's rounding error (+inf or NaN when a value does not fit f32);
// the squares, the sum and the root in FP32 rounded up (FP64 is slow here,
// its square root most of all).
__global__ void f32_copy_rows_kernel(const double *__restrict__ x, int64_t n, int d, float *__restrict__ x32,
                                     float *__restrict__ err) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n; r += nw) {
        float s = 0.f;
        for (int j = lane; j < d; j += 32) {
            const double v = x[r * d + j];
            const float f = __double2float_rn(v);
            x32[r * d + j] = f;
            const float e = round_err(v, f);
            s = __fadd_ru(s, __fmul_ru(e, e));
        }
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) s = __fadd_ru(s, __shfl_xor_sync(0xffffffffu, s, off));
        if (lane == 0) err[r] = __fsqrt_ru(s);
    }
}

// Per row: the centre with the smallest upper bound (ua, its lower bound la,
// its index ia), the smallest lower bound over the other centres (lb2), and
// whether any interval was not finite.
struct RowBound {
    float ua, la, lb2;
    int ia;
    bool bad;
};

__device__ __forceinline__ void rb_add(RowBound &r, float lb, float ub, int c) {
    if (!(lb <= ub)) r.bad = true;  // NaN
    if (ub < r.ua) {
        r.lb2 = fminf(r.lb2, r.la);
        r.ua = ub;
        r.la = lb;
        r.ia = c;
    } else {
        r.lb2 = fminf(r.lb2, lb);
    }
}

__device__ __forceinline__ void rb_merge(RowBound &r, const RowBound &o) {
    r.bad = r.bad || o.bad;
    if (o.ua < r.ua) {
        r.lb2 = fminf(fminf(r.lb2, o.lb2), r.la);
        r.ua = o.ua;
        r.la = o.la;
        r.ia = o.ia;
    } else {
        r.lb2 = fminf(fminf(r.lb2, o.lb2), o.la);
    }
}

// FP32 pass over 128-row tiles and every centre: decided rows get their label,
// open rows label -1 and a slot in the list.
__global__ void __launch_bounds__(PNT)
    f32_filter_kernel(const float *__restrict__ x32, const float *__restrict__ xerr, int64_t n, int d,
                      const float *__restrict__ c32, const float *__restrict__ cerr, int k,
                      int32_t *__restrict__ labels, int32_t *__restrict__ open_list,
                      unsigned long long *__restrict__ open_count) {
    __shared__ __align__(16) float xs[PDJ][PBM];
    __shared__ __align__(16) float cs[PDJ][PBN];
    const int tid = threadIdx.x;
    const int tx = tid & 15;  // centre group
    const int ty = tid >> 4;  // row group
    const int64_t row0 = (int64_t)blockIdx.x * PBM;
    RowBound rb[PTM];
    float ex[PTM];
#pragma unroll
    for (int a = 0; a < PTM; a++) {
        rb[a] = RowBound{INFINITY, INFINITY, INFINITY, -1, false};
        const int64_t gr = row0 + ty * PTM + a;
        ex[a] = gr < n ? xerr[gr] : 0.f;
    }
    for (int ct = 0; ct < k; ct += PBN) {
        float acc[PTM][PTN];
#pragma unroll
        for (int a = 0; a < PTM; a++)
#pragma unroll
            for (int b = 0; b < PTN; b++) acc[a][b] = 0.f;
        for (int j0 = 0; j0 < d; j0 += PDJ) {
#pragma unroll
            for (int e = 0; e < (PBM * PDJ) / PNT; e++) {
                const int idx = tid + e * PNT;
                const int r = idx / PDJ, jj = idx % PDJ;
                const int64_t gr = row0 + r;
                const int gj = j0 + jj;
                xs[jj][r] = (gr < n && gj < d) ? x32[gr * d + gj] : 0.f;
                const int gc = ct + r;
                cs[jj][r] = (gc < k && gj < d) ? c32[(int64_t)gc * d + gj] : 0.f;
            }
            __syncthreads();
            const int jn = min(PDJ, d - j0);
            for (int jj = 0; jj < jn; jj++) {
                float xv[PTM], cv[PTN];
#pragma unroll
                for (int a = 0; a < PTM; a++) xv[a] = xs[jj][ty * PTM + a];
#pragma unroll
                for (int b = 0; b < PTN; b++) cv[b] = cs[jj][tx * PTN + b];
#pragma unroll
                for (int a = 0; a < PTM; a++)
#pragma unroll
                    for (int b = 0; b < PTN; b++) {
                        const float t = xv[a] - cv[b];
                        acc[a][b] = fmaf(t, t, acc[a][b]);
                    }
            }
            __syncthreads();
        }
#pragma unroll
        for (int b = 0; b < PTN; b++) {
            const int gc = ct + tx * PTN + b;
            if (gc >= k) continue;
            const float ec = cerr[gc];
#pragma unroll
            for (int a = 0; a < PTM; a++) {
                const float bnd = bound32(acc[a][b], __fadd_ru(ex[a], ec), d);
                rb_add(rb[a], __fsub_rd(acc[a][b], bnd), __fadd_ru(acc[a][b], bnd), gc);
            }
        }
    }
    // merge over the 16 centre groups that share these rows (same half-warp)
#pragma unroll
    for (int a = 0; a < PTM; a++) {
        RowBound r = rb[a];
#pragma unroll
        for (int off = 8; off >= 1; off >>= 1) {
            RowBound o;
            o.ua = __shfl_xor_sync(0xffffffffu, r.ua, off);
            o.la = __shfl_xor_sync(0xffffffffu, r.la, off);
            o.lb2 = __shfl_xor_sync(0xffffffffu, r.lb2, off);
            o.ia = __shfl_xor_sync(0xffffffffu, r.ia, off);
            o.bad = __shfl_xor_sync(0xffffffffu, (int)r.bad, off) != 0;
            rb_merge(r, o);
        }
        const int64_t gr = row0 + ty * PTM + a;
        if (tx == 0 && gr < n) {
            const bool decided = !r.bad && r.ia >= 0 && r.lb2 > r.ua;
            labels[gr] = decided ? r.ia : -1;
            if (!decided) open_list[atomicAdd(open_count, 1ULL)] = (int32_t)gr;
        }
    }
}

// FP64 direct form of row x against centre c, in the reference's order.
__device__ __forceinline__ double sqeuc64_rn(const double *__restrict__ x, const double *__restrict__ c, int d) {
    double acc = 0.0;
    for (int j = 0; j < d; j++) {
        const double t = __dsub_rn(x[j], c[j]);
        acc = __dadd_rn(acc, __dmul_rn(t, t));
    }
    return acc;
}

// Decided rows: the FP64 distance to the label (open rows, label -1, are
// written by the exact pass).
__global__ void f64_label_dist_kernel(const double *__restrict__ x, int64_t n, int d, const double *__restrict__ c,
                                      const int32_t *__restrict__ labels, double *__restrict__ mind) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
        const int l = labels[r];
        if (l >= 0) mind[r] = sqeuc64_rn(x + r * d, c + (int64_t)l * d, d);
    }
}

// Open rows: one warp per row, lanes over the centres; the lowest index among
// the smallest FP64 distances strictly below F::MAX, else centre 0 at F::MAX.
__global__ void f64_open_rows_kernel(const double *__restrict__ x, int d, const double *__restrict__ c, int k,
                                     const int32_t *__restrict__ open_list,
                                     const unsigned long long *__restrict__ open_count, int32_t *__restrict__ labels,
                                     double *__restrict__ mind) {
    const int lane = threadIdx.x & 31;
    const unsigned long long cnt = *open_count;
    const unsigned long long nw = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
    for (unsigned long long q = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < cnt; q += nw) {
        const int64_t r = open_list[q];
        const double *xr = x + r * d;
        double bv = DBL_MAX;
        int bi = INT32_MAX;
        for (int cc = lane; cc < k; cc += 32) {
            const double v = sqeuc64_rn(xr, c + (int64_t)cc * d, d);
            if (v < DBL_MAX && (v < bv || (v == bv && cc < bi))) {
                bv = v;
                bi = cc;
            }
        }
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) {
            const double ov = __shfl_xor_sync(0xffffffffu, bv, off);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
            if (ov < bv || (ov == bv && oi < bi)) {
                bv = ov;
                bi = oi;
            }
        }
        if (lane == 0) {
            labels[r] = bi == INT32_MAX ? 0 : bi;
            if (mind) mind[r] = bi == INT32_MAX ? DBL_MAX : bv;
        }
    }
}

}  // namespace

void launch_f32_copy(Ctx &ctx, const double *x, int64_t n, int d, float *x32, float *err) {
    if (n == 0) return;
    f32_copy_rows_kernel<<<(unsigned)std::min<int64_t>((n + 7) / 8, (int64_t)ctx.num_sms * 8), 256, 0, ctx.stream>>>(
        x, n, d, x32, err);
    FK_LAUNCH_CHECK();
}

void launch_assign_f64_filtered(Ctx &ctx, const double *x, int64_t n, int d, const double *c, int k,
                                int32_t *labels, double *mind, bool fresh_x) {
    if (n == 0) return;
    cudaStream_t s = ctx.stream;
    float *x32 = (float *)ctx.get(BUF_PF_X32, sizeof(float) * (size_t)n * d);
    float *xerr = (float *)ctx.get(BUF_PF_XERR, sizeof(float) * (size_t)n);
    float *c32 = (float *)ctx.get(BUF_PF_C32, sizeof(float) * (size_t)k * d);
    float *cerr = (float *)ctx.get(BUF_PF_CERR, sizeof(float) * (size_t)k);
    int32_t *open_list = (int32_t *)ctx.get(BUF_PF_LIST, sizeof(int32_t) * (size_t)n);
    unsigned long long *open_count = (unsigned long long *)ctx.get(BUF_PF_CNT, sizeof(unsigned long long));
    const int grid_rows = ctx.num_sms * 8;
    if (fresh_x) {
        f32_copy_rows_kernel<<<grid_rows, 256, 0, s>>>(x, n, d, x32, xerr);
        FK_LAUNCH_CHECK();
    }
    f32_copy_rows_kernel<<<(unsigned)std::min<int64_t>((k + 7) / 8, grid_rows), 256, 0, s>>>(c, k, d, c32, cerr);
    FK_LAUNCH_CHECK();
    FK_CUDA(cudaMemsetAsync(open_count, 0, sizeof(unsigned long long), s));
    f32_filter_kernel<<<(unsigned)((n + PBM - 1) / PBM), PNT, 0, s>>>(x32, xerr, n, d, c32, cerr, k, labels,
                                                                      open_list, open_count);
    FK_LAUNCH_CHECK();
    if (mind) {
        f64_label_dist_kernel<<<grid_rows, 256, 0, s>>>(x, n, d, c, labels, mind);
        FK_LAUNCH_CHECK();
    }
    f64_open_rows_kernel<<<grid_rows, 256, 0, s>>>(x, d, c, k, open_list, open_count, labels, mind);
    FK_LAUNCH_CHECK();
}

}  // namespace fk
