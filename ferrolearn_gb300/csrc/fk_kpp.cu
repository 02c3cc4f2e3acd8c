// fk_kpp.cu -- greedy k-means++ on the GPU (kmeans.rs:169-253), with the
// reference's arithmetic: every sum is the sequential left fold in F.
//
// The reference forms three sums per new centre, each a left fold in F from
// zero in row order: the total of the D^2 array (kmeans.rs:201), the running
// cumsum that locates each trial's candidate (:215-223), and each trial's
// potential (:225-237). A fold in F is not associative, so a tree gives other
// roundings and, at scale, other candidates. Here each fold is computed
// exactly as the sequential one, in parallel:
//
//   While the running sum p stays in one binade [2^e, 2^(e+1)), p is an
//   integer P on that binade's ulp grid, and adding v >= 0 rounds to
//   P + round(v / ulp) -- except for an exact half, where round-to-nearest-even
//   picks the even result, so the step depends on P's parity. Each element is
//   therefore a map P -> P + a[P & 1], and so is any run of elements: these
//   maps compose (associatively), and a composed map is exact whenever the
//   final P stays below the binade's top (the sum only grows, so every
//   intermediate stayed inside too).
//
// kpp_compose_kernel forms, per chunk of KPP_CH values, the composed map for
// the three binades around the chunk's estimated starting sum (an f64 prefix
// of chunk sums; the estimate only steers speed, never the result).
// kpp_walk_kernel then walks the chunks with one warp per fold: a chunk whose
// map applies is one integer add; otherwise (the sum changes binade inside
// it, or is zero or non-finite) the warp walks the chunk 32 values at a time
// with a warp scan of the same maps, taking one exact F addition at each
// element where the binade changes. Every state it records is bit for bit
// the reference's running sum.
//
// Per new centre: kpp_select_kernel resolves the previous centre's trials
// (strictly smallest potential, first trial on ties: kmeans.rs:239-243),
// draws the thresholds u * total in F (:213-214) and finds each trial's
// candidate (the first row whose running sum reaches its threshold: a 32-ary
// search over the recorded chunk states, then the chunk walked exactly);
// kpp_trials_kernel forms min(D^2, d(x, candidate)) for every trial in one
// pass over X (direct-form distances, no FMA, identical to the reference);
// compose and walk give every trial's potential and its chunk states, which
// the next centre's search uses (the chosen trial's D^2 array becomes the new
// one without a copy: two buffers alternate). A non-positive total takes one
// uniform draw as a random row (:202-206).
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

constexpr int KPP_CH = 1024;      // values per fold chunk (and rows per trial-pass CTA)
constexpr int KPP_THREADS = 256;
constexpr int MAX_TRIALS = 16;
constexpr int KPP_DJ = 16;        // features staged per step of the trial pass
constexpr long long KPP_SAT = 1LL << 61;  // saturated increment: never applies

// ---------------------------------------------------- binade arithmetic --
template <typename T> struct Bits;
template <> struct Bits<float> {
    using U = uint32_t;
    static constexpr int MB = 23;      // stored mantissa bits
    static constexpr int EXPM = 0xFF;  // all-ones exponent (inf / NaN)
    static __device__ __forceinline__ U bits(float v) { return __float_as_uint(v); }
    static __device__ __forceinline__ float from(U b) { return __uint_as_float(b); }
};
template <> struct Bits<double> {
    using U = unsigned long long;
    static constexpr int MB = 52;
    static constexpr int EXPM = 0x7FF;
    static __device__ __forceinline__ U bits(double v) { return (U)__double_as_longlong(v); }
    static __device__ __forceinline__ double from(U b) { return __longlong_as_double((long long)b); }
};

// Biased exponent of a positive normal finite value, else 0.
template <typename T>
__device__ __forceinline__ int normal_exp(T p) {
    using B = Bits<T>;
    const typename B::U b = B::bits(p);
    const int be = (int)((b >> B::MB) & (typename B::U)B::EXPM);
    const bool neg = (b >> (sizeof(typename B::U) * 8 - 1)) != 0;
    return (!neg && be >= 1 && be < B::EXPM) ? be : 0;
}

template <typename T>
__device__ __forceinline__ bool is_inf_or_nan(T p) {
    using B = Bits<T>;
    return (int)((B::bits(p) >> B::MB) & (typename B::U)B::EXPM) == B::EXPM;
}

// Significand of a normal value as an integer in [2^MB, 2^(MB+1)).
template <typename T>
__device__ __forceinline__ long long significand(T p) {
    using B = Bits<T>;
    const typename B::U m = ((typename B::U)1 << B::MB) - 1;
    return (long long)((B::bits(p) & m) | ((typename B::U)1 << B::MB));
}

template <typename T>
__device__ __forceinline__ T from_parts(int be, long long P) {
    using B = Bits<T>;
    const typename B::U m = ((typename B::U)1 << B::MB) - 1;
    return B::from(((typename B::U)be << B::MB) | ((typename B::U)P & m));
}

__device__ __forceinline__ double pow2d(int s) {  // 2^s for s in [-1022, 1023]
    return __longlong_as_double((long long)(1023 + s) << 52);
}

// Increment map of one value v >= 0 on the grid of binade be: a0 / a1 for a
// running sum whose significand is even / odd.
struct Step {
    long long a0, a1;
};

__device__ __forceinline__ Step step_from_scaled(double s) {
    // s = v / ulp (exact); from 2^60 on (beyond any binade's 2^53 steps) saturate
    if (!(s < 1152921504606846976.0)) return {KPP_SAT, KPP_SAT};
    const double fl = floor(s);
    const double fr = s - fl;  // exact
    const long long q = (long long)fl;
    if (fr > 0.5) return {q + 1, q + 1};
    if (fr < 0.5) return {q, q};
    return {q + (q & 1), q + ((q + 1) & 1)};  // exact half: the even neighbour
}

__device__ __forceinline__ Step step_of(float v, int be) {
    const double vv = (double)v;
    if (!(vv <= 3.5e38)) return {KPP_SAT, KPP_SAT};  // inf or NaN (v is never negative)
    if (vv == 0.0) return {0, 0};
    return step_from_scaled(vv * pow2d(150 - be));  // ulp = 2^(be - 150), exact in f64
}

__device__ __forceinline__ Step step_of(double v, int be) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const int ev = (int)((b >> 52) & 0x7FF);
    if (ev == 0x7FF) return {KPP_SAT, KPP_SAT};  // inf or NaN
    if (v == 0.0) return {0, 0};
    if (ev > be + 1) return {KPP_SAT, KPP_SAT};  // v >= 2^(be-1021): leaves the binade
    if (ev < be - 55) return {0, 0};             // v < ulp / 4: rounds away, never a half
    double s;                                     // v / ulp, ulp = 2^(be - 1075)
    if (ev >= 1) {
        s = __longlong_as_double((long long)((b & 0xFFFFFFFFFFFFFULL) |
                                             ((unsigned long long)(ev - be + 1075) << 52)));
    } else {
        s = v * pow2d(1000) * pow2d(75 - be);  // subnormal v (then be <= 55): two exact scalings
    }
    return step_from_scaled(s);
}

// f then g
__device__ __forceinline__ Step compose(Step f, Step g) {
    const long long g0 = (f.a0 & 1) ? g.a1 : g.a0;      // even start: parity after f is f.a0's
    const long long g1 = ((1 + f.a1) & 1) ? g.a1 : g.a0;  // odd start
    long long h0 = f.a0 + g0, h1 = f.a1 + g1;
    if (h0 > KPP_SAT) h0 = KPP_SAT;
    if (h1 > KPP_SAT) h1 = KPP_SAT;
    return {h0, h1};
}

__device__ __forceinline__ Step shfl_up_step(Step s, int off) {
    return {(long long)__shfl_up_sync(0xffffffffu, (unsigned long long)s.a0, off),
            (long long)__shfl_up_sync(0xffffffffu, (unsigned long long)s.a1, off)};
}
__device__ __forceinline__ Step shfl_down_step(Step s, int off) {
    return {(long long)__shfl_down_sync(0xffffffffu, (unsigned long long)s.a0, off),
            (long long)__shfl_down_sync(0xffffffffu, (unsigned long long)s.a1, off)};
}

// One group of up to 32 values (lane i holds value i of the group, len of
// them valid) added to the running sum p in order, exactly as the sequential
// fold. Warp-uniform result. With thr given, *hit receives the first value
// index whose inclusive running sum reaches *thr (-1 if none).
template <typename T, bool SEARCH>
__device__ T walk_group(T p, T v, int len, T thr, int *hit) {
    const int lane = threadIdx.x & 31;
    constexpr long long TOP = 1LL << (Bits<T>::MB + 1);
    int start = 0;
    if (SEARCH) *hit = -1;
    while (start < len) {
        const bool live = lane >= start && lane < len;
        const int be = normal_exp(p);
        if (be == 0) {
            if (p != p) return p;  // a NaN sum stays NaN and reaches no threshold
            const T vs = __shfl_sync(0xffffffffu, v, start);
            if (is_inf_or_nan(p)) {
                // +inf stays +inf until a NaN value arrives, which makes it NaN
                if (SEARCH) {
                    const T p1 = kpp_add(p, vs);
                    if (p1 >= thr) {
                        *hit = start;
                        return p1;
                    }
                }
                const unsigned nanm = __ballot_sync(0xffffffffu, live && v != v);
                if (nanm) p = __shfl_sync(0xffffffffu, v, __ffs(nanm) - 1);
                return p;
            }
            // zero or subnormal sum: one exact addition
            p = kpp_add(p, vs);
            if (SEARCH && p >= thr) {
                *hit = start;
                return p;
            }
            start++;
            continue;
        }
        const long long P = significand(p);
        Step s = live ? step_of(v, be) : Step{0, 0};
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const Step o = shfl_up_step(s, off);
            if (lane >= off) s = compose(o, s);
        }
        const long long Pl = P + ((P & 1) ? s.a1 : s.a0);
        const unsigned badm = __ballot_sync(0xffffffffu, live && !(Pl < TOP));
        const int f0 = badm ? __ffs(badm) - 1 : len;  // first value that leaves the binade
        if (SEARCH) {
            const T pl = from_parts<T>(be, Pl < TOP ? Pl : P);
            const unsigned hm = __ballot_sync(0xffffffffu, live && lane < f0 && pl >= thr);
            if (hm) {
                *hit = __ffs(hm) - 1;
                return __shfl_sync(0xffffffffu, pl, *hit);
            }
        }
        if (f0 > start) {
            const long long Pb = (long long)__shfl_sync(0xffffffffu, (unsigned long long)Pl, f0 - 1);
            p = from_parts<T>(be, Pb);
        }
        if (f0 >= len) return p;
        const T vf = __shfl_sync(0xffffffffu, v, f0);
        p = kpp_add(p, vf);  // the one exact addition where the binade changes
        if (SEARCH && p >= thr) {
            *hit = f0;
            return p;
        }
        start = f0 + 1;
    }
    return p;
}

struct Comp {
    long long a[3][2];  // maps for binades e_lo, e_lo + 1, e_lo + 2
    int e_lo;           // -1: no map (walk the chunk)
    int pad;
};

struct KppState {
    long long cursor;  // uniform draws consumed so far
    int direct;        // the current centre was a uniform random row (no trials)
    int cur;           // buffer holding the current D^2 array ...
    int cur_trial;     // ... and its trial slice
    int pending;       // trial results not yet resolved into a centre
    int wbuf;          // buffer the pending trials were written to
    int ntr;           // their count
    int pcentre;       // their centre index (-1: the first D^2 array)
    int pad;
    long long cand[MAX_TRIALS];
    double thr[MAX_TRIALS];
    double pot[MAX_TRIALS];  // fold of each pending trial's array (F, widened)
    double total;            // fold of the current D^2 array
};

__device__ __forceinline__ long long draw_to_range(double u, long long n) {
    long long i = (long long)floor(u * (double)n);
    if (i < 0) i = 0;
    if (i >= n) i = n - 1;
    return i;
}

template <typename T>
__global__ void kpp_first_kernel(const T *__restrict__ x, long long n, int d, const double *__restrict__ draws,
                                 long long n_draws, KppState *st, T *__restrict__ centers) {
    __shared__ long long first;
    if (threadIdx.x == 0) {
        const double u = n_draws > 0 ? draws[0] : 0.0;
        first = draw_to_range(u, n);
        st->cursor = 1;
        st->direct = 0;
        st->cand[0] = first;
        st->pending = 1;  // the first D^2 array: no centre to resolve
        st->wbuf = 0;
        st->ntr = 1;
        st->pcentre = -1;
    }
    __syncthreads();
    for (int j = threadIdx.x; j < d; j += blockDim.x) centers[j] = x[first * d + j];
}

// One CTA per chunk of KPP_CH rows: every trial's min(D^2, d(x, candidate))
// (INIT: d(x, first row), the first D^2 array) and the chunk's f64 sums.
template <typename T, bool INIT>
__global__ void __launch_bounds__(KPP_THREADS)
    kpp_trials_kernel(const T *__restrict__ x, long long n, int d, T *__restrict__ chains, int tstride,
                      const KppState *__restrict__ st, int ntr, double *__restrict__ csum, long long nch) {
    if (!INIT && st->direct) return;
    __shared__ __align__(16) T xs[KPP_DJ][KPP_THREADS];
    __shared__ T cs[MAX_TRIALS][KPP_DJ];
    __shared__ double red[MAX_TRIALS][KPP_THREADS / 32];
    __shared__ long long cand[MAX_TRIALS];
    const int tid = threadIdx.x;
    if (tid < ntr) cand[tid] = st->cand[tid];
    const int cur = INIT ? 0 : st->cur, cur_trial = INIT ? 0 : st->cur_trial, wbuf = INIT ? 0 : 1 - cur;
    const T *mind = chains + ((long long)cur * tstride + cur_trial) * n;
    T *out = chains + (long long)wbuf * tstride * n;
    __syncthreads();
    double psum[MAX_TRIALS];
#pragma unroll
    for (int t = 0; t < MAX_TRIALS; t++) psum[t] = 0.0;
    const long long base = (long long)blockIdx.x * KPP_CH;
    for (int sub = 0; sub < KPP_CH / KPP_THREADS; sub++) {
        const long long r0 = base + (long long)sub * KPP_THREADS;
        if (r0 >= n) break;
        const long long row = r0 + tid;
        T acc[MAX_TRIALS];
#pragma unroll
        for (int t = 0; t < MAX_TRIALS; t++) acc[t] = T(0);
        for (int j0 = 0; j0 < d; j0 += KPP_DJ) {
            const int jn = min(KPP_DJ, d - j0);
            __syncthreads();
            for (int e = tid; e < KPP_THREADS * KPP_DJ; e += KPP_THREADS) {
                const int r = e / KPP_DJ, jj = e - r * KPP_DJ;
                const long long gr = r0 + r;
                xs[jj][r] = (gr < n && jj < jn) ? x[gr * d + j0 + jj] : T(0);
            }
            for (int e = tid; e < ntr * KPP_DJ; e += KPP_THREADS) {
                const int t = e / KPP_DJ, jj = e - t * KPP_DJ;
                cs[t][jj] = jj < jn ? x[cand[t] * d + j0 + jj] : T(0);
            }
            __syncthreads();
            for (int jj = 0; jj < jn; jj++) {
                const T xv = xs[jj][tid];
#pragma unroll
                for (int t = 0; t < MAX_TRIALS; t++) {
                    if (t < ntr) {
                        const T df = kpp_sub(xv, cs[t][jj]);
                        acc[t] = kpp_add(acc[t], kpp_mul(df, df));
                    }
                }
            }
        }
        if (row < n) {
            const T m = INIT ? T(0) : mind[row];
#pragma unroll
            for (int t = 0; t < MAX_TRIALS; t++) {
                if (t < ntr) {
                    const T v = acc[t];
                    const T r = INIT ? v : (v < m ? v : m);  // kmeans.rs:230-232
                    out[(long long)t * n + row] = r;
                    psum[t] += (double)r;
                }
            }
        }
    }
    const int lane = tid & 31, w = tid >> 5;
#pragma unroll
    for (int t = 0; t < MAX_TRIALS; t++) {
        if (t < ntr) {
            double v = psum[t];
#pragma unroll
            for (int off = 16; off >= 1; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
            if (lane == 0) red[t][w] = v;
        }
    }
    __syncthreads();
    if (tid < ntr) {
        double v = 0.0;
        for (int q = 0; q < KPP_THREADS / 32; q++) v += red[tid][q];
        csum[(long long)tid * nch + blockIdx.x] = v;
    }
}

// CTA (chunk j, trial t): the chunk's composed increment maps for the three
// binades around its estimated starting sum.
template <typename T>
__global__ void __launch_bounds__(KPP_THREADS)
    kpp_compose_kernel(const T *__restrict__ chains, long long n, int tstride, const KppState *__restrict__ st,
                       bool init, const double *__restrict__ csum, long long nch, Comp *__restrict__ comps) {
    if (!init && st->direct) return;
    const int t = blockIdx.y;
    const long long j = blockIdx.x;
    const int wbuf = init ? 0 : 1 - st->cur;
    const T *v = chains + ((long long)wbuf * tstride + t) * n;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    __shared__ double sh[KPP_THREADS / 32];
    __shared__ Step ws[KPP_THREADS / 32];
    __shared__ int e_lo_s;
    // estimated sum before the chunk: f64 sum of the earlier chunks' sums
    double e = 0.0;
    for (long long q = tid; q < j; q += KPP_THREADS) e += csum[(long long)t * nch + q];
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) e += __shfl_xor_sync(0xffffffffu, e, off);
    if (lane == 0) sh[w] = e;
    __syncthreads();
    if (tid == 0) {
        double s = 0.0;
        for (int q = 0; q < KPP_THREADS / 32; q++) s += sh[q];
        const T ef = (T)s;
        int lo = -1;
        const int be = normal_exp(ef);
        if (be > 0) {
            lo = be > 1 ? be - 1 : 1;
            if (lo + 2 >= Bits<T>::EXPM) lo = -1;
        }
        e_lo_s = lo;
    }
    __syncthreads();
    const int e_lo = e_lo_s;
    Comp *out = comps + (long long)t * nch + j;
    if (e_lo < 0) {
        if (tid == 0) out->e_lo = -1;
        return;
    }
    const long long i0 = j * KPP_CH + (long long)tid * (KPP_CH / KPP_THREADS);
    T vals[KPP_CH / KPP_THREADS];
#pragma unroll
    for (int q = 0; q < KPP_CH / KPP_THREADS; q++) vals[q] = i0 + q < n ? v[i0 + q] : T(0);
    for (int slot = 0; slot < 3; slot++) {
        const int be = e_lo + slot;
        Step s{0, 0};
#pragma unroll
        for (int q = 0; q < KPP_CH / KPP_THREADS; q++)
            if (i0 + q < n) s = compose(s, step_of(vals[q], be));
        // ordered warp reduction: lane i (earlier) absorbs lane i + off (later)
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const Step o = shfl_down_step(s, off);
            if ((lane & (2 * off - 1)) == 0) s = compose(s, o);
        }
        if (lane == 0) ws[w] = s;
        __syncthreads();
        if (tid == 0) {
            Step r = ws[0];
            for (int q = 1; q < KPP_THREADS / 32; q++) r = compose(r, ws[q]);
            out->a[slot][0] = r.a0;
            out->a[slot][1] = r.a1;
        }
        __syncthreads();
    }
    if (tid == 0) out->e_lo = e_lo;
}

// One warp per fold (blockIdx.x = trial): the running sum over every chunk,
// recorded at each chunk's end, and the whole fold (the trial's potential).
template <typename T>
__global__ void __launch_bounds__(32)
    kpp_walk_kernel(const T *__restrict__ chains, long long n, int tstride, KppState *__restrict__ st, bool init,
                    const Comp *__restrict__ comps, long long nch, T *__restrict__ states) {
    if (!init && st->direct) return;
    const int t = blockIdx.x;
    const int lane = threadIdx.x;
    const int wbuf = init ? 0 : 1 - st->cur;
    const T *v = chains + ((long long)wbuf * tstride + t) * n;
    const Comp *cp = comps + (long long)t * nch;
    T *sout = states + ((long long)wbuf * tstride + t) * nch;
    __shared__ Comp cc[32];
    constexpr long long TOP = 1LL << (Bits<T>::MB + 1);
    T p = T(0);
    int dummy;
    for (long long jb = 0; jb < nch; jb += 32) {
        __syncwarp();
        if (jb + lane < nch) cc[lane] = cp[jb + lane];
        __syncwarp();
        const int nb = (int)min(32LL, nch - jb);
        for (int jj = 0; jj < nb; jj++) {
            const long long j = jb + jj;
            const int e_lo = cc[jj].e_lo;
            const int be = normal_exp(p);
            bool done = false;
            if (be > 0 && e_lo >= 0) {
                const int slot = be - e_lo;
                if (slot >= 0 && slot < 3) {
                    const long long P = significand(p);
                    const long long a = (P & 1) ? cc[jj].a[slot][1] : cc[jj].a[slot][0];
                    const long long P2 = P + a;
                    if (P2 < TOP) {
                        p = from_parts<T>(be, P2);
                        done = true;
                    }
                }
            }
            if (!done) {
                const long long lo = j * KPP_CH, hi = min(n, lo + KPP_CH);
                for (long long g = lo; g < hi; g += 32) {
                    const int len = (int)min(32LL, hi - g);
                    const T val = lane < len ? v[g + lane] : T(0);
                    p = walk_group<T, false>(p, val, len, T(0), &dummy);
                }
            }
            if (lane == 0) sout[j] = p;
        }
    }
    if (lane == 0) st->pot[t] = (double)p;
}

// Single CTA, one warp per trial: resolve the pending trials into a centre,
// then (centre c < k) the thresholds and candidates of centre c.
template <typename T>
__global__ void __launch_bounds__(MAX_TRIALS * 32)
    kpp_select_kernel(const T *__restrict__ x, long long n, int d, const T *__restrict__ chains, int tstride,
                      const T *__restrict__ states, long long nch, const double *__restrict__ draws,
                      long long n_draws, int n_trials, int c, int k, KppState *__restrict__ st,
                      T *__restrict__ centers) {
    __shared__ long long copy_row;
    __shared__ int copy_centre;
    __shared__ int do_search;
    __shared__ T thr_s[MAX_TRIALS];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (tid == 0) {
        copy_row = -1;
        copy_centre = -1;
        do_search = 0;
        if (st->pending) {
            int best = 0;
            for (int t = 1; t < st->ntr; t++)
                if (st->pot[t] < st->pot[best]) best = t;  // strictly smaller: the first trial wins ties
            st->cur = st->wbuf;
            st->cur_trial = best;
            st->total = st->pot[best];
            if (st->pcentre >= 0) {
                copy_row = st->cand[best];
                copy_centre = st->pcentre;
            }
            st->pending = 0;
        }
    }
    __syncthreads();
    if (copy_row >= 0)
        for (int j = tid; j < d; j += blockDim.x) centers[(long long)copy_centre * d + j] = x[copy_row * d + j];
    __syncthreads();
    if (c >= k) return;
    if (tid == 0) {
        const T total = (T)st->total;
        long long cur = st->cursor;
        if (!(total > T(0))) {
            // kmeans.rs:202-206: a uniform random row, the D^2 array unchanged
            const double u = cur < n_draws ? draws[cur] : 0.0;
            copy_row = draw_to_range(u, n);
            copy_centre = c;
            st->direct = 1;
            cur += 1;
        } else {
            st->direct = 0;
            for (int t = 0; t < n_trials; t++) {
                const double u = cur < n_draws ? draws[cur] : 0.0;
                thr_s[t] = kpp_mul((T)u, total);
                st->thr[t] = (double)thr_s[t];
                cur += 1;
            }
            st->pending = 1;
            st->wbuf = 1 - st->cur;
            st->ntr = n_trials;
            st->pcentre = c;
            do_search = 1;
        }
        st->cursor = cur;
    }
    __syncthreads();
    if (!do_search) {
        for (int j = tid; j < d; j += blockDim.x) centers[(long long)copy_centre * d + j] = x[copy_row * d + j];
        return;
    }
    if (w >= n_trials) return;
    // trial w: the first row whose running sum reaches thr (kmeans.rs:215-223)
    const T thr = thr_s[w];
    const long long off = ((long long)st->cur * tstride + st->cur_trial);
    const T *S = states + off * nch;
    const T *v = chains + off * n;
    // First chunk whose end state is not below thr: a 32-ary search (the
    // states never decrease, and a NaN state stays NaN, so "not below" holds
    // from one chunk on); that chunk is then walked with the exact test.
    long long lo = 0, hi = nch;  // the answer lies in [lo, hi]; nch = none
    while (lo < hi) {
        const long long step = (hi - lo + 31) / 32;
        const long long pos = lo + (long long)lane * step;
        const unsigned m = __ballot_sync(0xffffffffu, pos < hi && !(S[pos] < thr));
        if (!m) {
            lo = lo + ((hi - 1 - lo) / step) * step + 1;  // past the last probe
        } else {
            const int f = __ffs(m) - 1;
            const long long pf = lo + (long long)f * step;
            if (f > 0) lo = lo + (long long)(f - 1) * step + 1;
            hi = pf;
        }
    }
    long long cand = n - 1;
    if (lo < nch) {
        const long long j = lo;
        T p = j > 0 ? S[j - 1] : T(0);
        const long long a = j * KPP_CH, b = min(n, a + KPP_CH);
        for (long long g = a; g < b; g += 32) {
            const int len = (int)min(32LL, b - g);
            const T val = lane < len ? v[g + lane] : T(0);
            int hit = -1;
            p = walk_group<T, true>(p, val, len, thr, &hit);
            if (hit >= 0) {
                cand = g + hit;
                break;
            }
        }
    }
    if (lane == 0) st->cand[w] = cand;
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
    const long long nch = (n + KPP_CH - 1) / KPP_CH;
    const int ts = n_trials;  // trial slices per buffer
    auto *st = (KppState *)ctx.get(BUF_KPP0, sizeof(KppState));
    T *chains = (T *)ctx.get(BUF_KPP1, sizeof(T) * (size_t)n * ts * 2);
    double *csum = (double *)ctx.get(BUF_KPP2, sizeof(double) * (size_t)nch * ts);
    Comp *comps = (Comp *)ctx.get(BUF_KPP3, sizeof(Comp) * (size_t)nch * ts + sizeof(T) * (size_t)nch * ts * 2 + 64);
    T *states = (T *)(comps + (size_t)nch * ts);
    FK_CUDA(cudaMemsetAsync(st, 0, sizeof(KppState), s));

    kpp_first_kernel<T><<<1, 128, 0, s>>>(x, n, d, draws_dev, n_draws, st, centers_out);
    FK_LAUNCH_CHECK();
    if (k == 1) {
        if (draws_used) *draws_used = 1;
        return;
    }
    // the first D^2 array (distances to the first centre) and its fold
    kpp_trials_kernel<T, true><<<(unsigned)nch, KPP_THREADS, 0, s>>>(x, n, d, chains, ts, st, 1, csum, nch);
    FK_LAUNCH_CHECK();
    kpp_compose_kernel<T><<<dim3((unsigned)nch, 1), KPP_THREADS, 0, s>>>(chains, n, ts, st, true, csum, nch, comps);
    FK_LAUNCH_CHECK();
    kpp_walk_kernel<T><<<1, 32, 0, s>>>(chains, n, ts, st, true, comps, nch, states);
    FK_LAUNCH_CHECK();
    for (int c = 1; c <= k; c++) {
        kpp_select_kernel<T><<<1, MAX_TRIALS * 32, 0, s>>>(x, n, d, chains, ts, states, nch, draws_dev, n_draws,
                                                            n_trials, c, k, st, centers_out);
        FK_LAUNCH_CHECK();
        if (c == k) break;
        kpp_trials_kernel<T, false><<<(unsigned)nch, KPP_THREADS, 0, s>>>(x, n, d, chains, ts, st, n_trials, csum,
                                                                          nch);
        FK_LAUNCH_CHECK();
        kpp_compose_kernel<T><<<dim3((unsigned)nch, (unsigned)n_trials), KPP_THREADS, 0, s>>>(chains, n, ts, st,
                                                                                             false, csum, nch, comps);
        FK_LAUNCH_CHECK();
        kpp_walk_kernel<T><<<(unsigned)n_trials, 32, 0, s>>>(chains, n, ts, st, false, comps, nch, states);
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
