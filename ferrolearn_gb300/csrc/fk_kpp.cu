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
// pass over X (direct-form distances, no FMA, identical to the reference; in
// f64, kpp_trials_f64f_kernel bounds them in FP32 first and forms the FP64
// distance only where the candidate may come closer than D^2);
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
constexpr int KPP_GROUPS = KPP_CH / 32;  // 32-value groups per chunk
constexpr int KPP_THREADS = 256;
constexpr int MAX_TRIALS = 16;
constexpr int KPP_PAD = 4;        // row padding of the staged X tile (16 bytes of f32)
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

// Increment map of one value v >= 0 on the grid of binade be: a0 / a1 for a
// running sum whose significand is even / odd. Integer arithmetic on the
// value's significand m and exponent: v / ulp = m * 2^(e - be), so the
// rounded increment is m shifted right by be - e, rounded to nearest, with
// an exact half left to the sum's parity (ties to even).
struct Step {
    long long a0, a1;
};

template <typename T>
__device__ __forceinline__ Step step_of(T v, int be) {
    using B = Bits<T>;
    using U = typename B::U;
    const U b = B::bits(v);
    const int ev = (int)((b >> B::MB) & (U)B::EXPM);
    if (ev == B::EXPM) return {KPP_SAT, KPP_SAT};  // inf or NaN
    const U mask = ((U)1 << B::MB) - 1;
    if (b >> (sizeof(U) * 8 - 1))                   // negative: only -0 is harmless
        return (b << 1) == 0 ? Step{0, 0} : Step{KPP_SAT, KPP_SAT};
    U m = b & mask;
    int e = ev;
    if (ev == 0) {
        if (m == 0) return {0, 0};
        e = 1;  // subnormal: no hidden bit, the exponent of the smallest normals
    } else {
        m |= (U)1 << B::MB;
    }
    const int sh = e - be;
    if (sh > 0) return {KPP_SAT, KPP_SAT};  // v >= 2^(be+1): the sum leaves the binade
    const int r = -sh;
    if (r == 0) return {(long long)m, (long long)m};
    if (r > B::MB + 2) return {0, 0};  // v < ulp / 2 by far: rounds away, never a half
    const long long q = (long long)(m >> r);
    const U rem = m & (((U)1 << r) - 1), half = (U)1 << (r - 1);
    if (rem > half) return {q + 1, q + 1};
    if (rem < half) return {q, q};
    return {q + (q & 1), q + ((q + 1) & 1)};  // exact half: the even neighbour
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

// Maps of one chunk or group for the three binades of its window.
struct Map3 {
    Step s[3];
};

__device__ __forceinline__ Step pick(const Map3 &m, int slot) {
    return slot == 0 ? m.s[0] : (slot == 1 ? m.s[1] : m.s[2]);
}

// Where the fold data of one buffer / trial slice live (kpp_layout on the host).
struct FoldSlices {
    int *elo;       // [2][ts][nch] lowest binade of each chunk's window (-1: none)
    Map3 *cmap;     // [2][ts][nch] chunk maps
    Map3 *gmap;     // [2][ts][nch][32] group maps
    void *states;   // [2][ts][nch] running sum at each chunk's end (T)
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

// The values of one chunk (clen of them) added to p in order, exactly as the
// sequential fold: the groups' maps scanned 32 at a time, and a group whose
// map does not apply walked value by value. With SEARCH, *hit receives the
// index (within the chunk) of the first value whose inclusive running sum
// reaches thr, or -1.
template <typename T, bool SEARCH>
__device__ T walk_chunk(T p, const T *__restrict__ cv, int clen, const Map3 *__restrict__ gm, int e_lo, T thr,
                        int *hit) {
    const int lane = threadIdx.x & 31;
    constexpr long long TOP = 1LL << (Bits<T>::MB + 1);
    const int ng = (clen + 31) / 32;
    Map3 g{};
    if (e_lo >= 0 && lane < ng) g = gm[lane];
    if (SEARCH) *hit = -1;
    int start = 0;
    while (start < ng) {
        const int be = normal_exp(p);
        const int slot = be - e_lo;
        if (!(be > 0 && e_lo >= 0 && slot >= 0 && slot < 3)) {
            // no map for this sum: the first remaining group value by value
            const int len = min(32, clen - start * 32);
            const T val = lane < len ? cv[start * 32 + lane] : T(0);
            int h = -1;
            p = walk_group<T, SEARCH>(p, val, len, thr, &h);
            if (SEARCH && h >= 0) {
                *hit = start * 32 + h;
                return p;
            }
            start++;
            continue;
        }
        const bool live = lane >= start && lane < ng;
        Step s = live ? pick(g, slot) : Step{0, 0};
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const Step o = shfl_up_step(s, off);
            if (lane >= off) s = compose(o, s);
        }
        const long long P = significand(p);
        const long long Pl = P + ((P & 1) ? s.a1 : s.a0);
        const unsigned badm = __ballot_sync(0xffffffffu, live && !(Pl < TOP));
        const int f0 = badm ? __ffs(badm) - 1 : ng;  // first group whose map does not apply
        int gsel = f0;                                 // the group to walk value by value
        if (SEARCH) {
            const unsigned hm = __ballot_sync(0xffffffffu, live && lane < f0 && from_parts<T>(be, Pl) >= thr);
            if (hm) gsel = __ffs(hm) - 1;              // the threshold is reached inside this group
        }
        if (gsel > start) {
            const long long Pb = (long long)__shfl_sync(0xffffffffu, (unsigned long long)Pl, gsel - 1);
            p = from_parts<T>(be, Pb);
        }
        if (gsel >= ng) return p;
        const int len = min(32, clen - gsel * 32);
        const T val = lane < len ? cv[gsel * 32 + lane] : T(0);
        int h = -1;
        p = walk_group<T, SEARCH>(p, val, len, thr, &h);
        if (SEARCH && h >= 0) {
            *hit = gsel * 32 + h;
            return p;
        }
        start = gsel + 1;
    }
    return p;
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

template <typename T> struct TrialTile;
template <> struct TrialTile<float> { static constexpr int DJ = 8; };
template <> struct TrialTile<double> { static constexpr int DJ = 4; };

// Two stages of the staged tile (rows and trial candidates), filled with
// asynchronous copies one feature round ahead.
template <typename T, int TT>
constexpr size_t trial_smem() {
    return 2 * sizeof(T) * ((size_t)TrialTile<T>::DJ * (KPP_CH + KPP_PAD) + (size_t)TrialTile<T>::DJ * TT);
}

// One element from global to shared memory, asynchronously (cp.async of 4
// or 8 bytes); ok == false writes zero (src-size 0: nothing is read).
template <typename T>
__device__ __forceinline__ void cp_async_elem(T *dst, const T *src, bool ok) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
    const int n = ok ? (int)sizeof(T) : 0;
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;" ::"r"(d), "l"(src), "n"((int)sizeof(T)), "r"(n)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// One CTA per chunk of KPP_CH rows, 4 rows per thread, all TT trial slots per
// thread (ntr <= TT of them live): every trial's min(D^2, d(x, candidate))
// (INIT: d(x, first row), the first D^2 array; kmeans.rs:188-195, 225-233)
// with the direct form folded over the features in order, and the chunk's
// sums (only an estimate for the fold's binade windows). The features come
// in rounds of DJ, staged in shared memory by asynchronous copies one round
// ahead of the arithmetic (two stages).
template <typename T, int TT, bool INIT>
__global__ void __launch_bounds__(KPP_THREADS)
    kpp_trials_kernel(const T *__restrict__ x, long long n, int d, T *__restrict__ chains, int tstride,
                      const KppState *__restrict__ st, int ntr, double *__restrict__ csum, long long nch) {
    if (!INIT && st->direct) return;
    constexpr int DJ = TrialTile<T>::DJ;
    constexpr int XS = KPP_CH + KPP_PAD;  // row length of the staged tile
    extern __shared__ __align__(16) unsigned char kpp_smem[];
    constexpr int STAGE = DJ * XS + DJ * TT;  // elements of one stage
    // stage q: xs = [DJ][XS] (feature-major, rows contiguous), then cs = [DJ][TT]
    T *const stages = reinterpret_cast<T *>(kpp_smem);
    __shared__ long long cand[TT];
    __shared__ double red[TT][KPP_THREADS / 32];
    const int tid = threadIdx.x;
    if (tid < TT) cand[tid] = tid < ntr ? st->cand[tid] : 0;
    const int cur = INIT ? 0 : st->cur, cur_trial = INIT ? 0 : st->cur_trial, wbuf = INIT ? 0 : 1 - cur;
    const T *mind = chains + ((long long)cur * tstride + cur_trial) * n;
    T *out = chains + (long long)wbuf * tstride * n;
    const long long base = (long long)blockIdx.x * KPP_CH;
    T acc[4][TT];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < TT; b++) acc[a][b] = T(0);
    __syncthreads();  // cand
    auto stage_round = [&](int j0, int q) {
        T *xs = stages + q * STAGE;
        T *cs = xs + DJ * XS;
        const int jn = min(DJ, d - j0);
        for (int e = tid; e < KPP_CH * DJ; e += KPP_THREADS) {
            const int r = e / DJ, jj = e - r * DJ;
            const long long gr = base + r;
            const bool ok = gr < n && jj < jn;
            cp_async_elem(xs + jj * XS + r, ok ? x + gr * d + j0 + jj : x, ok);
        }
        for (int e = tid; e < TT * DJ; e += KPP_THREADS) {
            const int t = e / DJ, jj = e - t * DJ;
            const bool ok = t < ntr && jj < jn;
            cp_async_elem(cs + jj * TT + t, ok ? x + cand[t] * d + j0 + jj : x, ok);
        }
        cp_async_commit();
    };
    stage_round(0, 0);
    for (int j0 = 0, q = 0; j0 < d; j0 += DJ, q ^= 1) {
        const int jn = min(DJ, d - j0);
        if (j0 + DJ < d) {
            stage_round(j0 + DJ, q ^ 1);  // the next round's copies fly during this round
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();  // every thread's copies of this round have landed
        const T *xs = stages + q * STAGE;
        const T *cs = xs + DJ * XS;
        for (int jj = 0; jj < jn; jj++) {
            T xv[4], cvv[TT];
#pragma unroll
            for (int a = 0; a < 4; a++) xv[a] = xs[jj * XS + tid * 4 + a];
#pragma unroll
            for (int b = 0; b < TT; b++) cvv[b] = cs[jj * TT + b];
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < TT; b++) {
                    const T df = kpp_sub(xv[a], cvv[b]);
                    acc[a][b] = kpp_add(acc[a][b], kpp_mul(df, df));
                }
        }
        __syncthreads();  // this stage is refilled by the next round's staging
    }
    double psum[TT];
#pragma unroll
    for (int b = 0; b < TT; b++) psum[b] = 0.0;
#pragma unroll
    for (int a = 0; a < 4; a++) {
        const long long row = base + tid * 4 + a;
        if (row < n) {
            const T m = INIT ? T(0) : mind[row];
#pragma unroll
            for (int b = 0; b < TT; b++) {
                if (b < ntr) {
                    const T v = acc[a][b];
                    const T r = INIT ? v : (v < m ? v : m);  // kmeans.rs:230-232
                    out[(long long)b * n + row] = r;
                    psum[b] += (double)r;
                }
            }
        }
    }
    const int lane = tid & 31, w = tid >> 5;
#pragma unroll
    for (int b = 0; b < TT; b++) {
        double v = psum[b];
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
        if (lane == 0) red[b][w] = v;
    }
    __syncthreads();
    if (tid < ntr) {
        double v = 0.0;
        for (int q = 0; q < KPP_THREADS / 32; q++) v += red[tid][q];
        csum[(long long)tid * nch + blockIdx.x] = v;
    }
}

// The direct form in FP64, in the reference's order (the loads run ahead of
// the dependent adds).
__device__ __forceinline__ double sqeuc_f64(const double *__restrict__ a, const double *__restrict__ b, int d) {
    double v = 0.0;
#pragma unroll 8
    for (int j = 0; j < d; j++) {
        const double df = __dsub_rn(a[j], b[j]);
        v = __dadd_rn(v, __dmul_rn(df, df));
    }
    return v;
}

constexpr int KPP_OPEN = 2048;  // listed open pairs a chunk (row within the chunk << 4 | trial)
static_assert(KPP_CH <= 4096, "a chunk row fits the list entry's 12 bits");

// The f64 trial pass through FP32 bounds: the same outputs as
// kpp_trials_kernel<double, TT, false>, bit for bit. The distances are first
// formed in FP32 from the rows' f32 copies (t = x - c, fma), with the
// rigorous bound b = bound32(d32, e_row + e_candidate, d) of their distance
// from the exact distance and from the FP64 direct form. Where d32 - b (down)
// exceeds the row's current D^2 value m, the FP64 distance v is larger too and
// min(v, m) is m (kmeans.rs:230-232); only the other (row, trial) pairs --
// rows the candidate may come closer to, non-finite values, values beyond the
// f32 range -- form v with the direct form in FP64, in the reference's order.
template <int TT>
__global__ void __launch_bounds__(KPP_THREADS)
    kpp_trials_f64f_kernel(const double *__restrict__ x, const float *__restrict__ x32,
                           const float *__restrict__ xerr, long long n, int d, double *__restrict__ chains,
                           int tstride, const KppState *__restrict__ st, int ntr, double *__restrict__ csum,
                           long long nch) {
    if (st->direct) return;
    constexpr int DJ = TrialTile<float>::DJ;
    constexpr int XS = KPP_CH + KPP_PAD;  // row length of the staged tile
    extern __shared__ __align__(16) unsigned char kpp_smem[];
    constexpr int STAGE = DJ * XS + DJ * TT;  // elements of one stage
    float *const stages = reinterpret_cast<float *>(kpp_smem);
    __shared__ long long cand[TT];
    __shared__ float cerr[TT];
    __shared__ double red[TT][KPP_THREADS / 32];
    __shared__ double open_sum[TT];
    __shared__ unsigned short open_pairs[KPP_OPEN];
    __shared__ int open_n;
    const int tid = threadIdx.x;
    if (tid < TT) {
        cand[tid] = tid < ntr ? st->cand[tid] : 0;
        cerr[tid] = tid < ntr ? xerr[st->cand[tid]] : 0.f;
        open_sum[tid] = 0.0;
    }
    if (tid == 0) open_n = 0;
    const int cur = st->cur, cur_trial = st->cur_trial, wbuf = 1 - cur;
    const double *mind = chains + ((long long)cur * tstride + cur_trial) * n;
    double *out = chains + (long long)wbuf * tstride * n;
    const long long base = (long long)blockIdx.x * KPP_CH;
    float acc[4][TT];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < TT; b++) acc[a][b] = 0.f;
    __syncthreads();  // cand, cerr
    auto stage_round = [&](int j0, int q) {
        float *xs = stages + q * STAGE;
        float *cs = xs + DJ * XS;
        const int jn = min(DJ, d - j0);
        for (int e = tid; e < KPP_CH * DJ; e += KPP_THREADS) {
            const int r = e / DJ, jj = e - r * DJ;
            const long long gr = base + r;
            const bool ok = gr < n && jj < jn;
            cp_async_elem(xs + jj * XS + r, ok ? x32 + gr * d + j0 + jj : x32, ok);
        }
        for (int e = tid; e < TT * DJ; e += KPP_THREADS) {
            const int t = e / DJ, jj = e - t * DJ;
            const bool ok = t < ntr && jj < jn;
            cp_async_elem(cs + jj * TT + t, ok ? x32 + cand[t] * d + j0 + jj : x32, ok);
        }
        cp_async_commit();
    };
    stage_round(0, 0);
    for (int j0 = 0, q = 0; j0 < d; j0 += DJ, q ^= 1) {
        const int jn = min(DJ, d - j0);
        if (j0 + DJ < d) {
            stage_round(j0 + DJ, q ^ 1);  // the next round's copies fly during this round
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();  // every thread's copies of this round have landed
        const float *xs = stages + q * STAGE;
        const float *cs = xs + DJ * XS;
        for (int jj = 0; jj < jn; jj++) {
            float xv[4], cvv[TT];
#pragma unroll
            for (int a = 0; a < 4; a++) xv[a] = xs[jj * XS + tid * 4 + a];
#pragma unroll
            for (int b = 0; b < TT; b++) cvv[b] = cs[jj * TT + b];
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < TT; b++) {
                    const float df = __fsub_rn(xv[a], cvv[b]);
                    acc[a][b] = __fmaf_rn(df, df, acc[a][b]);
                }
        }
        __syncthreads();  // this stage is refilled by the next round's staging
    }
    // Pairs the bounds leave open are listed (row within the chunk, trial)
    // and formed in FP64 by the whole block afterwards, one pair a thread:
    // a warp whose lanes waited on one lane's FP64 chain would run it for
    // nearly every row slot. A pair beyond the list's room is formed in place.
    double psum[TT];
#pragma unroll
    for (int b = 0; b < TT; b++) psum[b] = 0.0;
#pragma unroll
    for (int a = 0; a < 4; a++) {
        const long long row = base + tid * 4 + a;
        if (row < n) {
            const double m = mind[row];
            const float er = xerr[row];
#pragma unroll
            for (int b = 0; b < TT; b++) {
                if (b < ntr) {
                    const float bnd = bound32(acc[a][b], __fadd_ru(er, cerr[b]), d);
                    double r = m;  // v >= d32 - bnd > m: min(v, m) = m (kmeans.rs:230-232)
                    if (!((double)__fsub_rd(acc[a][b], bnd) > m)) {
                        const int slot = atomicAdd(&open_n, 1);
                        if (slot < KPP_OPEN) {
                            open_pairs[slot] = (unsigned short)(((tid * 4 + a) << 4) | b);
                            continue;
                        }
                        const double v = sqeuc_f64(x + row * d, x + cand[b] * d, d);
                        r = v < m ? v : m;
                    }
                    out[(long long)b * n + row] = r;
                    psum[b] += r;
                }
            }
        }
    }
    __syncthreads();  // the list is complete
    for (int q = tid; q < min(open_n, KPP_OPEN); q += KPP_THREADS) {
        const int e = open_pairs[q];
        const int b = e & 15;
        const long long row = base + (e >> 4);
        const double m = mind[row];
        const double v = sqeuc_f64(x + row * d, x + cand[b] * d, d);
        const double r = v < m ? v : m;
        out[(long long)b * n + row] = r;
        atomicAdd(&open_sum[b], r);  // the chunk sums only steer the folds' windows
    }
    const int lane = tid & 31, w = tid >> 5;
#pragma unroll
    for (int b = 0; b < TT; b++) {
        double vv = psum[b];
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) vv += __shfl_xor_sync(0xffffffffu, vv, off);
        if (lane == 0) red[b][w] = vv;
    }
    __syncthreads();
    if (tid < ntr) {
        double vv = open_sum[tid];
        for (int q = 0; q < KPP_THREADS / 32; q++) vv += red[tid][q];
        csum[(long long)tid * nch + blockIdx.x] = vv;
    }
}

// One warp per (chunk, trial): the maps of the chunk's 32 groups (lane g
// folds group g) and of the whole chunk (ordered warp reduction), each for
// the three binades around the chunk's estimated starting sum (an f64 sum of
// the earlier chunks' sums: only which maps get built depends on it).
template <typename T>
__global__ void __launch_bounds__(KPP_THREADS)
    kpp_compose_kernel(const T *__restrict__ chains, long long n, int tstride, const KppState *__restrict__ st,
                       bool init, const double *__restrict__ csum, long long nch, FoldSlices fs) {
    if (!init && st->direct) return;
    const int lane = threadIdx.x & 31;
    const int t = blockIdx.y;
    const long long j = (long long)blockIdx.x * (KPP_THREADS / 32) + (threadIdx.x >> 5);
    if (j >= nch) return;  // whole warps; no block-wide barrier below
    const int wbuf = init ? 0 : 1 - st->cur;
    const T *v = chains + ((long long)wbuf * tstride + t) * n + j * KPP_CH;
    const long long off = ((long long)wbuf * tstride + t) * nch + j;
    double e = 0.0;
    for (long long q = lane; q < j; q += 32) e += csum[(long long)t * nch + q];
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
    const int be = normal_exp((T)e);
    int lo = -1;
    if (be > 0) {
        lo = be > 1 ? be - 1 : 1;
        if (lo + 2 >= Bits<T>::EXPM) lo = -1;
    }
    if (lane == 0) fs.elo[off] = lo;
    if (lo < 0) return;
    const int clen = (int)min((long long)KPP_CH, n - j * KPP_CH);
    Step s0{0, 0}, s1{0, 0}, s2{0, 0};
    const int g0 = lane * 32;
    for (int q = 0; q < 32; q++) {
        const int i = g0 + q;
        if (i < clen) {
            const T val = v[i];
            s0 = compose(s0, step_of(val, lo));
            s1 = compose(s1, step_of(val, lo + 1));
            s2 = compose(s2, step_of(val, lo + 2));
        }
    }
    Map3 gm;
    gm.s[0] = s0;
    gm.s[1] = s1;
    gm.s[2] = s2;
    fs.gmap[off * KPP_GROUPS + lane] = gm;
    // ordered reduction: lane i (earlier groups) absorbs lane i + o (later)
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const Step r0 = shfl_down_step(s0, o), r1 = shfl_down_step(s1, o), r2 = shfl_down_step(s2, o);
        if ((lane & (2 * o - 1)) == 0) {
            s0 = compose(s0, r0);
            s1 = compose(s1, r1);
            s2 = compose(s2, r2);
        }
    }
    if (lane == 0) {
        Map3 cm;
        cm.s[0] = s0;
        cm.s[1] = s1;
        cm.s[2] = s2;
        fs.cmap[off] = cm;
    }
}

// One warp per fold (blockIdx.x = trial): the running sum over every chunk,
// recorded at each chunk's end, and the whole fold (the trial's potential).
// The chunk maps are scanned 32 chunks at a time; a chunk whose map does not
// apply (the sum changes binade inside it, or has no map) is walked by its
// groups (walk_chunk).
template <typename T>
__global__ void __launch_bounds__(32)
    kpp_walk_kernel(const T *__restrict__ chains, long long n, int tstride, KppState *__restrict__ st, bool init,
                    long long nch, FoldSlices fs) {
    if (!init && st->direct) return;
    const int t = blockIdx.x;
    const int lane = threadIdx.x;
    const int wbuf = init ? 0 : 1 - st->cur;
    const long long slice = (long long)wbuf * tstride + t;
    const T *v = chains + slice * n;
    const int *elo = fs.elo + slice * nch;
    const Map3 *cmap = fs.cmap + slice * nch;
    const Map3 *gmap = fs.gmap + slice * nch * KPP_GROUPS;
    T *sout = reinterpret_cast<T *>(fs.states) + slice * nch;
    constexpr long long TOP = 1LL << (Bits<T>::MB + 1);
    T p = T(0);
    int e_cur = -1;
    Map3 m_cur{};
    if (lane < nch) {
        e_cur = elo[lane];
        if (e_cur >= 0) m_cur = cmap[lane];
    }
    for (long long jb = 0; jb < nch; jb += 32) {
        // the next 32 chunks' maps load while these are scanned
        int e_nxt = -1;
        Map3 m_nxt{};
        if (jb + 32 + lane < nch) {
            e_nxt = elo[jb + 32 + lane];
            if (e_nxt >= 0) m_nxt = cmap[jb + 32 + lane];
        }
        const int nb = (int)min(32LL, nch - jb);
        int start = 0;
        while (start < nb) {
            const int be = normal_exp(p);
            const bool live = lane >= start && lane < nb;
            const int slot = be - e_cur;
            const bool ok = be > 0 && e_cur >= 0 && slot >= 0 && slot < 3;
            Step s = !live ? Step{0, 0} : (ok ? pick(m_cur, slot) : Step{KPP_SAT, KPP_SAT});
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const Step o = shfl_up_step(s, off);
                if (lane >= off) s = compose(o, s);
            }
            const long long P = be > 0 ? significand(p) : 0;
            const long long Pl = P + ((P & 1) ? s.a1 : s.a0);
            const unsigned badm = __ballot_sync(0xffffffffu, live && !(be > 0 && Pl < TOP));
            const int f0 = badm ? __ffs(badm) - 1 : nb;
            if (live && lane < f0) sout[jb + lane] = from_parts<T>(be, Pl);
            if (f0 > start) {
                const long long Pb = (long long)__shfl_sync(0xffffffffu, (unsigned long long)Pl, f0 - 1);
                p = from_parts<T>(be, Pb);
            }
            if (f0 >= nb) break;
            const long long j = jb + f0;
            const int ej = __shfl_sync(0xffffffffu, e_cur, f0);
            const int clen = (int)min((long long)KPP_CH, n - j * KPP_CH);
            int dummy;
            p = walk_chunk<T, false>(p, v + j * KPP_CH, clen, gmap + j * KPP_GROUPS, ej, T(0), &dummy);
            if (lane == 0) sout[j] = p;
            start = f0 + 1;
        }
        e_cur = e_nxt;
        m_cur = m_nxt;
    }
    if (lane == 0) st->pot[t] = (double)p;
}

// Single CTA, one warp per trial: resolve the pending trials into a centre,
// then (centre c < k) the thresholds and candidates of centre c.
template <typename T>
__global__ void __launch_bounds__(MAX_TRIALS * 32)
    kpp_select_kernel(const T *__restrict__ x, long long n, int d, const T *__restrict__ chains, int tstride,
                      long long nch, FoldSlices fs, const double *__restrict__ draws, long long n_draws,
                      int n_trials, int c, int k, KppState *__restrict__ st, T *__restrict__ centers) {
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
    const long long slice = (long long)st->cur * tstride + st->cur_trial;
    const T *S = reinterpret_cast<const T *>(fs.states) + slice * nch;
    const T *v = chains + slice * n;
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
        const T p = j > 0 ? S[j - 1] : T(0);
        const int clen = (int)min((long long)KPP_CH, n - j * KPP_CH);
        int hit = -1;
        walk_chunk<T, true>(p, v + j * KPP_CH, clen, fs.gmap + (slice * nch + j) * KPP_GROUPS, fs.elo[slice * nch + j],
                            thr, &hit);
        if (hit >= 0) cand = j * KPP_CH + hit;
    }
    if (lane == 0) st->cand[w] = cand;
}

template <typename T, int TT, bool INIT>
void launch_trials(const T *x, long long n, int d, T *chains, int ts, const KppState *st, int ntr, double *csum,
                   long long nch, cudaStream_t s) {
    constexpr size_t smem = trial_smem<T, TT>();
    static_assert(smem <= 227 * 1024, "two stages of the trial tile fit in shared memory");
    FK_CUDA(cudaFuncSetAttribute((const void *)kpp_trials_kernel<T, TT, INIT>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kpp_trials_kernel<T, TT, INIT><<<(unsigned)nch, KPP_THREADS, smem, s>>>(x, n, d, chains, ts, st, ntr, csum, nch);
    FK_LAUNCH_CHECK();
}

template <int TT>
void launch_trials_f64f(const double *x, const float *x32, const float *xerr, long long n, int d, double *chains,
                        int ts, const KppState *st, int ntr, double *csum, long long nch, cudaStream_t s) {
    constexpr size_t smem = trial_smem<float, TT>();
    FK_CUDA(cudaFuncSetAttribute((const void *)kpp_trials_f64f_kernel<TT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem));
    kpp_trials_f64f_kernel<TT><<<(unsigned)nch, KPP_THREADS, smem, s>>>(x, x32, xerr, n, d, chains, ts, st, ntr,
                                                                        csum, nch);
    FK_LAUNCH_CHECK();
}

void launch_trials_f64f_any(const double *x, const float *x32, const float *xerr, long long n, int d,
                            double *chains, int ts, const KppState *st, int ntr, double *csum, long long nch,
                            cudaStream_t s) {
    switch (ntr) {
        case 1: launch_trials_f64f<1>(x, x32, xerr, n, d, chains, ts, st, ntr, csum, nch, s); break;
        case 2: launch_trials_f64f<2>(x, x32, xerr, n, d, chains, ts, st, ntr, csum, nch, s); break;
        case 3: launch_trials_f64f<3>(x, x32, xerr, n, d, chains, ts, st, ntr, csum, nch, s); break;
        case 4: launch_trials_f64f<4>(x, x32, xerr, n, d, chains, ts, st, ntr, csum, nch, s); break;
        case 5: launch_trials_f64f<5>(x, x32, xerr, n, d, chains, ts, st, ntr, csum, nch, s); break;
        case 6: launch_trials_f64f<6>(x, x32, xerr, n, d, chains, ts, st, ntr, csum, nch, s); break;
        case 7: launch_trials_f64f<7>(x, x32, xerr, n, d, chains, ts, st, ntr, csum, nch, s); break;
        case 8: launch_trials_f64f<8>(x, x32, xerr, n, d, chains, ts, st, ntr, csum, nch, s); break;
        case 9: launch_trials_f64f<9>(x, x32, xerr, n, d, chains, ts, st, ntr, csum, nch, s); break;
        case 10: launch_trials_f64f<10>(x, x32, xerr, n, d, chains, ts, st, ntr, csum, nch, s); break;
        case 11: launch_trials_f64f<11>(x, x32, xerr, n, d, chains, ts, st, ntr, csum, nch, s); break;
        case 12: launch_trials_f64f<12>(x, x32, xerr, n, d, chains, ts, st, ntr, csum, nch, s); break;
        default: launch_trials_f64f<16>(x, x32, xerr, n, d, chains, ts, st, ntr, csum, nch, s); break;
    }
}

// The trial pass with the smallest trial-slot count that holds ntr trials.
template <typename T>
void launch_trials_any(const T *x, long long n, int d, T *chains, int ts, const KppState *st, int ntr, double *csum,
                       long long nch, cudaStream_t s) {
    switch (ntr) {
        case 1: launch_trials<T, 1, false>(x, n, d, chains, ts, st, ntr, csum, nch, s); break;
        case 2: launch_trials<T, 2, false>(x, n, d, chains, ts, st, ntr, csum, nch, s); break;
        case 3: launch_trials<T, 3, false>(x, n, d, chains, ts, st, ntr, csum, nch, s); break;
        case 4: launch_trials<T, 4, false>(x, n, d, chains, ts, st, ntr, csum, nch, s); break;
        case 5: launch_trials<T, 5, false>(x, n, d, chains, ts, st, ntr, csum, nch, s); break;
        case 6: launch_trials<T, 6, false>(x, n, d, chains, ts, st, ntr, csum, nch, s); break;
        case 7: launch_trials<T, 7, false>(x, n, d, chains, ts, st, ntr, csum, nch, s); break;
        case 8: launch_trials<T, 8, false>(x, n, d, chains, ts, st, ntr, csum, nch, s); break;
        case 9: launch_trials<T, 9, false>(x, n, d, chains, ts, st, ntr, csum, nch, s); break;
        case 10: launch_trials<T, 10, false>(x, n, d, chains, ts, st, ntr, csum, nch, s); break;
        case 11: launch_trials<T, 11, false>(x, n, d, chains, ts, st, ntr, csum, nch, s); break;
        case 12: launch_trials<T, 12, false>(x, n, d, chains, ts, st, ntr, csum, nch, s); break;
        default: launch_trials<T, 16, false>(x, n, d, chains, ts, st, ntr, csum, nch, s); break;
    }
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
    const size_t slices = 2 * (size_t)ts * (size_t)nch;  // per-chunk entries over both buffers
    auto *st = (KppState *)ctx.get(BUF_KPP0, sizeof(KppState));
    T *chains = (T *)ctx.get(BUF_KPP1, sizeof(T) * (size_t)n * ts * 2);
    double *csum = (double *)ctx.get(BUF_KPP2, sizeof(double) * (size_t)nch * ts);
    const size_t b_gmap = sizeof(Map3) * slices * KPP_GROUPS, b_cmap = sizeof(Map3) * slices,
                 b_states = sizeof(T) * slices, b_elo = sizeof(int) * slices;
    unsigned char *fold = (unsigned char *)ctx.get(BUF_KPP3, b_gmap + b_cmap + b_states + b_elo + 256);
    FoldSlices fs;
    fs.gmap = reinterpret_cast<Map3 *>(fold);
    fs.cmap = reinterpret_cast<Map3 *>(fold + b_gmap);
    fs.states = fold + b_gmap + b_cmap;
    fs.elo = reinterpret_cast<int *>(fold + b_gmap + b_cmap + b_states);
    FK_CUDA(cudaMemsetAsync(st, 0, sizeof(KppState), s));

    kpp_first_kernel<T><<<1, 128, 0, s>>>(x, n, d, draws_dev, n_draws, st, centers_out);
    FK_LAUNCH_CHECK();
    // f64: the rows' f32 copies and rounding-error norms for the trials' FP32 bounds
    float *x32 = nullptr, *xerr = nullptr;
    if constexpr (std::is_same<T, double>::value) {
        if (k > 1) {
            x32 = (float *)ctx.get(BUF_PF_X32, sizeof(float) * (size_t)n * d);
            xerr = (float *)ctx.get(BUF_PF_XERR, sizeof(float) * (size_t)n);
            launch_f32_copy(ctx, x, n, d, x32, xerr);
        }
    }
    if (k == 1) {
        if (draws_used) *draws_used = 1;
        return;
    }
    const unsigned cgrid = (unsigned)((nch + KPP_THREADS / 32 - 1) / (KPP_THREADS / 32));
    // the first D^2 array (distances to the first centre) and its fold
    launch_trials<T, 1, true>(x, n, d, chains, ts, st, 1, csum, nch, s);
    kpp_compose_kernel<T><<<dim3(cgrid, 1), KPP_THREADS, 0, s>>>(chains, n, ts, st, true, csum, nch, fs);
    FK_LAUNCH_CHECK();
    kpp_walk_kernel<T><<<1, 32, 0, s>>>(chains, n, ts, st, true, nch, fs);
    FK_LAUNCH_CHECK();
    for (int c = 1; c <= k; c++) {
        kpp_select_kernel<T><<<1, MAX_TRIALS * 32, 0, s>>>(x, n, d, chains, ts, nch, fs, draws_dev, n_draws,
                                                            n_trials, c, k, st, centers_out);
        FK_LAUNCH_CHECK();
        if (c == k) break;
        if constexpr (std::is_same<T, double>::value)
            launch_trials_f64f_any(x, x32, xerr, n, d, chains, ts, st, n_trials, csum, nch, s);
        else
            launch_trials_any<T>(x, n, d, chains, ts, st, n_trials, csum, nch, s);
        kpp_compose_kernel<T><<<dim3(cgrid, (unsigned)n_trials), KPP_THREADS, 0, s>>>(chains, n, ts, st, false, csum,
                                                                                     nch, fs);
        FK_LAUNCH_CHECK();
        kpp_walk_kernel<T><<<(unsigned)n_trials, 32, 0, s>>>(chains, n, ts, st, false, nch, fs);
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
