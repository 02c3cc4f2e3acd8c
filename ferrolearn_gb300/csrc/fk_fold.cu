// fk_fold.cu -- sequential left folds in F, computed exactly in parallel.
//
// The reference sums in row order with one rounding per addition: the 2-means
// centre sums of BisectingKMeans (bisecting_kmeans.rs:264-298, and
// compute_cluster_stats :192-211) and its SSE folds (:300-309, :443-463). On
// this GPU a dependent FP64 addition takes 64 cycles, so folding 10^5 values
// one after the other costs milliseconds per chain. The folds here return the
// same bits as the sequential loop:
//
//   While the running sum p keeps its sign s and its binade [2^e, 2^(e+1)),
//   p = s * P * ulp with P an integer in [2^MB, 2^(MB+1)), and adding v
//   rounds to P + a: a = round(s * v / ulp), and for an exact half the even
//   neighbour, so a depends on P's parity. Every value is thus a map
//   P -> P + a[P & 1], and so is any run of values (the maps compose). As the
//   sum can fall as well as rise, a composed map also carries the smallest
//   and largest running increment (lo, hi); it applies exactly when the
//   whole path stays inside the binade: 2^MB < P + lo and P + hi < 2^(MB+1).
//
// fold_sums_kernel forms per (chain, chunk of 1024 values) an f64 sum and a
// count; fold_compose_kernel the chunk's map for the sign and three binades
// around the chunk's estimated starting sum (the f64 prefix of the chunk sums
// -- it steers speed, never the result); fold_walk_kernel walks each chain
// with one warp: 32 chunk maps scanned at a time, a chunk whose map does not
// apply walked by its 32-value groups (its values staged in shared memory,
// the groups' maps recomputed for the sum's current sign and binade), a group
// whose map does not apply walked value by value, with one exact F addition
// where the sign or the binade changes (and, after a second change within 32
// values, exact additions for the rest of them).
//
// A chain is a strided array with an optional mask: chain c folds
// base[i * stride] over i in [0, m) in order, skipping i where
// mask != null and mask[i] != mval.
#include <cfloat>
#include <cmath>

#include "fk_internal.cuh"

namespace fk {
namespace {

constexpr int FCH = 1024;             // values per chunk
constexpr int FWARPS = 8;             // chains per CTA in the sums / compose passes
constexpr long long FSAT = 1LL << 61;  // saturated increment (never applies)

template <typename T> struct FB;
template <> struct FB<float> {
    using U = uint32_t;
    static constexpr int MB = 23;
    static constexpr int EXPM = 0xFF;
    static __device__ __forceinline__ U bits(float v) { return __float_as_uint(v); }
    static __device__ __forceinline__ float from(U b) { return __uint_as_float(b); }
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
};
template <> struct FB<double> {
    using U = unsigned long long;
    static constexpr int MB = 52;
    static constexpr int EXPM = 0x7FF;
    static __device__ __forceinline__ U bits(double v) { return (U)__double_as_longlong(v); }
    static __device__ __forceinline__ double from(U b) { return __longlong_as_double((long long)b); }
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
};

// Sign (+1 / -1), biased exponent and significand of a nonzero normal finite
// value; false for zero, subnormals, inf and NaN.
template <typename T>
__device__ __forceinline__ bool split(T p, int &s, int &be, long long &P) {
    using B = FB<T>;
    const typename B::U b = B::bits(p);
    be = (int)((b >> B::MB) & (typename B::U)B::EXPM);
    if (be == 0 || be == B::EXPM) return false;
    s = (b >> (sizeof(typename B::U) * 8 - 1)) ? -1 : 1;
    P = (long long)((b & (((typename B::U)1 << B::MB) - 1)) | ((typename B::U)1 << B::MB));
    return true;
}

template <typename T>
__device__ __forceinline__ T join(int s, int be, long long P) {
    using B = FB<T>;
    typename B::U b = ((typename B::U)be << B::MB) | ((typename B::U)P & (((typename B::U)1 << B::MB) - 1));
    if (s < 0) b |= (typename B::U)1 << (sizeof(typename B::U) * 8 - 1);
    return B::from(b);
}

// A map for a running sum of sign s in binade be: per parity of P, the total
// increment a and the smallest / largest running increment lo / hi.
struct SMap {
    long long a[2], lo[2], hi[2];
};

__device__ __forceinline__ SMap smap_ident() { return {{0, 0}, {FSAT, FSAT}, {-FSAT, -FSAT}}; }
__device__ __forceinline__ SMap smap_bad() { return {{FSAT, FSAT}, {-FSAT, -FSAT}, {FSAT, FSAT}}; }
__device__ __forceinline__ long long fsat(long long v) { return v > FSAT ? FSAT : (v < -FSAT ? -FSAT : v); }

template <typename T>
__device__ __forceinline__ SMap smap_of(T v, int be, int s) {
    using B = FB<T>;
    using U = typename B::U;
    const U b = B::bits(v);
    const int ev = (int)((b >> B::MB) & (U)B::EXPM);
    if (ev == B::EXPM) return smap_bad();  // inf or NaN
    U m = b & (((U)1 << B::MB) - 1);
    int e = ev;
    if (ev == 0) {
        if (m == 0) return smap_ident();  // +-0 changes nothing
        e = 1;
    } else {
        m |= (U)1 << B::MB;
    }
    const int sh = e - be;
    if (sh > 0) return smap_bad();  // |v| >= 2^(be+1): leaves the binade
    const int r = -sh;
    if (r > B::MB + 2) return smap_ident();  // below half an ulp by far: rounds away, never a half
    const int sig = ((b >> (sizeof(U) * 8 - 1)) ? -1 : 1) * s;
    long long q;
    bool tie = false;
    if (r == 0) {
        q = (long long)m;
    } else {
        q = (long long)(m >> r);
        const U rem = m & (((U)1 << r) - 1), half = (U)1 << (r - 1);
        if (rem > half) q += 1;
        tie = rem == half;
    }
    SMap o;
#pragma unroll
    for (int par = 0; par < 2; par++) {
        const long long t = tie ? ((par + q) & 1) : 0;
        const long long a = sig > 0 ? q + t : -q - t;
        o.a[par] = a;
        o.lo[par] = a;
        o.hi[par] = a;
    }
    return o;
}

// f then g
__device__ __forceinline__ SMap smap_compose(const SMap &f, const SMap &g) {
    SMap o;
#pragma unroll
    for (int par = 0; par < 2; par++) {
        const long long d1 = f.a[par];
        const int p1 = (int)((par + d1) & 1);
        o.a[par] = fsat(d1 + g.a[p1]);
        o.lo[par] = min(f.lo[par], fsat(d1 + g.lo[p1]));
        o.hi[par] = max(f.hi[par], fsat(d1 + g.hi[p1]));
    }
    return o;
}

// P after the map, or -1 when the path would leave the binade (or the sign).
template <typename T>
__device__ __forceinline__ long long smap_apply(long long P, const SMap &m) {
    const int par = (int)(P & 1);
    const long long low = (1LL << FB<T>::MB) + 1, top = (1LL << (FB<T>::MB + 1)) - 1;
    if (P + m.lo[par] >= low && P + m.hi[par] <= top) return P + m.a[par];
    return -1;
}

__device__ __forceinline__ SMap shfl_up_smap(const SMap &m, int off) {
    SMap o;
#pragma unroll
    for (int q = 0; q < 2; q++) {
        o.a[q] = (long long)__shfl_up_sync(0xffffffffu, (unsigned long long)m.a[q], off);
        o.lo[q] = (long long)__shfl_up_sync(0xffffffffu, (unsigned long long)m.lo[q], off);
        o.hi[q] = (long long)__shfl_up_sync(0xffffffffu, (unsigned long long)m.hi[q], off);
    }
    return o;
}

__device__ __forceinline__ SMap shfl_down_smap(const SMap &m, int off) {
    SMap o;
#pragma unroll
    for (int q = 0; q < 2; q++) {
        o.a[q] = (long long)__shfl_down_sync(0xffffffffu, (unsigned long long)m.a[q], off);
        o.lo[q] = (long long)__shfl_down_sync(0xffffffffu, (unsigned long long)m.lo[q], off);
        o.hi[q] = (long long)__shfl_down_sync(0xffffffffu, (unsigned long long)m.hi[q], off);
    }
    return o;
}

// Inclusive warp scan of maps in lane order (lane i holds value i's map).
__device__ __forceinline__ SMap scan_smap(SMap m) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const SMap o = shfl_up_smap(m, off);
        if (lane >= off) m = smap_compose(o, m);
    }
    return m;
}

// The chain descriptor (FoldChain, fk_internal.cuh) read with its values' type.
template <typename T>
struct Chain {
    const T *base;
    int64_t stride;
    const uint8_t *mask;
    int32_t mval;
    int32_t active_slot;
};
static_assert(sizeof(Chain<double>) == sizeof(FoldChain) && sizeof(Chain<float>) == sizeof(FoldChain),
              "Chain mirrors FoldChain");

template <typename T>
__device__ __forceinline__ bool takes(const Chain<T> &c, int64_t i) {
    return c.mask == nullptr || c.mask[i] == (uint8_t)c.mval;
}

// Up to 32 values (lane i holds value i, `live` marks the chain's values,
// len values in all) added to p in order, exactly as the sequential fold:
// the values' maps for p's sign and binade scanned at once, one exact F
// addition where the sum leaves them, one more scan for the rest; a sum that
// leaves its binade twice in 32 values (a fold near zero, where the binade
// changes every few values) takes the rest one exact addition at a time,
// which costs less than a scan per change.
template <typename T>
__device__ T walk_values(T p, T v, bool live, int len) {
    using B = FB<T>;
    const int lane = threadIdx.x & 31;
    int start = 0;
    for (int scans = 0; scans < 2 && start < len; scans++) {
        const unsigned rest = __ballot_sync(0xffffffffu, live && lane >= start && lane < len);
        if (!rest) return p;
        start = __ffs(rest) - 1;  // the next value of the chain
        int s, be;
        long long P;
        if (!split(p, s, be, P)) {
            // zero, subnormal, inf or NaN sum: one exact addition
            p = B::add(p, __shfl_sync(0xffffffffu, v, start));
            start++;
            continue;
        }
        const bool mine = live && lane >= start && lane < len;
        SMap m = mine ? smap_of(v, be, s) : smap_ident();
        m = scan_smap(m);
        const long long Pl = smap_apply<T>(P, m);
        const unsigned badm = __ballot_sync(0xffffffffu, mine && Pl < 0);
        const int f0 = badm ? __ffs(badm) - 1 : len;  // the first value that leaves the binade or sign
        if (f0 > start) {
            // the state after value f0 - 1 (lanes without a value carry it on)
            const long long Pb = (long long)__shfl_sync(0xffffffffu, (unsigned long long)Pl, f0 - 1);
            p = join<T>(s, be, Pb);
        }
        if (f0 >= len) return p;
        p = B::add(p, __shfl_sync(0xffffffffu, v, f0));  // the one exact addition there
        start = f0 + 1;
    }
    // the rest in order, one exact addition each
    for (unsigned rest = __ballot_sync(0xffffffffu, live && lane >= start && lane < len); rest; rest &= rest - 1u)
        p = B::add(p, __shfl_sync(0xffffffffu, v, __ffs(rest) - 1));
    return p;
}

// Per (chain, chunk): f64 sum and count of the chain's values (CTA: FWARPS
// chains of one chunk, a warp per chain, lane g over values g, g+32, ...).
template <typename T>
__global__ void __launch_bounds__(FWARPS * 32)
    fold_sums_kernel(const Chain<T> *__restrict__ chains, int nchains, int64_t m, const int *__restrict__ active,
                     int64_t nch, double *__restrict__ csum, int32_t *__restrict__ ccnt) {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int c = blockIdx.y * FWARPS + w;
    const int64_t j = blockIdx.x;
    if (c >= nchains) return;
    const Chain<T> ch = chains[c];
    if (ch.active_slot >= 0 && !active[ch.active_slot]) return;
    const int64_t lo = j * FCH, hi = min(m, lo + FCH);
    double s = 0.0;
    int cnt = 0;
    for (int64_t i = lo + lane; i < hi; i += 32) {
        if (takes(ch, i)) {
            s += (double)ch.base[i * ch.stride];
            cnt++;
        }
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    }
    if (lane == 0) {
        csum[(int64_t)c * nch + j] = s;
        ccnt[(int64_t)c * nch + j] = cnt;
    }
}

// Chunk maps for the three binades around the estimated start, with its sign.
struct CMap {
    SMap s[3];
    int e_lo;  // -1: no map
    int sign;
};

// Per (chain, chunk): the chunk's maps (lane g composes values g*32 ..
// g*32+31 of the chunk, then an ordered warp reduction).
template <typename T>
__global__ void __launch_bounds__(FWARPS * 32)
    fold_compose_kernel(const Chain<T> *__restrict__ chains, int nchains, int64_t m, const int *__restrict__ active,
                        int64_t nch, const double *__restrict__ csum, CMap *__restrict__ cmaps) {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int c = blockIdx.y * FWARPS + w;
    const int64_t j = blockIdx.x;
    if (c >= nchains) return;
    const Chain<T> ch = chains[c];
    if (ch.active_slot >= 0 && !active[ch.active_slot]) return;
    double e = 0.0;
    for (int64_t q = lane; q < j; q += 32) e += csum[(int64_t)c * nch + q];
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
    CMap *out = cmaps + (int64_t)c * nch + j;
    int s = 1, be;
    long long P;
    const T ef = (T)e;
    int lo = -1;
    if (split(ef, s, be, P)) {
        lo = be > 1 ? be - 1 : 1;
        if (lo + 2 >= FB<T>::EXPM) lo = -1;
    }
    if (lane == 0) {
        out->e_lo = lo;
        out->sign = s;
    }
    if (lo < 0) return;
    SMap m0 = smap_ident(), m1 = smap_ident(), m2 = smap_ident();
    const int64_t g0 = j * FCH + (int64_t)lane * 32;
    for (int q = 0; q < 32; q++) {
        const int64_t i = g0 + q;
        if (i < m && takes(ch, i)) {
            const T v = ch.base[i * ch.stride];
            m0 = smap_compose(m0, smap_of(v, lo, s));
            m1 = smap_compose(m1, smap_of(v, lo + 1, s));
            m2 = smap_compose(m2, smap_of(v, lo + 2, s));
        }
    }
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const SMap r0 = shfl_down_smap(m0, o), r1 = shfl_down_smap(m1, o), r2 = shfl_down_smap(m2, o);
        if ((lane & (2 * o - 1)) == 0) {
            m0 = smap_compose(m0, r0);
            m1 = smap_compose(m1, r1);
            m2 = smap_compose(m2, r2);
        }
    }
    if (lane == 0) {
        out->s[0] = m0;
        out->s[1] = m1;
        out->s[2] = m2;
    }
}

// One chunk (values [lo, lo + len) of the chain) added to p exactly: the
// chunk's values and take flags staged in shared memory (independent loads,
// issued together), the 32 groups' maps for p's current sign and binade
// scanned at once, a group whose map does not apply walked value by value.
template <typename T>
__device__ T walk_chunk_values(T p, const Chain<T> &ch, int64_t lo, int len, T *__restrict__ sv,
                               uint8_t *__restrict__ sm) {
    const int lane = threadIdx.x & 31;
    const int ng = (len + 31) / 32;
#pragma unroll 8
    for (int q = 0; q < 32; q++) {
        const int i = q * 32 + lane;
        if (i < len) {
            sv[i] = ch.base[(lo + i) * ch.stride];
            sm[i] = takes(ch, lo + i) ? 1 : 0;
        }
    }
    __syncwarp();
    int start = 0;
    while (start < ng) {
        int s, be;
        long long P;
        if (!split(p, s, be, P)) {
            // no binade: the next group value by value
            const int i = start * 32 + lane;
            const bool live = lane < min(32, len - start * 32) && sm[i];
            const T v = live ? sv[i] : T(0);
            p = walk_values<T>(p, v, live, 32);
            start++;
            continue;
        }
        // this lane's group map for the current sign and binade
        SMap g = smap_ident();
        if (lane >= start && lane < ng) {
            const int g0 = lane * 32;
            const int gl = min(32, len - lane * 32);
            for (int q = 0; q < gl; q++)
                if (sm[g0 + q]) g = smap_compose(g, smap_of(sv[g0 + q], be, s));
        }
        const SMap sc = scan_smap(g);
        const long long Pl = smap_apply<T>(P, sc);
        const unsigned badm = __ballot_sync(0xffffffffu, lane >= start && lane < ng && Pl < 0);
        const int f0 = badm ? __ffs(badm) - 1 : ng;
        if (f0 > start) p = join<T>(s, be, (long long)__shfl_sync(0xffffffffu, (unsigned long long)Pl, f0 - 1));
        if (f0 >= ng) break;
        const int i = f0 * 32 + lane;
        const bool live = lane < min(32, len - f0 * 32) && sm[i];
        const T v = live ? sv[i] : T(0);
        p = walk_values<T>(p, v, live, 32);
        start = f0 + 1;
    }
    __syncwarp();  // the staging area is refilled by the next slow chunk
    return p;
}

// One warp per chain: the whole fold and the count of the chain's values.
template <typename T>
__global__ void __launch_bounds__(32)
    fold_walk_kernel(const Chain<T> *__restrict__ chains, int nchains, int64_t m, const int *__restrict__ active,
                     int64_t nch, const CMap *__restrict__ cmaps, const int32_t *__restrict__ ccnt,
                     T *__restrict__ result, long long *__restrict__ count) {
    __shared__ T stage_v[FCH];
    __shared__ uint8_t stage_m[FCH];
    const int c = blockIdx.x;
    const int lane = threadIdx.x;
    const Chain<T> ch = chains[c];
    if (ch.active_slot >= 0 && !active[ch.active_slot]) return;
    const CMap *cm = cmaps + (int64_t)c * nch;
    T p = T(0);
    long long cnt = 0;
    for (int64_t jb = 0; jb < nch; jb += 32) {
        const int nb = (int)min((int64_t)32, nch - jb);
        int e_l = -1, sg = 1;
        SMap m0 = smap_bad(), m1 = smap_bad(), m2 = smap_bad();
        if (lane < nb) {
            e_l = cm[jb + lane].e_lo;
            sg = cm[jb + lane].sign;
            if (e_l >= 0) {
                m0 = cm[jb + lane].s[0];
                m1 = cm[jb + lane].s[1];
                m2 = cm[jb + lane].s[2];
            }
            cnt += ccnt[(int64_t)c * nch + jb + lane];
        }
        int start = 0;
        while (start < nb) {
            int s, be;
            long long P;
            const bool normal = split(p, s, be, P);
            const int slot = be - e_l;
            const bool ok = normal && e_l >= 0 && sg == s && slot >= 0 && slot < 3;
            const bool live = lane >= start && lane < nb;
            SMap mm = !live ? smap_ident() : (ok ? (slot == 0 ? m0 : (slot == 1 ? m1 : m2)) : smap_bad());
            mm = scan_smap(mm);
            const long long Pl = normal ? smap_apply<T>(P, mm) : -1;
            const unsigned badm = __ballot_sync(0xffffffffu, live && Pl < 0);
            const int f0 = badm ? __ffs(badm) - 1 : nb;
            if (f0 > start)
                p = join<T>(s, be, (long long)__shfl_sync(0xffffffffu, (unsigned long long)Pl, f0 - 1));
            if (f0 >= nb) break;
            const int64_t lo = (jb + f0) * FCH;
            p = walk_chunk_values<T>(p, ch, lo, (int)min((int64_t)FCH, m - lo), stage_v, stage_m);
            start = f0 + 1;
        }
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if (lane == 0) {
        result[c] = p;
        count[c] = cnt;
    }
}

}  // namespace

template <typename T>
void run_exact_folds(Ctx &ctx, const FoldChain *chains, int nchains, int64_t m, const int *active, T *result,
                     long long *count) {
    if (nchains <= 0) return;
    cudaStream_t s = ctx.stream;
    const int64_t nch = m > 0 ? (m + FCH - 1) / FCH : 1;
    double *csum = (double *)ctx.get(BUF_FOLD_SUM, sizeof(double) * (size_t)nchains * nch);
    int32_t *ccnt = (int32_t *)ctx.get(BUF_FOLD_CNT, sizeof(int32_t) * (size_t)nchains * nch);
    CMap *cmaps = (CMap *)ctx.get(BUF_FOLD_MAP, sizeof(CMap) * (size_t)nchains * nch);
    const Chain<T> *ch = (const Chain<T> *)chains;
    if (m > 0) {
        dim3 grid((unsigned)nch, (unsigned)((nchains + FWARPS - 1) / FWARPS));
        fold_sums_kernel<T><<<grid, FWARPS * 32, 0, s>>>(ch, nchains, m, active, nch, csum, ccnt);
        FK_LAUNCH_CHECK();
        fold_compose_kernel<T><<<grid, FWARPS * 32, 0, s>>>(ch, nchains, m, active, nch, csum, cmaps);
        FK_LAUNCH_CHECK();
    } else {
        FK_CUDA(cudaMemsetAsync(ccnt, 0, sizeof(int32_t) * (size_t)nchains, s));
    }
    fold_walk_kernel<T><<<(unsigned)nchains, 32, 0, s>>>(ch, nchains, m > 0 ? m : 0, active, m > 0 ? nch : 0, cmaps,
                                                         ccnt, result, count);
    FK_LAUNCH_CHECK();
}

template void run_exact_folds<double>(Ctx &, const FoldChain *, int, int64_t, const int *, double *, long long *);
template void run_exact_folds<float>(Ctx &, const FoldChain *, int, int64_t, const int *, float *, long long *);

}  // namespace fk
