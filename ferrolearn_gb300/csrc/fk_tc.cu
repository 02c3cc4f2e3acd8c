// fk_tc.cu -- fused BF16 / FP8 assignment on the 5th-generation tensor cores.
//
// One persistent launch, one CTA per SM (10 warps, up to ~215 KB shared
// memory, 512 TMEM columns). The centres are cut into `parts` slices of kp
// centres; CTA (slice p, index q) keeps its slice resident in shared memory
// for the whole launch and streams the row tiles q, q+Q, q+2Q, ... of X
// through a TMA ring -- two whole-tile stages where they fit beside the
// slice, else one stage used as a ring of its 16 KB atoms with a full /
// empty mbarrier each, so the next tile's first atoms load while the MMAs
// read this tile's last ones -- so X is read once per slice (the other
// slices' CTAs find it in L2) and the n x k score matrix never leaves the
// SM.
//
//   warp 0   TMA producer: the resident slice once, then 128-row X tiles
//            (cp.async.bulk.tensor, 128-byte swizzle, mbarrier complete_tx);
//            FP8 also loads each tile's per-row augmentation rows.
//   warp 1   TMEM allocator and MMA issuer: per (tile, 256-centre block),
//            tcgen05.mma M=128 N=256 (kind::f16 K=16 for BF16, kind::f8f6f4
//            K=32 for E4M3) over d_pad, plus one BF16 K=16 MMA that adds
//            a_c = BIG - ||c'||^2/2 (ones operand for BF16, the row's scale
//            for FP8); tcgen05.commit signals the epilogue. Two TMEM
//            accumulators (2 x 256 columns) alternate, so the MMAs of block
//            b+1 overlap the epilogue of block b.
//   warps 2-9 epilogue: tcgen05.ld (32x32b, one row per thread). The
//            top-2 pass turns every score into a key -- rounded to a 128-ulp
//            grid with the column code in the freed 7 bits (three FMA-pipe
//            operations; all scores of a launch share one binade) -- and
//            keeps a running top-2 with a bound of the rest (three-input
//            float max); the grid quantum is part of the error bound of the
//            re-check. The count and mask passes mark the centres scoring at
//            least a per-row threshold (one saturating FMA per score) and
//            keep their number, first mask words and the largest score, or
//            write the row's mask.
//
// Every wait on an mbarrier is bounded (about two seconds of SM clock); on
// expiry the CTA records an error word, stops issuing work, drains what it
// has in flight and frees its TMEM, so a fault in the pipeline can never hang
// the GPU. The host turns the error word into FK_ERR_TIMEOUT.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>

#include "fk_internal.cuh"

namespace fk {
namespace {

constexpr int BM = 128;           // rows per tile = TMEM lanes
constexpr int BN = 256;           // centres per accumulator block
// Threads of a launch: the TMA warp, the MMA warp and 4 x EP epilogue warps
// (EP parts of an accumulator block's 256 columns per TMEM lane quarter).
__host__ __device__ constexpr int tc_threads(int ep) { return 64 + ep * 128; }
constexpr uint32_t TMEM_COLS = 512;
constexpr uint32_t X_ATOM_BYTES = BM * 128;  // 128 rows x 64 BF16
constexpr uint32_t ONES_BYTES = BM * 32;     // 128 rows x 16 BF16
// Half 1's top-2 record as it crosses to half 0: the keys, and both centre
// indices relative to the slice in 16 bits each (0xFFFF: none).
struct alignas(16) HalfRec {
    uint32_t v1, v2, u;
    uint32_t ids;
};
__device__ __forceinline__ uint32_t pack_local(int i, int base) { return i < 0 ? 0xFFFFu : (uint32_t)(i - base); }
__device__ __forceinline__ int unpack_local(uint32_t l, int base) { return l == 0xFFFFu ? -1 : base + (int)l; }

// Shared-memory exchange between the epilogue parts of a row: for the top-2
// pass, `slots` rotating slots (see the tile merge in the kernel) of EP - 1
// records per row -- whole records for BF16 with two parts, 16-byte ones
// otherwise (FP8, whose larger X stages leave less room, and four parts) --
// none for the mask pass, whose parts write their own words of the row's
// candidate mask; the count pass rotates its slots like the top-2 pass, with
// SliceCount records.
__host__ __device__ constexpr uint32_t merge_bytes(int topk, bool fp8, int ep, int slots) {
    return topk == 1   ? 0u
           : topk == 2 ? BM * (uint32_t)slots * (uint32_t)(ep - 1) *
                             (uint32_t)((fp8 || ep > 2) ? sizeof(HalfRec) : sizeof(Top2))
                       : BM * (uint32_t)slots * (uint32_t)(ep - 1) * (uint32_t)sizeof(SliceCount);
}

// The record of one slot (FP8: HalfRec; BF16: Top2, no packing).
template <bool FP8> struct MergeSlot;
template <> struct MergeSlot<true> {
    HalfRec r;
    __device__ __forceinline__ void put(uint32_t v1, int i1, uint32_t v2, int i2, uint32_t u, int base) {
        r = HalfRec{v1, v2, u, pack_local(i1, base) | (pack_local(i2, base) << 16)};
    }
    __device__ __forceinline__ void get(uint32_t &v1, int &i1, uint32_t &v2, int &i2, uint32_t &u, int base) const {
        v1 = r.v1;
        v2 = r.v2;
        u = r.u;
        i1 = unpack_local(r.ids & 0xFFFFu, base);
        i2 = unpack_local(r.ids >> 16, base);
    }
};
template <> struct MergeSlot<false> {
    Top2 r;
    __device__ __forceinline__ void put(uint32_t v1, int i1, uint32_t v2, int i2, uint32_t u, int) {
        r = Top2{__uint_as_float(v1), __uint_as_float(v2), __uint_as_float(u), 0.f, i1, i2, 0, 0};
    }
    __device__ __forceinline__ void get(uint32_t &v1, int &i1, uint32_t &v2, int &i2, uint32_t &u, int) const {
        v1 = __float_as_uint(r.v1);
        v2 = __float_as_uint(r.v2);
        u = __float_as_uint(r.u3);
        i1 = r.i1;
        i2 = r.i2;
    }
};
constexpr uint32_t BAR_BYTES = 256;
constexpr uint32_t ATOM_RING = 4;  // atom slots of a one-stage ring (d_pad <= 4 atoms)
constexpr long long WAIT_LIMIT_CYCLES = 4000000000LL;

// Instruction descriptor, kind::f16: D = F32 (bits 4-5 = 1), A = B = BF16
// (bits 7-9 = 1, 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at
// bits 24-28.
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                           ((uint32_t)(BM >> 4) << 24);
// kind::f8f6f4 with A = B = E4M3 (format 0), D = F32, same shape fields.
constexpr uint32_t IDESC_FP8 = (1u << 4) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
constexpr uint32_t XAUG_BYTES = BM * 32;     // per-row augmentation tile (FP8): 128 rows x 16 BF16
constexpr uint32_t LAYOUT_SW128 = 2;
constexpr uint32_t LAYOUT_SW32 = 6;

struct TcParams {
    int64_t n;                       // rows (or the capacity when n_dev is set)
    int64_t tiles;
    const unsigned long long *n_dev; // optional: the row count is read here at launch
    int64_t out_stride;              // records of slice p start at p * out_stride
    int n_atoms;       // d_pad / 64
    int kp;            // centres per slice
    int nblocks;       // kp / 256
    int parts;
    int ctas_per_part;
    int slots;         // rotating tile-merge slots (top-2 pass)
    uint32_t off_c, off_x, off_aug, off_ones, off_merge, off_bar;
    uint32_t c_atom_bytes;  // kp * 128
    uint32_t x_stage_bytes;
    uint32_t c_tx_bytes;
    SliceTop2 *out;           // top-2 records (main pass)
    unsigned long long *err;
    const MixedStats *stats;  // cgrid, ulp of this launch
    const float *rowscale;    // FP8: per-row power of two 1/(s_i t) that maps scores to this row's units
    uint32_t off_xaug;        // FP8: per-stage augmentation tiles
    float *dump;  // optional: raw accumulators of the first tile of CTA 0 (tests only)
    uint32_t *masks;       // mask pass: wpr words per row, bit per centre (layout at mask_chunk)
    const float *thresh;   // mask and count passes: per-row threshold in score units
    SliceCount *outc;      // count pass records
    int wpr;               // mask words per row (k_pad / 32)
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait: false if the CTA is aborting or this wait ran out of time.
// The first test is inlined at every call site; only a wait that does not
// succeed at once pays for the call (the epilogue waits once per block).
__device__ __noinline__ bool mbar_wait_slow(uint32_t bar, uint32_t parity, volatile uint32_t *abort_flag,
                                            unsigned long long *err, unsigned long long code) {
    const long long t0 = clock64();
    uint32_t spins = 0;
    while (true) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((++spins & 63u) == 0u) {
            if (*abort_flag) return false;
            if (clock64() - t0 > WAIT_LIMIT_CYCLES) {
                *abort_flag = 1u;
                atomicOr(err, code);
                return false;
            }
        }
    }
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile uint32_t *abort_flag,
                                          unsigned long long *err, unsigned long long code) {
    return mbar_try_wait(bar, parity) || mbar_wait_slow(bar, parity, abort_flag, err, code);
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, uint32_t bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::
            "r"(dst),
        "l"((uint64_t)map), "r"(bar), "r"(x), "r"(y)
        : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor (sm_100 format): start address >> 4 in
// bits 0-13, leading-byte offset >> 4 in 16-29 (unused for swizzled K-major
// tiles whose K extent fits one atom), stride-byte offset >> 4 in 32-45
// (distance between 8-row groups), version 1 at bit 46, layout at 61-63.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t sbo, uint32_t layout) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1u << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1u << 46;
    d |= (uint64_t)layout << 61;
    return d;
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(IDESC), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_fp8(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(IDESC_FP8), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

// 32 consecutive columns of this thread's TMEM lane (asynchronous: the
// registers are valid only after tmem_wait on the same array).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
}

// Waits for every outstanding TMEM load; tied to r so that no use of r can be
// scheduled before it.
__device__ __forceinline__ void tmem_wait(uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.wait::ld.sync.aligned;"
        : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
          "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15]),
          "+r"(r[16]), "+r"(r[17]), "+r"(r[18]), "+r"(r[19]), "+r"(r[20]), "+r"(r[21]), "+r"(r[22]), "+r"(r[23]),
          "+r"(r[24]), "+r"(r[25]), "+r"(r[26]), "+r"(r[27]), "+r"(r[28]), "+r"(r[29]), "+r"(r[30]), "+r"(r[31])
        :
        : "memory");
}

__device__ __forceinline__ void tmem_ld(uint32_t taddr, uint32_t (&r)[32]) { tmem_ld32(taddr, r); }

// Columns per TMEM load in the top-2 epilogue. 64-column loads (32x32b.x64,
// two 64-register buffers) were tried: they exceed the 168 registers a thread
// of a 320-thread CTA can hold and spill, so the epilogue loads 32 columns at
// a time.
constexpr int TOP2_LOAD_COLS = 32;

__device__ __forceinline__ float fmax3(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// Running top-2 merge with a bound of the rest. (R1 >= R2, I1, I2) are the
// best two keys so far and U bounds every key seen but not kept. The merged
// result (w1 >= w2, j1, j2) comes with wu, a bound of its own rest (wu <= w2).
__device__ __forceinline__ void merge_res(uint32_t &R1, int &I1, uint32_t &R2, int &I2, uint32_t &U, uint32_t w1,
                                          int j1, uint32_t w2, int j2, uint32_t wu) {
    if (w1 > R1) {
        if (R1 > w2) {
            U = max(U, max(R2, w2));
            R2 = R1;
            I2 = I1;
        } else {
            U = max(U, max(R1, wu));
            R2 = w2;
            I2 = j2;
        }
        R1 = w1;
        I1 = j1;
    } else if (w1 > R2) {
        U = max(U, max(R2, w2));
        R2 = w1;
        I2 = j1;
    } else {
        U = max(U, w1);
    }
}

// Key of one score: every score of the launch lies in [2^E, 2^(E+1)), so
// (T + cgrid) - cgrid rounds it to a multiple of 128 ulp (its low 7 bits
// become zero) and adding code * ulp writes the column code (127 - the column
// within the half) into those bits exactly. Both steps run on the FMA pipe;
// keys are positive floats, so their float and unsigned orders agree. Padded
// columns (T = 0) get tiny keys; NaN scores (NaN rows) give NaN keys, ignored
// by fminf/fmaxf (such rows have non-finite bound ingredients and are always
// re-scored in full).
//
// Four scores per step: their top-2 as a small tournament (the quad's second
// is max3(loser of the final, loser of each pair): the winner's pair partner
// or the other pair's best), then one merge into the running top-2. The same
// 2.5 ALU operations per score as pairwise ranking, but the running chain
// advances once per four scores, so more of each warp's work is independent.
template <int COL0, int E, int N>
__device__ __forceinline__ void rank_quad(const uint32_t (&r)[N], float cgrid, float ulp, float &a1, float &a2) {
    uint64_t p0, p1, cg2;
    asm("mov.b64 %0, {%1, %2};" : "=l"(p0) : "r"(r[E]), "r"(r[E + 1]));
    asm("mov.b64 %0, {%1, %2};" : "=l"(p1) : "r"(r[E + 2]), "r"(r[E + 3]));
    asm("mov.b64 %0, {%1, %1};" : "=l"(cg2) : "f"(cgrid));
    asm("add.rn.f32x2 %0, %0, %1;" : "+l"(p0) : "l"(cg2));
    asm("add.rn.f32x2 %0, %0, %1;" : "+l"(p1) : "l"(cg2));
    asm("sub.rn.f32x2 %0, %0, %1;" : "+l"(p0) : "l"(cg2));
    asm("sub.rn.f32x2 %0, %0, %1;" : "+l"(p1) : "l"(cg2));
    float t0, t1, t2, t3;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(t0), "=f"(t1) : "l"(p0));
    asm("mov.b64 {%0, %1}, %2;" : "=f"(t2), "=f"(t3) : "l"(p1));
    const float k0 = __fmaf_rn(ulp, (float)(127 - ((COL0 + E) & 127)), t0);
    const float k1 = __fmaf_rn(ulp, (float)(127 - ((COL0 + E + 1) & 127)), t1);
    const float k2 = __fmaf_rn(ulp, (float)(127 - ((COL0 + E + 2) & 127)), t2);
    const float k3 = __fmaf_rn(ulp, (float)(127 - ((COL0 + E + 3) & 127)), t3);
    const float m01 = fmaxf(k0, k1), l01 = fminf(k0, k1);
    const float m23 = fmaxf(k2, k3), l23 = fminf(k2, k3);
    const float M = fmaxf(m01, m23), L = fminf(m01, m23);
    const float S = fmax3(L, l01, l23);
    a2 = fmax3(fminf(a1, M), a2, S);
    a1 = fmaxf(a1, M);
}

constexpr int NCH = 1;  // top-2 chains per rank pass (measured: 1 ~ 2 < 4 < 8 in time; the ALU pipe bounds it)

// Ranks the N scores of one TMEM load whose first column is COL0 within the part.
template <int COL0, int E, int N>
struct RankChunk {
    static __device__ __forceinline__ void run(const uint32_t (&r)[N], float cg, float ulp, float (&a1)[NCH],
                                               float (&a2)[NCH]) {
        rank_quad<COL0, E, N>(r, cg, ulp, a1[(E >> 2) & (NCH - 1)], a2[(E >> 2) & (NCH - 1)]);
        RankChunk<COL0, E + 4, N>::run(r, cg, ulp, a1, a2);
    }
};
template <int COL0, int N>
struct RankChunk<COL0, N, N> {
    static __device__ __forceinline__ void run(const uint32_t (&)[N], float, float, float (&)[NCH], float (&)[NCH]) {}
};

// ------------------------------------------------ mask (second pass) --
// One 32-column chunk of a row's candidate mask: column e is a candidate
// when its score T_e > th. fma.sat(T, S, C) with S = 8 / ulp and C = -th S
// is exactly 0 or 1: T and th are floats of at least 2^(E-2) (the caller
// sends every lower threshold to -inf), so a nonzero T - th is a multiple
// of 2^(E-25) and (T - th) S a nonzero multiple of 2, whose rounding keeps
// its sign; T = th gives 0; a padded column (T = 0) gives 0, or 1 with th =
// -inf; NaN gives 0. Every threshold lies strictly below the scores that
// can win (its margin holds 384 ulp, and its roundings go down), so the
// strict comparison loses no candidate. Horner steps on packed pairs, acc = 2 acc + (bit even, bit
// odd), exact below 2^16, put the even columns 2j in bits 15 - j of the low
// half and the odd columns 2j + 1 in bits 31 - j: one saturating FMA per
// score and one packed FMA per two scores, no ALU instruction. The steps
// run as two independent 8-step chains (columns 0-15 and 16-31) joined by
// acc = hi 2^8 + lo, which halves the dependent chain (count pass 0.778 ->
// 0.759 ms at n = 4M, d = 128, k = 1024; four 4-step chains 0.791 ms).
// (Also tried and slower: a magic-number add and a byte permute in place of
// the two conversions, a branch-free word record, four max chains.)
__device__ __forceinline__ uint32_t mask_chunk(const uint32_t (&r)[32], float S, float C, uint64_t two2) {
    uint64_t hi = 0ull, lo = 0ull, s256;
    asm("mov.b64 %0, {%1, %1};" : "=l"(s256) : "f"(256.f));
#pragma unroll
    for (int j = 0; j < 8; j++) {
        float b0, b1, b2, b3;
        asm("fma.rn.sat.f32 %0, %1, %2, %3;" : "=f"(b0) : "f"(__uint_as_float(r[2 * j])), "f"(S), "f"(C));
        asm("fma.rn.sat.f32 %0, %1, %2, %3;" : "=f"(b1) : "f"(__uint_as_float(r[2 * j + 1])), "f"(S), "f"(C));
        asm("fma.rn.sat.f32 %0, %1, %2, %3;" : "=f"(b2) : "f"(__uint_as_float(r[2 * j + 16])), "f"(S), "f"(C));
        asm("fma.rn.sat.f32 %0, %1, %2, %3;" : "=f"(b3) : "f"(__uint_as_float(r[2 * j + 17])), "f"(S), "f"(C));
        uint64_t bb, bc;
        asm("mov.b64 %0, {%1, %2};" : "=l"(bb) : "f"(b0), "f"(b1));
        asm("mov.b64 %0, {%1, %2};" : "=l"(bc) : "f"(b2), "f"(b3));
        asm("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(hi) : "l"(two2), "l"(bb));
        asm("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(lo) : "l"(two2), "l"(bc));
    }
    uint64_t acc;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(acc) : "l"(hi), "l"(s256), "l"(lo));
    float e, o;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(e), "=f"(o) : "l"(acc));
    return (uint32_t)e | ((uint32_t)o << 16);
}

// Count pass: one 32-column chunk folded into a row's running state -- the
// largest score (three-input max on the raw accumulators; NaN is ignored,
// and real scores are positive, so 0 means none), the number of marked
// centres, and the first two nonzero mask words with their word index gw.
struct CountState {
    float vmax;
    uint32_t cnt, w1, w2;
    int wi1, wi2;
};

__device__ __forceinline__ void count_add_word(CountState &s, uint32_t word, int gw) {
    if (word) {
        if (!s.w1) {
            s.w1 = word;
            s.wi1 = gw;
        } else if (!s.w2) {
            s.w2 = word;
            s.wi2 = gw;
        }
    }
}

__device__ __forceinline__ void count_chunk(const uint32_t (&r)[32], float S, float C, uint64_t two2, int gw,
                                            CountState &s) {
    const uint32_t word = mask_chunk(r, S, C, two2);
    float m0 = s.vmax, m1 = 0.f;  // two chains: more independent work per step
#pragma unroll
    for (int e = 0; e < 32; e += 4) {
        m0 = fmax3(m0, __uint_as_float(r[e]), __uint_as_float(r[e + 1]));
        m1 = fmax3(m1, __uint_as_float(r[e + 2]), __uint_as_float(r[e + 3]));
    }
    s.vmax = fmaxf(m0, m1);
    s.cnt += (uint32_t)__popc(word);
    count_add_word(s, word, gw);
}

__device__ __forceinline__ SliceCount count_pack(const CountState &s) {
    const uint32_t c = s.cnt < 0xFFFFu ? s.cnt : 0xFFFFu;
    return SliceCount{s.vmax, c | ((uint32_t)(s.w1 ? s.wi1 : 0xFF) << 16) | ((uint32_t)(s.w2 ? s.wi2 : 0xFF) << 24),
                      s.w1, s.w2};
}

__device__ __forceinline__ void count_merge(CountState &s, const SliceCount &o) {
    s.vmax = fmaxf(s.vmax, o.vmax);
    s.cnt += o.meta & 0xFFFFu;
    count_add_word(s, o.w1, (int)((o.meta >> 16) & 0xFFu));
    count_add_word(s, o.w2, (int)(o.meta >> 24));
}

// FP8: X and the centres are E4M3 (1 byte, 128 per swizzle atom) and the
// augmentation operand is a per-row BF16 tile loaded with each X tile (the
// row's scale times [1,1,1,0,...]); BF16: a constant ones tile.
template <int TOPK, bool FP8, int XST, int EP>
__global__ void __launch_bounds__(tc_threads(EP), 1)
    tc_assign_kernel(const __grid_constant__ CUtensorMap tm_x, const __grid_constant__ CUtensorMap tm_c,
                     const __grid_constant__ CUtensorMap tm_aug, const __grid_constant__ CUtensorMap tm_ones,
                     TcParams p) {
    if (p.n_dev) {
        const unsigned long long cnt = *p.n_dev;
        p.n = (int64_t)(cnt < (unsigned long long)p.n ? cnt : (unsigned long long)p.n);
        p.tiles = (p.n + BM - 1) / BM;
    }
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const uint32_t sb = smem_u32(smem);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int part = blockIdx.x % p.parts;
    const int64_t q = blockIdx.x / p.parts;
    const int64_t tstride = p.ctas_per_part;

    // With one X stage the stage is a ring of its atoms (at most ATOM_RING),
    // each with its own full / empty barrier: the next tile's first atoms load
    // while the MMAs still read this tile's last ones.
    constexpr uint32_t NXB = XST == 1 ? ATOM_RING : XST;  // X barriers of each kind
    const uint32_t bar_c = sb + p.off_bar;
    auto bar_xfull = [&](int s) { return bar_c + 8u * (1u + (uint32_t)s); };
    auto bar_xempty = [&](int s) { return bar_c + 8u * (1u + NXB + (uint32_t)s); };
    auto bar_afull = [&](int b) { return bar_c + 8u * (1u + 2 * NXB + (uint32_t)b); };
    auto bar_aempty = [&](int b) { return bar_c + 8u * (3u + 2 * NXB + (uint32_t)b); };
    uint32_t *slot = (uint32_t *)(smem + p.off_bar + 128);
    volatile uint32_t *abort_flag = slot + 1;

    if (threadIdx.x == 0) {
        mbar_init(bar_c, 1);
        for (int s = 0; s < (XST == 1 ? p.n_atoms : XST); s++) {
            mbar_init(bar_xfull(s), 1);
            mbar_init(bar_xempty(s), 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(bar_afull(b), 1);
            mbar_init(bar_aempty(b), 4 * EP);
        }
        *abort_flag = 0u;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *slot;

    if (warp == 0) {
        if (lane == 0) {
            // Resident slice of the centres, its augmentation rows, and the ones tile.
            mbar_expect_tx(bar_c, p.c_tx_bytes);
            const int crow0 = part * p.kp;
            for (int a = 0; a < p.n_atoms; a++)
                for (int r = 0; r < p.kp; r += BN)
                    tma_load_2d(sb + p.off_c + (uint32_t)a * p.c_atom_bytes + (uint32_t)r * 128u, &tm_c, bar_c,
                                a * (FP8 ? 128 : 64), crow0 + r);
            for (int r = 0; r < p.kp; r += BN) tma_load_2d(sb + p.off_aug + (uint32_t)r * 32u, &tm_aug, bar_c, 0, crow0 + r);
            if (!FP8) tma_load_2d(sb + p.off_ones, &tm_ones, bar_c, 0, 0);
            // ring entries: whole tiles (two stages) or single atoms (one stage)
            const int nring = XST == 1 ? p.n_atoms : XST;
            int it = 0;
            bool stop = false;
            for (int64_t t = q; t < p.tiles && !stop; t += tstride) {
                if constexpr (XST == 1) {
                    for (int a = 0; a < p.n_atoms; a++, ++it) {
                        const uint32_t ph = (uint32_t)(it / nring) & 1u;  // it % nring == a
                        if (!mbar_wait(bar_xempty(a), ph ^ 1u, abort_flag, p.err, 1ull)) {
                            stop = true;
                            break;
                        }
                        // FP8: the tile's augmentation rows ride with its last atom
                        const bool aug = FP8 && a == p.n_atoms - 1;
                        mbar_expect_tx(bar_xfull(a), X_ATOM_BYTES + (aug ? XAUG_BYTES : 0u));
                        tma_load_2d(sb + p.off_x + (uint32_t)a * X_ATOM_BYTES, &tm_x, bar_xfull(a),
                                    a * (FP8 ? 128 : 64), (int)(t * BM));
                        if (aug) tma_load_2d(sb + p.off_xaug, &tm_ones, bar_xfull(a), 0, (int)(t * BM));
                    }
                } else {
                    const int s = it % XST;
                    const uint32_t ph = (uint32_t)(it / XST) & 1u;
                    if (!mbar_wait(bar_xempty(s), ph ^ 1u, abort_flag, p.err, 1ull)) break;
                    mbar_expect_tx(bar_xfull(s), p.x_stage_bytes + (FP8 ? XAUG_BYTES : 0u));
                    for (int a = 0; a < p.n_atoms; a++)
                        tma_load_2d(sb + p.off_x + (uint32_t)s * p.x_stage_bytes + (uint32_t)a * X_ATOM_BYTES, &tm_x,
                                    bar_xfull(s), a * (FP8 ? 128 : 64), (int)(t * BM));
                    if (FP8)
                        tma_load_2d(sb + p.off_xaug + (uint32_t)s * XAUG_BYTES, &tm_ones, bar_xfull(s), 0,
                                    (int)(t * BM));
                    ++it;
                }
            }
            // Drain: every issued X load must land before the CTA can exit.
            const int issued = it;
            for (int j = issued > nring ? issued - nring : 0; j < issued; j++)
                mbar_wait(bar_xfull(j % nring), (uint32_t)(j / nring) & 1u, abort_flag, p.err, 0ull);
            mbar_wait(bar_c, 0u, abort_flag, p.err, 0ull);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            int it = 0;
            uint32_t item = 0;
            int last_s = -1;
            uint32_t last_ph = 0;
            if (mbar_wait(bar_c, 0u, abort_flag, p.err, 2ull)) {
                tc_fence_after();
                bool ok = true;
                for (int64_t t = q; t < p.tiles && ok; t += tstride, ++it) {
                    // one stage: ring entry (it, a) is atom slot a in phase it & 1
                    const int s = XST == 1 ? 0 : it % XST;
                    const uint32_t ph = (uint32_t)(XST == 1 ? it : it / XST) & 1u;
                    if (XST != 1) {
                        if (!mbar_wait(bar_xfull(s), ph, abort_flag, p.err, 4ull)) break;
                        tc_fence_after();
                    }
                    const uint32_t xs = sb + p.off_x + (uint32_t)s * p.x_stage_bytes;
                    for (int b = 0; b < p.nblocks; b++, item++) {
                        const int buf = (int)(item & 1u);
                        const uint32_t aph = (item >> 1) & 1u;
                        if (!mbar_wait(bar_aempty(buf), aph ^ 1u, abort_flag, p.err, 8ull)) {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                        const bool last_b = b == p.nblocks - 1;
                        const uint32_t dt = tmem + (uint32_t)buf * BN;
                        const uint32_t cs = sb + p.off_c + (uint32_t)b * BN * 128u;
                        for (int a = 0; a < p.n_atoms; a++) {
                            if (XST == 1 && b == 0) {
                                if (!mbar_wait(bar_xfull(a), ph, abort_flag, p.err, 4ull)) {
                                    ok = false;
                                    break;
                                }
                                tc_fence_after();
                            }
#pragma unroll
                            for (int kk = 0; kk < 4; kk++) {
                                const uint64_t ad = sdesc(xs + (uint32_t)a * X_ATOM_BYTES + kk * 32u, 1024u, LAYOUT_SW128);
                                const uint64_t bd = sdesc(cs + (uint32_t)a * p.c_atom_bytes + kk * 32u, 1024u, LAYOUT_SW128);
                                if (FP8)
                                    mma_fp8(dt, ad, bd, (a | kk) != 0 ? 1u : 0u);
                                else
                                    mma_bf16(dt, ad, bd, (a | kk) != 0 ? 1u : 0u);
                            }
                            // the tile's last block has read this atom: its slot is free
                            // (FP8: the last atom's slot also holds the augmentation rows)
                            if (XST == 1 && last_b && !(FP8 && a == p.n_atoms - 1)) {
                                mma_commit(bar_xempty(a));
                                last_s = a;
                                last_ph = ph;
                            }
                        }
                        if (!ok) break;
                        const uint32_t aug_a = FP8 ? sb + p.off_xaug + (uint32_t)s * XAUG_BYTES : sb + p.off_ones;
                        mma_bf16(dt, sdesc(aug_a, 256u, LAYOUT_SW32),
                                 sdesc(sb + p.off_aug + (uint32_t)b * BN * 32u, 256u, LAYOUT_SW32), 1u);
                        if (XST == 1 && FP8 && last_b) {
                            mma_commit(bar_xempty(p.n_atoms - 1));
                            last_s = p.n_atoms - 1;
                            last_ph = ph;
                        }
                        mma_commit(bar_afull(buf));
                    }
                    if (!ok) break;
                    if (XST != 1) {
                        mma_commit(bar_xempty(s));
                        last_s = s;
                        last_ph = ph;
                    }
                }
            }
            // Drain: the last commit covers every MMA issued before it.
            if (last_s >= 0) mbar_wait(bar_xempty(last_s), last_ph, abort_flag, p.err, 0ull);
        }
    } else if constexpr (TOPK == 1) {
        // Mask pass: every part writes its 128 columns' words of each row's
        // mask straight to global memory (no exchange between the parts).
        constexpr int CP = BN / EP;
        constexpr int NCK = CP / 32;
        static_assert(NCK == 4, "the mask pass runs with two epilogue parts");
        const int ew = warp - 2;
        const int quarter = warp & 3;
        const int prt = ew >> 2;
        const int row_local = quarter * 32 + lane;
        const uint32_t lane_addr = tmem + ((uint32_t)(quarter * 32) << 16);
        const float S = 8.f / p.stats->ulp;  // a power of two
        uint64_t two2;
        asm("mov.b64 %0, {%1, %1};" : "=l"(two2) : "f"(2.f));
        uint32_t item = 0;
        bool dead = false;
        float th_next = q * BM + row_local < p.n ? p.thresh[q * BM + row_local] : INFINITY;  // one tile ahead
        for (int64_t t = q; t < p.tiles; t += tstride) {
            const int64_t row = t * BM + row_local;
            const float th = th_next;
            {
                const int64_t nrow = (t + tstride) * BM + row_local;
                th_next = nrow < p.n ? p.thresh[nrow] : INFINITY;
            }
            const float C = -(th * S);  // exact: a float times a power of two
            for (int b = 0; b < p.nblocks; b++, item++) {
                const int buf = (int)(item & 1u);
                const uint32_t aph = (item >> 1) & 1u;
                if (!dead && !mbar_wait(bar_afull(buf), aph, abort_flag, p.err, 16ull)) dead = true;
                dead = __any_sync(0xffffffffu, dead);
                if (dead) continue;
                tc_fence_after();
                const uint32_t col = lane_addr + (uint32_t)buf * BN + (uint32_t)prt * CP;
                uint32_t ra[32], rb[32];
                uint4 w;
                tmem_ld32(col, ra);
                tmem_wait(ra);
                tmem_ld32(col + 32, rb);
                w.x = mask_chunk(ra, S, C, two2);
                tmem_wait(rb);
                tmem_ld32(col + 64, ra);
                w.y = mask_chunk(rb, S, C, two2);
                tmem_wait(ra);
                tmem_ld32(col + 96, rb);
                w.z = mask_chunk(ra, S, C, two2);
                tmem_wait(rb);
                // every column of this block is in registers: release the buffer
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(bar_aempty(buf));
                w.w = mask_chunk(rb, S, C, two2);
                if (row < p.n) {
                    const int word = (part * p.kp + b * BN + prt * CP) / 32;  // a multiple of 4
                    *reinterpret_cast<uint4 *>(p.masks + row * (int64_t)p.wpr + word) = w;
                }
            }
        }
    } else if constexpr (TOPK == 3) {
        // Count pass: per row, against the row's threshold, the largest score
        // and the marked centres' number and first mask words; the parts of a
        // row meet once per tile through the rotating slots, as in the top-2
        // pass below.
        constexpr int CP = BN / EP;
        constexpr int NCK = CP / 32;
        static_assert(NCK == 2 || NCK == 4, "two or four epilogue parts");
        constexpr int EPI = 4 * EP * 32;  // epilogue threads (the named barriers' count)
        const int ew = warp - 2;
        const int quarter = warp & 3;
        const int prt = ew >> 2;
        const int row_local = quarter * 32 + lane;
        const uint32_t lane_addr = tmem + ((uint32_t)(quarter * 32) << 16);
        SliceCount *merge = (SliceCount *)(smem + p.off_merge);
        const float S = 8.f / p.stats->ulp;  // a power of two
        uint64_t two2;
        asm("mov.b64 %0, {%1, %1};" : "=l"(two2) : "f"(2.f));
        uint32_t item = 0, tile_it = 0;
        bool dead = false;
        // the row's threshold (and FP8 scale) one tile ahead, so that no tile
        // starts on a global load
        float th_next = INFINITY, rs_next = 1.f;
        if (q * BM + row_local < p.n) {
            th_next = p.thresh[q * BM + row_local];
            if (FP8) rs_next = p.rowscale[q * BM + row_local];
        }
        for (int64_t t = q; t < p.tiles; t += tstride, tile_it++) {
            const int64_t row = t * BM + row_local;
            const float th = th_next, rs = rs_next;
            {
                const int64_t nrow = (t + tstride) * BM + row_local;
                th_next = nrow < p.n ? p.thresh[nrow] : INFINITY;
                if (FP8) rs_next = nrow < p.n ? p.rowscale[nrow] : 1.f;
            }
            const float C = -(th * S);  // exact: a float times a power of two
            // FP8 accumulators are the row's scores times rs (a power of two):
            // T_acc (S / rs) - th S is exactly (T - th) S
            const float Sr = FP8 ? S / rs : S;
            CountState st{0.f, 0u, 0u, 0u, 0, 0};
            for (int b = 0; b < p.nblocks; b++, item++) {
                const int buf = (int)(item & 1u);
                const uint32_t aph = (item >> 1) & 1u;
                if (!dead && !mbar_wait(bar_afull(buf), aph, abort_flag, p.err, 16ull)) dead = true;
                dead = __any_sync(0xffffffffu, dead);  // warp-uniform, for the barriers below
                if (dead) continue;
                tc_fence_after();
                const uint32_t col = lane_addr + (uint32_t)buf * BN + (uint32_t)prt * CP;
                const int wbase = (b * BN + prt * CP) / 32;  // word index within the slice
                uint32_t ra[32], rb[32];
                tmem_ld32(col, ra);
                tmem_wait(ra);
                tmem_ld32(col + 32, rb);
                count_chunk(ra, Sr, C, two2, wbase, st);
                tmem_wait(rb);
                if (NCK == 4) {
                    tmem_ld32(col + 64, ra);
                    count_chunk(rb, Sr, C, two2, wbase + 1, st);
                    tmem_wait(ra);
                    tmem_ld32(col + 96, rb);
                    count_chunk(ra, Sr, C, two2, wbase + 2, st);
                    tmem_wait(rb);
                }
                // every column of this block is in registers: release the buffer
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(bar_aempty(buf));
                count_chunk(rb, Sr, C, two2, wbase + NCK - 1, st);
            }
            // tile merge: the slot and barrier protocol of the top-2 pass
            const uint32_t sl = tile_it % (uint32_t)p.slots;
            SliceCount *slot = merge + sl * (uint32_t)(EP - 1) * BM;
            if (prt > 0) {
                slot[(prt - 1) * BM + row_local] = count_pack(st);
                if (dead)
                    asm volatile("bar.sync %0, %1;" ::"r"(1u + sl), "r"(EPI) : "memory");
                else
                    asm volatile("bar.arrive %0, %1;" ::"r"(1u + sl), "r"(EPI) : "memory");
            } else {
                asm volatile("bar.sync %0, %1;" ::"r"(1u + sl), "r"(EPI) : "memory");
#pragma unroll
                for (int o = 1; o < EP; o++) count_merge(st, slot[(o - 1) * BM + row_local]);
                if (row < p.n && !dead) p.outc[(int64_t)part * p.out_stride + row] = count_pack(st);
            }
        }
    } else {
        static_assert(TOPK == 2, "pass kinds: 1 masks, 2 top-2, 3 count");
        constexpr int CP = BN / EP;   // columns of one part
        constexpr int NCK = CP / 32;  // its 32-column chunks
        static_assert(NCK == 2 || NCK == 4, "two or four epilogue parts");
        constexpr int LDW = TOP2_LOAD_COLS;  // columns per TMEM load
        static_assert(CP / LDW == 2 || CP / LDW == 4, "two or four loads per part");
        constexpr int EPI = 4 * EP * 32;  // epilogue threads (the named barriers' count)
        using Slot = MergeSlot<FP8 || (EP > 2)>;
        const int ew = warp - 2;
        const int quarter = warp & 3;
        const int prt = ew >> 2;
        const int row_local = quarter * 32 + lane;
        const uint32_t lane_addr = tmem + ((uint32_t)(quarter * 32) << 16);
        Slot *merge = (Slot *)(smem + p.off_merge);
        const int slice0 = part * p.kp;  // the slice's first centre
        const float cgrid = p.stats->cgrid, ulp = p.stats->ulp;
        const int64_t my_tiles = q < p.tiles ? (p.tiles - 1 - q) / tstride + 1 : 0;
        const uint32_t items = (uint32_t)(my_tiles * p.nblocks);
        uint32_t item = 0, tile_it = 0;
        bool dead = false;
        // Software pipeline across accumulator blocks: a block's buffer goes
        // back to the MMA warp as soon as its last 32 columns are in
        // registers, and the next block's first 32 columns start loading
        // (when its MMAs have already committed) while those last columns
        // are ranked, so the warps of a sub-partition do not all wait on a
        // fresh TMEM load at every block. pre: ra holds that load.
        uint32_t ra[LDW], rb[LDW];
        bool pre = false;
        // FP8: the row's scale one tile ahead, so that no tile starts on a global load
        float rs_next = 1.f;
        if (FP8 && q * BM + row_local < p.n) rs_next = p.rowscale[q * BM + row_local];
        for (int64_t t = q; t < p.tiles; t += tstride, tile_it++) {
            uint32_t R1 = 0u, R2 = 0u, U = 0u;
            int I1 = -1, I2 = -1;
            float cg = cgrid, ul = ulp;
            if (FP8) {
                const float rs = rs_next;
                const int64_t nrow = (t + tstride) * BM + row_local;
                rs_next = nrow < p.n ? p.rowscale[nrow] : 1.f;
                cg = cgrid * rs;
                ul = ulp * rs;
            }
            for (int b = 0; b < p.nblocks; b++, item++) {
                const int buf = (int)(item & 1u);
                const uint32_t aph = (item >> 1) & 1u;
                const uint32_t col = lane_addr + (uint32_t)buf * BN + (uint32_t)prt * CP;
                if (!pre) {
                    if (!dead && !mbar_wait(bar_afull(buf), aph, abort_flag, p.err, 16ull)) dead = true;
                    dead = __any_sync(0xffffffffu, dead);  // warp-uniform, for the barriers below
                    if (dead) continue;
                    tc_fence_after();
                    tmem_ld(col, ra);
                }
                pre = false;
                if (p.dump && blockIdx.x == 0 && t == q) {
                    for (int ch = 0; ch < NCK; ch++) {
                        uint32_t r[32];
                        tmem_ld32(col + ch * 32, r);
                        tmem_wait(r);
                        for (int e = 0; e < 32; e++)
                            p.dump[(int64_t)row_local * (p.nblocks * BN) + b * BN + prt * CP + ch * 32 + e] =
                                __uint_as_float(r[e]);
                    }
                }
                float a1[NCH], a2[NCH];
#pragma unroll
                for (int qd = 0; qd < NCH; qd++) a1[qd] = a2[qd] = 0.f;
                tmem_wait(ra);
                tmem_ld(col + LDW, rb);
                RankChunk<0, 0, LDW>::run(ra, cg, ul, a1, a2);
                tmem_wait(rb);
                if (CP / LDW == 4) {
                    tmem_ld(col + 2 * LDW, ra);
                    RankChunk<LDW, 0, LDW>::run(rb, cg, ul, a1, a2);
                    tmem_wait(ra);
                    tmem_ld(col + 3 * LDW, rb);
                    RankChunk<2 * LDW, 0, LDW>::run(ra, cg, ul, a1, a2);
                    tmem_wait(rb);
                }
                // every column of this block is in registers: release the buffer
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(bar_aempty(buf));
                if (item + 1 < items) {
                    const int nbuf = (int)((item + 1) & 1u);
                    const uint32_t naph = ((item + 1) >> 1) & 1u;
                    if (__all_sync(0xffffffffu, mbar_try_wait(bar_afull(nbuf), naph))) {
                        tc_fence_after();
                        tmem_ld(lane_addr + (uint32_t)nbuf * BN + (uint32_t)prt * CP, ra);
                        pre = true;
                    }
                }
                RankChunk<CP - LDW, 0, LDW>::run(rb, cg, ul, a1, a2);
                uint32_t b1 = __float_as_uint(a1[0]), b2 = __float_as_uint(a2[0]), bu = b2;
                int d1 = 0, d2 = 0;  // indices are carried inside the keys
#pragma unroll
                for (int qd = 1; qd < NCH; qd++)
                    merge_res(b1, d1, b2, d2, bu, __float_as_uint(a1[qd]), 0, __float_as_uint(a2[qd]), 0,
                              __float_as_uint(a2[qd]));
                const int base = part * p.kp + b * BN + prt * CP + 127;
                merge_res(R1, I1, R2, I2, U, b1 & 0xFFFFFF80u, base - (int)(b1 & 0x7Fu), b2 & 0xFFFFFF80u,
                          base - (int)(b2 & 0x7Fu), bu & 0xFFFFFF80u);
            }
            // Tile merge: parts 1.. publish their records in slot
            // tile_it % slots and arrive on named barrier 1 + that slot
            // without waiting; part 0 waits there, merges and stores. A part
            // cannot reach the same slot and barrier again before part 0 has
            // passed this merge: that tile's accumulators need every epilogue
            // warp to have released the buffer of an earlier tile of this
            // CTA (three slots when a tile is one accumulator block, two
            // otherwise: the host plans which). An aborting warp is no longer
            // held back by the MMAs, so it waits instead.
            const uint32_t sl = tile_it % (uint32_t)p.slots;
            Slot *slot = merge + sl * (uint32_t)(EP - 1) * BM;
            if (prt > 0) {
                slot[(prt - 1) * BM + row_local].put(R1, I1, R2, I2, U, slice0);
                if (dead)
                    asm volatile("bar.sync %0, %1;" ::"r"(1u + sl), "r"(EPI) : "memory");
                else
                    asm volatile("bar.arrive %0, %1;" ::"r"(1u + sl), "r"(EPI) : "memory");
            } else {
                asm volatile("bar.sync %0, %1;" ::"r"(1u + sl), "r"(EPI) : "memory");
#pragma unroll
                for (int o = 1; o < EP; o++) {
                    uint32_t w1, w2, wu;
                    int j1, j2;
                    slot[(o - 1) * BM + row_local].get(w1, j1, w2, j2, wu, slice0);
                    merge_res(R1, I1, R2, I2, U, w1, j1, w2, j2, wu);
                }
                const int64_t row = t * BM + row_local;
                if (row < p.n && !dead)
                    p.out[(int64_t)part * p.out_stride + row] =
                        SliceTop2{__uint_as_float(R1), __uint_as_float(R2), __uint_as_float(U),
                                  pack_local(I1, slice0) | (pack_local(I2, slice0) << 16)};
            }
        }
        if (pre) tmem_wait(ra);  // a load issued for an item that never ran completes before exit
    }

    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    }
}

// --------------------------------------------- tensor-core peak loop --
// Dense tensor-core throughput of this GPU with the contraction's own MMA
// shape: M=128, N=256, K=16 (BF16) or K=32 (E4M3) from 128-byte-swizzled
// shared memory into a TMEM accumulator. One CTA per SM; one thread issues
// iters x 4 MMAs back to back (one swizzle atom of K per iteration), commits
// once and waits (bounded) for completion. The operands are fixed finite
// patterns written by the threads (then made visible to the tensor core's
// proxy); only the time matters.
constexpr uint32_t PEAK_A_BYTES = BM * 128u, PEAK_B_BYTES = BN * 128u;

template <bool FP8>
__global__ void __launch_bounds__(128, 1) tc_peak_kernel(int iters, unsigned long long *err) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const uint32_t sb = smem_u32(smem);
    const uint32_t bar = sb + PEAK_A_BYTES + PEAK_B_BYTES;
    uint32_t *slot = (uint32_t *)(smem + PEAK_A_BYTES + PEAK_B_BYTES + 64);
    volatile uint32_t *abort_flag = slot + 1;
    uint32_t *words = (uint32_t *)smem;
    for (uint32_t i = threadIdx.x; i < (PEAK_A_BYTES + PEAK_B_BYTES) / 4; i += blockDim.x) {
        const uint32_t v = (i * 2654435761u) >> 27;  // 0..31
        // E4M3 bytes 0x30..0x3F (0.5 .. 0.94) or BF16 halves 0x3F80..0x3F9F (1.0 .. 1.24)
        words[i] = FP8 ? 0x30303030u + v * 0x00010101u : (0x3F803F80u + (v << 16) + (v ^ 7u));
    }
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        *abort_flag = 0u;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the threads' stores, seen by the MMAs
    if (threadIdx.x < 32) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                     "r"(256u)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *slot;
    if (threadIdx.x == 0) {
        for (int it = 0; it < iters; it++) {
#pragma unroll
            for (int kk = 0; kk < 4; kk++) {
                const uint64_t ad = sdesc(sb + kk * 32u, 1024u, LAYOUT_SW128);
                const uint64_t bd = sdesc(sb + PEAK_A_BYTES + kk * 32u, 1024u, LAYOUT_SW128);
                if (FP8)
                    mma_fp8(tmem, ad, bd, (it | kk) != 0 ? 1u : 0u);
                else
                    mma_bf16(tmem, ad, bd, (it | kk) != 0 ? 1u : 0u);
            }
        }
        mma_commit(bar);
        mbar_wait(bar, 0u, abort_flag, err, 32ull);
    }
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x < 32) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(256u) : "memory");
    }
}

// ------------------------------------------------------------- host side --
PFN_cuTensorMapEncodeTiled_v12000 get_encode(Ctx &ctx) {
    if (!ctx.tmap_fn) {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult qr;
        FK_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &qr));
        if (!fn || qr != cudaDriverEntryPointSuccess) {
            set_error("cuTensorMapEncodeTiled is not available from the CUDA driver");
            fail(FK_ERR_CUDA);
        }
        ctx.tmap_fn = fn;
    }
    return (PFN_cuTensorMapEncodeTiled_v12000)ctx.tmap_fn;
}

void encode_2d(Ctx &ctx, void *out, const void *ptr, uint64_t inner, uint64_t outer, uint64_t row_bytes,
               uint32_t box_inner, uint32_t box_outer, CUtensorMapSwizzle swz,
               CUtensorMapDataType dt = CU_TENSOR_MAP_DATA_TYPE_BFLOAT16) {
    auto enc = get_encode(ctx);
    CUtensorMap m;
    cuuint64_t dims[2] = {inner, outer};
    cuuint64_t strides[1] = {row_bytes};
    cuuint32_t box[2] = {box_inner, box_outer};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(&m, dt, 2, const_cast<void *>(ptr), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, swz, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed (%d) for a %llux%llu tensor", (int)r, (unsigned long long)outer,
                  (unsigned long long)inner);
        fail(FK_ERR_CUDA);
    }
    memcpy(out, &m, sizeof(m));
}

constexpr size_t SMEM_LIMIT = 227 * 1024;

}  // namespace

// The launch shape of one tensor-core pass (host arithmetic only): the X
// ring depth, the resident slice of centres that fits next to it, the grid.
// kp_fixed > 0 imposes the slice size of another plan (the mask pass reads
// the main pass's centre operands, so it must slice them the same way).
void plan_shape(MixedPlan &mp, int64_t n, int d, int k, bool fp8, int topk, int sms, int kp_fixed) {
    mp.n = n;
    mp.d = d;
    mp.k = k;
    mp.fp8 = fp8;
    mp.topk = topk;
    const int per_atom = fp8 ? 128 : 64;  // elements per 128-byte swizzle atom
    mp.d_pad = (d + per_atom - 1) / per_atom * per_atom;
    const int n_atoms = mp.d_pad / per_atom;
    const size_t x_stage = (size_t)n_atoms * X_ATOM_BYTES;
    const size_t per_centre = (size_t)n_atoms * 128 + 32;
    // two X stages when 256 resident centres still fit, else one (run as a
    // ring of its atoms)
    // Two epilogue parts per lane quarter (8 epilogue warps, three merge
    // slots). The kernel also takes four (16 warps, 64 columns each, two
    // slots when a tile has two blocks or more), measured slower at n = 4M,
    // d = 128, k = 1024: top-2 pass 1.351 against 1.020 ms (96 registers a
    // thread, four-way merges), count pass 0.873 against 0.812 ms.
    mp.ep = 2;
    mp.slots = 3;
    size_t fixed = 0;
    for (;;) {
        int xst = 2;
        for (; xst >= 1; xst--) {
            fixed = 1024 + xst * x_stage + (fp8 ? xst * XAUG_BYTES : ONES_BYTES) +
                    merge_bytes(topk, fp8, mp.ep, mp.slots) + BAR_BYTES;
            if (fixed + (size_t)(kp_fixed > 0 ? kp_fixed : BN) * per_centre <= SMEM_LIMIT) break;
        }
        if (xst < 1) {
            set_error("the resident-slice tensor-core kernel supports d <= %d for this precision (got %d)",
                      fp8 ? 512 : 256, d);
            fail(FK_ERR_UNSUPPORTED);
        }
        mp.xst = xst;
        if (xst == 1 && n_atoms > (int)ATOM_RING) {
            set_error("one-stage tensor-core plan with %d atoms (the ring holds %u)", n_atoms, ATOM_RING);
            fail(FK_ERR_UNSUPPORTED);
        }
        const int kp_max = kp_fixed > 0 ? kp_fixed : (int)((SMEM_LIMIT - fixed) / per_centre) / BN * BN;
        mp.parts = (k + kp_max - 1) / kp_max;
        mp.kp = ((k + mp.parts - 1) / mp.parts + BN - 1) / BN * BN;
        mp.k_pad = mp.parts * mp.kp;
        mp.nblocks = mp.kp / BN;
        if ((topk == 2 || topk == 3) && mp.nblocks < 2 && mp.slots < 3) {
            mp.slots = 3;
            continue;
        }
        if (topk == 3 && mp.ep == 4 && mp.nblocks >= 2 && mp.slots == 3) {
            mp.slots = 2;  // a smaller exchange; the slice stays as planned
            continue;
        }
        break;
    }
    mp.tiles = (n + BM - 1) / BM;
    if (sms < 1) sms = 1;
    mp.ctas_per_part = sms / mp.parts > 0 ? sms / mp.parts : 1;
    if ((int64_t)mp.ctas_per_part > mp.tiles) mp.ctas_per_part = (int)mp.tiles;
    mp.grid = mp.ctas_per_part * mp.parts;
    mp.smem = fixed + (size_t)mp.kp * per_centre;
}

// The plan changes only once everything it needs exists: the ones tile is
// allocated, filled and mapped first (a failure frees it and leaves the plan
// as it was, e.g. a synchronous copy refused while the stream is captured).
void plan_tc(Ctx &ctx, MixedPlan &mp, int64_t n, int d, int k, bool fp8, int topk, int kp_fixed) {
    if (!mp.ones) {
        uint16_t h[BM * 16];
        for (int r = 0; r < BM; r++)
            for (int j = 0; j < 16; j++) h[r * 16 + j] = j < 3 ? 0x3F80 : 0;  // BF16 1.0 = 0x3F80
        void *ones = nullptr;
        FK_CUDA(cudaMalloc(&ones, sizeof(h)));
        try {
            FK_CUDA(cudaMemcpy(ones, h, sizeof(h), cudaMemcpyHostToDevice));
            encode_2d(ctx, mp.tm_ones, ones, 16, BM, 32, 16, BM, CU_TENSOR_MAP_SWIZZLE_32B);
        } catch (...) {
            cudaFree(ones);
            throw;
        }
        mp.ones = ones;
    }
    plan_shape(mp, n, d, k, fp8, topk, ctx.num_sms, kp_fixed);
    mp.tm_x_ptr = mp.tm_c_ptr = mp.tm_aug_ptr = mp.tm_xaug_ptr = nullptr;
}

void launch_tc_assign(Ctx &ctx, MixedPlan &mp, const void *xb, const void *cb, const void *caug, SliceTop2 *out,
                      DevScalars *sc, const MixedStats *stats, float *dump,
                      const unsigned long long *n_dev, const void *xaug, const float *rowscale, uint32_t *masks,
                      const float *thresh, SliceCount *outc) {
    const bool fp8 = mp.fp8;
    if ((mp.topk == 2) != (out != nullptr) || (mp.topk == 1) != (masks != nullptr) || (mp.topk == 3) != (outc != nullptr) ||
        ((mp.topk == 1 || mp.topk == 3) != (thresh != nullptr)) || (mp.topk == 1 && fp8)) {
        set_error("tensor-core launch: records do not match the plan");
        fail(FK_ERR_INVALID_PARAMETER);
    }
    const CUtensorMapDataType dt = fp8 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
    const uint64_t es = fp8 ? 1 : 2;
    const uint32_t box_in = fp8 ? 128 : 64;
    if (mp.tm_x_ptr != xb) {
        encode_2d(ctx, mp.tm_x, xb, (uint64_t)mp.d_pad, (uint64_t)mp.n, (uint64_t)mp.d_pad * es, box_in, BM,
                  CU_TENSOR_MAP_SWIZZLE_128B, dt);
        mp.tm_x_ptr = xb;
    }
    if (mp.tm_c_ptr != cb) {
        encode_2d(ctx, mp.tm_c, cb, (uint64_t)mp.d_pad, (uint64_t)mp.k_pad, (uint64_t)mp.d_pad * es, box_in, BN,
                  CU_TENSOR_MAP_SWIZZLE_128B, dt);
        mp.tm_c_ptr = cb;
    }
    if (mp.tm_aug_ptr != caug) {
        encode_2d(ctx, mp.tm_aug, caug, 16, (uint64_t)mp.k_pad, 32, 16, BN, CU_TENSOR_MAP_SWIZZLE_32B);
        mp.tm_aug_ptr = caug;
    }
    unsigned char *tmo = mp.tm_ones;
    if (fp8) {
        tmo = mp.tm_xaug;
        if (mp.tm_xaug_ptr != xaug) {
            encode_2d(ctx, mp.tm_xaug, xaug, 16, (uint64_t)mp.n, 32, 16, BM, CU_TENSOR_MAP_SWIZZLE_32B);
            mp.tm_xaug_ptr = xaug;
        }
    }
    TcParams p;
    memset(&p, 0, sizeof(p));
    p.n = mp.n;
    p.tiles = mp.tiles;
    p.n_atoms = (int)((uint64_t)mp.d_pad * es / 128);
    p.kp = mp.kp;
    p.nblocks = mp.nblocks;
    p.parts = mp.parts;
    p.ctas_per_part = mp.ctas_per_part;
    p.c_atom_bytes = (uint32_t)mp.kp * 128u;
    p.x_stage_bytes = (uint32_t)p.n_atoms * X_ATOM_BYTES;
    p.off_c = 0;
    p.off_x = p.off_c + (uint32_t)p.n_atoms * p.c_atom_bytes;
    p.off_aug = p.off_x + (uint32_t)mp.xst * p.x_stage_bytes;
    p.off_ones = p.off_aug + (uint32_t)mp.kp * 32u;
    p.off_xaug = p.off_ones;
    p.off_merge = p.off_ones + (fp8 ? (uint32_t)mp.xst * XAUG_BYTES : ONES_BYTES);
    p.off_bar = p.off_merge + merge_bytes(mp.topk, mp.fp8, mp.ep, mp.slots);
    p.slots = mp.slots;
    p.c_tx_bytes = (uint32_t)p.n_atoms * p.c_atom_bytes + (uint32_t)mp.kp * 32u + (fp8 ? 0u : ONES_BYTES);
    p.out = out;
    p.n_dev = n_dev;
    p.out_stride = mp.n;
    p.err = &sc->error_word;
    p.stats = stats;
    p.rowscale = rowscale;
    p.dump = dump;
    p.masks = masks;
    p.thresh = thresh;
    p.outc = outc;
    p.wpr = mp.k_pad / 32;
    const size_t smem = (size_t)p.off_bar + BAR_BYTES + 1024;
    if (smem > SMEM_LIMIT) {
        set_error("tensor-core plan needs %zu bytes of shared memory", smem);
        fail(FK_ERR_UNSUPPORTED);
    }
    const CUtensorMap *tx = (const CUtensorMap *)mp.tm_x, *tcm = (const CUtensorMap *)mp.tm_c,
                      *ta = (const CUtensorMap *)mp.tm_aug, *to = (const CUtensorMap *)tmo;
    auto go = [&](auto kern) {
        FK_CUDA(cudaFuncSetAttribute((const void *)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kern<<<mp.grid, tc_threads(mp.ep), smem, ctx.stream>>>(*tx, *tcm, *ta, *to, p);
    };
    // Instantiations, each with one or two X stages: the top-2 and count
    // passes in BF16 and FP8, the mask pass in BF16.
    if (mp.topk == 1) {
        mp.xst == 2 ? go(tc_assign_kernel<1, false, 2, 2>) : go(tc_assign_kernel<1, false, 1, 2>);
    } else if (mp.topk == 3) {
        if (fp8)
            mp.xst == 2 ? go(tc_assign_kernel<3, true, 2, 2>) : go(tc_assign_kernel<3, true, 1, 2>);
        else if (mp.ep == 4)
            mp.xst == 2 ? go(tc_assign_kernel<3, false, 2, 4>) : go(tc_assign_kernel<3, false, 1, 4>);
        else
            mp.xst == 2 ? go(tc_assign_kernel<3, false, 2, 2>) : go(tc_assign_kernel<3, false, 1, 2>);
    } else if (mp.topk != 2) {
        set_error("tensor-core launch: unknown pass kind %d", mp.topk);
        fail(FK_ERR_INVALID_PARAMETER);
    } else if (fp8) {
        mp.xst == 2 ? go(tc_assign_kernel<2, true, 2, 2>) : go(tc_assign_kernel<2, true, 1, 2>);
    } else {
        mp.xst == 2 ? go(tc_assign_kernel<2, false, 2, 2>) : go(tc_assign_kernel<2, false, 1, 2>);
    }
    FK_LAUNCH_CHECK();
}


// Dense BF16 and E4M3 flop/s of tc_peak_kernel (best of three timed launches
// after one warm-up, CUDA events on the context's stream): out[0] BF16,
// out[1] E4M3.
void measure_tc_peaks(Ctx &ctx, double *out) {
    unsigned long long *err = (unsigned long long *)ctx.get(BUF_OUT2, 64);
    FK_CUDA(cudaMemsetAsync(err, 0, sizeof(unsigned long long), ctx.stream));
    const size_t smem = PEAK_A_BYTES + PEAK_B_BYTES + 1024 + 128;
    const int iters = 4096;
    for (int fp8 = 0; fp8 < 2; fp8++) {
        const void *fn = fp8 ? (const void *)tc_peak_kernel<true> : (const void *)tc_peak_kernel<false>;
        FK_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        auto launch = [&](int it) {
            if (fp8)
                tc_peak_kernel<true><<<ctx.num_sms, 128, smem, ctx.stream>>>(it, err);
            else
                tc_peak_kernel<false><<<ctx.num_sms, 128, smem, ctx.stream>>>(it, err);
            FK_LAUNCH_CHECK();
        };
        launch(64);
        double best = 0.0;
        for (int rep = 0; rep < 3; rep++) {
            Events<2> ev;
            FK_CUDA(cudaEventRecord(ev[0], ctx.stream));
            launch(iters);
            FK_CUDA(cudaEventRecord(ev[1], ctx.stream));
            FK_CUDA(cudaEventSynchronize(ev[1]));
            float ms = 0.f;
            FK_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
            const double flops = (double)ctx.num_sms * iters * 4.0 * 2.0 * BM * BN * (fp8 ? 32.0 : 16.0);
            best = std::max(best, flops / (ms * 1e-3));
        }
        out[fp8] = best;
    }
    unsigned long long h = 0;
    FK_CUDA(cudaMemcpyAsync(&h, err, sizeof(h), cudaMemcpyDeviceToHost, ctx.stream));
    FK_CUDA(cudaStreamSynchronize(ctx.stream));
    if (h) {
        set_error("the tensor-core peak loop's bounded wait gave up (code %llu)", h);
        fail(FK_ERR_TIMEOUT);
    }
}

}  // namespace fk
