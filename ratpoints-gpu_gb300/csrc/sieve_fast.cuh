// Fast-plan sieve kernels (this project's plan; see plan.hpp).
//
// Class-strided layout.  For a denominator d only some numerator classes
// a = r (mod M) can hold points, M = 64 * q with q the curve's class prime
// (q = 1: M = 64):
//   - r mod 64 must make F(r, d) a square mod 64 (and r odd when d is even);
//   - r mod q must make f(r/d) a square mod q, or, when q | d, be nonzero
//     (gcd) with c_n a square mod q for even degree.
// Each admissible class is swept on its own: word w of class r holds the 64
// sites a = a0 + S w + M j (j = bit, S = 64 M), a0 the least a >= -H in the
// class.  For an odd modulus m prime to M, S is invertible mod m, so the mask
// of m is periodic in w with period m and one table row per (m, d mod m)
// serves every class: class r starts at row index a0 * S^-1 (mod m).  Tables
// therefore do not depend on H.
//
// Stage 1 ANDs the rows of NS composite moduli of small primes (chosen per
// curve), staged in shared memory per denominator; surviving words go through
// a per-warp queue to stage 2, which checks the reference's 32 selected
// primes (same selection as the reference plan: the 32 largest of its 36
// candidates that do not divide d) from class-layout tables in global memory,
// then emits (a, d).  Survivors are a subset of the reference plan's.
//
// Warp-specialized pipeline: warp 0 produces denominators (prime selection,
// class layout from the per-curve class-start table, TMA copies of the rows)
// into one of two slots; the other warps consume a slot's sweep items once
// its full barrier completes and release it through its empty barrier, so a
// slot is refilled while the other is swept and no barrier spans the CTA.
#pragma once

#include "plan.hpp"
#include "sieve_device.cuh"

namespace rpg {
namespace dev {

constexpr int kFastSlots = kMaxFastSlots;  // stage-1 moduli (at most)
constexpr int kFastMaxFactors = 4;         // primes per stage-1 modulus
constexpr int kFK = 4;                     // words per lane per step (lanes 32 apart)
constexpr int kFWarps = 12;                // warp 0 produces, the others sweep
constexpr int kFThreads = kFWarps * kWarpSize;
constexpr int kFConsumers = kFWarps - 1;
constexpr int kFMaxSlotCount = 3;                          // denominators in flight per CTA: 2 or 3
constexpr int kFChunk = 16;                                // parameters per producer fetch (one per lane)
constexpr int kFSteps = 4;                                 // steps per work item
constexpr int kFItemWords = kWarpSize * kFK * kFSteps;     // 512 words per item
constexpr int kFExt = kWarpSize * (kFK - 1);               // row extension
constexpr int kFQueue = 64;
constexpr int kFStage2Group = 6;                           // stage-2 primes loaded together
constexpr long long kFMaxClassWords = 1LL << 23;           // class words of a launch's tile (24-bit field)
constexpr int kFAdmQ = 16;                                 // admissible-residue words for q <= 13
constexpr int kFBadBase = 64 + kFAdmQ;                     // first denominator-prime word of admissible


struct FastModulus {
    int m;                         // modulus (odd, prime to the class modulus)
    int nf;                        // number of prime factors
    int q[kFastMaxFactors];        // prime factors
    int length;                    // row length in words (m + kFExt, even)
    long long offset;              // word offset of row 0 in the table
    int smem_offset;               // word offset of the staged row in shared memory
    u32 inv_stride;                // (64 M)^-1 mod m
    u32 neg_h;                     // (-H) mod m
    u32 wlo_mod;                   // first word of the launch's tile, mod m
    u32 step;                      // (32 * kFK) mod m: row advance per step
    unsigned long long magic;      // ceil(2^64 / m) for 32-bit n mod m
    u32 step8;                     // 8 step: byte advance of a lane's offset per step
    u32 mod8;                      // 8 m
    u32 soff8;                     // 8 smem_offset: byte offset of the staged row in a slot
    u32 pad;
};

struct FastPrime {                 // one of the 36 reference candidates, class layout
    long long offset;              // word offset of row 0 (rows of length p)
    int p;
    u32 inv_stride;                // (64 M)^-1 mod p
    u32 neg_h;                     // (-H) mod p
    u32 magic;                     // magic40(p)
    u32 wlo_mod;                   // first word of the launch's tile, mod p
};

// Per class residue r mod M: the row index of class word 0 for each modulus,
// (a0 S^-1) mod m with a0 = -H + ofs, and ofs = (r + H) mod M.
struct FastClassStart {
    unsigned short start[kFastSlots];
    unsigned short ofs;
    unsigned short pad[3];
};
static_assert(sizeof(FastClassStart) == 32, "two 16-byte loads per class");
static_assert(kFExt == kFastRowExtension, "the planner sizes rows with the kernel's extension");

struct FastRun;

struct FastTables {
    const FastClassStart *class_starts;  // [M]
    int max_classes;               // most admissible classes of any denominator
    // Class lists by denominator class k = (d mod 64) q + (d mod q), for
    // launches over whole class rows (null otherwise): list_count[k] classes
    // and their runs list_runs[k max_classes ..], copied into a slot with its
    // rows.  A denominator's classes
    // depend on k alone, so the producer looks them up instead of laying them
    // out.  Every class of a whole row has list_ipc sweep items (its words
    // differ from another class's by at most one, and a class with fewer
    // words finds nothing to sweep in its last item), so item i of a list is
    // item i mod list_ipc of class i / list_ipc.
    const FastRun *list_runs;
    const int *list_count;
    int list_ipc;
    const u64 *rows;               // stage-1 modulus tables
    const u64 *prime_rows;         // reference candidate tables (class layout)
    const u64 *admissible;         // [64] 2-adic classes by d mod 64, then [kFAdmQ] residues by d mod q,
                                   // then nbad pairs (p, ceil(2^64 / p)): the denominator primes
    int nbad;                      // denominator primes: p < 512, p != q, c_n not a square mod p (even degree)
    int class_prime;               // q (1: none)
    int class_mod;                 // M = 64 q
    int h_mod_m;                   // H mod M
    int inv64_q;                   // 64^-1 mod q (CRT), 0 when q = 1
    long long stride;              // S = 64 M: numerator step between words of a class
    long long count_q;             // 2H = count_q * M + count_r: a class with offset
    int count_r;                   //   ofs <= count_r holds count_q + 1 sites, else count_q
    unsigned char crt[13 * 13];    // [r64 mod q][rq] -> t with r = r64 + 64 t (mod 64 q)
    unsigned char mod_q[64];       // r64 mod q
    FastModulus mod[kFastSlots];
    FastPrime prime[kCandidatePrimes];
    int slots;                     // stage-1 moduli in use
    int smem_words;                // staged row words
    int min_modulus;               // smallest stage-1 modulus
};

// Position of the n-th set bit (n counted from 0) of a 64-bit mask.
__device__ __forceinline__ int nth_set_bit(u64 mask, int n) {
    for (int i = 0; i < n; ++i) mask &= mask - 1;
    return __ffsll((long long)mask) - 1;
}

// One test of one site class for prime q: rho = d mod q, x = a mod q.
__device__ __forceinline__ bool prime_bit(const unsigned char *affine, const unsigned short *inverse,
                                          int q, int rho, int lead_ok, int x) {
    if (rho == 0) return x != 0 && lead_ok;  // q | d: need q !| a, and c_n square mod q (even n)
    return affine[(x * inverse[rho]) % q] != 0;
}

// Bit patterns of one prime q used by the class-layout tables: for each
// rho in [0, q), bit k of row rho is prime_bit(.., rho, (k step) mod q) for
// k in [0, q + 64), step = M mod q (k taken mod q), `words` words per row.
// Bit j of a table word whose first site has residue x0 is then bit
// (x0 step^-1 mod q) + j of the row: one 64-bit window instead of 64 tests.
struct ClassPatternSpec {
    long long out;                 // word offset of row 0
    int q;
    int words;                     // words per row: ceil((q + 64) / 64) + 1
    int factor_base;               // offset of q's affine/inverse arrays
    int lead_ok;
    int step;                      // M mod q
    int pad;
};

__global__ void pattern_rows_kernel(u64 *patterns, const ClassPatternSpec *specs, int nspecs,
                                    const unsigned char *affine, const unsigned short *inverse,
                                    long long total) {
    const long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (id >= total) return;
    int lo = 0, hi = nspecs - 1;  // last spec with out <= id
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (specs[mid].out <= id) lo = mid;
        else hi = mid - 1;
    }
    const ClassPatternSpec &P = specs[lo];
    const long long rel = id - P.out;
    const int rho = int(rel / P.words);
    const int wi = int(rel % P.words);
    const unsigned char *aff = affine + P.factor_base;
    const unsigned short *inv = inverse + P.factor_base;
    u64 word = 0;
    int k = (64 * wi) % P.q;
    for (int j = 0; j < 64; ++j) {
        const int x = int((long long)k * P.step % P.q);
        if (prime_bit(aff, inv, P.q, rho, P.lead_ok, x)) word |= u64(1) << j;
        if (++k == P.q) k = 0;
    }
    patterns[id] = word;
}

// Description of one class-layout table: m rows of `length` words, bit j of
// word u of row rho = AND over the prime factors q of
// prime_bit(.., rho mod q, (S u + M j) mod q), read from q's pattern rows.
struct TableSpec {
    long long offset;
    int m;
    int nf;
    int q[kFastMaxFactors];
    int length;
    long long pattern[kFastMaxFactors];  // word offset of q's pattern row 0
    int pattern_words[kFastMaxFactors];
    int s_mod[kFastMaxFactors];          // S mod q
    int step_inv[kFastMaxFactors];       // (M mod q)^-1 mod q
};

__global__ void class_table_kernel(u64 *rows, const TableSpec *specs, int nspecs, const u64 *patterns,
                                   long long total) {
    const long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (id >= total) return;
    int lo = 0, hi = nspecs - 1;  // last spec with offset <= id
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (specs[mid].offset <= id) lo = mid;
        else hi = mid - 1;
    }
    const TableSpec &S = specs[lo];
    const long long rel = id - S.offset;
    const int rho = int(rel / S.length);
    const int u = int(rel % S.length) % S.m;
    u64 word = ~u64(0);
    for (int f = 0; f < S.nf; ++f) {
        const int q = S.q[f];
        const int x0 = int((long long)S.s_mod[f] * u % q);
        const int k0 = int((long long)x0 * S.step_inv[f] % q);
        const u64 *row = patterns + S.pattern[f] + (long long)(rho % q) * S.pattern_words[f];
        const int w = k0 >> 6, sh = k0 & 63;
        const u64 lo_word = __ldg(row + w), hi_word = __ldg(row + w + 1);
        word &= sh ? (lo_word >> sh) | (hi_word << (64 - sh)) : lo_word;
    }
    rows[id] = word;
}

// One admissible class of the slot's denominator: its words inside the
// launch's tile, where its last word is (or -1), and that word's valid bits.
struct FastRun {
    u32 words_last;                // words in the tile (bits 0..23), last word in the tile (bit 24),
                                   // valid bits of the class's last word (bits 25..31, 1..64)
    unsigned short ofs;            // (r + H) mod M
    unsigned short start[kFastSlots];  // row index of the tile's first class word, per modulus
    unsigned short pad;
};
static_assert(sizeof(FastRun) == 32, "packed class run");

// A denominator in flight: written by the producer warp, read by the others.
// Its class runs and item prefix are its class list in global memory, or laid
// out by the producer in dynamic shared memory (launches over part of the
// class rows), sized by the plan's largest class count.
struct FastSlot {
    long long d;                   // denominator; -1: no more work
    const FastRun *runs;
    const int *prefix;             // sweep-item prefix of laid-out classes (null for class lists)
    int nclass;
    int items;                     // sweep items of the denominator
    int rot;                       // items handed out in this CTA before these, mod the consumer count
};

// A consumer warp's queued words carry one of kFCtx context indices; the
// context holds their denominator, so a slot can be refilled before those
// words go through stage 2.  Sixteen contexts per warp let its queue fill up
// across many denominators before it is drained.
constexpr int kFCtx = 16;
constexpr int kFTagShift = 56;             // context index in bits 56..59 of a queued position

// One group of stage 2: candidates ci0, ci0-1, .., ci0-COUNT+1 (descending),
// each tested on the words whose denominator it does not divide; ndiv counts
// the candidates that divide it.  The group's table words are loaded together.
template <int COUNT>
__device__ __forceinline__ void fast_stage2_group(const FastTables &T, int ci0, u32 hi, u32 lo, u32 d,
                                                  u64 &m, int &ndiv) {
    u64 rows[COUNT];
    bool skip[COUNT];
#pragma unroll
    for (int t = 0; t < COUNT; ++t) {
        const FastPrime &P = T.prime[ci0 - t];
        const u32 p = u32(P.p);
        const u32 rho = mod_small(d, p, P.magic);
        u32 r = mod_small(hi, p, P.magic);
        r = mod_small((r << 16) | lo, p, P.magic);  // pos mod p
        r += P.neg_h;                               // a mod p
        if (r >= p) r -= p;
        const u32 u = mod_small(r * P.inv_stride, p, P.magic);
        skip[t] = rho == 0;
        ndiv += skip[t] ? 1 : 0;
        rows[t] = __ldg(T.prime_rows + P.offset + (long long)rho * p + u);
    }
#pragma unroll
    for (int t = 0; t < COUNT; ++t) m &= skip[t] ? ~u64(0) : rows[t];
}

// Stage 2 for up to 32 queued words (one per lane), then emission.  A queued
// word carries its context (bits 56..59) and the position pos = a - (-H) of
// its bit 0 (bits 0..55): its sites are a = -H + pos + M j, and the
// class-layout row index of prime p is (a mod p) S^-1 mod p in row d mod p.
// A word meets the reference's selection, the 32 largest of the 36
// candidates that do not divide d: the 32 largest candidates (six at a time
// in a loop that is not unrolled, which keeps the kernel's code compact; the
// warp stops once its words are empty), skipping those dividing d, then, one
// at a time and only for words where some of those divided d, the four
// smallest until 32 have been tested.
__device__ __forceinline__ void fast_drain(const u64 *qmask, const u64 *qpos, int start, int n,
                                           const FastTables &T, const SieveArgs &A, const int *ctx_d) {
    const int lane = threadIdx.x & 31;
    u64 m = 0, pos = 0;
    if (lane < n) {
        m = qmask[start + lane];
        pos = qpos[start + lane];
    }
    __syncwarp();
    // lanes past n hold no word: any denominator keeps their row indices in range
    const u32 d = lane < n ? u32(ctx_d[int(pos >> kFTagShift) & (kFCtx - 1)]) : 1u;
    const u64 p56 = pos & ((u64(1) << kFTagShift) - 1);
    const u32 hi = u32(p56 >> 16), lo = u32(p56 & 0xFFFF);
    static_assert(kCandidatePrimes == 36 && kSelectedPrimes == 32, "stage-2 group schedule");
    int ndiv = 0;  // of the candidates tested so far, those dividing d
#pragma unroll 1
    for (int g = 0; g + kFStage2Group <= kSelectedPrimes; g += kFStage2Group) {
        if (!__any_sync(kFullMask, m != 0)) break;
        fast_stage2_group<kFStage2Group>(T, kCandidatePrimes - 1 - g, hi, lo, d, m, ndiv);
    }
    constexpr int kRest = kSelectedPrimes % kFStage2Group;
    if (kRest > 0 && __any_sync(kFullMask, m != 0))
        fast_stage2_group<kRest>(T, kCandidatePrimes - 1 - (kSelectedPrimes - kRest), hi, lo, d, m, ndiv);
    // candidates 3, 2, 1, 0 make up for the larger ones that divide d
#pragma unroll
    for (int ci = 3; ci >= 0; --ci) {
        if (!__any_sync(kFullMask, m != 0 && ndiv > 0)) break;
        const FastPrime &P = T.prime[ci];
        const u32 p = u32(P.p);
        const u32 rho = mod_small(d, p, P.magic);
        if (m != 0 && ndiv > 0 && rho != 0) {
            u32 r = mod_small(hi, p, P.magic);
            r = mod_small((r << 16) | lo, p, P.magic);
            r += P.neg_h;
            if (r >= p) r -= p;
            const u32 u = mod_small(r * P.inv_stride, p, P.magic);
            m &= __ldg(T.prime_rows + P.offset + (long long)rho * p + u);
            --ndiv;  // one of the 32 taken by a smaller candidate
        }
    }
    // emission: a = -H + pos + M j
    u32 cnt = __popcll(m);
    if (!__any_sync(kFullMask, cnt != 0)) return;
    u32 incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        u32 v = __shfl_up_sync(kFullMask, incl, o);
        if (lane >= o) incl += v;
    }
    const u32 total = __shfl_sync(kFullMask, incl, 31);
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(A.out_count, (unsigned long long)total);
    base = __shfl_sync(kFullMask, base, 0);
    unsigned long long at = base + incl - cnt;
    const long long abase = -A.bound + (long long)p56;
    while (m) {
        const int bit = __ffsll((long long)m) - 1;
        m &= m - 1;
        if (at < A.capacity) {
            A.out_a[at] = abase + (long long)T.class_mod * bit;
            A.out_d[at] = int(d);
        }
        ++at;
    }
}

// Producer work for denominator d into slot S (the whole warp): the
// admissible classes and their sweep items (a prefix scan, 32 classes per
// pass) in shared memory.  Returns the item count.
__device__ __forceinline__ int fast_setup(const FastTables &T, const SieveArgs &A, long long d,
                                           FastSlot &S, FastRun *runs, int *prefix) {
    const int lane = threadIdx.x & 31;
    const u32 du = u32(d);
    const int q = T.class_prime;
    const int M = T.class_mod;
    const u64 classes2 = __ldg(T.admissible + (du & 63));
    const u64 classesq =
        q > 1 ? __ldg(T.admissible + 64 + int(mod_u32(du, u32(q), (~0ull) / u32(q) + 1))) : u64(1);
    const int nq = __popcll(classesq);
    const int nclass = __popcll(classes2) * nq;
    int carry = 0;
    for (int base = 0; base < nclass; base += 32) {
        const int c = base + lane;
        int items = 0;
        if (c < nclass) {
            const int i2 = nq == 1 ? c : c / nq;
            const int r64 = nth_bit64(classes2, i2);
            int r = r64;
            if (q > 1) {
                const int rq = nth_bit64(classesq, c - i2 * nq);
                r = r64 + 64 * int(T.crt[T.mod_q[r64] * 13 + rq]);
            }
            const FastClassStart cs = T.class_starts[r];
            const int ofs = cs.ofs;
            // sites of class r: a = -H + ofs + M t, t in [0, count)
            const long long count = T.count_q + (ofs <= T.count_r ? 1 : 0);
            const long long words = (count + 63) >> 6;
            const long long lo = A.w_lo < words ? A.w_lo : words;
            const long long hi = A.w_hi < words ? A.w_hi : words;
            FastRun run;
            const u32 tile_words = u32(hi - lo);
            const bool has_last = hi == words && words > 0 && hi > lo;
            const u32 last_bits = has_last ? u32(count - 64 * (words - 1)) : 64u;
            run.words_last = tile_words | (has_last ? 1u << 24 : 0u) | ((last_bits - 1) << 25);
            run.ofs = (unsigned short)ofs;
#pragma unroll
            for (int sl = 0; sl < kFastSlots; ++sl) {
                // tile word 0 is class word w_lo: (a0 S^-1 + w_lo) mod m
                const FastModulus &Md = T.mod[sl];
                u32 st = u32(cs.start[sl]) + Md.wlo_mod;  // both below m
                if (st >= u32(Md.m)) st -= u32(Md.m);
                run.start[sl] = (unsigned short)st;
            }
            runs[c] = run;
            items = int((tile_words + kFItemWords - 1) / kFItemWords);
        }
        int incl = items;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(kFullMask, incl, o);
            if (lane >= o) incl += v;
        }
        if (c < nclass) prefix[c] = carry + incl - items;
        carry += __shfl_sync(kFullMask, incl, 31);
    }
    if (lane == 0) {
        prefix[nclass] = carry;
        S.runs = runs;
        S.prefix = prefix;
        S.nclass = nclass;
        S.items = carry;
        S.d = d;
    }
    return carry;
    (void)M;
}

// Four 64-bit shared words of one staged row, 256 bytes apart (a lane's kFK
// words, 32 apart), as 32-bit halves: one address register, immediate offsets.
__device__ __forceinline__ void lds_row4(u32 a, u32 (&lo)[kFK], u32 (&hi)[kFK]) {
    static_assert(kFK == 4, "four words per lane per step");
    asm volatile(
        "ld.shared.v2.u32 {%0, %1}, [%8];\n\t"
        "ld.shared.v2.u32 {%2, %3}, [%8+256];\n\t"
        "ld.shared.v2.u32 {%4, %5}, [%8+512];\n\t"
        "ld.shared.v2.u32 {%6, %7}, [%8+768];"
        : "=r"(lo[0]), "=r"(hi[0]), "=r"(lo[1]), "=r"(hi[1]), "=r"(lo[2]), "=r"(hi[2]), "=r"(lo[3]),
          "=r"(hi[3])
        : "r"(a));
}

template <int NS, int SLOTS>
__global__ void __launch_bounds__(kFThreads, 2) fast_sieve_kernel(FastTables T, SieveArgs A,
                                                               unsigned long long *work) {
    extern __shared__ __align__(16) u64 smem[];
    const int row_stride = T.smem_words;  // even: buffers stay 16-byte aligned
    u64 *qmask = smem + SLOTS * row_stride;
    u64 *qpos = qmask + kFConsumers * kFQueue;
    FastRun *runs0 = reinterpret_cast<FastRun *>(qpos + kFConsumers * kFQueue);  // [slots][max_classes]
    int *prefix0 = reinterpret_cast<int *>(runs0 + SLOTS * T.max_classes);  // [slots][max_classes + 1]

    __shared__ FastSlot slot[SLOTS];
    __shared__ int s_ctx[kFConsumers][kFCtx];  // denominators of each warp's contexts
    __shared__ __align__(8) unsigned long long s_full[SLOTS];
    __shared__ __align__(8) unsigned long long s_empty[SLOTS];

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        for (int b = 0; b < SLOTS; ++b) {
            mbar_init(smem_addr(&s_full[b]), 1);
            mbar_init(smem_addr(&s_empty[b]), kFConsumers);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    if (warp == 0) {
        // ---- producer: next live denominator into the next free slot ----
        // Parameters come kFChunk at a time from the launch's work counter, the
        // next chunk's fetch issued before this chunk is handed out so that its
        // latency is hidden; lane j classifies parameter j of a chunk (class
        // list length by d mod 64 and d mod q), and the live ones go to the
        // slots in order.  The row copies of a slot are issued by lanes
        // 0 .. NS-1, one row each.
        const int q = T.class_prime;
        const unsigned long long magic_q = (~0ull) / u32(q) + 1;  // q >= 1: mod_u32 constant
        const bool lists = T.list_count != nullptr;
        int uses[SLOTS] = {};      // fills of each slot so far
        int b = 0;
        bool failed = false;
        int rot = 0;               // sweep items handed out so far, mod kFConsumers
        unsigned long long next_chunk = 0;
        if (lane == 0) next_chunk = atomicAdd(work, (unsigned long long)kFChunk);
        // waits until slot b is released by every consumer (false: gave up)
        auto acquire_slot = [&]() -> bool {
            int used = 0;
#pragma unroll
            for (int t = 0; t < SLOTS; ++t) used = t == b ? uses[t] : used;
            return used == 0 || mbar_wait(smem_addr(&s_empty[b]), u32(used - 1) & 1u);
        };
        for (;;) {
            const long long chunk = (long long)__shfl_sync(kFullMask, next_chunk, 0);
            if (chunk >= A.k_count) break;
            if (lane == 0) next_chunk = atomicAdd(work, (unsigned long long)kFChunk);
            static_assert(2 * kFChunk == kWarpSize, "lanes 16..31 mirror the chunk's parameters");
            const long long idx = chunk + (lane & (kFChunk - 1));
            const bool in_range = idx < A.k_count;
            const bool valid = lane < kFChunk && in_range;
            const long long k = A.k_first + (in_range ? idx : 0);
            const long long dd = A.square ? k * k : k;
            const u32 du = u32(dd);
            const int combo = int(du & 63) * q + (q > 1 ? int(mod_u32(du, u32(q), magic_q)) : 0);
            int list_n = 0;
            if (valid) {
                if (lists) {
                    list_n = __ldg(T.list_count + combo);
                } else {
                    const bool adm = __ldg(T.admissible + (du & 63)) != 0 &&
                                     (q == 1 || __ldg(T.admissible + 64 + int(mod_u32(du, u32(q), magic_q))) != 0);
                    list_n = adm ? 1 : 0;
                }
            }
            if (T.nbad > 0) {
                // Denominator primes: for p | d and p !| a, F(a, d) = c_n a^n
                // (mod p), which is not a square when c_n is not and n is
                // even, so d holds no points.  p | k^2 iff p | k; the two
                // half-warps test a parameter against alternate primes.
                const u32 ku = u32(k);
                int hit = 0;
                for (int i = lane >> 4; i < T.nbad; i += 2) {
                    const u32 p = u32(__ldg(T.admissible + kFBadBase + 2 * i));
                    const unsigned long long mg = __ldg(T.admissible + kFBadBase + 2 * i + 1);
                    hit |= mod_u32(ku, p, mg) == 0 ? 1 : 0;
                }
                hit |= __shfl_xor_sync(kFullMask, hit, kFChunk);
                if (hit) list_n = 0;
            }
            u32 live = __ballot_sync(kFullMask, list_n > 0);
            while (live) {
                const int j = __ffs(live) - 1;
                live &= live - 1;
                const long long d = __shfl_sync(kFullMask, dd, j);
                const int combo_j = __shfl_sync(kFullMask, combo, j);
                const int n_j = __shfl_sync(kFullMask, list_n, j);
                if (!acquire_slot()) {
                    failed = true;
                    break;
                }
                FastSlot &S = slot[b];
                const u32 full = smem_addr(&s_full[b]);
                int items;
                if (lists) {
                    items = n_j * T.list_ipc;
                    if (lane == 0) {
                        S.runs = runs0 + b * T.max_classes;
                        S.prefix = nullptr;
                        S.nclass = n_j;
                        S.items = items;
                        S.d = d;
                    }
                } else {
                    items = fast_setup(T, A, d, S, runs0 + b * T.max_classes, prefix0 + b * (T.max_classes + 1));
                }
                if (lane == 0) S.rot = rot;
                rot = int((rot + (unsigned)items) % unsigned(kFConsumers));
                __syncwarp();
                const u32 run_bytes = lists ? u32(n_j) * u32(sizeof(FastRun)) : 0u;
                if (lane == 0) {
                    __threadfence_block();
                    mbar_arrive_expect_tx(full, u32(T.smem_words) * 8u + run_bytes);
                }
                __syncwarp();
                if (lane < NS) {
                    // the consumers' reads of this slot's previous rows are
                    // ordered before the asynchronous copies that overwrite them
                    fence_proxy_async_shared();
                    const FastModulus &Md = T.mod[lane];
                    const u32 rho = mod_u32(u32(d), u32(Md.m), Md.magic);
                    bulk_copy_to_shared(smem_addr(smem + b * row_stride) + u32(Md.smem_offset) * 8u,
                                        T.rows + Md.offset + (long long)rho * Md.length,
                                        u32(Md.length) * 8u, full);
                }
                if (lists && lane == 31) {
                    // the class list's runs go next to the slot with the rows, so
                    // the consumers read them from shared memory
                    fence_proxy_async_shared();
                    bulk_copy_to_shared(smem_addr(runs0 + b * T.max_classes),
                                        T.list_runs + (long long)combo_j * T.max_classes, run_bytes, full);
                }
#pragma unroll
                for (int t = 0; t < SLOTS; ++t) uses[t] += t == b ? 1 : 0;
                b = b + 1 == SLOTS ? 0 : b + 1;
            }
            if (failed) break;
        }
        if (!failed) {
            // no more work: an empty slot fill tells the consumers to finish
            if (acquire_slot()) {
                if (lane == 0) {
                    slot[b].d = -1;
                    __threadfence_block();
                    mbar_arrive(smem_addr(&s_full[b]));
                }
            } else {
                failed = true;
            }
        }
        if (failed) {
            if (A.error && lane == 0) atomicOr(A.error, 1ull);
            // let the copies already issued land (bounded) before leaving
#pragma unroll
            for (int t = 0; t < SLOTS; ++t)
                if (lane == 0 && uses[t] > 0) mbar_wait(smem_addr(&s_full[t]), u32(uses[t] - 1) & 1u);
        }
        return;
    }

    // ---- consumers: sweep the items of each filled slot in turn ----
    // Items are dealt round-robin over the consumer warps, continuing across
    // denominators (the slot's rot): consumer cw sweeps items i of a fill with
    // (i + rot) mod kFConsumers = cw.  No counter is shared, and a warp with
    // no item in a fill only releases the slot.
    const int cw = warp - 1;
    u64 *wq_mask = qmask + cw * kFQueue;
    u64 *wq_pos = qpos + cw * kFQueue;
    int *ctx = s_ctx[cw];
    u32 phase = 0;   // bit b: parity of slot b's next fill
    int b = 0;
    int qn = 0;      // queued words (kept across denominators)
    int seq = 0;     // slot fills this warp has taken items from
    int oldest = 0;  // oldest context that may still have queued words
    auto drain_all = [&]() {
        while (qn > 0) {
            const int n = qn < 32 ? qn : 32;
            __syncwarp();
            fast_drain(wq_mask, wq_pos, qn - n, n, T, A, ctx);
            qn -= n;
        }
    };
    for (;;) {
        if (!mbar_wait(smem_addr(&s_full[b]), (phase >> b) & 1u)) {  // bounded wait
            if (A.error && lane == 0) atomicOr(A.error, 1ull);
            return;
        }
        phase ^= 1u << b;
        const FastSlot &S = slot[b];
        if (S.d < 0) {  // the producer has no more work
            drain_all();
            return;
        }
        const int total_items = S.items;
        int item = cw - S.rot;
        if (item < 0) item += kFConsumers;
        if (item < total_items) {
            // context k replaces the one taken kFCtx fills ago: its queued words go first
            const int k = seq & (kFCtx - 1);
            if (qn > 0 && seq - oldest >= kFCtx) drain_all();
            if (qn == 0) oldest = seq;
            __syncwarp();
            if (lane == 0) ctx[k] = int(S.d);
            __syncwarp();
            const u64 tag = u64(k) << kFTagShift;

            const unsigned char *sbase = reinterpret_cast<const unsigned char *>(smem + b * row_stride);
            const FastRun *runs = S.runs;
            const int *prefix = S.prefix;  // null: a class list, list_ipc items per class
            const int nclass = S.nclass;
            // laid-out classes, up to 31 of them: lane c keeps prefix[c], so
            // finding an item's class takes no memory access
            const bool lane_prefix = prefix != nullptr && nclass < kWarpSize;
            const int my_prefix = lane_prefix && lane <= nclass ? prefix[lane] : 0;
            const u32 slot_addr = smem_addr(sbase);
            int c = 0;  // this warp's items of a slot only increase: so do their classes
            for (; item < total_items; item += kFConsumers) {
                // class index: item / list_ipc for a class list; otherwise the
                // largest c with prefix[c] <= item (32 classes per probe, from
                // the last one on)
                int first_item;
                if (prefix == nullptr) {
                    const int ipc = T.list_ipc;
                    c = ipc == 1 ? item : item / ipc;
                    first_item = c * ipc;
                } else if (lane_prefix) {
                    const u32 bb = __ballot_sync(kFullMask, lane < nclass && my_prefix <= item);
                    c = 31 - __clz(bb);
                    first_item = __shfl_sync(kFullMask, my_prefix, c);
                } else {
                    for (int base = c; base < nclass; base += 32) {
                        const int cc = base + lane;
                        const u32 bb = __ballot_sync(kFullMask, cc < nclass && prefix[cc] <= item);
                        if (bb) c = base + 31 - __clz(bb);
                        if (bb != kFullMask) break;
                    }
                    first_item = prefix[c];
                }
                const int w0 = (item - first_item) * kFItemWords;
                const FastRun run = runs[c];
                const int wt = int(run.words_last & 0xFFFFFFu);
                const int last_word = (run.words_last >> 24) & 1u ? wt - 1 : -1;
                const u32 last_bits = (run.words_last >> 25) + 1;
                const u64 last_mask = last_bits >= 64 ? ~u64(0) : ((u64(1) << last_bits) - 1);
                // pos of word w of this class: ofs + S (w_lo + w)
                const u64 pos0 = u64(run.ofs) + u64(T.stride) * u64(A.w_lo);
                u32 o[NS];  // byte offset of this lane's word inside each staged row
                if (w0 == 0 && T.min_modulus >= kWarpSize) {
                    // a class's first item: start < m and lane < 32 <= m, one subtraction
#pragma unroll
                    for (int sl = 0; sl < NS; ++sl) {
                        const u32 v = 8u * (u32(run.start[sl]) + u32(lane));
                        o[sl] = min(v, v - T.mod[sl].mod8);
                    }
                } else {
#pragma unroll
                    for (int sl = 0; sl < NS; ++sl)
                        o[sl] = 8u * mod_u32(u32(run.start[sl]) + u32(w0 + lane), u32(T.mod[sl].m), T.mod[sl].magic);
                }
#pragma unroll 1
                for (int step = 0; step < kFSteps; ++step) {
                    const int ws = w0 + step * kWarpSize * kFK;
                    if (ws >= wt) break;
                    // stage 1: this lane's kFK words (32 apart) of each staged
                    // row, ANDed three at a time
                    u32 lo[kFK], hi[kFK];
                    lds_row4(slot_addr + T.mod[0].soff8 + o[0], lo, hi);
#pragma unroll
                    for (int sl = 1; sl + 1 < NS; sl += 2) {
                        u32 xl[kFK], xh[kFK], yl[kFK], yh[kFK];
                        lds_row4(slot_addr + T.mod[sl].soff8 + o[sl], xl, xh);
                        lds_row4(slot_addr + T.mod[sl + 1].soff8 + o[sl + 1], yl, yh);
#pragma unroll
                        for (int kk = 0; kk < kFK; ++kk) {
                            lo[kk] = and3(lo[kk], xl[kk], yl[kk]);
                            hi[kk] = and3(hi[kk], xh[kk], yh[kk]);
                        }
                    }
                    if (NS % 2 == 0) {
                        u32 xl[kFK], xh[kFK];
                        lds_row4(slot_addr + T.mod[NS - 1].soff8 + o[NS - 1], xl, xh);
#pragma unroll
                        for (int kk = 0; kk < kFK; ++kk) {
                            lo[kk] &= xl[kk];
                            hi[kk] &= xh[kk];
                        }
                    }
#pragma unroll
                    for (int sl = 0; sl < NS; ++sl) {
                        // advance (32 kFK) mod m words; unsigned min wraps into [0, m)
                        const u32 t = o[sl] + T.mod[sl].step8;
                        o[sl] = min(t, t - T.mod[sl].mod8);
                    }
                    const u32 any = or3(or3(lo[0], hi[0], lo[1]), or3(hi[1], lo[2], hi[2]), lo[3] | hi[3]);
                    if (!__ballot_sync(kFullMask, any != 0)) continue;
                    u64 acc[kFK];
#pragma unroll
                    for (int kk = 0; kk < kFK; ++kk) acc[kk] = (u64(hi[kk]) << 32) | lo[kk];
                    if (ws + kWarpSize * kFK >= wt) {
                        // the step reaches the class's last word in the tile:
                        // that word keeps its valid bits, words past it none
#pragma unroll
                        for (int kk = 0; kk < kFK; ++kk) {
                            const int w = ws + kWarpSize * kk + lane;
                            if (w == last_word) acc[kk] &= last_mask;
                            if (w >= wt) acc[kk] = 0;
                        }
                    }
#pragma unroll
                    for (int kk = 0; kk < kFK; ++kk) {
                        const bool live = acc[kk] != 0;
                        const u32 bb = __ballot_sync(kFullMask, live);
                        if (bb) {
                            const int at = qn + __popc(bb & lanemask_lt());
                            if (live) {
                                const int w = ws + kWarpSize * kk + lane;
                                wq_mask[at] = acc[kk];
                                wq_pos[at] = tag | (pos0 + u64(T.stride) * u64(w));
                            }
                            qn += __popc(bb);
                            if (qn >= 32) {
                                __syncwarp();
                                fast_drain(wq_mask, wq_pos, qn - 32, 32, T, A, ctx);
                                qn -= 32;
                                if (qn == 0) oldest = seq;
                            }
                        }
                    }
                }
            }
            ++seq;
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_addr(&s_empty[b]));  // this warp is done with slot b
        b = b + 1 == SLOTS ? 0 : b + 1;
    }
}

}  // namespace dev
}  // namespace rpg
