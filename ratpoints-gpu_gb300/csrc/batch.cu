// Batched many-curve sieve (batch.hpp): device kernels and host driver.
#include "batch.hpp"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <thread>

#include "exact.hpp"
#include "plan.hpp"
#include "preverify.hpp"
#include "sieve.hpp"
#include "sieve_device.cuh"
#include "tune.hpp"

namespace rpg {
namespace dev {

constexpr int kWideSlots = 6;                      // stage-1 moduli of a wide curve (padded)
constexpr int kWK = 4;                             // words per lane per step (lanes 32 apart)
constexpr int kWWarps = 12;                        // warp 0 produces, the others sweep
constexpr int kWThreads = kWWarps * kWarpSize;
constexpr int kWConsumers = kWWarps - 1;
constexpr int kWSlotCount = 2;                     // denominators in flight per CTA
constexpr int kWSteps = 4;
constexpr int kWItemWords = kWarpSize * kWK * kWSteps;  // class words per sweep item
constexpr int kWExt = kWarpSize * (kWK - 1);            // row extension
constexpr int kWMaxSmemWords = 6000;                    // staged row words per slot (two
                                                        // slots, 2 CTAs per SM)
constexpr int kQueue = 64;
constexpr long long kMaxClassWords = 1LL << 23;         // class words of a row (sweep-item arithmetic)
constexpr int kAdmQ = 16;                               // residue words for class primes <= 13
constexpr int kNarrowSlots = 8;
constexpr int kNK = 4;                                  // consecutive row words per lane
constexpr int kND = 4;                                  // consecutive parameters per warp fetch
constexpr int kNWarps = 8;
constexpr int kNThreads = kNWarps * kWarpSize;
constexpr int kNarrowTableWords = 7680;                 // sum of m (m + kNK - 1) per curve
constexpr int kAffWords = kCandidatePrimes * 8;         // the 36 candidate bitmasks
constexpr int kRefWords = 8;                            // u64 words of a bitmask over [0, 512)
constexpr int kMaxFactors = 4;
constexpr int kMaxIntervals = 8;                        // more: sweep the whole row


// The odd primes below 512 with ceil(2^64 / p) (mod_u32): a curve's
// denominator primes are a bit mask over this table.
constexpr int kOddPrimes = 96;
struct OddPrime {
    u32 p;
    u32 pad;
    unsigned long long magic;
};

struct Modulus {                   // one stage-1 modulus of a wide curve (class layout)
    long long offset;              // word offset of row 0 in the table pool
    unsigned long long magic;      // mod_u32 constant (all ones for m = 1)
    int m;
    int length;                    // row length in words (m + kWExt, even)
    int smem_offset;               // word offset of the staged row
    u32 inv_stride;                // S^-1 mod m
    u32 neg_h;                     // (-H) mod m
    u32 step;                      // (32 kWK) mod m
};

struct WideCurve {
    long long bound;               // H
    long long stride;              // S = 64 M: numerator step between words of a class
    long long count_q;             // 2H = count_q M + count_r
    long long aff;                 // u64 offset of the 36 candidate bitmasks
    long long cls;                 // index of the curve's ClassStart[M] block
    // class lists by denominator class k = (d mod 64) q + (d mod q): counts at
    // list_count + k, runs at list_runs + k list_max, item prefixes at
    // list_prefix + k (list_max + 1); list_count = -1 for curves with x
    // intervals (their classes are clipped per denominator)
    long long list_count, list_runs, list_prefix;
    Modulus mod[kWideSlots];
    u64 admissible[64 + kAdmQ];    // 2-adic classes by d mod 64, residues mod q by d mod q
    int count_r;
    int class_prime;               // q (1: 2-adic classes only)
    int class_mod;                 // M = 64 q
    int h_mod_m;                   // H mod M
    int inv64_q;                   // 64^-1 mod q (CRT)
    int smem_words;
    int list_max;                  // class-list stride: most classes of one denominator
    int list_steps;                // classes of at most 128 words: 32-word steps per class
                                   // (their items are kWK classes swept side by side); else 0
    int square;
    int index;                     // position in the caller's curve list
    int rows;                      // stage-1 moduli in use (the others are padding)
    int pad0;
    u64 denom_primes[2];           // bit i: odd prime i of the OddPrime table is a denominator prime
    unsigned short neg_h[kCandidatePrimes];   // (-H) mod p
    unsigned short s_mod[kCandidatePrimes];   // S mod p
    unsigned short m_mod[kCandidatePrimes];   // M mod p
    unsigned char crt[13 * 13];    // [r64 mod q][rq] -> t with r = r64 + 64 t (mod 64 q)
    unsigned char mod_q[64];       // r64 mod q
    int nint;                      // x intervals (0: the whole row)
    double lo[kMaxIntervals];      // ascending lower bounds (-inf: none)
    double hi[kMaxIntervals];      // upper bounds (+inf: none)
};

struct NarrowCurve {
    long long bound;
    long long words;               // W: dense 64-site words per denominator row
    long long tables;              // word offset of the curve's table block (even)
    long long aff;
    unsigned long long magic[kNarrowSlots];
    u64 dense2[64];                // by d mod 64: bit j set iff a = -H + j (mod 64) may hold points
    int table_words;               // even
    int square;
    int index;
    int rows;                      // stage-1 moduli in use (the others are padding)
    u64 denom_primes[2];           // bit i: odd prime i of the OddPrime table is a denominator prime
    int m[kNarrowSlots];           // moduli (1: padding)
    int off[kNarrowSlots];         // word offset of each table inside the block
    int len[kNarrowSlots];         // row length m + kNK - 1 (rows repeat their first words)
    u32 shift[kNarrowSlots];       // (-H) 64^-1 mod m: table word of row word 0
    u32 step[kNarrowSlots];        // (32 kNK) mod m
    unsigned short neg_h[kCandidatePrimes];
    int nint;
    double lo[kMaxIntervals];
    double hi[kMaxIntervals];
};

static_assert(sizeof(WideCurve) % 4 == 0 && sizeof(NarrowCurve) % 4 == 0, "u32 copies");

struct BatchItem {
    long long first;               // first parameter k
    int curve;                     // descriptor index
    int count;                     // parameters in this item
    int range;                     // which numerator range of each denominator (see x_ranges)
    int pad;
};

// Numerator ranges of denominator d for x in the curve's intervals: each
// interval [lo, hi] gives a in [floor(lo d) - 1, ceil(hi d) + 1] (widened by
// one so that double rounding never drops a site; the host applies the exact
// interval test), clipped to [-H, H]; overlapping ranges are merged.  Sets
// [L, U] to the want-th of the disjoint ascending ranges and returns false if
// there are not that many.  Without intervals the one range is [-H, H].
__device__ __forceinline__ bool x_range(const double *lo, const double *hi, int nint, long long H,
                                        long long d, int want, long long &L, long long &U) {
    if (nint == 0) {
        L = -H;
        U = H;
        return want == 0;
    }
    const double dd = double(d), h = double(H);
    int n = -1;
    long long cl = 0, cu = -1;
    for (int i = 0; i < nint; ++i) {
        const double x = floor(lo[i] * dd) - 1.0;
        const double y = ceil(hi[i] * dd) + 1.0;
        const long long l = !(x > -h) ? -H : (x > h ? H + 1 : (long long)x);
        const long long u = !(y < h) ? H : (y < -h ? -H - 1 : (long long)y);
        if (l > u) continue;
        if (n >= 0 && l <= cu + 1) {
            if (u > cu) cu = u;
            continue;
        }
        if (n == want) break;
        ++n;
        cl = l;
        cu = u;
    }
    if (n != want) return false;
    L = cl;
    U = cu;
    return true;
}

struct AffineSpec {                // bitmask of x in [0, p) with f(x) a square mod p
    long long out;                 // u64 offset of the 8-word output
    long long residues;            // offset of c_0 .. c_n mod p
    int p, n;
};

struct PatternSpec {               // q x q words: bit j of word (rho, u) tests x = (s u + t j) mod q
    long long offset;
    long long aff;
    int q, lead_ok, s, t;
};

struct CompositeSpec {             // m rows of `length` words: AND of the factor patterns
    long long offset;
    long long pattern[kMaxFactors];
    int m, length, nf;
    int q[kMaxFactors];
};

struct BatchOut {
    long long *a;
    int *d;
    int *curve;
    unsigned long long *count;
    unsigned long long capacity;
    unsigned long long *error;
};

struct Candidates {
    int p[kCandidatePrimes];
    u32 magic[kCandidatePrimes];
};

// ---------------------------------------------------------------------------
// Table construction

__global__ void affine_kernel(const AffineSpec *specs, long long nspecs,
                              const unsigned short *residues, const u64 *square_masks, u64 *out) {
    const long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (id >= nspecs * kRefWords) return;
    const AffineSpec S = specs[id / kRefWords];
    const int k = int(id % kRefWords);
    const int p = S.p;
    const unsigned short *c = residues + S.residues;
    const u64 *sq = square_masks + (long long)p * kRefWords;
    u64 word = 0;
    for (int b = 0; b < 64; ++b) {
        const int x = 64 * k + b;
        if (x >= p) break;
        int v = c[S.n];
        for (int i = S.n - 1; i >= 0; --i) v = (v * x + c[i]) % p;
        if ((sq[v >> 6] >> (v & 63)) & 1) word |= u64(1) << b;
    }
    out[S.out + k] = word;
}

// Index of the last spec whose offset is <= id (specs sorted by offset).
template <typename Spec>
__device__ __forceinline__ int find_spec(const Spec *specs, int nspecs, long long id) {
    int lo = 0, hi = nspecs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (specs[mid].offset <= id) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

constexpr int kPatternWords = 4;  // words per thread (see composite_kernel)

__global__ void pattern_kernel(const PatternSpec *specs, int nspecs, const u64 *affine,
                               const unsigned short *inv_table, u64 *patterns, long long total) {
    const long long base = (long long)blockIdx.x * blockDim.x * kPatternWords + threadIdx.x;
    if (base >= total) return;
    int s = find_spec(specs, nspecs, base);
    for (int i = 0; i < kPatternWords; ++i) {
        const long long id = base + (long long)i * blockDim.x;
        if (id >= total) break;
        while (s + 1 < nspecs && specs[s + 1].offset <= id) ++s;
        const PatternSpec S = specs[s];
        const int q = S.q;
        const int rel = int(id - S.offset);
        const int rho = rel / q;
        const int u = rel % q;
        const u64 *aff = affine + S.aff;
        const int inv = rho ? inv_table[q * kMaximumPrime + rho] : 0;
        int x = (S.s * u) % q;
        u64 word = 0;
        for (int j = 0; j < 64; ++j) {
            bool ok;
            if (rho == 0) {
                ok = x != 0 && S.lead_ok;  // q | d: q !| a, and c_n a square mod q for even degree
            } else {
                const int y = (x * inv) % q;
                ok = (__ldg(aff + (y >> 6)) >> (y & 63)) & 1;
            }
            if (ok) word |= u64(1) << j;
            x += S.t;
            if (x >= q) x -= q;
        }
        patterns[id] = word;
    }
}

// kCompositeWords words per thread, a block's threads interleaved (stores
// stay coalesced): one binary search over the specs per thread, then the
// spec index only moves forward.
constexpr int kCompositeWords = 16;

__global__ void composite_kernel(const CompositeSpec *specs, int nspecs, const u64 *patterns,
                                 u64 *rows, long long total) {
    const long long base = (long long)blockIdx.x * blockDim.x * kCompositeWords + threadIdx.x;
    if (base >= total) return;
    int s = find_spec(specs, nspecs, base);
    for (int i = 0; i < kCompositeWords; ++i) {
        const long long id = base + (long long)i * blockDim.x;
        if (id >= total) break;
        while (s + 1 < nspecs && specs[s + 1].offset <= id) ++s;
        const CompositeSpec &S = specs[s];
        const long long rel = id - S.offset;
        const int rho = int(rel / S.length);
        const int u = int(rel % S.length) % S.m;
        u64 word = ~u64(0);
        for (int f = 0; f < S.nf; ++f) {
            const int q = S.q[f];
            word &= __ldg(patterns + S.pattern[f] + (rho % q) * q + (u % q));
        }
        rows[id] = word;
    }
}

// ---------------------------------------------------------------------------
// Stage 2 and emission

// The 32 largest candidates not dividing d with 1/d mod p, by one warp: lane
// l tests candidate 35 - l, lanes 0..3 also candidate 3 - l.
__device__ __forceinline__ void select_warp(u32 du, const Candidates &cand,
                                            const unsigned short *inv_table, int *s_ci, u32 *s_dinv) {
    const int lane = threadIdx.x & 31;
    const int ch = kCandidatePrimes - 1 - lane;
    const u32 rh = mod_small(du, u32(cand.p[ch]), cand.magic[ch]);
    const u32 hi_div = __ballot_sync(kFullMask, rh == 0);
    const int cl = kCandidatePrimes - 1 - 32 - lane;
    const u32 rl = lane < kCandidatePrimes - 32 ? mod_small(du, u32(cand.p[cl]), cand.magic[cl]) : 1u;
    const u32 lo_div = __ballot_sync(kFullMask, rl == 0);
    const u32 below = lanemask_lt();
    const int rank_h = lane - __popc(hi_div & below);
    if (rh != 0 && rank_h < kSelectedPrimes) {
        s_ci[rank_h] = ch;
        s_dinv[rank_h] = __ldg(inv_table + cand.p[ch] * kMaximumPrime + rh);
    }
    const int rank_l = 32 - __popc(hi_div) + lane - __popc(lo_div & below);
    if (lane < kCandidatePrimes - 32 && rl != 0 && rank_l < kSelectedPrimes) {
        s_ci[rank_l] = cl;
        s_dinv[rank_l] = __ldg(inv_table + cand.p[cl] * kMaximumPrime + rl);
    }
    __syncwarp();
}

// Clears the bits j of m whose site a = base + step j fails one of the 32
// selected primes: f(a/d) mod p must be a square.  residue(ci, p, magic)
// returns base mod p; step_mod(ci) returns step mod p; aff holds the curve's
// 36 candidate bitmasks in shared memory.
template <typename Residue, typename StepMod, typename Index, typename Inverse>
__device__ __forceinline__ u64 stage2(u64 m, const Index *s_ci, const Inverse *s_dinv,
                                      const Candidates &cand, const u64 *aff, Residue residue,
                                      StepMod step_mod) {
    for (int s = 0; s < kSelectedPrimes && m; ++s) {
        const int ci = s_ci[s];
        const u32 p = u32(cand.p[ci]), magic = cand.magic[ci];
        const u32 dinv = s_dinv[s];
        const u32 x0 = mod_small(residue(ci, p, magic) * dinv, p, magic);
        const u32 dx = mod_small(step_mod(ci) * dinv, p, magic);
        const u64 *bits = aff + ci * kRefWords;
        u64 rest = m;
        while (rest) {
            const int j = __ffsll((long long)rest) - 1;
            rest &= rest - 1;
            const u32 x = mod_small(x0 + u32(j) * dx, p, magic);
            if (!((bits[x >> 6] >> (x & 63)) & 1)) m &= ~(u64(1) << j);
        }
    }
    return m;
}

// Warp-collective emission of sites a = base + step j for the set bits j of m.
__device__ __forceinline__ void emit(u64 m, long long base, long long step, long long d, int curve,
                                     const BatchOut &out) {
    const int lane = threadIdx.x & 31;
    const u32 cnt = __popcll(m);
    if (!__any_sync(kFullMask, cnt != 0)) return;
    u32 incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const u32 v = __shfl_up_sync(kFullMask, incl, o);
        if (lane >= o) incl += v;
    }
    const u32 total = __shfl_sync(kFullMask, incl, 31);
    unsigned long long pos = 0;
    if (lane == 0) pos = atomicAdd(out.count, (unsigned long long)total);
    pos = __shfl_sync(kFullMask, pos, 0) + incl - cnt;
    while (m) {
        const int j = __ffsll((long long)m) - 1;
        m &= m - 1;
        if (pos < out.capacity) {
            out.a[pos] = base + step * j;
            out.d[pos] = int(d);
            out.curve[pos] = curve;
        }
        ++pos;
    }
}

// Denominator primes: for p | d and p !| a, F(a, d) = c_n a^n (mod p), not a
// square when c_n is not and n is even, so a denominator with such a prime
// factor holds no points.  True if k (d = k or k^2: p | k^2 iff p | k) has a
// prime factor in the curve's mask (the loop is uniform over the warp).
__device__ __forceinline__ bool has_denominator_prime(u32 k, u64 mask0, u64 mask1, const OddPrime *odd) {
    bool hit = false;
    for (int w = 0; w < 2; ++w)
        for (u64 m = w ? mask1 : mask0; m; m &= m - 1) {
            const int i = 64 * w + __ffsll((long long)m) - 1;
            hit |= mod_u32(k, __ldg(&odd[i].p), __ldg(&odd[i].magic)) == 0;
        }
    return hit;
}

// ---------------------------------------------------------------------------
// Wide rows: class layout, warp-specialized like the single-curve fast
// kernel.  Warp 0 produces denominators into two slots: it takes work items
// (curve, parameter range, numerator range) from the device queue, skips
// parameters without admissible classes or with a denominator prime, points
// the slot at the curve's class list for the
// denominator's class k = (d mod 64) q + (d mod q) (or, for curves with x
// intervals, lays out the classes clipped to the numerator range in shared
// memory), and copies the curve's stage-1 rows into the slot by TMA.  The
// other warps sweep each filled slot's items and release it; queued words
// carry a private context (curve, d), so they wait past later
// denominators and curves.  No barrier spans the CTA.

// One class of one denominator in the numerator range being swept: class
// words [wbase, wbase + words); the first word drops its `first` low bits,
// the last keeps its `last` low bits; start[sl] is the row index of class word
// wbase for modulus sl.
struct WideRun {
    int wbase;
    int words;
    unsigned short ofs;            // (r + H) mod M: the class's least a is -H + ofs
    unsigned char first;
    unsigned char last;            // 1..64
    unsigned short start[kWideSlots];
    unsigned int pad[2];           // 32 bytes: class lists are copied by TMA in whole 16-byte units
};
static_assert(sizeof(WideRun) == 32, "packed class run");

// Item prefixes of a class list are stored at a stride of whole 16-byte
// units, so that a list's prefix row starts 16-byte aligned.
__host__ __device__ inline int wide_prefix_stride(int max_classes) { return (max_classes + 1 + 3) & ~3; }

// Per curve and class residue r mod M (precomputed on the host): the row
// index of class word 0 for each modulus, (a0 S^-1) mod m with a0 = -H + ofs.
struct ClassStart {
    unsigned short start[kWideSlots];
    unsigned short ofs;            // (r + H) mod M
    unsigned short pad;
};
static_assert(sizeof(ClassStart) == 16, "one 16-byte load per class");

// A denominator in flight: written by the producer warp, read by the others.
struct WideSlot {
    long long d;                   // -1: no more work
    const WideRun *runs;           // the denominator's class runs (shared memory)
    const int *prefix;             // sweep-item prefix of the runs
    unsigned long long magic[kWideSlots];  // the curve's stage-1 moduli: mod_u32 constants,
    u32 m[kWideSlots];             //   moduli,
    u32 step8[kWideSlots];         //   8 ((32 kWK) mod m): byte advance per step,
    u32 soff[kWideSlots];          //   byte offsets of the staged rows
    int curve;
    int nclass;
    int next;                      // sweep-item counter
    int steps;                     // > 0: items are groups of kWK short classes, this many steps
};

// A denominator a consumer warp still has queued words of.
constexpr int kWCtx = 8;
struct WideCtx {
    int d;
    int curve;
};

// Stage 2 and emission for up to 32 queued words.  A queued word carries its
// context (bits 56..58) and the position pos = a + H of its bit 0 (bits
// 0..55); its sites are a = -H + pos + M j.  A word meets the reference's
// selection, the 32 largest of the 36 candidates that do not divide its d:
// the candidates go largest first, the same one for the whole warp, each
// skipped where it divides d, until every word has met 32 or is empty.  The
// curve's descriptor and bitmasks are read through the read-only cache.
__device__ __forceinline__ void wide_drain(const u64 *qmask, const u64 *qpos, int start, int n,
                                           const WideCurve *curves, const u64 *affine,
                                           const Candidates &cand, const unsigned short *inv_table,
                                           const WideCtx *ctx, const BatchOut &out) {
    const int lane = threadIdx.x & 31;
    u64 m = 0, pos = 0;
    if (lane < n) {
        m = qmask[start + lane];
        pos = qpos[start + lane];
    }
    __syncwarp();
    const WideCtx &X = ctx[int(pos >> 56) & (kWCtx - 1)];
    const WideCurve *Cg = curves + (lane < n ? X.curve : 0);
    const u64 p56 = pos & ((u64(1) << 56) - 1);
    const u32 hi = u32(p56 >> 16), lo = u32(p56 & 0xFFFF);
    const u64 *aff = affine + __ldg(&Cg->aff);
    const u32 d = lane < n ? u32(X.d) : 1u;
    // the 32 largest candidates that do not divide d, largest first
    int tested = 0;
    for (int ci = kCandidatePrimes - 1; ci >= 0; --ci) {
        if (!__any_sync(kFullMask, m != 0 && tested < kSelectedPrimes)) break;
        const u32 p = u32(cand.p[ci]), magic = cand.magic[ci];
        const u32 rho = mod_small(d, p, magic);
        if (m != 0 && tested < kSelectedPrimes && rho != 0) {
            ++tested;
            const u32 dinv = __ldg(inv_table + p * kMaximumPrime + rho);
            u32 r = mod_small(hi, p, magic);
            r = mod_small((r << 16) | lo, p, magic);  // pos mod p
            r += __ldg(&Cg->neg_h[ci]);               // a mod p
            if (r >= p) r -= p;
            const u32 x0 = mod_small(r * dinv, p, magic);
            const u32 dx = mod_small(u32(__ldg(&Cg->m_mod[ci])) * dinv, p, magic);
            const u64 *bits = aff + ci * kRefWords;
            u64 rest = m;
            while (rest) {
                const int j = __ffsll((long long)rest) - 1;
                rest &= rest - 1;
                const u32 x = mod_small(x0 + u32(j) * dx, p, magic);
                if (!((__ldg(bits + (x >> 6)) >> (x & 63)) & 1)) m &= ~(u64(1) << j);
            }
        }
    }
    const bool any = __any_sync(kFullMask, m != 0);
    if (!any) return;
    emit(m, -__ldg(&Cg->bound) + (long long)p56, __ldg(&Cg->class_mod), X.d, __ldg(&Cg->index), out);
}

// Producer layout for curves with x intervals: denominator d's admissible
// classes clipped to the item's numerator range, into runs / prefix in
// shared memory (the whole warp; 32 classes per pass).
__device__ __forceinline__ int wide_layout(const WideCurve &C, const ClassStart *cstart, u32 du,
                                           long long d, int range, WideRun *runs, int *prefix) {
    const int lane = threadIdx.x & 31;
    const int q = C.class_prime;
    const int M = C.class_mod;
    const u64 classes2 = C.admissible[du & 63];
    const u64 classesq = q > 1 ? C.admissible[64 + int(du % u32(q))] : u64(1);
    const int nq = __popcll(classesq);
    const int nclass = __popcll(classes2) * nq;
    long long lo_a = -C.bound, hi_a = C.bound;
    if (C.nint > 0) x_range(C.lo, C.hi, C.nint, C.bound, d, range, lo_a, hi_a);
    int carry = 0;
    for (int base = 0; base < nclass; base += 32) {
        const int c = base + lane;
        int nitems_c = 0;
        if (c < nclass) {
            const int r64 = nth_bit64(classes2, c / nq);
            int r = r64;
            if (q > 1) {
                const int rq = nth_bit64(classesq, c % nq);
                r = r64 + 64 * int(C.crt[C.mod_q[r64] * 13 + rq]);
            }
            const ClassStart cs = cstart[r];
            const int ofs = cs.ofs;
            // sites of class r: a = -H + ofs + M t, t in [0, count); those in
            // [lo_a, hi_a] are t in [t_lo, t_hi]
            const long long count = C.count_q + (ofs <= C.count_r ? 1 : 0);
            const long long a0 = -C.bound + ofs;
            const long long below = lo_a - a0;
            const long long t_lo = below <= 0 ? 0 : (below + M - 1) / M;
            const long long above = hi_a - a0;
            const long long t_hi = above < 0 ? -1 : min(count - 1, above / M);
            WideRun run;
            run.ofs = (unsigned short)ofs;
            if (t_lo <= t_hi) {
                run.wbase = int(t_lo >> 6);
                run.words = int((t_hi >> 6) - (t_lo >> 6) + 1);
                run.first = (unsigned char)(t_lo & 63);
                run.last = (unsigned char)((t_hi & 63) + 1);
            } else {
                run.wbase = 0;
                run.words = 0;
                run.first = 0;
                run.last = 64;
            }
#pragma unroll
            for (int sl = 0; sl < kWideSlots; ++sl)
                run.start[sl] = (unsigned short)mod_u32(u32(cs.start[sl]) + u32(run.wbase), u32(C.mod[sl].m),
                                                        C.mod[sl].magic);
            runs[c] = run;
            nitems_c = (run.words + kWItemWords - 1) / kWItemWords;
        }
        int incl = nitems_c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(kFullMask, incl, o);
            if (lane >= o) incl += v;
        }
        if (c < nclass) prefix[c] = carry + incl - nitems_c;
        carry += __shfl_sync(kFullMask, incl, 31);
    }
    if (lane == 0) prefix[nclass] = carry;
    return nclass;
}

__global__ void __launch_bounds__(kWThreads, 2)
    wide_kernel(const WideCurve *__restrict__ curves, const BatchItem *__restrict__ items,
                int nitems, const u64 *__restrict__ pool, const u64 *__restrict__ affine,
                const ClassStart *__restrict__ class_starts, const WideRun *__restrict__ list_runs,
                const int *__restrict__ list_prefix, const int *__restrict__ list_count,
                const unsigned short *__restrict__ inv_table, const OddPrime *__restrict__ odd,
                Candidates cand, BatchOut out, int row_stride, int max_classes, unsigned long long *work,
                unsigned long long *swept) {
    extern __shared__ __align__(16) u64 smem[];
    u64 *qmask = smem + kWSlotCount * row_stride;
    u64 *qpos = qmask + kWConsumers * kQueue;
    WideRun *runs0 = reinterpret_cast<WideRun *>(qpos + kWConsumers * kQueue);  // [slots][max_classes]
    int *prefix0 = reinterpret_cast<int *>(runs0 + kWSlotCount * max_classes);  // [slots][prefix stride]
    const int pstride = wide_prefix_stride(max_classes);
    __shared__ WideSlot slot[kWSlotCount];
    __shared__ WideCtx s_ctx[kWConsumers][kWCtx];
    __shared__ unsigned long long s_swept[kWConsumers][2];
    __shared__ __align__(8) unsigned long long s_full[kWSlotCount];
    __shared__ __align__(8) unsigned long long s_empty[kWSlotCount];

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        for (int b = 0; b < kWSlotCount; ++b) {
            mbar_init(smem_addr(&s_full[b]), 1);
            mbar_init(smem_addr(&s_empty[b]), kWConsumers);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int i = threadIdx.x; i < kWConsumers * kWCtx; i += kWThreads) {
        s_ctx[i / kWCtx][i % kWCtx].d = 1;
        s_ctx[i / kWCtx][i % kWCtx].curve = 0;
    }
    __syncthreads();

    if (warp == 0) {
        // ---- producer ----
        // Work items come from the device queue with the next item's index
        // fetched ahead; lane j classifies parameter j of each 32 of an item,
        // and the live denominators go to the slots in order.  Lanes
        // 0 .. kWideSlots-1 copy one row each, lanes 30 and 31 the class list.
        int b = 0;
        int uses[kWSlotCount] = {};  // fills of each slot so far
        bool failed = false;
        int next_item = 0;
        if (lane == 0) next_item = int(atomicAdd(work, 1ull));
        auto acquire_slot = [&]() -> bool {
            int used = 0;
#pragma unroll
            for (int t = 0; t < kWSlotCount; ++t) used = t == b ? uses[t] : used;
            return used == 0 || mbar_wait(smem_addr(&s_empty[b]), u32(used - 1) & 1u);
        };
        for (;;) {
            const int idx = __shfl_sync(kFullMask, next_item, 0);
            if (idx >= nitems) break;
            if (lane == 0) next_item = int(atomicAdd(work, 1ull));
            const BatchItem item = items[idx];
            const WideCurve &C = curves[item.curve];
            const int q = C.class_prime;
            const long long lists = C.list_count;  // -1: classes laid out here
            const unsigned long long magic_q = (~0ull) / u32(q) + 1;
            const u64 bad0 = C.denom_primes[0], bad1 = C.denom_primes[1];
            for (int base = 0; base < item.count && !failed; base += kWarpSize) {
                const bool valid = base + lane < item.count;
                const long long k = item.first + base + (valid ? lane : 0);
                const long long dd = C.square ? k * k : k;
                const u32 dv = u32(dd);
                const int dq = q > 1 ? int(mod_u32(dv, u32(q), magic_q)) : 0;
                const int combo = int(dv & 63) * q + dq;
                int nlist = 0;
                bool live = false;
                if (valid) {
                    if (lists >= 0) {
                        nlist = __ldg(list_count + lists + combo);
                        live = nlist > 0;
                    } else {
                        long long L, U;
                        live = C.admissible[dv & 63] != 0 && (q == 1 || C.admissible[64 + dq] != 0) &&
                               (C.nint == 0 || x_range(C.lo, C.hi, C.nint, C.bound, dd, item.range, L, U));
                    }
                }
                if (bad0 | bad1) live = live && !has_denominator_prime(u32(k), bad0, bad1, odd);
                for (u32 todo = __ballot_sync(kFullMask, live); todo; todo &= todo - 1) {
                    const int j = __ffs(todo) - 1;
                    const long long d = __shfl_sync(kFullMask, dd, j);
                    const int combo_j = __shfl_sync(kFullMask, combo, j);
                    const int nlist_j = __shfl_sync(kFullMask, nlist, j);
                    if (!acquire_slot()) {
                        failed = true;
                        break;
                    }
                    WideSlot &S = slot[b];
                    const u32 full = smem_addr(&s_full[b]);
                    const u32 du = u32(d);
                    if (lane < kWideSlots) {
                        const Modulus &Md = C.mod[lane];
                        S.magic[lane] = Md.magic;
                        S.m[lane] = u32(Md.m);
                        S.step8[lane] = 8u * Md.step;
                        S.soff[lane] = 8u * u32(Md.smem_offset);
                    }
                    WideRun *runs = runs0 + b * max_classes;
                    int *prefix = prefix0 + b * pstride;
                    // a class list goes next to the slot by TMA with the rows
                    u32 list_bytes = 0, prefix_bytes = 0;
                    int nclass = nlist_j;
                    if (lists >= 0) {
                        list_bytes = u32(nlist_j) * u32(sizeof(WideRun));
                        prefix_bytes = u32(wide_prefix_stride(nlist_j)) * 4u;  // within the list's stride
                    } else {
                        nclass = wide_layout(C, class_starts + C.cls, du, d, item.range, runs, prefix);
                    }
                    __syncwarp();
                    if (lane == 0) {
                        S.runs = runs;
                        S.prefix = prefix;
                        S.nclass = nclass;
                        S.steps = lists >= 0 ? C.list_steps : 0;
                        S.d = d;
                        S.curve = item.curve;
                        S.next = 0;
                        __threadfence_block();
                        mbar_arrive_expect_tx(full, u32(C.smem_words) * 8u + list_bytes + prefix_bytes);
                    }
                    __syncwarp();
                    if (lane < kWideSlots) {
                        // the consumers' reads of this slot's previous contents are
                        // ordered before the asynchronous copies that overwrite them
                        fence_proxy_async_shared();
                        const Modulus &Md = C.mod[lane];
                        const u32 rho = mod_u32(du, u32(Md.m), Md.magic);
                        bulk_copy_to_shared(smem_addr(smem + b * row_stride) + u32(Md.smem_offset) * 8u,
                                            pool + Md.offset + (long long)rho * Md.length,
                                            u32(Md.length) * 8u, full);
                    } else if (list_bytes && lane >= kWarpSize - 2) {
                        fence_proxy_async_shared();
                        const int lm = C.list_max;
                        if (lane == kWarpSize - 2)
                            bulk_copy_to_shared(smem_addr(runs), list_runs + C.list_runs + (long long)combo_j * lm,
                                                list_bytes, full);
                        else
                            bulk_copy_to_shared(smem_addr(prefix),
                                                list_prefix + C.list_prefix + (long long)combo_j * wide_prefix_stride(lm),
                                                prefix_bytes, full);
                    }
#pragma unroll
                    for (int t = 0; t < kWSlotCount; ++t) uses[t] += t == b ? 1 : 0;
                    b = b + 1 == kWSlotCount ? 0 : b + 1;
                }
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
            if (out.error && lane == 0) atomicOr(out.error, 1ull);
            // let the copies already issued land (bounded) before leaving
#pragma unroll
            for (int t = 0; t < kWSlotCount; ++t)
                if (lane == 0 && uses[t] > 0) mbar_wait(smem_addr(&s_full[t]), u32(uses[t] - 1) & 1u);
        }
        return;
    }

    // ---- consumers ----
    const int cw = warp - 1;
    u64 *wq_mask = qmask + cw * kQueue;
    u64 *wq_pos = qpos + cw * kQueue;
    WideCtx *ctx = s_ctx[cw];
    u32 phase = 0;
    int b = 0;
    int qn = 0;      // queued words (kept across denominators and curves)
    int seq = 0;     // slot fills this warp has taken
    int oldest = 0;  // oldest context that may still have queued words
    auto drain_all = [&]() {
        while (qn > 0) {
            const int nd = qn < 32 ? qn : 32;
            __syncwarp();
            wide_drain(wq_mask, wq_pos, qn - nd, nd, curves, affine, cand, inv_table, ctx, out);
            qn -= nd;
        }
    };
    // class words this warp sweeps, and the stage-1 shared-memory bytes
    // they read (8 per word and row of the curve), kept in shared memory
    unsigned long long *my_swept = s_swept[cw];
    if (lane == 0) my_swept[0] = my_swept[1] = 0;
    for (;;) {
        if (!mbar_wait(smem_addr(&s_full[b]), (phase >> b) & 1u)) {  // bounded wait
            if (out.error && lane == 0) atomicOr(out.error, 1ull);
            return;
        }
        phase ^= 1u << b;
        const WideSlot &S = slot[b];
        if (S.d < 0) {
            drain_all();
            if (lane == 0) {
                atomicAdd(swept, my_swept[0]);
                atomicAdd(swept + 1, my_swept[1]);
            }
            return;
        }
        // context kc replaces the one taken kWCtx fills ago: its queued words go first
        const int kc = seq & (kWCtx - 1);
        if (qn > 0 && seq - oldest >= kWCtx) drain_all();
        if (qn == 0) oldest = seq;
        __syncwarp();
        if (lane == 0) {
            ctx[kc].d = int(S.d);
            ctx[kc].curve = S.curve;
        }
        __syncwarp();
        const u64 tag = u64(kc) << 56;
        const WideCurve &C = curves[S.curve];
        const unsigned char *sbase = reinterpret_cast<const unsigned char *>(smem + b * row_stride);
        const u64 stride = u64(C.stride);
        const u32 rows = u32(__ldg(&C.rows));
        const WideRun *runs = S.runs;
        const int *prefix = S.prefix;
        const int nclass = S.nclass;
        const int nsteps = S.steps;
        if (nsteps > 0) {
            // Short classes (at most 128 words): an item is kWK classes side
            // by side, group kk of a lane's words taken from class kk, so a
            // step covers 32 words of each; a lane's word w of a class is row
            // word (start + lane) mod m + 32 s, inside the row's 96-word
            // extension.  o holds byte offsets from the slot's row base.
            for (;;) {
                int g = 0;
                if (lane == 0) g = atomicAdd(const_cast<int *>(&S.next), 1);
                g = __shfl_sync(kFullMask, g, 0);
                if (g * kWK >= nclass) break;
                u32 o[kWideSlots][kWK];
                u32 meta[kWK];  // class words (bits 0..7), valid bits of its last word (8..15), ofs (16..31)
#pragma unroll
                for (int kk = 0; kk < kWK; ++kk) {
                    const int cc = g * kWK + kk;
                    meta[kk] = 0;
#pragma unroll
                    for (int sl = 0; sl < kWideSlots; ++sl) o[sl][kk] = S.soff[sl];
                    if (cc < nclass) {
                        const WideRun run = runs[cc];
                        meta[kk] = u32(run.words) | (u32(run.last) << 8) | (u32(run.ofs) << 16);
#pragma unroll
                        for (int sl = 0; sl < kWideSlots; ++sl) {
                            const u32 m = S.m[sl];
                            const u32 v = u32(run.start[sl]) + u32(lane);
                            o[sl][kk] += 8u * (m >= 32 ? (v >= m ? v - m : v) : mod_u32(v, m, S.magic[sl]));
                        }
                    }
                }
                if (lane == 0) {
                    const u32 words = (meta[0] & 0xFFu) + (meta[1] & 0xFFu) + (meta[2] & 0xFFu) + (meta[3] & 0xFFu);
                    my_swept[0] += words;
                    my_swept[1] += 8ull * words * rows;
                }
#pragma unroll 1
                for (int step = 0; step < nsteps; ++step) {
                    u64 acc[kWK];
#pragma unroll
                    for (int kk = 0; kk < kWK; ++kk)
                        acc[kk] = *reinterpret_cast<const u64 *>(sbase + o[0][kk] + 256 * step);
#pragma unroll
                    for (int sl = 1; sl < kWideSlots; ++sl) {
#pragma unroll
                        for (int kk = 0; kk < kWK; ++kk)
                            acc[kk] &= *reinterpret_cast<const u64 *>(sbase + o[sl][kk] + 256 * step);
                    }
                    const int w = kWarpSize * step + lane;
#pragma unroll
                    for (int kk = 0; kk < kWK; ++kk) {
                        const int wk = int(meta[kk] & 0xFFu);
                        if (w == wk - 1) {
                            const u32 last = (meta[kk] >> 8) & 0xFFu;
                            if (last < 64) acc[kk] &= (u64(1) << last) - 1;
                        }
                        if (w >= wk) acc[kk] = 0;
                    }
                    const u64 any = acc[0] | acc[1] | acc[2] | acc[3];
                    if (!__ballot_sync(kFullMask, any != 0)) continue;
#pragma unroll
                    for (int kk = 0; kk < kWK; ++kk) {
                        const bool live_word = acc[kk] != 0;
                        const u32 bb = __ballot_sync(kFullMask, live_word);
                        if (bb) {
                            const int at = qn + __popc(bb & lanemask_lt());
                            if (live_word) {
                                wq_mask[at] = acc[kk];
                                wq_pos[at] = tag | (u64(meta[kk] >> 16) + stride * u64(w));
                            }
                            qn += __popc(bb);
                            if (qn >= 32) {
                                __syncwarp();
                                wide_drain(wq_mask, wq_pos, qn - 32, 32, curves, affine, cand, inv_table, ctx, out);
                                qn -= 32;
                                if (qn == 0) oldest = seq;
                            }
                        }
                    }
                }
            }
        } else {
            u32 step8[kWideSlots], mod8[kWideSlots];
            const unsigned char *slot_base[kWideSlots];
#pragma unroll
            for (int sl = 0; sl < kWideSlots; ++sl) {
                step8[sl] = S.step8[sl];
                mod8[sl] = 8u * S.m[sl];
                slot_base[sl] = sbase + S.soff[sl];
            }
            const int total_items = prefix[nclass];
            int c = 0;  // this warp's items of a slot only increase: so do their classes
            for (;;) {
                int sweep = 0;
                if (lane == 0) sweep = atomicAdd(const_cast<int *>(&S.next), 1);
                sweep = __shfl_sync(kFullMask, sweep, 0);
                if (sweep >= total_items) break;
                // class index: largest c with prefix[c] <= sweep, from the last one on
                for (int base = c; base < nclass; base += 32) {
                    const int cc = base + lane;
                    const u32 bb = __ballot_sync(kFullMask, cc < nclass && prefix[cc] <= sweep);
                    if (bb) c = base + 31 - __clz(bb);
                    if (bb != kFullMask) break;
                }
                const int w0 = (sweep - prefix[c]) * kWItemWords;
                const WideRun run = runs[c];
                const int wt = run.words;
                if (lane == 0) {
                    const u32 words = u32(min(kWItemWords, wt - w0));
                    my_swept[0] += words;
                    my_swept[1] += 8ull * words * rows;
                }
                const u64 first_mask = ~u64(0) << run.first;
                const u64 last_mask = run.last >= 64 ? ~u64(0) : ((u64(1) << run.last) - 1);
                const u64 pos0 = u64(run.ofs) + stride * u64(run.wbase);
                u32 o[kWideSlots];
#pragma unroll
                for (int sl = 0; sl < kWideSlots; ++sl)
                    o[sl] = 8u * mod_u32(u32(run.start[sl]) + u32(w0 + lane), S.m[sl], S.magic[sl]);
#pragma unroll 1
                for (int step = 0; step < kWSteps; ++step) {
                    const int ws = w0 + step * kWarpSize * kWK;
                    if (ws >= wt) break;
                    // a class's last step often covers fewer than kWK groups of
                    // 32 words (short rows): the groups past its end are skipped
                    const int nk = min(kWK, (wt - ws + kWarpSize - 1) / kWarpSize);
                    u64 acc[kWK];
#pragma unroll
                    for (int kk = 0; kk < kWK; ++kk)
                        acc[kk] = kk < nk ? *reinterpret_cast<const u64 *>(slot_base[0] + o[0] + 256 * kk) : 0;
#pragma unroll
                    for (int sl = 1; sl < kWideSlots; ++sl) {
#pragma unroll
                        for (int kk = 0; kk < kWK; ++kk)
                            if (kk < nk) acc[kk] &= *reinterpret_cast<const u64 *>(slot_base[sl] + o[sl] + 256 * kk);
                    }
#pragma unroll
                    for (int sl = 0; sl < kWideSlots; ++sl) {
                        // advance (32 kWK) mod m words; unsigned min wraps into [0, m)
                        const u32 t = o[sl] + step8[sl];
                        o[sl] = min(t, t - mod8[sl]);
                    }
                    const u64 any = acc[0] | acc[1] | acc[2] | acc[3];
                    if (!__ballot_sync(kFullMask, any != 0)) continue;
#pragma unroll
                    for (int kk = 0; kk < kWK; ++kk) {
                        if (kk >= nk) break;
                        const int w = ws + kWarpSize * kk + lane;
                        u64 a = acc[kk];
                        if (w == 0) a &= first_mask;
                        if (w == wt - 1) a &= last_mask;
                        const bool live_word = a != 0 && w < wt;
                        const u32 bb = __ballot_sync(kFullMask, live_word);
                        if (bb) {
                            const int at = qn + __popc(bb & lanemask_lt());
                            if (live_word) {
                                wq_mask[at] = a;
                                wq_pos[at] = tag | (pos0 + stride * u64(w));
                            }
                            qn += __popc(bb);
                            if (qn >= 32) {
                                __syncwarp();
                                wide_drain(wq_mask, wq_pos, qn - 32, 32, curves, affine, cand, inv_table, ctx, out);
                                qn -= 32;
                                if (qn == 0) oldest = seq;
                            }
                        }
                    }
                }
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_addr(&s_empty[b]));  // this warp is done with slot b
        ++seq;
        b = b + 1 == kWSlotCount ? 0 : b + 1;
    }
}

// ---------------------------------------------------------------------------
// Narrow rows: dense layout, one warp per denominator, whole tables in shared memory.

__device__ __forceinline__ void narrow_drain(const u64 *qmask, const u32 *qword, int start, int n,
                                             const NarrowCurve &C, const Candidates &cand,
                                             const u64 *s_aff, const int *s_ci, const u32 *s_dinv,
                                             long long d, const BatchOut &out) {
    const int lane = threadIdx.x & 31;
    u64 m = 0;
    u32 w = 0;
    if (lane < n) {
        m = qmask[start + lane];
        w = qword[start + lane];
    }
    __syncwarp();
    if (m) {
        m = stage2(
            m, s_ci, s_dinv, cand, s_aff,
            [&](int ci, u32 p, u32 magic) {
                const u32 r = C.neg_h[ci] + mod_small(64u * mod_small(w, p, magic), p, magic);
                return r >= p ? r - p : r;
            },
            [&](int) { return 1u; });
    }
    emit(m, -C.bound + 64LL * w, 1, d, C.index, out);
}

__global__ void __launch_bounds__(kNThreads, 3)
    narrow_kernel(const NarrowCurve *__restrict__ curves, const BatchItem *__restrict__ items,
                  int nitems, const u64 *__restrict__ pool, const u64 *__restrict__ affine,
                  const unsigned short *__restrict__ inv_table, const OddPrime *__restrict__ odd,
                  Candidates cand, BatchOut out, unsigned long long *work, unsigned long long *swept) {
    extern __shared__ __align__(16) u64 smem[];
    __shared__ NarrowCurve C;
    __shared__ int s_item;
    __shared__ int s_next;
    __shared__ int s_abort;
    __shared__ int s_ci[kNWarps][kSelectedPrimes];
    __shared__ u32 s_dinv[kNWarps][kSelectedPrimes];
    __shared__ unsigned char s_lane_at[kNarrowSlots][kWarpSize];  // (shift + kNK lane) mod m
    __shared__ __align__(8) unsigned long long s_bar;

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const u64 *tab = smem;
    const u64 *s_aff = smem + kNarrowTableWords;  // the curve's 36 candidate bitmasks
    u64 *wq_mask = smem + kNarrowTableWords + kAffWords + warp * kQueue;
    u32 *wq_word =
        reinterpret_cast<u32 *>(smem + kNarrowTableWords + kAffWords + kNWarps * kQueue) + warp * kQueue;
    const u32 bar = smem_addr(&s_bar);
    u32 phase = 0;
    int cur = -1;
    // row words this warp sweeps and the stage-1 shared-memory bytes they read
    unsigned long long swept_words = 0, swept_bytes = 0;
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    for (;;) {
        if (threadIdx.x == 0) {
            s_item = int(atomicAdd(work, 1ull));
            s_next = 0;
        }
        __syncthreads();
        const int it = s_item;
        if (it >= nitems) break;
        const BatchItem item = items[it];
        if (item.curve != cur) {
            const u32 *src = reinterpret_cast<const u32 *>(curves + item.curve);
            u32 *dst = reinterpret_cast<u32 *>(&C);
            for (int i = threadIdx.x; i < int(sizeof(NarrowCurve) / 4); i += kNThreads) dst[i] = src[i];
            cur = item.curve;
            __syncthreads();
            // each lane's first table word per modulus for rows swept from word 0
            for (int t = threadIdx.x; t < kNarrowSlots * kWarpSize; t += kNThreads) {
                const int s = t / kWarpSize, l = t % kWarpSize;
                s_lane_at[s][l] = (unsigned char)((C.shift[s] + u32(kNK * l)) % u32(C.m[s]));
            }
            if (threadIdx.x == 0) {
                fence_proxy_async_shared();
                mbar_arrive_expect_tx(bar, u32(C.table_words + kAffWords) * 8u);
                bulk_copy_to_shared(smem_addr(smem), pool + C.tables, u32(C.table_words) * 8u, bar);
                bulk_copy_to_shared(smem_addr(smem + kNarrowTableWords), affine + C.aff,
                                    u32(kAffWords) * 8u, bar);
            }
            if (!mbar_wait(bar, phase)) {
                s_abort = 1;
                if (out.error) atomicOr(out.error, 1ull);
            }
            phase ^= 1u;
            __syncthreads();
            if (s_abort) {
                if (threadIdx.x == 0) mbar_wait(bar, phase ^ 1u);
                return;
            }
        }
        int *w_ci = s_ci[warp];
        u32 *w_dinv = s_dinv[warp];
        for (;;) {
            int idx0 = 0;
            if (lane == 0) idx0 = atomicAdd(&s_next, kND);
            idx0 = __shfl_sync(kFullMask, idx0, 0);
            if (idx0 >= item.count) break;
            const int jn = min(kND, item.count - idx0);
            u32 rho[kNarrowSlots];
            for (int j = 0; j < jn; ++j) {
                const long long k = item.first + idx0 + j;
                const long long d = C.square ? k * k : k;
                const u32 du = u32(d);
                // d mod m for every modulus: reduced for the first parameter of the
                // fetch (and for square denominators), else advanced by one
#pragma unroll
                for (int s = 0; s < kNarrowSlots; ++s) {
                    if (j == 0 || C.square) {
                        rho[s] = mod_u32(du, u32(C.m[s]), C.magic[s]);
                    } else {
                        rho[s] += 1;
                        if (rho[s] == u32(C.m[s])) rho[s] = 0;
                    }
                }
                const u64 mask2 = C.dense2[du & 63];
                if (!mask2) continue;
                // denominator primes (see has_denominator_prime), split over the lanes
                bool hit = false;
                for (int i = lane; i < kOddPrimes; i += kWarpSize)
                    if ((C.denom_primes[i >> 6] >> (i & 63)) & 1)
                        hit |= mod_u32(u32(k), __ldg(&odd[i].p), __ldg(&odd[i].magic)) == 0;
                if (__any_sync(kFullMask, hit)) continue;
                // words [w_lo, w_hi] hold the numerator range of this item: a in [L, U]
                long long L = -C.bound, U = C.bound;
                if (C.nint > 0 && !x_range(C.lo, C.hi, C.nint, C.bound, d, item.range, L, U)) continue;
                const int w_lo = int((L + C.bound) >> 6), w_hi = int((U + C.bound) >> 6);
                swept_words += u32(w_hi - w_lo + 1);
                swept_bytes += 8ull * u32(C.rows) * u32(w_hi - w_lo + 1);
                const u64 first_mask = ~u64(0) << ((L + C.bound) & 63);
                const int last_bits = int((U + C.bound) & 63) + 1;
                const u64 last_mask = last_bits >= 64 ? ~u64(0) : ((u64(1) << last_bits) - 1);
                // lane l takes words w0 + kNK l .. w0 + kNK l + kNK - 1 of each
                // 128-word step: rows repeat their first kNK - 1 words, so the kNK
                // words of a lane never wrap and one index per modulus advances
                u32 base[kNarrowSlots], at[kNarrowSlots], mods[kNarrowSlots], steps[kNarrowSlots];
#pragma unroll
                for (int s = 0; s < kNarrowSlots; ++s) {
                    const u32 m = u32(C.m[s]);
                    mods[s] = m;
                    steps[s] = C.step[s];
                    base[s] = u32(C.off[s]) + rho[s] * u32(C.len[s]);
                    at[s] = w_lo == 0 ? u32(s_lane_at[s][lane])
                                      : mod_u32(C.shift[s] + u32(w_lo + kNK * lane), m, C.magic[s]);
                }
                bool selected = false;
                int qn = 0;
                for (int w0 = w_lo; w0 <= w_hi; w0 += kWarpSize * kNK) {
                    u64 acc[kNK];
#pragma unroll
                    for (int k = 0; k < kNK; ++k) acc[k] = mask2;
#pragma unroll
                    for (int s = 0; s < kNarrowSlots; ++s) {
                        const u64 *row = tab + base[s] + at[s];
#pragma unroll
                        for (int k = 0; k < kNK; ++k) acc[k] &= row[k];
                        const u32 t = at[s] + steps[s];  // advance 32 kNK words mod m
                        at[s] = min(t, t - mods[s]);
                    }
                    const int wl = w0 + kNK * lane;
                    if (w0 == w_lo || w0 + kWarpSize * kNK - 1 > w_hi) {  // the range's first or last step
#pragma unroll
                        for (int k = 0; k < kNK; ++k) {
                            const int w = wl + k;
                            if (w > w_hi) acc[k] = 0;
                            if (w == w_lo) acc[k] &= first_mask;
                            if (w == w_hi) acc[k] &= last_mask;
                        }
                    }
                    if (!__ballot_sync(kFullMask, (acc[0] | acc[1] | acc[2] | acc[3]) != 0)) continue;
#pragma unroll
                    for (int k = 0; k < kNK; ++k) {
                        const u32 b = __ballot_sync(kFullMask, acc[k] != 0);
                        if (!b) continue;
                        const int pos = qn + __popc(b & lanemask_lt());
                        if (acc[k]) {
                            wq_mask[pos] = acc[k];
                            wq_word[pos] = u32(wl + k);
                        }
                        qn += __popc(b);
                        if (qn >= 32) {
                            if (!selected) {
                                select_warp(du, cand, inv_table, w_ci, w_dinv);
                                selected = true;
                            }
                            __syncwarp();
                            narrow_drain(wq_mask, wq_word, qn - 32, 32, C, cand, s_aff, w_ci, w_dinv, d,
                                         out);
                            qn -= 32;
                        }
                    }
                }
                if (qn) {
                    if (!selected) select_warp(du, cand, inv_table, w_ci, w_dinv);
                    __syncwarp();
                    narrow_drain(wq_mask, wq_word, 0, qn, C, cand, s_aff, w_ci, w_dinv, d, out);
                }
            }
        }
        __syncthreads();
    }
    if (lane == 0) {
        atomicAdd(swept, swept_words);
        atomicAdd(swept + 1, swept_bytes);
    }
}

}  // namespace dev

// ---------------------------------------------------------------------------
// Host driver

namespace {

using Clock = std::chrono::steady_clock;
double ms_since(Clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
}

// Grow-only device array: kept across runs, reallocated only when a run
// needs more room than it has.
template <typename T>
struct DeviceArray {
    T *p = nullptr;
    std::size_t cap = 0;
    DeviceArray() = default;
    DeviceArray(const DeviceArray &) = delete;
    DeviceArray &operator=(const DeviceArray &) = delete;
    ~DeviceArray() { cudaFree(p); }
    void ensure(std::size_t count, const char *what) {
        count = std::max<std::size_t>(count, 1);
        if (count <= cap) return;
        cudaFree(p);
        p = nullptr;
        cap = 0;
        check_cuda(cudaMalloc(&p, count * sizeof(T)), what);
        cap = count;
    }
    void upload(const std::vector<T> &v, cudaStream_t s, unsigned long long &bytes, const char *what) {
        ensure(v.size(), what);
        if (!v.empty())
            check_cuda(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s),
                       what);
        bytes += v.size() * sizeof(T);
    }
};

// Runs fn(i) for i in [0, n) on the host's threads; rethrows the first exception.
template <typename F>
void parallel_for(std::size_t n, F &&fn) {
    const unsigned threads = std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), 64));
    if (n < 2 || threads == 1) {
        for (std::size_t i = 0; i < n; ++i) fn(i);
        return;
    }
    std::atomic<std::size_t> next{0};
    std::vector<std::thread> pool;
    std::exception_ptr error;
    std::mutex error_mutex;
    for (unsigned t = 0; t < std::min<std::size_t>(threads, n); ++t) {
        pool.emplace_back([&] {
            for (std::size_t i; (i = next.fetch_add(1)) < n;) {
                try {
                    fn(i);
                } catch (...) {
                    std::lock_guard<std::mutex> lock(error_mutex);
                    if (!error) error = std::current_exception();
                }
            }
        });
    }
    for (auto &th : pool) th.join();
    if (error) std::rethrow_exception(error);
}

long long gcd_ll(long long a, long long b) {
    if (a < 0) a = -a;
    while (b) {
        const long long t = a % b;
        a = b;
        b = t;
    }
    return a;
}

bool is_small_prime(int n) {
    if (n < 2) return false;
    for (int f = 2; f * f <= n; ++f)
        if (n % f == 0) return false;
    return true;
}

unsigned long long host_magic(int m) {
    return m == 1 ? ~0ull : (~0ull) / (unsigned long long)m + 1;
}

// Position of the odd prime p in the list of odd primes (3 -> 0, 5 -> 1, ...).
int odd_prime_index(int p) {
    int i = 0;
    for (int f = 3; f < p; f += 2) i += is_small_prime(f) ? 1 : 0;
    return i;
}

// Bit i set iff the i-th odd prime p below 512 (p != skip) is a denominator
// prime of the curve: even degree and c_n a nonzero non-square mod p (a
// denominator divisible by one holds no points).
void denominator_prime_mask(const std::vector<std::string> &coefficients, int skip, dev::u64 out[2]) {
    out[0] = out[1] = 0;
    if ((coefficients.size() - 1) % 2) return;
    int i = 0;
    for (int p = 3; p < kMaximumPrime; p += 2) {
        if (!is_small_prime(p)) continue;
        const int lc = decimal_mod(coefficients.back(), p);
        if (p != skip && lc != 0 && !square_mod(lc, p)) out[i >> 6] |= dev::u64(1) << (i & 63);
        ++i;
    }
}

// Position of the k-th set bit (k counted from 0) of a 64-bit mask.
int nth_bit_host(dev::u64 mask, int k) {
    for (int i = 0; i < k; ++i) mask &= mask - 1;
    return __builtin_ctzll(mask);
}

bool lead_is_square(const std::vector<std::string> &coefficients, int q) {
    const int n = int(coefficients.size()) - 1;
    if (n % 2) return true;  // odd degree: F(a, d) = d (...) vanishes mod q | d
    const int lc = decimal_mod(coefficients.back(), q);
    for (int v = 0; v < q; ++v)
        if ((v * v) % q == lc) return true;
    return false;
}

int round_even(long long v) { return int((v + 1) & ~1LL); }

// A rational bound as a double (leading 18 digits of numerator and
// denominator), +-inf beyond 1e300: the device widens every range by one site,
// far more than this rounding can move a bound that matters (|x d| <= 2^36).
double approx_value(const Rational &r) {
    auto split = [](const BigInt &v, double &mant, long &exp10) {
        std::string t = v.to_string();
        const bool neg = !t.empty() && t[0] == '-';
        if (neg) t.erase(0, 1);
        const std::size_t keep = std::min<std::size_t>(t.size(), 18);
        mant = std::stod(t.substr(0, keep));
        exp10 = long(t.size() - keep);
        if (neg) mant = -mant;
    };
    double mn, md;
    long en, ed;
    split(r.num, mn, en);
    split(r.den, md, ed);
    if (mn == 0) return 0.0;
    const long e = en - ed;
    if (e > 300) return mn > 0 ? HUGE_VAL : -HUGE_VAL;
    if (e < -300) return 0.0;
    return mn / md * std::pow(10.0, double(e));
}

// The intervals as ascending (lo, hi) doubles for the device ranges; false
// when there are none or more than the device takes (then rows are swept whole).
bool device_intervals(const std::vector<SearchInterval> &intervals, int &nint, double *lo, double *hi) {
    nint = 0;
    if (intervals.empty() || intervals.size() > std::size_t(dev::kMaxIntervals)) return false;
    std::vector<std::pair<double, double>> v;
    for (const auto &iv : intervals)
        v.push_back({iv.lower_infinite ? -HUGE_VAL : approx_value(iv.lower),
                     iv.upper_infinite ? HUGE_VAL : approx_value(iv.upper)});
    std::sort(v.begin(), v.end());
    for (const auto &p : v) {
        lo[nint] = p.first;
        hi[nint] = p.second;
        ++nint;
    }
    return true;
}

struct CurveWork {
    bool ok = false;
    bool wide = false;
    std::unique_ptr<ExactPolynomial> poly;
    FastPlan plan;
    long long words = 0;       // dense 64-site words per row
    long long swept = 0;       // words a denominator sweeps after interval narrowing (estimate)
    long long count = 0;       // parameters
    dev::u64 adm2[64] = {};    // 2-adic admissible classes by d mod 64
    int classes = 1;           // wide curves: most numerator classes of one denominator
    std::unique_ptr<FastPlanner> planner;  // wide curves, until planned
    std::vector<unsigned short> cand_residues;  // c_i mod p for the 36 candidates, candidate-major
    dev::u64 denom_primes[2] = {};             // the curve's denominator primes (no class prime removed)
};

// Words of one denominator's row that the sieve sweeps: the whole row, or with
// x intervals the interval numerators at a middle denominator (each interval
// [lo, hi] covers about (hi - lo) d / 64 words).  Picks the kernel shape.
long long swept_row_words(const BatchCurveSpec &c, long long words) {
    if (c.intervals.empty() || c.intervals.size() > std::size_t(dev::kMaxIntervals)) return words;
    const double dmid = 0.5 * double(c.first) + 0.5 * double(std::max(c.first, c.last));
    const double d = c.square ? dmid * dmid : dmid;
    double total = 0;
    for (const auto &iv : c.intervals) {
        if (iv.lower_infinite || iv.upper_infinite) return words;
        const double len = approx_value(iv.upper) - approx_value(iv.lower);
        if (len < 0) continue;
        total += std::min(double(words), len * d / 64.0 + 2.0);
    }
    return std::min(words, (long long)std::ceil(total));
}

// Narrow plan: every odd prime up to kBatchNarrowModulus that filters at
// least 0.15 bit, strongest first, each joining the slot whose product stays
// within the cap (smallest product first) or opening a new slot, while the
// tables (m rows of m + kNK - 1 words per slot) fit shared memory.
FastPlan narrow_plan(const std::vector<std::string> &coefficients) {
    std::vector<std::pair<double, int>> strength;
    for (int q = 3; q <= kBatchNarrowModulus; q += 2) {
        if (!is_small_prime(q)) continue;
        const double rate = pass_rate(q, coefficients);
        const double bits = rate > 0 ? -std::log2(rate) : 8.0;
        if (bits >= 0.15) strength.push_back({bits, q});
    }
    std::sort(strength.begin(), strength.end(), [](const auto &a, const auto &b) {
        return a.first != b.first ? a.first > b.first : a.second < b.second;
    });
    auto words = [](long long m) { return m * (m + dev::kNK - 1); };
    FastPlan plan;
    long long used = 0;
    for (const auto &sq : strength) {
        const int q = sq.second;
        int join = -1;
        for (std::size_t i = 0; i < plan.moduli.size(); ++i)
            if (plan.moduli[i] * q <= kBatchNarrowModulus &&
                (join < 0 || plan.moduli[i] < plan.moduli[std::size_t(join)]))
                join = int(i);
        if (join >= 0) {
            const long long m = plan.moduli[std::size_t(join)];
            const long long grown = used - words(m) + words(m * q);
            if (grown + dev::kNK * (dev::kNarrowSlots - long(plan.moduli.size())) >
                dev::kNarrowTableWords - 1)  // one word may pad the block to an even length
                continue;
            used = grown;
            plan.moduli[std::size_t(join)] *= q;
            plan.slots[std::size_t(join)].push_back(q);
        } else {
            if (int(plan.moduli.size()) == dev::kNarrowSlots) continue;
            const long long grown = used + words(q);
            if (grown + dev::kNK * (dev::kNarrowSlots - long(plan.moduli.size()) - 1) >
                dev::kNarrowTableWords - 1)
                continue;
            used = grown;
            plan.moduli.push_back(q);
            plan.slots.push_back({q});
        }
        plan.bits += sq.first;
    }
    return plan;
}

// Wide plan: moduli capped so that tables stay small against the curve's
// work, and the staged rows fit the shared-memory budget.
// Staged row words a wide curve may use (both buffers together) so that a
// CTA stays within a third of an SM's shared memory: static arrays, queues,
// and two sets of class runs and item prefixes for max_classes classes.
long long wide_row_budget(int max_classes) {
    const long long per_cta = 228 * 1024 / 2 - 1024;
    const long long fixed = 6 * 1024 +  // static shared memory of the kernel (5 KB) and slack
                            (long long)dev::kWConsumers * dev::kQueue * 16 +
                            (long long)dev::kWSlotCount * max_classes * (long long)sizeof(dev::WideRun) +
                            (long long)dev::kWSlotCount * dev::wide_prefix_stride(max_classes) * 4;
    return std::max(2LL * 64, (per_cta - fixed) / 8);
}

// Admissible residues mod the class prime q by d mod q: bit r of out[dq] is
// set iff f(r / dq) is a square mod q, or (q | d) r != 0 and c_n is a square.
void class_prime_residues(const std::vector<std::string> &coefficients, int q, dev::u64 *out) {
    const auto aff = affine_mask(q, coefficients);
    const bool lead = lead_is_square(coefficients, q);
    for (int dq = 0; dq < q; ++dq) {
        out[dq] = 0;
        for (int r = 0; r < q; ++r) {
            const bool ok = dq == 0 ? (r != 0 && lead) : aff[(r * mod_inverse(dq, q)) % q] != 0;
            if (ok) out[dq] |= dev::u64(1) << r;
        }
    }
}

// Most numerator classes of any one denominator of a wide curve: admissible
// 2-adic classes times admissible residues of the class prime.
int wide_classes(const std::vector<std::string> &coefficients, const dev::u64 adm2[64], int q) {
    int most2 = 0, mostq = 1;
    for (int dd = 0; dd < 64; ++dd) most2 = std::max(most2, __builtin_popcountll(adm2[dd]));
    if (q > 1) {
        dev::u64 admq[13];
        class_prime_residues(coefficients, q, admq);
        mostq = 0;
        for (int dq = 0; dq < q; ++dq) mostq = std::max(mostq, __builtin_popcountll(admq[dq]));
    }
    return most2 * std::max(1, mostq);
}

// max_classes: the most classes of a denominator of any wide curve in the
// launch, which sizes the slots' class arrays and so the share of shared
// memory left for rows.
FastPlan wide_plan(const FastPlanner &planner, long double work, int max_classes) {
    int cap = int(std::min<long double>(kMaxModulus, std::max<long double>(64, std::sqrt(work / 48.0L))));
    // two slots of staged rows
    const long long smem_budget =
        std::min<long long>(dev::kWMaxSmemWords, wide_row_budget(max_classes) / dev::kWSlotCount);
    for (;;) {
        FastPlan plan = planner.plan(cap, dev::kWideSlots, 1LL << 40, false);
        long long smem = 0;
        for (int sl = 0; sl < dev::kWideSlots; ++sl) {
            const int m = sl < int(plan.moduli.size()) ? plan.moduli[sl] : 1;
            smem += round_even(m + dev::kWExt);
        }
        if (smem <= smem_budget || cap <= 64) return plan;
        cap = cap * 7 / 8;
    }
}

}  // namespace

namespace {

// Everything one batched run launches: per-curve descriptors, table specs
// and work items, built on the host from the curves' plans.
struct BatchPlan {
    std::vector<CurveWork> work;
    std::vector<dev::WideCurve> wide;
    std::vector<dev::NarrowCurve> narrow;
    std::vector<dev::AffineSpec> aspecs;
    std::vector<unsigned short> residues;
    std::vector<dev::PatternSpec> pspecs;
    std::vector<dev::CompositeSpec> cspecs;
    std::vector<dev::BatchItem> wide_items, narrow_items;
    std::vector<dev::ClassStart> class_starts;
    std::vector<dev::WideRun> list_runs;       // class lists of wide curves without x intervals
    std::vector<int> list_prefix, list_count;
    long long aff_words = 0, pattern_words = 0, row_words = 0;
    int wide_smem_words = 0;
    int wide_max_classes = 1;   // most classes of a denominator of any wide curve
};

// Validation and per-curve plans (one curve per task), then descriptors,
// table specs and work items in the order the kernels take them.
void build_plan(const std::vector<BatchCurveSpec> &curves, std::vector<BatchCurveResult> &results,
                BatchPlan &P, BatchStats &stats, int items_per_kernel) {
    P.work.resize(curves.size());
    parallel_for(curves.size(), [&](std::size_t i) {
        const BatchCurveSpec &c = curves[i];
        BatchCurveResult &r = results[i];
        CurveWork &cw = P.work[i];
        try {
            if (c.coefficients.size() < 2) throw std::invalid_argument("polynomial must have degree >= 1");
            if (c.bound < 1) throw std::invalid_argument("numerator bound must be positive");
            if (c.first < 1) throw std::invalid_argument("denominators start at 1");
            if (c.last > (c.square ? 46340LL : 2147483647LL))
                throw std::invalid_argument("denominator range too large for 32-bit denominators");
            if (c.bound > (1LL << 33))
                throw std::invalid_argument("numerator bound too large for the batched search");
            cw.poly.reset(new ExactPolynomial(c.coefficients));
            if (!cw.poly->is_squarefree()) {
                r.status = 6;
                r.error = "polynomial is not squarefree";
                return;
            }
            cw.words = word_count64(c.bound);
            cw.count = c.last >= c.first ? c.last - c.first + 1 : 0;
            cw.swept = swept_row_words(c, cw.words);
            cw.wide = cw.swept >= kBatchWideWords;
            two_adic_classes(c.coefficients, cw.adm2);
            if (cw.wide) {
                cw.planner.reset(new FastPlanner(c.coefficients, c.bound, true, kFastPrimeLimit));
                cw.classes = wide_classes(c.coefficients, cw.adm2, cw.planner->class_prime());
            } else {
                cw.plan = narrow_plan(c.coefficients);
            }
            denominator_prime_mask(c.coefficients, 1, cw.denom_primes);
            {
                const auto &cps = candidate_primes();
                cw.cand_residues.reserve(kCandidatePrimes * c.coefficients.size());
                for (int ci = 0; ci < kCandidatePrimes; ++ci)
                    for (const auto &coef : c.coefficients)
                        cw.cand_residues.push_back((unsigned short)decimal_mod(coef, cps[ci]));
            }
            cw.ok = true;
        } catch (const std::exception &e) {
            r.status = 1;
            r.error = e.what();
        }
    });
    // wide plans: one row budget for the launch, from the largest class count
    // of its curves (each slot holds its denominator's classes)
    int max_classes = 1;
    for (std::size_t i = 0; i < curves.size(); ++i)
        if (P.work[i].ok && P.work[i].wide) max_classes = std::max(max_classes, P.work[i].classes);
    parallel_for(curves.size(), [&](std::size_t i) {
        CurveWork &cw = P.work[i];
        if (!cw.ok) return;
        if (cw.wide) {
            cw.plan = wide_plan(*cw.planner, (long double)cw.words * cw.count, max_classes);
            cw.planner.reset();
        }
        results[i].wide = cw.wide;
        results[i].class_prime = cw.plan.class_prime;
        results[i].moduli = cw.plan.moduli;
    });

    const auto &cands = candidate_primes();
    auto add_affine = [&](int p, const std::vector<std::string> &coeffs) {
        dev::AffineSpec A{};
        A.out = P.aff_words;
        A.residues = (long long)P.residues.size();
        A.p = p;
        A.n = int(coeffs.size()) - 1;
        for (const auto &c : coeffs) P.residues.push_back((unsigned short)decimal_mod(c, p));
        P.aspecs.push_back(A);
        P.aff_words += dev::kRefWords;
        return A.out;
    };
    // largest work first, so that the persistent kernels end on small items
    std::vector<std::size_t> order;
    for (std::size_t i = 0; i < curves.size(); ++i)
        if (P.work[i].ok && P.work[i].count > 0) order.push_back(i);
    std::stable_sort(order.begin(), order.end(), [&](std::size_t a, std::size_t b) {
        return (long double)P.work[a].words * P.work[a].count >
               (long double)P.work[b].words * P.work[b].count;
    });
    std::vector<std::pair<std::size_t, std::size_t>> list_curves;  // (descriptor, curve) with class lists
    // items: large enough that building and fetching them stays cheap, small
    // enough that a small batch still spreads over the device (about
    // items_per_kernel items per kernel): up to 2^21 row words (wide) and 2^18
    // swept words (narrow), at least one denominator per warp; one set per
    // numerator range
    long double wide_work = 0, narrow_work = 0;
    for (std::size_t i : order) {
        const CurveWork &cw = P.work[i];
        (cw.wide ? wide_work : narrow_work) += (long double)(cw.wide ? cw.words : cw.swept) * cw.count;
    }
    const long long wide_item =
        (long long)std::min<long double>(1LL << 21, std::max<long double>(1LL << 14, wide_work / items_per_kernel));
    const long long narrow_item =
        (long long)std::min<long double>(1LL << 18, std::max<long double>(1LL << 12, narrow_work / items_per_kernel));
    auto item_chunk = [&](const CurveWork &cw) -> long long {
        return cw.wide ? std::max(1LL, std::min<long long>(1 << 16, wide_item / cw.words))
                       : std::max<long long>(dev::kNWarps,
                                             std::min<long long>(1 << 16, narrow_item / std::max(1LL, cw.swept)));
    };
    {
        // sizes first, so that the vectors grow once
        std::size_t wide_items = 0, narrow_items = 0;
        for (std::size_t i : order) {
            const CurveWork &cw = P.work[i];
            const std::size_t n = curves[i].intervals.size();
            const long long ranges = n > 0 && n <= std::size_t(dev::kMaxIntervals) ? (long long)n : 1;
            const long long chunk = item_chunk(cw);
            (cw.wide ? wide_items : narrow_items) += std::size_t(ranges * ((cw.count + chunk - 1) / chunk));
        }
        P.wide_items.reserve(wide_items);
        P.narrow_items.reserve(narrow_items);
    }
    long long list_count_total = 0, list_runs_total = 0, list_prefix_total = 0;
    for (std::size_t i : order) {
        const BatchCurveSpec &c = curves[i];
        CurveWork &cw = P.work[i];
        const FastPlan &plan = cw.plan;
        const long long H = c.bound;
        const long long aff_base = P.aff_words;
        {
            // the 36 candidate bitmasks, residues computed in the parallel phase
            const std::size_t nc = c.coefficients.size();
            for (int ci = 0; ci < kCandidatePrimes; ++ci) {
                dev::AffineSpec A{};
                A.out = P.aff_words;
                A.residues = (long long)P.residues.size();
                A.p = cands[ci];
                A.n = int(nc) - 1;
                P.residues.insert(P.residues.end(), cw.cand_residues.begin() + std::ptrdiff_t(ci * nc),
                                  cw.cand_residues.begin() + std::ptrdiff_t((ci + 1) * nc));
                P.aspecs.push_back(A);
                P.aff_words += dev::kRefWords;
            }
        }
        // per-prime patterns of this curve's stage-1 factors
        const long long M = cw.wide ? 64LL * plan.class_prime : 1;
        const long long S = cw.wide ? 64LL * M : 64;
        std::vector<long long> pattern_of(kFastPrimeLimit, -1);
        for (const auto &slot : plan.slots)
            for (int q : slot) {
                if (pattern_of[q] >= 0) continue;
                dev::PatternSpec Q{};
                Q.offset = P.pattern_words;
                Q.aff = add_affine(q, c.coefficients);
                Q.q = q;
                Q.lead_ok = lead_is_square(c.coefficients, q) ? 1 : 0;
                Q.s = int(S % q);
                Q.t = int(M % q);
                P.pspecs.push_back(Q);
                pattern_of[q] = P.pattern_words;
                P.pattern_words += (long long)q * q;
            }
        auto add_composite = [&](int sl, int length) {
            dev::CompositeSpec T{};
            T.offset = P.row_words;
            if (sl < int(plan.moduli.size())) {
                T.m = plan.moduli[sl];
                T.nf = int(plan.slots[sl].size());
                for (int f = 0; f < T.nf; ++f) {
                    T.q[f] = plan.slots[sl][f];
                    T.pattern[f] = pattern_of[T.q[f]];
                }
            } else {
                T.m = 1;  // padding: a row of ones
                T.nf = 0;
            }
            T.length = length < 0 ? T.m : length;
            P.cspecs.push_back(T);
            P.row_words += (long long)T.m * T.length;
            return T;
        };
        stats.rectangle_sites += (long double)(2 * H + 1) * (long double)cw.count;
        stats.denominators += (unsigned long long)cw.count;
        stats.words += (unsigned long long)(cw.words * cw.count);
        if (cw.wide) {
            dev::WideCurve C{};
            const int q = plan.class_prime;
            C.bound = H;
            C.stride = S;
            C.count_q = (2 * H) / M;
            C.count_r = int((2 * H) % M);
            C.class_prime = q;
            C.class_mod = int(M);
            C.h_mod_m = int(H % M);
            C.inv64_q = q > 1 ? int(mod_inverse(64 % q, q)) : 0;
            C.square = c.square ? 1 : 0;
            C.index = int(i);
            C.rows = int(plan.moduli.size());
            // the class prime's classes already leave q | d without sites
            C.denom_primes[0] = cw.denom_primes[0] & ~(q > 1 ? dev::u64(1) << odd_prime_index(q) : 0);
            C.denom_primes[1] = cw.denom_primes[1];
            C.aff = aff_base;
            if (C.count_q / 64 + 2 >= dev::kMaxClassWords)
                throw std::invalid_argument("numerator bound too large for the batched search");
            int smem = 0;
            for (int sl = 0; sl < dev::kWideSlots; ++sl) {
                const int m = sl < int(plan.moduli.size()) ? plan.moduli[sl] : 1;
                const dev::CompositeSpec T = add_composite(sl, round_even(m + dev::kWExt));
                dev::Modulus &Md = C.mod[sl];
                Md.offset = T.offset;
                Md.magic = host_magic(m);
                Md.m = m;
                Md.length = T.length;
                Md.smem_offset = smem;
                smem += T.length;
                Md.inv_stride = m > 1 ? dev::u32(mod_inverse(S % m, m)) : 0;
                Md.neg_h = dev::u32((m - H % m) % m);
                Md.step = dev::u32((dev::kWarpSize * dev::kWK) % m);
            }
            C.smem_words = smem;
            P.wide_smem_words = std::max(P.wide_smem_words, round_even(smem));
            std::copy(cw.adm2, cw.adm2 + 64, C.admissible);
            if (q > 1) {
                class_prime_residues(c.coefficients, q, C.admissible + 64);
                for (int a = 0; a < q; ++a)
                    for (int rq = 0; rq < q; ++rq)
                        C.crt[a * 13 + rq] = (unsigned char)(((rq - a + q) % q) * C.inv64_q % q);
            }
            for (int r64 = 0; r64 < 64; ++r64) C.mod_q[r64] = (unsigned char)(q > 1 ? r64 % q : 0);
            // class starts for every residue r mod M: ofs = (r + H) mod M, and per
            // modulus the row index ((-H + ofs) S^-1) mod m of class word 0
            C.cls = (long long)P.class_starts.size();
            for (long long r = 0; r < M; ++r) {
                dev::ClassStart cs{};
                const long long ofs = (r + H % M) % M;
                cs.ofs = (unsigned short)ofs;
                for (int sl = 0; sl < dev::kWideSlots; ++sl) {
                    const dev::Modulus &Md = C.mod[sl];
                    const long long m = Md.m;
                    cs.start[sl] = (unsigned short)((Md.neg_h + ofs) % m * Md.inv_stride % m);
                }
                P.class_starts.push_back(cs);
            }
            for (int ci = 0; ci < kCandidatePrimes; ++ci) {
                const int p = cands[ci];
                C.neg_h[ci] = (unsigned short)((p - H % p) % p);
                C.s_mod[ci] = (unsigned short)(S % p);
                C.m_mod[ci] = (unsigned short)(M % p);
            }
            device_intervals(c.intervals, C.nint, C.lo, C.hi);
            C.list_max = std::max(1, cw.classes);
            if (C.nint == 0) {
                // room for the curve's class lists (64 q denominator classes)
                const int lm = C.list_max;
                const std::size_t ncombo = std::size_t(64) * std::size_t(q);
                C.list_count = list_count_total;
                C.list_runs = list_runs_total;
                C.list_prefix = list_prefix_total;  // a multiple of 4: rows start 16-byte aligned
                list_count_total += (long long)ncombo;
                list_runs_total += (long long)ncombo * lm;
                list_prefix_total += (long long)ncombo * dev::wide_prefix_stride(lm);
                list_curves.push_back({P.wide.size(), i});  // filled below, in parallel
                // classes of at most 128 words are swept kWK at a time
                const long long max_words = (C.count_q + 1 + 63) >> 6;
                C.list_steps = max_words <= 4 * dev::kWarpSize ? int((max_words + dev::kWarpSize - 1) / dev::kWarpSize) : 0;
            } else {
                C.list_steps = 0;
                C.list_count = -1;
            }
            P.wide_max_classes = std::max(P.wide_max_classes, cw.classes);
            const long long chunk = item_chunk(cw);
            for (int range = 0; range < std::max(1, C.nint); ++range)
                for (long long f = c.first; f <= c.last; f += chunk)
                    P.wide_items.push_back({f, int(P.wide.size()), int(std::min(chunk, c.last - f + 1)),
                                            range, 0});
            P.wide.push_back(C);
            stats.wide_curves += 1;
        } else {
            dev::NarrowCurve C{};
            C.bound = H;
            C.words = cw.words;
            C.square = c.square ? 1 : 0;
            C.index = int(i);
            C.rows = int(plan.moduli.size());
            C.denom_primes[0] = cw.denom_primes[0];
            C.denom_primes[1] = cw.denom_primes[1];
            C.aff = aff_base;
            if (P.row_words % 2) P.row_words += 1;  // 16-byte aligned bulk copy
            C.tables = P.row_words;
            int used = 0;
            for (int sl = 0; sl < dev::kNarrowSlots; ++sl) {
                const int m = sl < int(plan.moduli.size()) ? plan.moduli[sl] : 1;
                const dev::CompositeSpec T = add_composite(sl, m + dev::kNK - 1);
                C.m[sl] = m;
                C.off[sl] = used;
                C.len[sl] = T.length;
                used += m * T.length;
                C.magic[sl] = host_magic(m);
                const long long inv64 = m > 1 ? mod_inverse(64 % m, m) : 0;
                C.shift[sl] = dev::u32(((m - H % m) % m) * inv64 % m);
                C.step[sl] = dev::u32((dev::kWarpSize * dev::kNK) % m);
            }
            if (used % 2) {
                P.row_words += 1;
                used += 1;
            }
            if (used > dev::kNarrowTableWords) throw std::logic_error("narrow tables exceed shared memory");
            C.table_words = used;
            // dense layout: bit j of a word holds a = -H + 64 w + j, so a = j - H (mod 64)
            const dev::u64 *by_class = cw.adm2;
            const int h64 = int(H % 64);
            for (int dd = 0; dd < 64; ++dd)  // bit j = class bit (j - H) mod 64: a rotation
                C.dense2[dd] = h64 ? (by_class[dd] << h64) | (by_class[dd] >> (64 - h64)) : by_class[dd];
            for (int ci = 0; ci < kCandidatePrimes; ++ci) {
                const int p = cands[ci];
                C.neg_h[ci] = (unsigned short)((p - H % p) % p);
            }
            device_intervals(c.intervals, C.nint, C.lo, C.hi);
            const long long chunk = item_chunk(cw);
            for (int range = 0; range < std::max(1, C.nint); ++range)
                for (long long f = c.first; f <= c.last; f += chunk)
                    P.narrow_items.push_back({f, int(P.narrow.size()),
                                              int(std::min(chunk, c.last - f + 1)), range, 0});
            P.narrow.push_back(C);
        }
        stats.curves += 1;
    }
    // class lists by denominator class k = (d mod 64) q + (d mod q), in the
    // order the producer lays out classes for interval curves
    P.list_count.resize(std::size_t(list_count_total));
    P.list_runs.resize(std::size_t(list_runs_total));
    P.list_prefix.resize(std::size_t(list_prefix_total));
    parallel_for(list_curves.size(), [&](std::size_t j) {
        const dev::WideCurve &C = P.wide[list_curves[j].first];
        const CurveWork &cw = P.work[list_curves[j].second];
        const int q = C.class_prime;
        const int lm = C.list_max;
        for (int dd = 0; dd < 64; ++dd)
            for (int dq = 0; dq < q; ++dq) {
                const std::size_t k = std::size_t(dd) * std::size_t(q) + std::size_t(dq);
                const dev::u64 classes2 = cw.adm2[dd];
                const dev::u64 classesq = q > 1 ? C.admissible[64 + dq] : dev::u64(1);
                const int nq = __builtin_popcountll(classesq);
                const int nclass = __builtin_popcountll(classes2) * nq;
                if (nclass > lm) throw std::logic_error("class list longer than its stride");
                dev::WideRun *runs = P.list_runs.data() + C.list_runs + k * std::size_t(lm);
                int *prefix = P.list_prefix.data() + C.list_prefix + k * std::size_t(dev::wide_prefix_stride(lm));
                int items = 0;
                for (int cidx = 0; cidx < nclass; ++cidx) {
                    const int r64 = nth_bit_host(classes2, cidx / nq);
                    int r = r64;
                    if (q > 1) r = r64 + 64 * int(C.crt[C.mod_q[r64] * 13 + nth_bit_host(classesq, cidx % nq)]);
                    const dev::ClassStart &cs = P.class_starts[std::size_t(C.cls + r)];
                    const long long count = C.count_q + (cs.ofs <= C.count_r ? 1 : 0);
                    const long long words = (count + 63) >> 6;
                    dev::WideRun &run = runs[cidx];
                    run.wbase = 0;
                    run.words = int(words);
                    run.ofs = cs.ofs;
                    run.first = 0;
                    run.last = (unsigned char)(words > 0 ? count - 64 * (words - 1) : 64);
                    for (int sl = 0; sl < dev::kWideSlots; ++sl) run.start[sl] = cs.start[sl];
                    prefix[cidx] = items;
                    items += int((words + dev::kWItemWords - 1) / dev::kWItemWords);
                }
                prefix[nclass] = items;
                P.list_count[std::size_t(C.list_count) + k] = nclass;
            }
    });
    stats.wide_items = P.wide_items.size();
    stats.narrow_items = P.narrow_items.size();
    stats.table_words = (unsigned long long)P.row_words;
}

}  // namespace

struct BatchEngine::Impl {
    int device = 0;
    int sms = 0;
    cudaStream_t stream = nullptr, side = nullptr;
    cudaEvent_t ev[6] = {};    // tables, wide kernel, narrow kernel (start, end)
    cudaEvent_t fork = nullptr, join = nullptr;
    // device counters of a run: survivors, wide and narrow work items, error
    // word, survivors kept by pre-verification, words swept, stage-1
    // shared-memory bytes read
    static constexpr int kCounters = 7;
    unsigned long long *h_counters = nullptr;
    unsigned long long capacity = 1ull << 20;
    dev::Candidates cand{};
    DeviceArray<dev::WideCurve> d_wide;
    DeviceArray<dev::NarrowCurve> d_narrow;
    DeviceArray<dev::BatchItem> d_witems, d_nitems;
    DeviceArray<dev::AffineSpec> d_aspecs;
    DeviceArray<dev::PatternSpec> d_pspecs;
    DeviceArray<dev::CompositeSpec> d_cspecs;
    DeviceArray<dev::ClassStart> d_cls;
    DeviceArray<dev::WideRun> d_lruns;
    DeviceArray<int> d_lprefix, d_lcount;
    DeviceArray<unsigned short> d_res, d_inv;
    DeviceArray<dev::u64> d_sq, d_aff, d_patterns, d_rows;
    DeviceArray<dev::OddPrime> d_odd;
    // [0] survivors [1] wide work [2] narrow work [3] error [4] pre-verified survivors
    DeviceArray<unsigned long long> d_counters;
    DeviceArray<long long> d_a, d_pa;        // survivors, and those kept by pre-verification
    DeviceArray<int> d_d, d_c, d_pd, d_pc;
    DeviceArray<unsigned long long> d_curve_modular;  // per-curve modular survivors
    Preverifier pre;

    explicit Impl(int dev_ordinal) {
        if (dev_ordinal >= 0) check_cuda(cudaSetDevice(dev_ordinal), "cudaSetDevice");
        check_cuda(cudaGetDevice(&device), "cudaGetDevice");
        check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device),
                   "cudaDeviceGetAttribute");
        check_cuda(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
        check_cuda(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking), "cudaStreamCreate");
        for (auto &e : ev) check_cuda(cudaEventCreate(&e), "cudaEventCreate");
        check_cuda(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming), "cudaEventCreate");
        check_cuda(cudaEventCreateWithFlags(&join, cudaEventDisableTiming), "cudaEventCreate");
        check_cuda(cudaMallocHost(&h_counters, 8 * sizeof(unsigned long long)), "cudaMallocHost");
        // RPG_BATCH_CAPACITY overrides the first survivor capacity (tests use a
        // small one to exercise the rerun after an overflow)
        if (const char *env = std::getenv("RPG_BATCH_CAPACITY"))
            capacity = (unsigned long long)std::max(1LL, std::atoll(env));
        const auto &cands = candidate_primes();
        for (int ci = 0; ci < kCandidatePrimes; ++ci) {
            cand.p[ci] = cands[ci];
            cand.magic[ci] = dev::magic40(dev::u32(cands[ci]));
        }
        // curve-independent tables: inverses and squares modulo every prime below 512
        std::vector<unsigned short> inv_table(std::size_t(kMaximumPrime) * kMaximumPrime, 0);
        std::vector<dev::u64> square_masks(std::size_t(kMaximumPrime) * dev::kRefWords, 0);
        for (int p = 2; p < kMaximumPrime; ++p) {
            if (!is_small_prime(p)) continue;
            for (int r = 1; r < p; ++r)
                inv_table[std::size_t(p) * kMaximumPrime + r] = (unsigned short)mod_inverse(r, p);
            for (long long v = 0; v < p; ++v) {
                const int sq = int(v * v % p);
                square_masks[std::size_t(p) * dev::kRefWords + sq / 64] |= dev::u64(1) << (sq % 64);
            }
        }
        std::vector<dev::OddPrime> odd;
        for (int p = 3; p < kMaximumPrime; p += 2)
            if (is_small_prime(p)) odd.push_back({dev::u32(p), 0, host_magic(p)});
        if (odd.size() != std::size_t(dev::kOddPrimes)) throw std::logic_error("odd prime table");
        unsigned long long bytes = 0;
        d_inv.upload(inv_table, stream, bytes, "upload inverses");
        d_sq.upload(square_masks, stream, bytes, "upload squares");
        d_odd.upload(odd, stream, bytes, "upload odd primes");
        d_counters.ensure(kCounters, "cudaMalloc(batch counters)");
        ensure_output(capacity);
        check_cuda(cudaStreamSynchronize(stream), "batch engine setup");
    }

    ~Impl() {
        if (stream) cudaStreamSynchronize(stream);
        if (side) cudaStreamSynchronize(side);
        for (auto &e : ev)
            if (e) cudaEventDestroy(e);
        if (fork) cudaEventDestroy(fork);
        if (join) cudaEventDestroy(join);
        if (h_counters) cudaFreeHost(h_counters);
        if (stream) cudaStreamDestroy(stream);
        if (side) cudaStreamDestroy(side);
    }

    void ensure_output(unsigned long long cap) {
        d_a.ensure(cap, "cudaMalloc(batch survivors)");
        d_d.ensure(cap, "cudaMalloc(batch survivors)");
        d_c.ensure(cap, "cudaMalloc(batch survivors)");
        d_pa.ensure(cap, "cudaMalloc(batch survivors)");
        d_pd.ensure(cap, "cudaMalloc(batch survivors)");
        d_pc.ensure(cap, "cudaMalloc(batch survivors)");
    }

    std::vector<BatchCurveResult> run(const std::vector<BatchCurveSpec> &curves, BatchStats *stats_out,
                                      bool use_graph, bool preverify, int items_per_kernel);
};

std::vector<BatchCurveResult> BatchEngine::Impl::run(const std::vector<BatchCurveSpec> &curves,
                                                     BatchStats *stats_out, bool use_graph, bool preverify,
                                                     int items_per_kernel) {
    const auto started = Clock::now();
    BatchStats stats;
    if (items_per_kernel <= 0) {
        items_per_kernel = tuned_batch_items(curves);
        stats.items_from_cache = items_per_kernel > 0;
        if (items_per_kernel <= 0) items_per_kernel = kDefaultBatchItems;
    }
    stats.items_per_kernel = items_per_kernel;
    std::vector<BatchCurveResult> results(curves.size());
    check_cuda(cudaSetDevice(device), "cudaSetDevice");
    // Curves with huge rows fill the device on their own: batching gains them
    // nothing, and the single-curve kernel (row count compiled in, stage 2
    // from class-layout tables) sweeps them faster.  They are validated with
    // the others, then searched one by one in a thread beside the batched
    // kernels.
    std::vector<BatchCurveSpec> batched(curves);
    std::vector<std::size_t> solo;
    std::vector<char> is_solo(curves.size(), 0);
    for (std::size_t i = 0; i < curves.size(); ++i)
        if (curves[i].last >= curves[i].first && curves[i].bound >= 1 &&
            word_count64(curves[i].bound) >= kBatchSoloWords) {
            solo.push_back(i);
            is_solo[i] = 1;
            batched[i].first = 1;
            batched[i].last = 0;
        }
    BatchPlan P;
    const auto t_plan = Clock::now();
    build_plan(batched, results, P, stats, items_per_kernel);
    stats.plan_ms = ms_since(t_plan);
    const std::vector<CurveWork> &work = P.work;
    std::exception_ptr solo_error;
    std::thread solo_thread;
    struct Joiner {
        std::thread &t;
        ~Joiner() {
            if (t.joinable()) t.join();
        }
    } joiner{solo_thread};
    if (!solo.empty())
        solo_thread = std::thread([&] {
            try {
                check_cuda(cudaSetDevice(device), "cudaSetDevice");
                for (std::size_t i : solo) {
                    if (results[i].status != 0) continue;
                    const BatchCurveSpec &c = curves[i];
                    SearchOptions o;
                    o.coefficients = c.coefficients;
                    o.numerator_bound = c.bound;
                    o.first = c.first;
                    o.last = c.last;
                    o.intervals = c.intervals;
                    o.include_infinity = false;  // added below with the batched curves'
                    o.devices = {device};
                    o.square = c.square;
                    o.plan = PlanKind::fast;
                    o.device_preverify = preverify;
                    PointSearch search(o);
                    std::vector<PointPair> found;
                    const SearchMetrics m = search.run([&](const PointPair &p) {
                        found.push_back(p);
                        return true;
                    });
                    results[i].points = std::move(found);
                    results[i].survivors = m.modular_survivors;
                    results[i].wide = true;
                    results[i].solo = true;
                }
            } catch (...) {
                solo_error = std::current_exception();
            }
        });

    if (!P.wide.empty() || !P.narrow.empty()) {
        d_wide.upload(P.wide, stream, stats.h2d_bytes, "upload wide curves");
        d_narrow.upload(P.narrow, stream, stats.h2d_bytes, "upload narrow curves");
        d_witems.upload(P.wide_items, stream, stats.h2d_bytes, "upload work items");
        d_nitems.upload(P.narrow_items, stream, stats.h2d_bytes, "upload work items");
        d_aspecs.upload(P.aspecs, stream, stats.h2d_bytes, "upload bitmask specs");
        d_pspecs.upload(P.pspecs, stream, stats.h2d_bytes, "upload pattern specs");
        d_cspecs.upload(P.cspecs, stream, stats.h2d_bytes, "upload table specs");
        d_res.upload(P.residues, stream, stats.h2d_bytes, "upload residues");
        d_cls.upload(P.class_starts, stream, stats.h2d_bytes, "upload class starts");
        d_lruns.upload(P.list_runs, stream, stats.h2d_bytes, "upload class lists");
        d_lprefix.upload(P.list_prefix, stream, stats.h2d_bytes, "upload class lists");
        d_lcount.upload(P.list_count, stream, stats.h2d_bytes, "upload class lists");
        d_aff.ensure(std::size_t(P.aff_words), "cudaMalloc(batch bitmasks)");
        d_patterns.ensure(std::size_t(P.pattern_words), "cudaMalloc(batch patterns)");
        d_rows.ensure(std::size_t(P.row_words), "cudaMalloc(batch tables)");
        if (preverify) {
            std::vector<const std::vector<std::string> *> coefs(curves.size(), nullptr);
            for (std::size_t i = 0; i < curves.size(); ++i)
                if (work[i].ok) coefs[i] = &curves[i].coefficients;
            pre.prepare(coefs, stream);
            stats.h2d_bytes += pre.upload_bytes();
            d_curve_modular.ensure(std::max<std::size_t>(1, curves.size()), "cudaMalloc(batch counters)");
        }

        const int wide_smem_words = P.wide_smem_words;
        const int wide_max_classes = P.wide_max_classes;
        const std::size_t wide_smem = std::size_t(dev::kWSlotCount) * std::size_t(wide_smem_words) * 8 +
                                      std::size_t(dev::kWConsumers) * dev::kQueue * 16 +
                                      std::size_t(dev::kWSlotCount) * std::size_t(wide_max_classes) *
                                          sizeof(dev::WideRun) +
                                      std::size_t(dev::kWSlotCount) * std::size_t(dev::wide_prefix_stride(wide_max_classes)) * 4;
        const std::size_t narrow_smem = std::size_t(dev::kNarrowTableWords + dev::kAffWords) * 8 +
                                        std::size_t(dev::kNWarps) * dev::kQueue * 12;
        int wide_grid = 0, narrow_grid = 0;
        if (!P.wide.empty()) {
            int per_sm = 0;
            check_cuda(cudaFuncSetAttribute(dev::wide_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            int(wide_smem)),
                       "cudaFuncSetAttribute");
            check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dev::wide_kernel,
                                                                     dev::kWThreads, wide_smem),
                       "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
            wide_grid = std::max(1, std::min<int>(sms * std::max(1, per_sm), int(P.wide_items.size())));
        }
        if (!P.narrow.empty()) {
            int per_sm = 0;
            check_cuda(cudaFuncSetAttribute(dev::narrow_kernel,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize, int(narrow_smem)),
                       "cudaFuncSetAttribute");
            check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dev::narrow_kernel,
                                                                     dev::kNThreads, narrow_smem),
                       "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
            narrow_grid = std::max(1, std::min<int>(sms * std::max(1, per_sm), int(P.narrow_items.size())));
        }

        // external records become event nodes when the stream is captured
        bool capturing = false;
        auto record = [&](cudaEvent_t e, cudaStream_t s) {
            check_cuda(capturing ? cudaEventRecordWithFlags(e, s, cudaEventRecordExternal)
                                 : cudaEventRecord(e, s),
                       "cudaEventRecord");
        };
        auto enqueue_sieve = [&]() {
            const dev::BatchOut out{d_a.p, d_d.p, d_c.p, d_counters.p, capacity, d_counters.p + 3};
            check_cuda(cudaMemsetAsync(d_counters.p, 0, kCounters * sizeof(unsigned long long), stream),
                       "cudaMemsetAsync");
            if (preverify)
                check_cuda(cudaMemsetAsync(d_curve_modular.p, 0, curves.size() * sizeof(unsigned long long), stream),
                           "cudaMemsetAsync");
            check_cuda(cudaEventRecord(fork, stream), "cudaEventRecord");
            check_cuda(cudaStreamWaitEvent(side, fork, 0), "cudaStreamWaitEvent");
            record(ev[2], stream);
            if (wide_grid) {
                dev::wide_kernel<<<wide_grid, dev::kWThreads, wide_smem, stream>>>(
                    d_wide.p, d_witems.p, int(P.wide_items.size()), d_rows.p, d_aff.p, d_cls.p, d_lruns.p,
                    d_lprefix.p, d_lcount.p, d_inv.p, d_odd.p, cand, out, wide_smem_words, wide_max_classes,
                    d_counters.p + 1, d_counters.p + 5);
                check_cuda(cudaGetLastError(), "wide_kernel launch");
            }
            record(ev[3], stream);
            record(ev[4], side);
            if (narrow_grid) {
                dev::narrow_kernel<<<narrow_grid, dev::kNThreads, narrow_smem, side>>>(
                    d_narrow.p, d_nitems.p, int(P.narrow_items.size()), d_rows.p, d_aff.p, d_inv.p,
                    d_odd.p, cand, out, d_counters.p + 2, d_counters.p + 5);
                check_cuda(cudaGetLastError(), "narrow_kernel launch");
            }
            record(ev[5], side);
            check_cuda(cudaEventRecord(join, side), "cudaEventRecord");
            check_cuda(cudaStreamWaitEvent(stream, join, 0), "cudaStreamWaitEvent");
            if (preverify)
                pre.launch(d_a.p, d_d.p, d_c.p, d_counters.p, capacity, d_pa.p, d_pd.p, d_pc.p, d_counters.p + 4,
                           d_curve_modular.p, stream);
            check_cuda(cudaMemcpyAsync(h_counters, d_counters.p, kCounters * sizeof(unsigned long long),
                                       cudaMemcpyDeviceToHost, stream),
                       "download batch counters");
        };
        auto enqueue_all = [&]() {
            record(ev[0], stream);
            const long long aff_threads = (long long)P.aspecs.size() * dev::kRefWords;
            if (aff_threads) {
                dev::affine_kernel<<<unsigned((aff_threads + 255) / 256), 256, 0, stream>>>(
                    d_aspecs.p, (long long)P.aspecs.size(), d_res.p, d_sq.p, d_aff.p);
                check_cuda(cudaGetLastError(), "affine_kernel launch");
            }
            if (P.pattern_words) {
                dev::pattern_kernel<<<unsigned((P.pattern_words + 256 * dev::kPatternWords - 1) /
                                               (256 * dev::kPatternWords)),
                                      256, 0, stream>>>(
                    d_pspecs.p, int(P.pspecs.size()), d_aff.p, d_inv.p, d_patterns.p, P.pattern_words);
                check_cuda(cudaGetLastError(), "pattern_kernel launch");
            }
            if (P.row_words) {
                dev::composite_kernel<<<unsigned((P.row_words + 256 * dev::kCompositeWords - 1) /
                                                 (256 * dev::kCompositeWords)),
                                        256, 0, stream>>>(
                    d_cspecs.p, int(P.cspecs.size()), d_patterns.p, d_rows.p, P.row_words);
                check_cuda(cudaGetLastError(), "composite_kernel launch");
            }
            record(ev[1], stream);
            enqueue_sieve();
        };
        if (use_graph) {
            cudaGraph_t graph = nullptr;
            cudaGraphExec_t exec = nullptr;
            check_cuda(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal),
                       "cudaStreamBeginCapture");
            capturing = true;
            try {
                enqueue_all();
            } catch (...) {
                capturing = false;
                cudaStreamEndCapture(stream, &graph);
                if (graph) cudaGraphDestroy(graph);
                throw;
            }
            capturing = false;
            check_cuda(cudaStreamEndCapture(stream, &graph), "cudaStreamEndCapture");
            const cudaError_t inst = cudaGraphInstantiate(&exec, graph, 0);
            cudaGraphDestroy(graph);
            check_cuda(inst, "cudaGraphInstantiate");
            const cudaError_t launched = cudaGraphLaunch(exec, stream);
            const cudaError_t synced = cudaStreamSynchronize(stream);
            cudaGraphExecDestroy(exec);
            check_cuda(launched, "cudaGraphLaunch");
            check_cuda(synced, "batch graph");
            stats.graph = true;
        } else {
            enqueue_all();
            check_cuda(cudaStreamSynchronize(stream), "batch sieve");
        }
        stats.launches += (P.aspecs.empty() ? 0 : 1) + (P.pattern_words ? 1 : 0) + (P.row_words ? 1 : 0) +
                          (wide_grid ? 1 : 0) + (narrow_grid ? 1 : 0) + (preverify ? 1 : 0);
        auto elapsed = [&](int a, int b) {
            float ms = 0;
            cudaEventElapsedTime(&ms, ev[a], ev[b]);
            return double(ms);
        };
        stats.table_ms = elapsed(0, 1);
        stats.wide_ms = elapsed(2, 3);
        stats.narrow_ms = elapsed(4, 5);
        stats.sieve_ms = std::max(elapsed(2, 3), elapsed(2, 5));
        if (h_counters[3]) throw DeviceTimeout("batched sieve: a bounded wait for a table copy timed out");
        while (h_counters[0] > capacity) {  // survivors did not fit: run again with room for all
            capacity = h_counters[0] + (h_counters[0] >> 3) + 1024;
            ensure_output(capacity);
            enqueue_sieve();
            check_cuda(cudaStreamSynchronize(stream), "batch sieve");
            stats.sieve_ms += std::max(elapsed(2, 3), elapsed(2, 5));
            stats.launches += (wide_grid ? 1 : 0) + (narrow_grid ? 1 : 0) + (preverify ? 1 : 0);
            if (h_counters[3]) throw DeviceTimeout("batched sieve: a bounded wait timed out");
        }
        stats.survivors = h_counters[0];
        stats.swept_words = h_counters[5];
        stats.smem_bytes = h_counters[6];
        // survivors for the host: those kept by pre-verification, or all
        const std::size_t n = std::size_t(preverify ? h_counters[4] : h_counters[0]);
        stats.host_candidates = n;
        std::vector<long long> ha(n);
        std::vector<int> hd(n), hc(n);
        std::vector<unsigned long long> curve_modular(preverify ? curves.size() : 0);
        if (n) {
            check_cuda(cudaMemcpyAsync(ha.data(), preverify ? d_pa.p : d_a.p, n * sizeof(long long),
                                       cudaMemcpyDeviceToHost, stream),
                       "download batch survivors");
            check_cuda(cudaMemcpyAsync(hd.data(), preverify ? d_pd.p : d_d.p, n * sizeof(int),
                                       cudaMemcpyDeviceToHost, stream),
                       "download batch survivors");
            check_cuda(cudaMemcpyAsync(hc.data(), preverify ? d_pc.p : d_c.p, n * sizeof(int),
                                       cudaMemcpyDeviceToHost, stream),
                       "download batch survivors");
        }
        if (!curve_modular.empty())
            check_cuda(cudaMemcpyAsync(curve_modular.data(), d_curve_modular.p,
                                       curve_modular.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                       stream),
                       "download batch survivor counts");
        check_cuda(cudaStreamSynchronize(stream), "download batch survivors");
        stats.d2h_bytes += n * (sizeof(long long) + 2 * sizeof(int)) + kCounters * sizeof(unsigned long long) +
                           curve_modular.size() * sizeof(unsigned long long);

        // ---- exact verification per curve, in single-search order ----
        const auto t_verify = Clock::now();
        std::vector<std::vector<std::size_t>> by_curve(curves.size());
        for (std::size_t s = 0; s < n; ++s) by_curve[std::size_t(hc[s])].push_back(s);
        parallel_for(curves.size(), [&](std::size_t i) {
            if (!work[i].ok) return;
            BatchCurveResult &r = results[i];
            const ExactPolynomial &poly = *work[i].poly;
            std::vector<PointPair> found;
            std::string root;
            for (std::size_t s : by_curve[i]) {
                if (gcd_ll(ha[s], hd[s]) != 1) continue;
                if (poly.square_root(ha[s], hd[s], root)) found.push_back(PointPair{ha[s], root, hd[s]});
            }
            std::sort(found.begin(), found.end(), [](const PointPair &a, const PointPair &b) {
                return a.denominator != b.denominator ? a.denominator < b.denominator
                                                      : a.numerator < b.numerator;
            });
            SearchOptions filter;
            filter.intervals = curves[i].intervals;
            for (auto &p : found)
                if (filter.accepts(p.numerator, p.denominator)) r.points.push_back(std::move(p));
            r.survivors = preverify ? curve_modular[i] : by_curve[i].size();
        });
        stats.verify_ms = ms_since(t_verify);
    }
    // the point at infinity first, as a single search reports it
    parallel_for(curves.size(), [&](std::size_t i) {
        if (!work[i].ok || !curves[i].include_infinity || is_solo[i]) return;
        std::string root;
        if (work[i].poly->square_root(1, 0, root))
            results[i].points.insert(results[i].points.begin(), PointPair{1, root, 0});
    });
    if (solo_thread.joinable()) solo_thread.join();
    if (solo_error) std::rethrow_exception(solo_error);
    for (std::size_t i : solo)
        if (results[i].status == 0) {
            const BatchCurveSpec &c = curves[i];
            const long long count = c.last - c.first + 1;
            ++stats.solo_curves;
            ++stats.curves;
            ++stats.wide_curves;
            stats.survivors += results[i].survivors;
            stats.denominators += (unsigned long long)count;
            stats.rectangle_sites += (long double)(2 * c.bound + 1) * (long double)count;
        }
    // the point at infinity first, as a single search reports it
    parallel_for(solo.size(), [&](std::size_t j) {
        const std::size_t i = solo[j];
        if (!work[i].ok || !curves[i].include_infinity) return;
        std::string root;
        if (work[i].poly->square_root(1, 0, root))
            results[i].points.insert(results[i].points.begin(), PointPair{1, root, 0});
    });
    for (const auto &r : results) stats.points += r.points.size();
    stats.wall_ms = ms_since(started);
    if (stats_out) *stats_out = stats;
    return results;
}

BatchEngine::BatchEngine(int device) : impl_(new Impl(device)) {}
BatchEngine::~BatchEngine() = default;

std::vector<BatchCurveResult> BatchEngine::run(const std::vector<BatchCurveSpec> &curves,
                                               BatchStats *stats, bool use_graph, bool preverify,
                                               int items_per_kernel) {
    return impl_->run(curves, stats, use_graph, preverify, items_per_kernel);
}

int BatchEngine::device() const { return impl_->device; }

unsigned long long BatchEngine::estimate_bytes(const BatchCurveSpec &c) {
    const long long words = word_count64(std::max(1LL, c.bound));
    const long long count = c.last >= c.first ? c.last - c.first + 1 : 0;
    long long table;
    if (words >= kBatchWideWords) {
        const double cap = std::min<double>(kMaxModulus, std::max(64.0, std::sqrt(double(words) * count / 48.0)));
        table = (long long)(6.0 * cap * (cap + dev::kWExt));
    } else {
        table = dev::kNarrowTableWords;
    }
    // tables, bitmasks, patterns, descriptor and items (8-byte words)
    return (unsigned long long)(table + 2 * dev::kAffWords + 6 * 127 * 127 + 1024 +
                                std::max(1LL, count * std::max(1LL, (long long)c.intervals.size()) /
                                                  64)) * 8ull;
}

std::vector<BatchCurveResult> batch_search(const std::vector<BatchCurveSpec> &curves, int device,
                                           BatchStats *stats, bool use_graph, bool preverify) {
    BatchEngine engine(device);
    return engine.run(curves, stats, use_graph, preverify);
}

}  // namespace rpg
