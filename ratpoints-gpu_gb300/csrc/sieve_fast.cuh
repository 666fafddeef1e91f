// Fast-plan sieve kernels (this project's plan; see plan.hpp).
//
// Class-strided layout.  For a denominator d only the numerator classes
// a = r (mod 64) with F(r, d) a square modulo 64 (and r odd when d is even)
// can hold points.  Each admissible class is swept on its own: word w of class
// r holds the 64 sites a = a0 + 4096 w + 64 j (j = bit), a0 the least a >= -H
// with a = r (mod 64).  For an odd modulus m, 4096 is invertible, so along a
// class the mask of m is periodic in w with period m and one table row per
// (m, d mod m) serves every class: class r starts at row index
// s = a0 * 4096^-1 (mod m).  Tables therefore do not depend on H.
//
// Stage 1 ANDs the rows of up to kFastSlots composite moduli of small primes,
// staged in shared memory per denominator; surviving words go through a
// per-warp queue to stage 2, which checks the reference's 32 selected primes
// (same selection as the reference plan) from class-layout tables in global
// memory, then emits (a, d).  Survivors are a subset of the reference plan's.
#pragma once

#include "plan.hpp"
#include "sieve_device.cuh"

namespace rpg {
namespace dev {

constexpr int kFastSlots = 5;       // stage-1 moduli
constexpr int kFastMaxFactors = 3;  // primes per stage-1 modulus
constexpr int kFK = 2;              // words per lane per step (lanes 32 apart)
constexpr int kFWarps = 4;
constexpr int kFThreads = kFWarps * kWarpSize;
constexpr int kFSteps = 8;                                 // steps per work item
constexpr int kFItemWords = kWarpSize * kFK * kFSteps;     // 512 words per item
constexpr int kFExt = kWarpSize * (kFK - 1);               // row extension
constexpr int kFQueue = 64;
constexpr int kFClassBits = 6;                             // 64 classes
constexpr long long kFMaxClassWords = 1LL << 25;           // word offset fits 26 bits
constexpr int kFFetch = 4;                                 // denominators per fetch

struct FastModulus {
    int m;                         // modulus (odd)
    int nf;                        // number of prime factors
    int q[kFastMaxFactors];        // prime factors
    int length;                    // row length in words (m + kFExt, even)
    long long offset;              // word offset of row 0 in the table
    int smem_offset;               // word offset of the staged row in shared memory
    u32 inv4096;                   // 4096^-1 mod m
    u32 neg_h;                     // (-H) mod m
    u32 wlo_mod;                   // first word of the launch's tile, mod m
    unsigned long long magic;      // ceil(2^64 / m) for 32-bit n mod m
};

struct FastPrime {                 // one of the 36 reference candidates, class layout
    long long offset;              // word offset of row 0 (rows of length p)
    int p;
    u32 inv4096;                   // 4096^-1 mod p
    u32 neg_h;                     // (-H) mod p
    u32 magic;                     // magic40(p)
    u32 wlo_mod;                   // first word of the launch's tile, mod p
};

struct FastTables {
    const u64 *rows;               // stage-1 modulus tables
    const u64 *prime_rows;         // reference candidate tables (class layout)
    const u64 *admissible;         // [64]: bit r set iff class r may hold points for d = index (mod 64)
    FastModulus mod[kFastSlots];
    int h_mod64;                   // H mod 64
    FastPrime prime[kCandidatePrimes];
    int slots;                     // stage-1 moduli in use
    int smem_words;                // staged row words
};

__device__ __forceinline__ u32 mod_u32(u32 n, u32 m, unsigned long long magic) {
    u32 q = u32(__umul64hi((unsigned long long)n, magic));
    u32 r = n - q * m;
    return r >= m ? r - m : r;
}

// One 64-bit word of a class-layout row: bit j for the sites congruent to
// 4096 u + 64 j (mod q) of a denominator with residue rho (mod q).
__device__ __forceinline__ bool prime_bit(const unsigned char *affine, const unsigned short *inverse,
                                          int q, int rho, int lead_ok, int x) {
    if (rho == 0) return x != 0 && lead_ok;  // q | d: need q !| a, and c_n square mod q (even n)
    return affine[(x * inverse[rho]) % q] != 0;
}


// Description of one class-layout table: m rows of `length` words, bit j of
// word u of row rho = AND over the prime factors q of prime_bit(.., rho mod q,
// (4096 u + 64 j) mod q).
struct TableSpec {
    long long offset;
    int m;
    int nf;
    int q[kFastMaxFactors];
    int length;
    int factor_base[kFastMaxFactors];   // offset of q's affine/inverse arrays
    int lead_ok[kFastMaxFactors];
};

__global__ void class_table_kernel(u64 *rows, const TableSpec *specs, int nspecs,
                                   const unsigned char *affine, const unsigned short *inverse,
                                   long long total) {
    const long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (id >= total) return;
    int t = 0;
    while (t + 1 < nspecs && specs[t + 1].offset <= id) ++t;
    const TableSpec &S = specs[t];
    const long long rel = id - S.offset;
    const int rho = int(rel / S.length);
    const int u = int(rel % S.length) % S.m;
    u64 word = ~u64(0);
    for (int f = 0; f < S.nf; ++f) {
        const int q = S.q[f];
        const unsigned char *aff = affine + S.factor_base[f];
        const unsigned short *inv = inverse + S.factor_base[f];
        const int rq = rho % q;
        int x = int((4096LL * u) % q);
        const int step = 64 % q;
        u64 bits = 0;
        for (int j = 0; j < 64; ++j) {
            if (prime_bit(aff, inv, q, rq, S.lead_ok[f], x)) bits |= u64(1) << j;
            x += step;
            if (x >= q) x -= q;
        }
        word &= bits;
    }
    rows[id] = word;
}

// Stage 2 for up to 32 queued class words (one per lane), then emission.
__device__ __forceinline__ void fast_drain(const u64 *qmask, const u32 *qinfo, int start, int n,
                                           const FastTables &T, const SieveArgs &A,
                                           int denominator, const int *s_sel,
                                           const long long *s_prow) {
    const int lane = threadIdx.x & 31;
    u64 m = 0;
    u32 info = 0;
    if (lane < n) {
        m = qmask[start + lane];
        info = qinfo[start + lane];
    }
    __syncwarp();
    const u32 off = info >> kFClassBits;
    const int r = int(info & ((1u << kFClassBits) - 1));
    const int ofs = (r + T.h_mod64) & 63;             // (r + H) mod 64
    const long long a0 = -A.bound + ofs;              // least a >= -H in class r
    const long long w = A.w_lo + off;
    if (m) {
        for (int s = 0; s < kSelectedPrimes; ++s) {
            const FastPrime &P = T.prime[s_sel[s]];
            const u32 p = u32(P.p);
            u32 a0m = P.neg_h + u32(ofs);
            if (a0m >= p) a0m -= p;
            u32 u = mod_small(a0m * P.inv4096, p, P.magic);
            u += P.wlo_mod;
            if (u >= p) u -= p;
            u += mod_small(off, p, P.magic);
            if (u >= p) u -= p;
            m &= __ldg(T.prime_rows + s_prow[s] + u);
            if (!m) break;
        }
    }
    // emission: a = a0 + 4096 w + 64 j
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
    unsigned long long pos = base + incl - cnt;
    const long long abase = a0 + 4096LL * w;
    while (m) {
        const int bit = __ffsll((long long)m) - 1;
        m &= m - 1;
        if (pos < A.capacity) {
            A.out_a[pos] = abase + 64LL * bit;
            A.out_d[pos] = denominator;
        }
        ++pos;
    }
}

__global__ void __launch_bounds__(kFThreads) fast_sieve_kernel(FastTables T, SieveArgs A,
                                                               unsigned long long *work) {
    extern __shared__ __align__(16) u64 smem[];
    u64 *rows = smem;
    u64 *qmask = rows + T.smem_words;
    u32 *qinfo = reinterpret_cast<u32 *>(qmask + kFWarps * kFQueue);

    __shared__ long long s_items[kFFetch];
    __shared__ int s_nitems;
    __shared__ int s_nclass;
    __shared__ unsigned char s_class[64];
    __shared__ int s_wtile[64];           // words of the class inside this launch's tile
    __shared__ int s_last_bits[64];       // valid bits of the class's last word (64 if full)
    __shared__ int s_last_word[64];       // tile offset of the class's last word, or -1
    __shared__ int s_prefix[65];          // work items before class index c
    __shared__ u32 s_start[64][kFastSlots];
    __shared__ int s_sel[kSelectedPrimes];
    __shared__ long long s_prow[kSelectedPrimes];
    __shared__ int s_next;

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    u64 *wq_mask = qmask + warp * kFQueue;
    u32 *wq_info = qinfo + warp * kFQueue;
    const long long class_sites_total = 2 * A.bound + 1;

    for (;;) {
        if (threadIdx.x == 0) {
            const unsigned long long base = atomicAdd(work, (unsigned long long)kFFetch);
            int n = 0;
            for (int i = 0; i < kFFetch; ++i)
                if (base + i < (unsigned long long)A.k_count) s_items[n++] = (long long)base + i;
            s_nitems = n;
        }
        __syncthreads();
        const int nitems = s_nitems;
        if (nitems == 0) break;
        for (int it = 0; it < nitems; ++it) {
            const long long k = A.k_first + s_items[it];
            const long long d = A.square ? k * k : k;
            const u64 classes = __ldg(T.admissible + (d & 63));
            if (!classes) continue;

            // ---- per-denominator setup ----
            if (warp == 0) {
                // The 32 largest candidates not dividing d (d < 2^31): lane l tests
                // candidate 35 - l, lanes 0..3 also candidate 3 - l.
                const u32 du = u32(d);
                const int ch = kCandidatePrimes - 1 - lane;
                const u32 rh = du % u32(T.prime[ch].p);
                const u32 hi_div = __ballot_sync(kFullMask, rh == 0);
                const int cl = kCandidatePrimes - 1 - 32 - lane;
                const u32 rl = lane < kCandidatePrimes - 32 ? du % u32(T.prime[cl].p) : 1u;
                const u32 lo_div = __ballot_sync(kFullMask, rl == 0);
                const u32 below = lanemask_lt();
                const int rank_h = lane - __popc(hi_div & below);
                if (rh != 0 && rank_h < kSelectedPrimes) {
                    s_sel[rank_h] = ch;
                    s_prow[rank_h] = T.prime[ch].offset + (long long)rh * T.prime[ch].p;
                }
                const int rank_l = 32 - __popc(hi_div) + lane - __popc(lo_div & below);
                if (lane < kCandidatePrimes - 32 && rl != 0 && rank_l < kSelectedPrimes) {
                    s_sel[rank_l] = cl;
                    s_prow[rank_l] = T.prime[cl].offset + (long long)rl * T.prime[cl].p;
                }
                if (lane == 0) {
                    s_nclass = __popcll(classes);
                    s_next = 0;
                }
            }
            if (threadIdx.x < 64 && ((classes >> threadIdx.x) & 1)) {
                const int r = threadIdx.x;
                const int c = __popcll(classes & ((u64(1) << r) - 1));
                const int ofs = (r + T.h_mod64) & 63;
                // sites of class r: a = -H + ofs + 64 t, t in [0, count)
                const long long count = ofs < class_sites_total ? (class_sites_total - 1 - ofs) / 64 + 1 : 0;
                const long long words = (count + 63) / 64;
                const long long lo = A.w_lo < words ? A.w_lo : words;  // tile start (class words)
                const long long hi = A.w_hi < words ? A.w_hi : words;
                s_class[c] = (unsigned char)r;
                s_wtile[c] = int(hi - lo);
                const bool has_last = hi == words && words > 0 && hi > lo;
                s_last_word[c] = has_last ? int(words - 1 - lo) : -1;
                s_last_bits[c] = has_last ? int(count - 64 * (words - 1)) : 64;
                for (int sl = 0; sl < T.slots; ++sl) {
                    // row index of tile word 0: (a0 * 4096^-1 + w_lo) mod m, a0 = -H + ofs
                    const FastModulus &M = T.mod[sl];
                    const u32 a0m = mod_u32(M.neg_h + u32(ofs), u32(M.m), M.magic);
                    s_start[c][sl] = mod_u32(a0m * M.inv4096 + M.wlo_mod, u32(M.m), M.magic);
                }
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                int acc = 0;
                for (int c = 0; c < s_nclass; ++c) {
                    s_prefix[c] = acc;
                    acc += (s_wtile[c] + kFItemWords - 1) / kFItemWords;
                }
                s_prefix[s_nclass] = acc;
            }
            // stage the stage-1 rows of this denominator
            for (int sl = 0; sl < T.slots; ++sl) {
                const FastModulus &M = T.mod[sl];
                const int rho = int(d % M.m);
                const uint4 *src = reinterpret_cast<const uint4 *>(T.rows + M.offset + (long long)rho * M.length);
                uint4 *dst = reinterpret_cast<uint4 *>(rows + M.smem_offset);
                const int n16 = M.length >> 1;
                for (int t = threadIdx.x; t < n16; t += kFThreads) dst[t] = __ldg(src + t);
            }
            __syncthreads();

            // ---- sweep: warps take work items (class, 256-word chunk) ----
            const int nclass = s_nclass;
            const int total_items = s_prefix[nclass];
            int qn = 0;
            for (;;) {
                int item = 0;
                if (lane == 0) item = atomicAdd(&s_next, 1);
                item = __shfl_sync(kFullMask, item, 0);
                if (item >= total_items) break;
                // class index: largest c with s_prefix[c] <= item
                int c = 0;
                {
                    const int c0 = lane, c1 = lane + 32;
                    const bool b0 = c0 < nclass && s_prefix[c0] <= item;
                    const bool b1 = c1 < nclass && s_prefix[c1] <= item;
                    const u32 m0 = __ballot_sync(kFullMask, b0);
                    const u32 m1 = __ballot_sync(kFullMask, b1);
                    c = m1 ? 32 + 31 - __clz(m1) : 31 - __clz(m0);
                }
                const int w0 = (item - s_prefix[c]) * kFItemWords;
                const int wt = s_wtile[c];
                const int last_word = s_last_word[c];
                const u64 last_mask = s_last_bits[c] >= 64 ? ~u64(0) : ((u64(1) << s_last_bits[c]) - 1);
                const u32 cls = s_class[c];
                u32 o[kFastSlots];
                u32 mo[kFastSlots];
#pragma unroll
                for (int sl = 0; sl < kFastSlots; ++sl) {
                    if (sl < T.slots) {
                        const FastModulus &M = T.mod[sl];
                        const u32 r0 = mod_u32(s_start[c][sl] + u32(w0 + lane), u32(M.m), M.magic);
                        o[sl] = r0;
                        mo[sl] = u32(M.m);
                    } else {
                        o[sl] = 0;
                        mo[sl] = 1u << 30;
                    }
                }
#pragma unroll 1
                for (int step = 0; step < kFSteps; ++step) {
                    const int ws = w0 + step * kWarpSize * kFK;
                    if (ws >= wt) break;
                    u64 acc0 = ~u64(0), acc1 = ~u64(0);
#pragma unroll
                    for (int sl = 0; sl < kFastSlots; ++sl) {
                        if (sl < T.slots) {
                            const u64 *row = rows + T.mod[sl].smem_offset + o[sl];
                            acc0 &= row[0];
                            acc1 &= row[kWarpSize];
                            u32 t = o[sl] + kWarpSize * kFK;
                            o[sl] = t >= mo[sl] ? t - mo[sl] : t;
                        }
                    }
#pragma unroll
                    for (int kk = 0; kk < kFK; ++kk) {
                        const int w = ws + kWarpSize * kk + lane;
                        u64 acc = kk == 0 ? acc0 : acc1;
                        if (w == last_word) acc &= last_mask;
                        const bool live = acc != 0 && w < wt;
                        const u32 b = __ballot_sync(kFullMask, live);
                        if (b) {
                            const int pos = qn + __popc(b & lanemask_lt());
                            if (live) {
                                wq_mask[pos] = acc;
                                wq_info[pos] = (u32(w) << kFClassBits) | cls;
                            }
                            qn += __popc(b);
                            if (qn >= 32) {
                                __syncwarp();
                                fast_drain(wq_mask, wq_info, qn - 32, 32, T, A, int(d), s_sel, s_prow);
                                qn -= 32;
                            }
                        }
                    }
                }
            }
            __syncwarp();
            fast_drain(wq_mask, wq_info, 0, qn, T, A, int(d), s_sel, s_prow);
            __syncthreads();
        }
        __syncthreads();
    }
}

}  // namespace dev
}  // namespace rpg
