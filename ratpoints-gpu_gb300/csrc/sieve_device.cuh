// Device-side pieces of the modular square sieve shared by the sieve kernels.
//
// Site layout: for a search bound H, the numerators a in [-H, H] of one
// denominator d form a row of 64-site words; word w holds a = -H + 64 w + j in
// bit j.  The reference uses 32-site words (src/sieve.cu:179-181); the site set
// and the survivor set are the same.
#pragma once

#include <cstdint>

namespace rpg {
namespace dev {

using u32 = std::uint32_t;
using u64 = std::uint64_t;

constexpr int kWarpSize = 32;
constexpr unsigned kFullMask = 0xffffffffu;

// Arguments of one sieve launch: parameters k_first .. k_first + k_count - 1
// (denominators k, or k*k when square), word range [w_lo, w_hi) of each row,
// and the survivor output (structure of arrays, capacity entries).
struct SieveArgs {
    long long bound;     // H
    long long words;     // words per denominator row (64-site words)
    long long w_lo;
    long long w_hi;
    long long k_first;
    int k_count;
    int square;
    long long *out_a;
    int *out_d;
    unsigned long long *out_count;
    unsigned long long capacity;
    unsigned long long *error;   // set nonzero if a bounded device wait ran out (may be null)
};

// Quotient estimate for n mod p with n < 2^31 and 257 <= p < 2^9 (the
// reference's candidate primes): q = (n * ceil(2^40 / p)) >> 40 is exact in
// that range.  Below 257, ceil(2^40 / p) does not fit 32 bits: use mod_u32.
__host__ __device__ inline u32 magic40(u32 p) {
    return u32(((u64(1) << 40) + p - 1) / p);
}
__device__ __forceinline__ u32 mod_small(u32 n, u32 p, u32 magic) {
    u32 q = u32((u64(n) * magic) >> 40);
    return n - q * p;
}

__device__ __forceinline__ u32 mod_u32(u32 n, u32 m, unsigned long long magic) {
    u32 q = u32(__umul64hi((unsigned long long)n, magic));
    u32 r = n - q * m;
    return r >= m ? r - m : r;
}

// Three-input AND and OR (one lop3 each).
__device__ __forceinline__ u32 and3(u32 a, u32 b, u32 c) {
    u32 d;
    asm("lop3.b32 %0, %1, %2, %3, 0x80;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}
__device__ __forceinline__ u32 or3(u32 a, u32 b, u32 c) {
    u32 d;
    asm("lop3.b32 %0, %1, %2, %3, 0xFE;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}

// Shared-memory address, mbarrier and bulk-copy (TMA, non-tensor) helpers.
__device__ __forceinline__ u32 smem_addr(const void *p) {
    return u32(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(u32 bar, u32 count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(u32 bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(u32 bar, u32 bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(u32 bar, u32 parity) {
    u32 done;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; "
        "selp.u32 %0, 1, 0, p; }"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    return done != 0;
}
// Bounded wait for the phase with the given parity; false if the limit ran out.
constexpr int kMbarPolls = 1 << 24;
__device__ __forceinline__ bool mbar_wait(u32 bar, u32 parity, int polls = kMbarPolls) {
    for (int i = 0; i < polls; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void bulk_copy_to_shared(u32 dst, const void *src, u32 bytes, u32 bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            dst),
        "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}
__device__ __forceinline__ void fence_proxy_async_shared() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Position of the n-th set bit (n counted from 0) of a 64-bit mask that has
// more than n set bits, by halving with population counts.
__device__ __forceinline__ int nth_bit64(u64 mask, int n) {
    int pos = 0;
    int c = __popc(u32(mask));
    if (n >= c) {
        n -= c;
        mask >>= 32;
        pos = 32;
    }
    u32 m = u32(mask);
    c = __popc(m & 0xFFFFu);
    if (n >= c) { n -= c; m >>= 16; pos += 16; }
    c = __popc(m & 0xFFu);
    if (n >= c) { n -= c; m >>= 8; pos += 8; }
    c = __popc(m & 0xFu);
    if (n >= c) { n -= c; m >>= 4; pos += 4; }
    c = __popc(m & 0x3u);
    if (n >= c) { n -= c; m >>= 2; pos += 2; }
    if (n >= int(m & 1u)) pos += 1;
    return pos;
}

__device__ __forceinline__ u32 lanemask_lt() {
    u32 m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Warp-wide emission of surviving sites.  Every lane of the warp calls this
// with its word index and final mask (0 if none).  One atomicAdd per warp
// reserves output slots; slots past capacity are counted but not written, so
// the host sees count > capacity and re-runs the work in smaller pieces.
__device__ __forceinline__ void emit_survivors(u64 mask, long long word, long long bound,
                                               int denominator, long long *out_a, int *out_d,
                                               unsigned long long *out_count,
                                               unsigned long long capacity) {
    const int lane = threadIdx.x & 31;
    u32 n = __popcll(mask);
    if (!__any_sync(kFullMask, n != 0)) return;
    u32 incl = n;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        u32 v = __shfl_up_sync(kFullMask, incl, off);
        if (lane >= off) incl += v;
    }
    u32 total = __shfl_sync(kFullMask, incl, 31);
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(out_count, (unsigned long long)total);
    base = __shfl_sync(kFullMask, base, 0);
    unsigned long long pos = base + incl - n;
    long long a0 = -bound + 64 * word;
    while (mask) {
        int bit = __ffsll((long long)mask) - 1;
        mask &= mask - 1;
        if (pos < capacity) {
            out_a[pos] = a0 + bit;
            out_d[pos] = denominator;
        }
        ++pos;
    }
}

}  // namespace dev
}  // namespace rpg
