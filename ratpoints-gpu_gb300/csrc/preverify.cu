#include "preverify.hpp"

#include <algorithm>
#include <stdexcept>

#include "sieve.hpp"

namespace rpg {
namespace pre {

using u64 = unsigned long long;
using u32 = unsigned int;

constexpr int kGroups = 4;        // products of small primes below 2^32
constexpr int kSmallPrimes = 24;  // 3 .. 97
constexpr int kLarge = 4;         // primes just below 2^31

// Group g holds the small primes [group_first(g), group_first(g + 1)).
__host__ __device__ constexpr int group_first(int g) { return g == 0 ? 0 : g == 1 ? 9 : g == 2 ? 14 : g == 3 ? 19 : 24; }
__host__ __device__ constexpr u32 small_prime(int i) {
    return i == 0 ? 3 : i == 1 ? 5 : i == 2 ? 7 : i == 3 ? 11 : i == 4 ? 13 : i == 5 ? 17 : i == 6 ? 19
         : i == 7 ? 23 : i == 8 ? 29 : i == 9 ? 31 : i == 10 ? 37 : i == 11 ? 41 : i == 12 ? 43
         : i == 13 ? 47 : i == 14 ? 53 : i == 15 ? 59 : i == 16 ? 61 : i == 17 ? 67 : i == 18 ? 71
         : i == 19 ? 73 : i == 20 ? 79 : i == 21 ? 83 : i == 22 ? 89 : 97;
}
// products of each group's primes: 3..29, 31..47, 53..71, 73..97
__host__ __device__ constexpr u32 group_modulus(int g) {
    return g == 0 ? 3234846615u : g == 1 ? 95041567u : g == 2 ? 907383479u : 4132280413u;
}
__host__ __device__ constexpr u32 large_prime(int l) {
    return l == 0 ? 2147483647u : l == 1 ? 2147483629u : l == 2 ? 2147483587u : 2147483579u;
}

struct PreCurve {
    long long coef;  // first coefficient in the PreCoef array
    int n;           // coefficient count (degree + 1)
    int pad;
};
struct PreCoef {
    u64 wrap;                  // c mod 2^64
    u32 r[kGroups + kLarge];   // c mod group_modulus(g), then c mod large_prime(l)
};
struct PreMasks {
    u64 bits[kSmallPrimes][2];  // bit r set iff r is a square mod small_prime(i)
};

__host__ __device__ inline u64 mul_hi(u64 a, u64 b) {
#ifdef __CUDA_ARCH__
    return __umul64hi(a, b);
#else
    return u64((unsigned __int128)a * b >> 64);
#endif
}

// x * y mod m for x, y < m < 2^32 by Barrett reduction with
// magic = floor((2^64 - 1) / m): the quotient estimate is low by at most 1.
__host__ __device__ inline u32 mul_mod(u32 x, u32 y, u32 m, u64 magic) {
    const u64 p = u64(x) * y;
    const u64 r = p - mul_hi(p, magic) * m;
    return u32(r >= m ? r - m : r);
}
__host__ __device__ inline u32 add_mod(u32 x, u32 y, u32 m) {
    const u64 s = u64(x) + y;
    return u32(s >= m ? s - m : s);
}
__host__ __device__ inline u32 signed_mod(long long v, u32 m) {
    const u64 r = (v < 0 ? u64(0) - u64(v) : u64(v)) % m;
    return u32(v < 0 && r ? m - r : r);
}

__host__ __device__ inline int ctz64(u64 x) {
#ifdef __CUDA_ARCH__
    return __ffsll((long long)x) - 1;
#else
    return __builtin_ctzll(x);
#endif
}

__host__ __device__ inline u64 gcd64(u64 x, u64 y) {
    if (x == 0) return y;
    if (y == 0) return x;
    const int shift = ctz64(x | y);
    x >>= ctz64(x);
    while (y) {
        y >>= ctz64(y);
        if (x > y) {
            const u64 t = x;
            x = y;
            y = t;
        }
        y -= x;
    }
    return x << shift;
}

// x is the value mod 2^64 of a square iff x = 0, or its 2-adic valuation v
// is even and its odd part is 1 mod 8 (1 mod 4 when v = 62, where only two
// bits of it are known).
__host__ __device__ inline bool square_mod_2_64(u64 x) {
    if (x == 0) return true;
    const int v = ctz64(x);
    if (v & 1) return false;
    const u64 odd = x >> v;
    return v == 62 ? (odd & 3u) == 1u : (odd & 7u) == 1u;
}

// F(a, d) mod m by Horner in a with the powers of d accumulated; slot
// selects the coefficients' residues mod m.
__host__ __device__ inline u32 value_mod(const PreCoef *c, int n, int slot, u32 am, u32 dm, u32 m, u64 magic) {
    u32 v = c[n - 1].r[slot], pw = 1u % m;
    for (int i = n - 2; i >= 0; --i) {
        v = mul_mod(v, am, m, magic);
        pw = mul_mod(pw, dm, m, magic);
        v = add_mod(v, mul_mod(c[i].r[slot], pw, m, magic), m);
    }
    if ((n & 1) == 0) v = mul_mod(v, dm, m, magic);
    return v;
}

__host__ __device__ inline bool may_be_point(long long a, long long d, const PreCoef *c, int n,
                                             const PreMasks &masks) {
    if (gcd64(a < 0 ? u64(0) - u64(a) : u64(a), u64(d)) != 1) return false;
    {
        const u64 ua = u64(a), ud = u64(d);
        u64 v = c[n - 1].wrap, pw = 1;
        for (int i = n - 2; i >= 0; --i) {
            v *= ua;
            pw *= ud;
            v += c[i].wrap * pw;
        }
        if ((n & 1) == 0) v *= ud;
        if (!square_mod_2_64(v)) return false;
    }
#pragma unroll
    for (int g = 0; g < kGroups; ++g) {
        const u32 m = group_modulus(g);
        const u64 magic = ~0ull / m;
        const u32 v = value_mod(c, n, g, signed_mod(a, m), signed_mod(d, m), m, magic);
#pragma unroll
        for (int i = group_first(g); i < group_first(g + 1); ++i) {
            const u32 r = v % small_prime(i);
            if (!((masks.bits[i][r >> 6] >> (r & 63)) & 1u)) return false;
        }
    }
#pragma unroll 1
    for (int l = 0; l < kLarge; ++l) {
        const u32 p = large_prime(l);
        const u64 magic = ~0ull / p;
        const u32 v = value_mod(c, n, kGroups + l, signed_mod(a, p), signed_mod(d, p), p, magic);
        if (v == 0) continue;
        // Euler's criterion: v^((p-1)/2) is 1 for a nonzero square, p - 1 otherwise
        u32 e = (p - 1) / 2, base = v, acc = 1;
        while (e) {
            if (e & 1u) acc = mul_mod(acc, base, p, magic);
            base = mul_mod(base, base, p, magic);
            e >>= 1;
        }
        if (acc != 1) return false;
    }
    return true;
}

constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) preverify_kernel(
    const long long *a, const int *d, const int *curve, const unsigned long long *count,
    unsigned long long capacity, const PreCurve *curves, const PreCoef *coefs, PreMasks masks,
    long long *out_a, int *out_d, int *out_curve, unsigned long long *out_count,
    unsigned long long *curve_modular) {
    const unsigned long long n = *count < capacity ? *count : capacity;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long base = (unsigned long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u);
         base < n; base += stride) {
        const unsigned long long i = base + lane;
        bool keep = false;
        long long ai = 0;
        int di = 0, ci = 0;
        if (i < n) {
            ai = a[i];
            di = d[i];
            ci = curve ? curve[i] : 0;
            const PreCurve C = curves[ci];
            keep = may_be_point(ai, di, coefs + C.coef, C.n, masks);
        }
        if (curve_modular) {  // one atomic per curve present in the warp
            const unsigned live = __ballot_sync(0xffffffffu, i < n);
            const unsigned same = __match_any_sync(0xffffffffu, i < n ? ci : -1);
            if (i < n && lane == unsigned(__ffs(same) - 1))
                atomicAdd(curve_modular + ci, (unsigned long long)__popc(same & live));
        }
        const unsigned vote = __ballot_sync(0xffffffffu, keep);
        if (!vote) continue;
        unsigned long long slot = 0;
        if (lane == 0) slot = atomicAdd(out_count, (unsigned long long)__popc(vote));
        slot = __shfl_sync(0xffffffffu, slot, 0) + __popc(vote & ((1u << lane) - 1u));
        if (keep) {
            out_a[slot] = ai;
            out_d[slot] = di;
            if (out_curve) out_curve[slot] = ci;
        }
    }
}

const PreMasks &host_masks() {
    static const PreMasks masks = [] {
        PreMasks m{};
        for (int i = 0; i < kSmallPrimes; ++i) {
            const u32 p = small_prime(i);
            for (u32 v = 0; v < p; ++v) {
                const u32 r = v * v % p;
                m.bits[i][r >> 6] |= u64(1) << (r & 63);
            }
        }
        return m;
    }();
    return masks;
}

// c mod m for decimal text c (sign folded in), m < 2^32.
u32 text_mod(const std::string &text, u32 m) {
    std::size_t i = 0;
    const bool negative = !text.empty() && text[0] == '-';
    if (!text.empty() && (text[0] == '-' || text[0] == '+')) i = 1;
    u64 r = 0;
    for (; i < text.size(); ++i) {
        if (text[i] < '0' || text[i] > '9') throw std::invalid_argument("coefficients must be decimal integers");
        r = (r * 10 + u64(text[i] - '0')) % m;
    }
    return u32(negative && r ? m - r : r);
}

// c mod 2^64 (two's complement of the signed value).
u64 text_wrap(const std::string &text) {
    std::size_t i = 0;
    const bool negative = !text.empty() && text[0] == '-';
    if (!text.empty() && (text[0] == '-' || text[0] == '+')) i = 1;
    u64 r = 0;
    for (; i < text.size(); ++i) r = r * 10 + u64(text[i] - '0');
    return negative ? u64(0) - r : r;
}

PreCoef coef_residues(const std::string &text) {
    PreCoef c{};
    c.wrap = text_wrap(text);
    for (int g = 0; g < kGroups; ++g) c.r[g] = text_mod(text, group_modulus(g));
    for (int l = 0; l < kLarge; ++l) c.r[kGroups + l] = text_mod(text, large_prime(l));
    return c;
}

}  // namespace pre

Preverifier::~Preverifier() { release(); }

void Preverifier::release() {
    cudaFree(curves_);
    cudaFree(coefs_);
    curves_ = coefs_ = nullptr;
    curves_cap_ = coefs_cap_ = 0;
}

void Preverifier::prepare(const std::vector<const std::vector<std::string> *> &curves, cudaStream_t stream) {
    std::vector<pre::PreCurve> hc(curves.size());
    std::vector<pre::PreCoef> hk;
    for (std::size_t i = 0; i < curves.size(); ++i) {
        hc[i].coef = (long long)hk.size();
        hc[i].n = curves[i] ? int(curves[i]->size()) : 0;
        if (curves[i])
            for (const auto &t : *curves[i]) hk.push_back(pre::coef_residues(t));
    }
    if (hk.empty()) hk.push_back(pre::PreCoef{});
    auto grow = [](void *&p, std::size_t &cap, std::size_t bytes) {
        if (cap >= bytes) return;
        cudaFree(p);
        p = nullptr;
        cap = 0;
        check_cuda(cudaMalloc(&p, bytes), "cudaMalloc(pre-verification tables)");
        cap = bytes;
    };
    grow(curves_, curves_cap_, std::max<std::size_t>(1, hc.size()) * sizeof(pre::PreCurve));
    grow(coefs_, coefs_cap_, hk.size() * sizeof(pre::PreCoef));
    // pageable sources: the copies complete before these calls return
    if (!hc.empty())
        check_cuda(cudaMemcpyAsync(curves_, hc.data(), hc.size() * sizeof(pre::PreCurve), cudaMemcpyHostToDevice,
                                   stream),
                   "upload pre-verification tables");
    check_cuda(cudaMemcpyAsync(coefs_, hk.data(), hk.size() * sizeof(pre::PreCoef), cudaMemcpyHostToDevice, stream),
               "upload pre-verification tables");
    check_cuda(cudaStreamSynchronize(stream), "upload pre-verification tables");
    upload_bytes_ = hc.size() * sizeof(pre::PreCurve) + hk.size() * sizeof(pre::PreCoef);
    if (!blocks_) {
        int device = 0, sms = 0;
        check_cuda(cudaGetDevice(&device), "cudaGetDevice");
        check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "cudaDeviceGetAttribute");
        blocks_ = sms * 8;
    }
}

void Preverifier::launch(const long long *a, const int *d, const int *curve, const unsigned long long *count,
                         unsigned long long capacity, long long *out_a, int *out_d, int *out_curve,
                         unsigned long long *out_count, unsigned long long *curve_modular,
                         cudaStream_t stream) const {
    if (!coefs_) throw std::logic_error("pre-verification tables not prepared");
    pre::preverify_kernel<<<blocks_, pre::kThreads, 0, stream>>>(
        a, d, curve, count, capacity, static_cast<const pre::PreCurve *>(curves_),
        static_cast<const pre::PreCoef *>(coefs_), pre::host_masks(), out_a, out_d, out_curve, out_count,
        curve_modular);
    check_cuda(cudaGetLastError(), "preverify_kernel launch");
}

bool preverify_host(const std::vector<std::string> &coefficients, long long a, long long d) {
    if (coefficients.size() < 2) throw std::invalid_argument("polynomial must have degree >= 1");
    std::vector<pre::PreCoef> c;
    for (const auto &t : coefficients) c.push_back(pre::coef_residues(t));
    return pre::may_be_point(a, d, c.data(), int(c.size()), pre::host_masks());
}

}  // namespace rpg
