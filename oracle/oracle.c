/*
 * oracle.c - CPU restatement of the reference ratpoints_gpu modular sieve.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA sieve: it
 * is compiled into oracle/_build/liboracle.so and loaded by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg.  No product
 * code path links, loads or calls it.
 *
 * It restates, in scalar C, the reference's algorithm for the survivor set of
 * one search box:
 *   - candidate primes: the 36 largest primes below 512
 *     (src/sieve_plan.cpp:83-100, 115-116; src/sieve_plan.hpp:27-30);
 *   - per-denominator selection of the 32 largest candidates that do not
 *     divide the denominator d (d = b, or k*k in square-denominator mode)
 *     (src/sieve_plan.cpp:128-145);
 *   - coefficient residues from decimal text (src/sieve_plan.cpp:70-81);
 *   - the affine square table of f mod p (src/sieve_plan.cpp:170-193);
 *   - modular inverses by extended Euclid (src/sieve_plan.cpp:153-168);
 *   - the 32-bit word masks: bit j of word w for denominator residue r is
 *     affine[((-H + 32 w + j) * r^-1) mod p], row r = 0 all zero
 *     (src/sieve.cu:141-172);
 *   - the sieve: per denominator, AND the 32 selected masks for every word,
 *     clear bits past +H in the last word, and emit (a, d) for each set bit
 *     with a = -H + 32 w + j (src/sieve.cu:221-388, 174-194, 324-330).
 * Survivors are emitted in (d ascending, a ascending) order; the reference
 * leaves emission order unspecified (include/sieve.hpp:41-47), so callers
 * compare sets.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define RPO_CANDIDATES 36
#define RPO_SELECTED 32
#define RPO_MAX_PRIME 512

int rpo_candidate_primes(int *out) {
    /* Eratosthenes below 512, then keep the largest 36 (sieve_plan.cpp:83-100, 115-116). */
    unsigned char composite[RPO_MAX_PRIME];
    int primes[RPO_MAX_PRIME];
    int count = 0;
    memset(composite, 0, sizeof composite);
    for (int n = 2; n < RPO_MAX_PRIME; ++n) {
        if (composite[n]) continue;
        primes[count++] = n;
        for (int m = n * n; m < RPO_MAX_PRIME; m += n) composite[m] = 1;
    }
    for (int i = 0; i < RPO_CANDIDATES; ++i) out[i] = primes[count - RPO_CANDIDATES + i];
    return RPO_CANDIDATES;
}

int rpo_decimal_mod(const char *text, int modulus) {
    /* Leading sign, then base-10 digits reduced on the fly (sieve_plan.cpp:70-81). */
    const char *c = text;
    int negative = *c == '-';
    if (*c == '-' || *c == '+') ++c;
    long long value = 0;
    for (; *c; ++c) value = (10 * value + (*c - '0')) % modulus;
    return negative && value ? (int)(modulus - value) : (int)value;
}

long long rpo_mod_inverse(long long value, long long modulus) {
    /* Extended Euclid, result normalised into [0, modulus) (sieve_plan.cpp:153-168). */
    long long r0 = value, r1 = modulus, s0 = 1, s1 = 0;
    while (r1) {
        long long q = r0 / r1, t = r0 - q * r1;
        r0 = r1; r1 = t;
        t = s0 - q * s1; s0 = s1; s1 = t;
    }
    return (s0 % modulus + modulus) % modulus;
}

void rpo_affine_mask(int prime, const char *const *coefficients, int count, unsigned char *out) {
    /* out[x] = [f(x) mod p is a square, 0 included] by Horner (sieve_plan.cpp:170-193). */
    int residues[128];
    unsigned char square[RPO_MAX_PRIME];
    for (int i = 0; i < count; ++i) residues[i] = rpo_decimal_mod(coefficients[i], prime);
    memset(square, 0, sizeof square);
    for (long long v = 0; v < prime; ++v) square[v * v % prime] = 1;
    for (int x = 0; x < prime; ++x) {
        long long value = 0;
        for (int i = count - 1; i >= 0; --i) value = (value * x + residues[i]) % prime;
        out[x] = square[value];
    }
}

int rpo_select(long long denominator, int *out_indices) {
    /* Indices (into the ascending candidate list) of the 32 largest candidates not
     * dividing the denominator, largest first (sieve_plan.cpp:128-145). */
    int primes[RPO_CANDIDATES];
    rpo_candidate_primes(primes);
    int n = 0;
    for (int i = RPO_CANDIDATES - 1; i >= 0 && n < RPO_SELECTED; --i)
        if (denominator % primes[i] != 0) out_indices[n++] = i;
    return n == RPO_SELECTED ? 0 : -1;
}

typedef struct rpo_ctx {
    long long bound;           /* H */
    long long words;           /* floor((2H + 32) / 32)  (sieve_plan.cpp:109) */
    int primes[RPO_CANDIDATES];
    long long offsets[RPO_CANDIDATES];
    uint32_t *masks;           /* sum p*p words, row-major [residue][word residue] */
} rpo_ctx;

static uint32_t basis_word(const unsigned char *affine, const int *inverses, int prime,
                           int residue, int word_residue, long long bound) {
    /* One word of the mask basis (sieve.cu:141-172). */
    if (residue == 0) return 0;
    int inverse = inverses[residue];
    long long numerator = (-bound + 32LL * word_residue) % prime;
    if (numerator < 0) numerator += prime;
    int x = (int)(numerator * inverse % prime);
    uint32_t packed = 0;
    for (int bit = 0; bit < 32; ++bit) {
        if (affine[x]) packed |= 1u << bit;
        x += inverse;
        if (x >= prime) x -= prime;
    }
    return packed;
}

rpo_ctx *rpo_create(const char *const *coefficients, int count, long long bound) {
    if (count < 1 || count > 128 || bound < 1) return NULL;
    rpo_ctx *ctx = (rpo_ctx *)calloc(1, sizeof *ctx);
    if (!ctx) return NULL;
    ctx->bound = bound;
    ctx->words = (2 * bound + 32) / 32;
    rpo_candidate_primes(ctx->primes);
    long long total = 0;
    for (int i = 0; i < RPO_CANDIDATES; ++i) {
        ctx->offsets[i] = total;
        total += (long long)ctx->primes[i] * ctx->primes[i];
    }
    ctx->masks = (uint32_t *)malloc((size_t)total * sizeof(uint32_t));
    if (!ctx->masks) { free(ctx); return NULL; }
    for (int i = 0; i < RPO_CANDIDATES; ++i) {
        int p = ctx->primes[i];
        unsigned char affine[RPO_MAX_PRIME];
        int inverses[RPO_MAX_PRIME];
        rpo_affine_mask(p, coefficients, count, affine);
        inverses[0] = 0;
        for (int v = 1; v < p; ++v) inverses[v] = (int)rpo_mod_inverse(v, p);
        for (int r = 0; r < p; ++r)
            for (int u = 0; u < p; ++u)
                ctx->masks[ctx->offsets[i] + (long long)r * p + u] =
                    basis_word(affine, inverses, p, r, u, bound);
    }
    return ctx;
}

void rpo_destroy(rpo_ctx *ctx) {
    if (!ctx) return;
    free(ctx->masks);
    free(ctx);
}

long long rpo_words(const rpo_ctx *ctx) { return ctx->words; }

uint32_t rpo_mask_word(const rpo_ctx *ctx, int candidate, int residue, long long word) {
    int p = ctx->primes[candidate];
    return ctx->masks[ctx->offsets[candidate] + (long long)residue * p + word % p];
}

/* Order-independent digest of a survivor set; the same formula is restated in
 * the Python test helpers so device output can be compared without sorting. */
static inline uint64_t mix_pair(long long a, long long d) {
    uint64_t z = (uint64_t)a * 0x9E3779B97F4A7C15ull ^ ((uint64_t)d << 1) ^ 0x632BE59BD9B4E019ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

uint64_t rpo_mix_pair(long long a, long long d) { return mix_pair(a, d); }

/* Sieve denominators [first, last] (parameters k, d = k*k if square).  Writes at
 * most cap survivors into out_a/out_d (either may be NULL), returns the total
 * count, and adds mix_pair over all survivors into *checksum. */
static long long sieve_range(const rpo_ctx *ctx, long long first, long long last, int square,
                             long long *out_a, int *out_d, long long cap, uint64_t *checksum) {
    long long count = 0;
    uint64_t sum = 0;
    const long long words = ctx->words, bound = ctx->bound;
    for (long long k = first; k <= last; ++k) {
        long long d = square ? k * k : k;
        int sel[RPO_SELECTED];
        if (rpo_select(d, sel) != 0) return -1;
        const uint32_t *row[RPO_SELECTED];
        int prime[RPO_SELECTED], pos[RPO_SELECTED];
        for (int s = 0; s < RPO_SELECTED; ++s) {
            int i = sel[s], p = ctx->primes[i];
            prime[s] = p;
            row[s] = ctx->masks + ctx->offsets[i] + (long long)(d % p) * p;
            pos[s] = 0;
        }
        for (long long w = 0; w < words; ++w) {
            uint32_t surviving = 0xffffffffu;
            for (int s = 0; s < RPO_SELECTED; ++s) {
                surviving &= row[s][pos[s]];
                if (++pos[s] == prime[s]) pos[s] = 0;
            }
            if (surviving && w == words - 1) {
                long long valid = bound - (-bound + 32 * w) + 1;
                if (valid < 32) surviving &= (1u << valid) - 1;
            }
            while (surviving) {
                int bit = __builtin_ctz(surviving);
                surviving &= surviving - 1;
                long long a = -bound + 32 * w + bit;
                if (count < cap) {
                    if (out_a) out_a[count] = a;
                    if (out_d) out_d[count] = (int)d;
                }
                sum += mix_pair(a, d);
                ++count;
            }
        }
    }
    if (checksum) *checksum += sum;
    return count;
}

typedef struct {
    const rpo_ctx *ctx;
    long long first, last;
    int square;
    long long count;
    uint64_t checksum;
} range_job;

static void *run_job(void *arg) {
    range_job *job = (range_job *)arg;
    job->checksum = 0;
    job->count = sieve_range(job->ctx, job->first, job->last, job->square, NULL, NULL, 0,
                             &job->checksum);
    return NULL;
}

long long rpo_sieve(const rpo_ctx *ctx, long long first, long long last, int square,
                    long long *out_a, int *out_d, long long cap, uint64_t *checksum) {
    if (!ctx || first < 1 || last < first) return -1;
    if (checksum) *checksum = 0;
    return sieve_range(ctx, first, last, square, out_a, out_d, cap, checksum);
}

/* Count and digest only, split over `threads` POSIX threads by denominator. */
long long rpo_sieve_count_mt(const rpo_ctx *ctx, long long first, long long last, int square,
                             int threads, uint64_t *checksum) {
    if (!ctx || first < 1 || last < first || threads < 1) return -1;
    long long n = last - first + 1;
    if (threads > n) threads = (int)n;
    range_job *jobs = (range_job *)calloc((size_t)threads, sizeof *jobs);
    pthread_t *ids = (pthread_t *)calloc((size_t)threads, sizeof *ids);
    long long start = first;
    for (int t = 0; t < threads; ++t) {
        long long size = n / threads + (t < n % threads);
        jobs[t].ctx = ctx;
        jobs[t].first = start;
        jobs[t].last = start + size - 1;
        jobs[t].square = square;
        start += size;
        pthread_create(&ids[t], NULL, run_job, &jobs[t]);
    }
    long long total = 0;
    uint64_t sum = 0;
    for (int t = 0; t < threads; ++t) {
        pthread_join(ids[t], NULL);
        if (jobs[t].count < 0) total = -1;
        else if (total >= 0) total += jobs[t].count;
        sum += jobs[t].checksum;
    }
    free(jobs);
    free(ids);
    if (checksum) *checksum = sum;
    return total;
}
