// Sieve plans: which moduli reject which (a, d) sites, and the host-side
// tables the device kernels are built from.
//
// The reference plan restates the reference's SievePlan (src/sieve_plan.hpp:27-46,
// src/sieve_plan.cpp:83-151, 153-193): candidate primes are the 36 largest
// primes below 512; a denominator d uses the 32 largest that do not divide d;
// a site survives iff f(a/d) mod p is a square (0 included) for all 32.  Its
// survivor set is the reference's, unreduced pairs included.
//
// The fast plan (this project's) keeps every reference test and adds filters
// that no point can fail, so its survivors are a subset of the reference's
// that still holds every point:
//   - gcd(a, d) = 1 for the primes 2, 3, 5, 7 and every other small prime q | d;
//   - F(a, d) is a square modulo 64;
//   - f(a/d) mod q is a square for the small primes q in the wheel and the
//     composite moduli (or, when q | d, c_n is a square mod q for even n).
#pragma once

#include <array>
#include <cstdint>
#include <string>
#include <utility>
#include <vector>

namespace rpg {

constexpr int kCandidatePrimes = 36;   // sieve_plan.hpp:29 (NUM_PRIMES + 4)
constexpr int kSelectedPrimes = 32;    // sieve_plan.hpp:11 (NUM_PRIMES)
constexpr int kMaximumPrime = 512;     // sieve_plan.hpp:30

const std::array<int, kCandidatePrimes> &candidate_primes();  // ascending, 293 .. 509

// Residue of a decimal integer modulo m (m < 2^31), sign folded into [0, m).
int decimal_mod(const std::string &text, int modulus);
long long mod_inverse(long long value, long long modulus);
// out[v] = v^-1 mod p for 0 < v < p and out[0] = 0, for a prime p < 65536.
void modular_inverses(int p, unsigned short *out);
// value mod p is a square (0 included), for a prime p < 2^31.
bool square_mod(long long value, int p);

// affine[x] = 1 iff f(x) mod p is a square (0 included), for x in [0, p).
std::vector<std::uint8_t> affine_mask(int prime, const std::vector<std::string> &coefficients);

// Indices into candidate_primes() of the 32 largest candidates not dividing
// denominator, largest first.  Returns false if fewer than 32 qualify.
bool select_primes(long long denominator, int *indices);

// ceil((2H + 1) / 64): 64-site words covering a in [-H, H].
long long word_count64(long long bound);
// floor((2H + 32) / 32): the reference's 32-site word count (sieve_plan.cpp:109),
// reported by the -v metrics line.
long long word_count32(long long bound);

// Fraction of x in [0, q) with f(x) a square mod q (0 included): the share of
// sites (a, d), q !| d, that pass the test mod q.
double pass_rate(int q, const std::vector<std::string> &coefficients);

// 2-adic admissible classes by d mod 64: bit r of out[d mod 64] is set iff
// F(r, d) is a square mod 64, with r odd when d is even (gcd).
void two_adic_classes(const std::vector<std::string> &coefficients, std::uint64_t out[64]);

// Per-curve choice of the fast plan's filters (this project's autotuner).
// Numerator classes are taken modulo 64 * class_prime (2-adic classes crossed
// with the admissible residues mod class_prime; class_prime 1 means 2-adic
// classes only); the first-stage rows are products of the other primes (odd,
// below the planner's prime limit), at most max_slots of them, each below
// kMaxModulus.  The number of rows is chosen by a cost model of the fast
// kernel: stage 1 costs kStageRowCost per row and swept word, stage 2
// kSurvivorWordCost per word that survives stage 1 (SM cycles, measured on
// GB300).  Curves that are squares modulo most small primes (dense curves)
// get more rows, of primes up to 509.
constexpr int kMaxFastSlots = 12;
constexpr int kMaxModulus = 1500;
constexpr int kMaxFastClasses = 256;
constexpr int kFastPrimeLimit = 128;   // primes of the class prime and the batch's rows: 3 .. 127
constexpr int kStagePrimeLimit = 512;  // primes of the single-curve rows: 3 .. 509
constexpr int kFastRowExtension = 96;  // words a staged row extends past its period
constexpr double kDenseCurveBits = 10.0;  // below this from six small-prime rows: try large primes
constexpr double kStageRowCost = 0.16;
constexpr double kSurvivorWordCost = 40.0;
struct FastPlan {
    int class_prime = 1;
    std::vector<std::vector<int>> slots;   // prime factors of each stage-1 modulus
    std::vector<int> moduli;               // their products
    double bits = 0;                       // expected filtering of the stage-1 rows (bits)
    int row_slots = 2;                     // single-curve kernel: denominators staged per CTA (2 or 3)
};
// max_modulus caps each stage-1 modulus (table size grows as its square);
// class_prime false keeps the plan to 2-adic classes (the dense layout of the
// batched search, 64 consecutive numerators per word).
FastPlan choose_fast_plan(const std::vector<std::string> &coefficients, long long bound,
                          int max_modulus = kMaxModulus, bool class_prime = true);

// The autotuner's per-curve work done once (pass rates of every small prime,
// the class prime), for callers that try several modulus caps.
class FastPlanner {
public:
    FastPlanner(const std::vector<std::string> &coefficients, long long bound, bool class_prime = true,
                int prime_limit = kStagePrimeLimit);
    // The cheapest plan (cost model above) with at most max_slots rows whose
    // staged row words, sum of (m + kFastRowExtension) rounded up to even,
    // stay within row_budget.  by_cost false: the plan with the most filtering
    // bits in max_slots rows (kernels that sweep a fixed number of rows).
    FastPlan plan(int max_modulus = kMaxModulus, int max_slots = kMaxFastSlots,
                  long long row_budget = 1LL << 40, bool by_cost = true) const;
    int class_prime() const { return class_prime_; }

private:
    std::vector<std::pair<double, int>> strength_;  // (bits, prime) of the odd primes below the limit
    int class_prime_ = 1;
    int prime_limit_ = kStagePrimeLimit;
};

}  // namespace rpg
