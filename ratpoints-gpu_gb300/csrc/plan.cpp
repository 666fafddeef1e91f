#include "plan.hpp"

#include <algorithm>
#include <cmath>

namespace rpg {

const std::array<int, kCandidatePrimes> &candidate_primes() {
    static const std::array<int, kCandidatePrimes> primes = [] {
        std::array<int, kCandidatePrimes> out{};
        std::vector<int> all;
        std::vector<bool> composite(kMaximumPrime, false);
        for (int n = 2; n < kMaximumPrime; ++n) {
            if (composite[n]) continue;
            all.push_back(n);
            for (int m = n * n; m < kMaximumPrime; m += n) composite[m] = true;
        }
        for (int i = 0; i < kCandidatePrimes; ++i)
            out[i] = all[all.size() - kCandidatePrimes + i];
        return out;
    }();
    return primes;
}

int decimal_mod(const std::string &text, int modulus) {
    std::size_t i = 0;
    bool negative = i < text.size() && text[i] == '-';
    if (i < text.size() && (text[i] == '-' || text[i] == '+')) ++i;
    long long value = 0;
    for (; i < text.size(); ++i) value = (10 * value + (text[i] - '0')) % modulus;
    return negative && value ? int(modulus - value) : int(value);
}

long long mod_inverse(long long value, long long modulus) {
    long long r0 = value, r1 = modulus, s0 = 1, s1 = 0;
    while (r1) {
        long long q = r0 / r1;
        long long t = r0 - q * r1;
        r0 = r1;
        r1 = t;
        t = s0 - q * s1;
        s0 = s1;
        s1 = t;
    }
    return (s0 % modulus + modulus) % modulus;
}

void modular_inverses(int p, unsigned short *out) {
    out[0] = 0;
    if (p > 1) out[1] = 1;
    // v^-1 = -(p / v) (p mod v)^-1 (mod p), from p = (p / v) v + p mod v
    for (int v = 2; v < p; ++v) {
        const int t = int((long long)(p / v) * out[p % v] % p);
        out[v] = (unsigned short)(t ? p - t : 0);
    }
}

bool square_mod(long long value, int p) {
    long long v = value % p;
    if (v < 0) v += p;
    if (v == 0 || p == 2) return true;
    long long result = 1;  // Euler's criterion: v^((p-1)/2) = 1
    for (long long e = (p - 1) / 2, b = v; e; e >>= 1, b = b * b % p)
        if (e & 1) result = result * b % p;
    return result == 1;
}

std::vector<std::uint8_t> affine_mask(int prime, const std::vector<std::string> &coefficients) {
    std::vector<int> residues(coefficients.size());
    for (std::size_t i = 0; i < coefficients.size(); ++i)
        residues[i] = decimal_mod(coefficients[i], prime);
    std::vector<std::uint8_t> square(prime, 0);
    // v^2 mod p for v <= p / 2 (the rest repeat them): (v + 1)^2 = v^2 + 2v + 1
    for (long long v = 0, sq = 0; 2 * v <= prime; ++v) {
        square[sq] = 1;
        sq += 2 * v + 1;
        while (sq >= prime) sq -= prime;
    }
    std::vector<std::uint8_t> affine(prime, 0);
    auto evaluate = [&](long long x) {
        long long value = 0;
        for (std::size_t i = residues.size(); i-- > 0;) value = (value * x + residues[i]) % prime;
        return value;
    };
    const int degree = int(residues.size()) - 1;
    if (prime <= 2 * (degree + 1)) {
        for (int x = 0; x < prime; ++x) affine[x] = square[evaluate(x)];
        return affine;
    }
    // Forward differences: f(x + 1) from f(x) with degree additions mod p
    // instead of a Horner evaluation (a division per coefficient) at every x.
    std::vector<long long> diff(std::size_t(degree) + 1);
    for (int x = 0; x <= degree; ++x) diff[std::size_t(x)] = evaluate(x);
    for (int k = 1; k <= degree; ++k)  // diff[k] = k-th difference at 0
        for (int x = degree; x >= k; --x) {
            long long v = diff[std::size_t(x)] - diff[std::size_t(x) - 1];
            diff[std::size_t(x)] = v < 0 ? v + prime : v;
        }
    for (int x = 0; x < prime; ++x) {
        affine[x] = square[diff[0]];
        for (int k = 0; k < degree; ++k) {
            long long v = diff[std::size_t(k)] + diff[std::size_t(k) + 1];
            diff[std::size_t(k)] = v >= prime ? v - prime : v;
        }
    }
    return affine;
}

bool select_primes(long long denominator, int *indices) {
    const auto &primes = candidate_primes();
    int n = 0;
    for (int i = kCandidatePrimes - 1; i >= 0 && n < kSelectedPrimes; --i)
        if (denominator % primes[i] != 0) indices[n++] = i;
    return n == kSelectedPrimes;
}

long long word_count64(long long bound) {
    long long sites = 2 * bound + 1;  // cannot overflow for bound <= (LLONG_MAX - 32) / 2
    return sites / 64 + (sites % 64 != 0);
}
long long word_count32(long long bound) { return (2 * bound + 32) / 32; }

double pass_rate(int q, const std::vector<std::string> &coefficients) {
    const auto aff = affine_mask(q, coefficients);
    int n = 0;
    for (auto v : aff) n += v;
    return double(n) / q;
}

void two_adic_classes(const std::vector<std::string> &coefficients, std::uint64_t out[64]) {
    const int n = int(coefficients.size()) - 1;
    std::vector<int> c64(coefficients.size());
    for (std::size_t i = 0; i < coefficients.size(); ++i) c64[i] = decimal_mod(coefficients[i], 64);
    bool square64[64] = {};
    for (int v = 0; v < 64; ++v) square64[(v * v) & 63] = true;
    for (int dd = 0; dd < 64; ++dd) {
        out[dd] = 0;
        for (int r = 0; r < 64; ++r) {
            if (dd % 2 == 0 && r % 2 == 0) continue;
            int value = c64[n], power = 1;
            for (int i = n - 1; i >= 0; --i) {
                value = (value * r) & 63;
                power = (power * dd) & 63;
                value = (value + c64[i] * power) & 63;
            }
            if (n % 2 == 1) value = (value * dd) & 63;
            if (square64[value]) out[dd] |= std::uint64_t(1) << r;
        }
    }
}

FastPlanner::FastPlanner(const std::vector<std::string> &coefficients, long long bound,
                         bool class_layout, int prime_limit)
    : prime_limit_(std::min(prime_limit, kFastPrimeLimit)) {
    auto add_primes = [&](int lo, int hi) {
        for (int q = lo | 1; q < hi; q += 2) {
            bool prime = q > 2;
            for (int f = 3; f * f <= q; f += 2) prime = prime && q % f;
            if (!prime) continue;
            const double rate = pass_rate(q, coefficients);
            strength_.push_back({rate > 0 ? -std::log2(rate) : 8.0, q});
        }
    };
    add_primes(3, prime_limit_);
    // Class prime: of 3..13 whose classes stay long enough (at least 256
    // words of 64 sites per class) and few enough (admissible 2-adic classes
    // times admissible residues mod q, over all d), the one whose class
    // layout sweeps the smallest share of the (d, r) residue pairs mod q:
    // A = q x pass rate residues for each of the q - 1 classes of d prime to
    // q, and for q | d every r != 0 when F(r, d) = c_n r^n is a square mod q
    // (c_n a square or zero, or n odd, where F vanishes), none otherwise.
    const long double sites = 2.0L * bound + 1.0L;
    const int degree = int(coefficients.size()) - 1;
    double best = 0.45;  // below ~0.45 bits a class prime does not pay for its classes
    int worst2 = -1;
    for (const auto &s : strength_) {
        const int q = s.second;
        if (!class_layout || q > 13) continue;
        if (sites / (64.0L * 64.0L * q) < 256.0L) continue;
        if (worst2 < 0) {
            std::uint64_t adm2[64];
            two_adic_classes(coefficients, adm2);
            worst2 = 0;
            for (auto m : adm2) worst2 = std::max(worst2, __builtin_popcountll(m));
        }
        const int admissible = int(std::lround(std::exp2(-s.first) * q));
        const bool lead = degree % 2 == 1 || square_mod(decimal_mod(coefficients.back(), q), q);
        const int divides = lead ? q - 1 : 0;
        if (worst2 * std::max(admissible, divides) > kMaxFastClasses) continue;
        const int swept = (q - 1) * admissible + divides;
        const double bits = swept > 0 ? std::log2(double(q) * q / swept) : 16.0;
        if (bits > best) {
            best = bits;
            class_prime_ = q;
        }
    }
    // Larger primes (rows of one prime each, about one bit) only for curves
    // that small primes filter weakly: with at least kDenseCurveBits from six
    // rows of small primes the cost model never takes them, and computing
    // their pass rates is most of the planning time of high-degree curves.
    if (prime_limit > prime_limit_ && plan(kMaxModulus, 6, 1LL << 40, false).bits < kDenseCurveBits) {
        add_primes(prime_limit_, prime_limit);
        prime_limit_ = prime_limit;
    }
}

FastPlan choose_fast_plan(const std::vector<std::string> &coefficients, long long bound,
                          int max_modulus, bool class_layout) {
    return FastPlanner(coefficients, bound, class_layout).plan(max_modulus);
}

FastPlan FastPlanner::plan(int max_modulus, int max_slots, long long row_budget, bool by_cost) const {
    FastPlan plan;
    plan.class_prime = class_prime_;
    const std::vector<std::pair<double, int>> &strength = strength_;
    // Stage-1 moduli: pack primes into at most `slots` products below
    // max_modulus.  Each packing puts a prime into the open modulus with the
    // most headroom that it fits, else opens a new one; it is tried with the
    // primes ordered by bits and by bits per bit of size, over primes below 72,
    // 128 and the planner's limit, and the packing with the most bits is kept.
    // the two orders, sorted once for every packing below
    std::vector<std::pair<double, int>> by_bits(strength), by_density(strength);
    std::sort(by_bits.begin(), by_bits.end(), [](const std::pair<double, int> &a, const std::pair<double, int> &b) {
        return a.first != b.first ? a.first > b.first : a.second < b.second;
    });
    std::sort(by_density.begin(), by_density.end(),
              [](const std::pair<double, int> &a, const std::pair<double, int> &b) {
                  const double da = a.first / std::log2(double(a.second));
                  const double db = b.first / std::log2(double(b.second));
                  return da != db ? da > db : a.second < b.second;
              });
    // A packing in fixed arrays (no allocation: the search below runs a few
    // hundred of them); odd primes multiply past 2^31 after eight factors.
    struct Packing {
        int count = 0;
        int modulus[kMaxFastSlots];
        int factors[kMaxFastSlots];
        int factor[kMaxFastSlots][8];
        double bits = 0;
    };
    auto pack = [&](const std::vector<std::pair<double, int>> &order, int limit, int slots, int cap,
                    Packing &out) {
        out.count = 0;
        out.bits = 0;
        for (const auto &s : order) {
            const int q = s.second;
            if (q >= limit || q == plan.class_prime || s.first < 0.3 || q > cap) continue;
            int target = -1;
            long long headroom = -1;
            for (int i = 0; i < out.count; ++i) {
                const long long product = (long long)out.modulus[i] * q;
                if (product <= cap && (long long)cap - product > headroom) {
                    headroom = cap - product;
                    target = i;
                }
            }
            if (target < 0) {
                if (out.count == slots) continue;
                target = out.count++;
                out.modulus[target] = 1;
                out.factors[target] = 0;
            }
            out.modulus[target] *= q;
            out.factor[target][out.factors[target]++] = q;
            out.bits += s.first;
        }
    };
    auto row_words = [](const Packing &p) {
        long long rows = 0;
        for (int i = 0; i < p.count; ++i) rows += (p.modulus[i] + kFastRowExtension + 1) & ~1;
        return rows;
    };
    // one packing per row count, its moduli capped (from max_modulus down by
    // 1/8 steps) until its rows fit the budget; the cheapest by the cost model
    // (limits that coincide give the same packing: each is tried once)
    const int limits[3] = {std::min(72, prime_limit_), std::min(kFastPrimeLimit, prime_limit_), prime_limit_};
    Packing best, candidate, packed;
    double best_cost = 0;
    bool found = false;
    const int top = std::min(max_slots, kMaxFastSlots);
    for (int slots = by_cost ? 1 : top; slots <= top; ++slots) {
        for (int cap = max_modulus;; cap = cap * 7 / 8) {
            candidate.count = 0;
            candidate.bits = -1;
            for (int li = 0; li < 3; ++li) {
                if (li > 0 && limits[li] == limits[li - 1]) continue;
                for (const auto *order : {&by_bits, &by_density}) {
                    pack(*order, limits[li], slots, cap, packed);
                    if (packed.bits > candidate.bits) candidate = packed;
                }
            }
            if (row_words(candidate) <= row_budget || cap <= 64) break;
        }
        if (candidate.count == 0) continue;
        if (row_words(candidate) > row_budget) continue;
        const double word_survives = 1.0 - std::pow(1.0 - std::exp2(-candidate.bits), 64.0);
        const double cost = kStageRowCost * double(candidate.count) + kSurvivorWordCost * word_survives;
        if (!found || cost < best_cost - 1e-9) {
            best = candidate;
            best_cost = cost;
            found = true;
        }
    }
    FastPlan best_plan = plan;
    if (found) {
        best_plan.bits = best.bits;
        for (int i = 0; i < best.count; ++i) {
            best_plan.moduli.push_back(best.modulus[i]);
            best_plan.slots.emplace_back(best.factor[i], best.factor[i] + best.factors[i]);
        }
    }
    plan = best_plan;
    if (plan.moduli.empty()) {  // every small prime is weak: keep one modulus anyway
        // (prime to the class prime, so that the class layout can use it)
        std::vector<int> pair = plan.class_prime == 5   ? std::vector<int>{3, 7}
                                : plan.class_prime == 7 ? std::vector<int>{3, 5}
                                                        : std::vector<int>{5, 7};
        plan.moduli.push_back(pair[0] * pair[1]);
        plan.slots.push_back(pair);
    }
    return plan;
}

}  // namespace rpg
