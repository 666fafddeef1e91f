#include "plan.hpp"

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

std::vector<std::uint8_t> affine_mask(int prime, const std::vector<std::string> &coefficients) {
    std::vector<int> residues(coefficients.size());
    for (std::size_t i = 0; i < coefficients.size(); ++i)
        residues[i] = decimal_mod(coefficients[i], prime);
    std::vector<std::uint8_t> square(prime, 0);
    for (long long v = 0; v < prime; ++v) square[v * v % prime] = 1;
    std::vector<std::uint8_t> affine(prime, 0);
    for (int x = 0; x < prime; ++x) {
        long long value = 0;
        for (std::size_t i = residues.size(); i-- > 0;) value = (value * x + residues[i]) % prime;
        affine[x] = square[value];
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

}  // namespace rpg
