#include "exact.hpp"

#include <algorithm>
#include <cmath>
#include <stdexcept>

namespace rpg {

namespace {

// 3 * 5 * 7 * ... * 53: the odd primes whose quadratic residues prefilter
// candidate values before the exact square root.
constexpr u64 kSmallModulus = 16294579238595022365ull;
constexpr int kSmallPrimes[] = {3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53};

struct ResidueTables {
    u64 square_bits[sizeof(kSmallPrimes) / sizeof(int)];
    ResidueTables() {
        for (std::size_t i = 0; i < sizeof(kSmallPrimes) / sizeof(int); ++i) {
            int q = kSmallPrimes[i];
            u64 bits = 0;
            for (int v = 0; v < q; ++v) bits |= u64(1) << (v * v % q);
            square_bits[i] = bits;
        }
    }
};
const ResidueTables kTables;

inline u64 mulmod(u64 a, u64 b, u64 m) { return u64(u128(a) * b % m); }
inline u64 addmod(u64 a, u64 b, u64 m) {
    u64 s = a + b;
    return (s < a || s >= m) ? s - m : s;
}
inline u64 to_mod(long long v, u64 m) {
    if (v >= 0) return u64(v) % m;
    u64 r = (u64(0) - u64(v)) % m;
    return r ? m - r : 0;
}

// A non-negative integer whose value mod 2^64 is x can be a square only if x
// is zero or its 2-adic valuation is even with odd part = 1 mod 8 (when at
// least three bits of that odd part are known).
inline bool two_adic_square(u64 x) {
    if (x == 0) return true;
    int v = __builtin_ctzll(x);
    if (v & 1) return false;
    if (v > 61) return true;
    return ((x >> v) & 7u) == 1u;
}

// --- squarefreeness by modular gcd ---------------------------------------

u64 powmod(u64 b, u64 e, u64 m) {
    u64 r = 1 % m;
    for (; e; e >>= 1, b = mulmod(b, b, m))
        if (e & 1) r = mulmod(r, b, m);
    return r;
}

bool is_prime_u64(u64 n) {
    if (n < 2) return false;
    for (u64 p : {2ull, 3ull, 5ull, 7ull, 11ull, 13ull, 17ull, 19ull, 23ull, 29ull, 31ull, 37ull}) {
        if (n % p == 0) return n == p;
    }
    u64 d = n - 1;
    int s = 0;
    while ((d & 1) == 0) { d >>= 1; ++s; }
    for (u64 a : {2ull, 3ull, 5ull, 7ull, 11ull, 13ull, 17ull, 19ull, 23ull, 29ull, 31ull, 37ull}) {
        u64 x = powmod(a, d, n);
        if (x == 1 || x == n - 1) continue;
        bool composite = true;
        for (int r = 1; r < s; ++r) {
            x = mulmod(x, x, n);
            if (x == n - 1) { composite = false; break; }
        }
        if (composite) return false;
    }
    return true;
}

void trim_poly(std::vector<u64> &p) {
    while (!p.empty() && p.back() == 0) p.pop_back();
}

// Degree of gcd(f, g) over F_p (p prime); f, g trimmed, g nonempty.
int gcd_degree_mod(std::vector<u64> f, std::vector<u64> g, u64 p) {
    while (!g.empty()) {
        u64 inv = powmod(g.back(), p - 2, p);
        while (f.size() >= g.size()) {
            std::size_t shift = f.size() - g.size();
            u64 factor = mulmod(f.back(), inv, p);
            for (std::size_t i = 0; i < g.size(); ++i) {
                u64 sub = mulmod(factor, g[i], p);
                u64 &x = f[i + shift];
                x = x >= sub ? x - sub : x + (p - sub);
            }
            trim_poly(f);
            if (f.empty()) break;
        }
        std::swap(f, g);
    }
    return int(f.size()) - 1;
}

}  // namespace

ExactPolynomial::ExactPolynomial(const std::vector<std::string> &coefficients) {
    if (coefficients.empty()) throw std::invalid_argument("empty polynomial");
    coeffs_.resize(coefficients.size());
    fits_i64_ = true;
    for (std::size_t i = 0; i < coefficients.size(); ++i) {
        if (!BigInt::parse(coefficients[i], coeffs_[i]))
            throw std::invalid_argument("coefficients must be decimal integers");
        if (coeffs_[i].limbs() > 1 ||
            (coeffs_[i].limbs() == 1 && (coeffs_[i].magnitude()[0] >> 63)))
            fits_i64_ = false;
    }
    mod_wrap_.resize(coeffs_.size());
    mod_small_.resize(coeffs_.size());
    small_.resize(coeffs_.size());
    for (std::size_t i = 0; i < coeffs_.size(); ++i) {
        const BigInt &c = coeffs_[i];
        u64 low = c.limbs() ? c.magnitude()[0] : 0;
        mod_wrap_[i] = c.negative() ? u64(0) - low : low;
        mod_small_[i] = c.mod(kSmallModulus);
        small_[i] = fits_i64_ ? (long long)mod_wrap_[i] : 0;
    }
}

bool ExactPolynomial::passes_residue_tests(long long a, long long b) const {
    // F mod 2^64 by wrapping Horner, then F mod the odd-prime product.
    const std::size_t n = coeffs_.size();
    u64 ua = u64(a), ub = u64(b);
    u64 value = mod_wrap_[n - 1], power = 1;
    for (std::size_t i = n - 1; i-- > 0;) {
        value *= ua;
        power *= ub;
        value += mod_wrap_[i] * power;
    }
    if (n % 2 == 0) value *= ub;
    if (!two_adic_square(value)) return false;
    const u64 m = kSmallModulus;
    u64 am = to_mod(a, m), bm = to_mod(b, m);
    u64 v = mod_small_[n - 1], pw = 1 % m;
    for (std::size_t i = n - 1; i-- > 0;) {
        v = mulmod(v, am, m);
        pw = mulmod(pw, bm, m);
        v = addmod(v, mulmod(mod_small_[i], pw, m), m);
    }
    if (n % 2 == 0) v = mulmod(v, bm, m);
    for (std::size_t i = 0; i < sizeof(kSmallPrimes) / sizeof(int); ++i) {
        if (!((kTables.square_bits[i] >> (v % u64(kSmallPrimes[i]))) & 1u)) return false;
    }
    return true;
}

BigInt ExactPolynomial::evaluate(long long a, long long b) const {
    // Horner in a with an accumulated power of b (exact_polynomial.cpp:25-36).
    const std::size_t n = coeffs_.size();
    BigInt value = coeffs_[n - 1];
    BigInt power(1);
    for (std::size_t i = n - 1; i-- > 0;) {
        value.mul_small(a);
        power.mul_small(b);
        if (!coeffs_[i].is_zero()) value.add(BigInt::mul(coeffs_[i], power));
    }
    if (n % 2 == 0) value.mul_small(b);
    return value;
}

bool ExactPolynomial::is_point(long long a, long long b) const {
    if (!passes_residue_tests(a, b)) return false;
    BigInt value = evaluate(a, b);
    if (value.negative()) return false;
    bool exact = false;
    value.isqrt(exact);
    return exact;
}

bool ExactPolynomial::square_root(long long a, long long b, std::string &root) const {
    if (!passes_residue_tests(a, b)) return false;
    BigInt value = evaluate(a, b);
    if (value.negative()) return false;
    bool exact = false;
    BigInt r = value.isqrt(exact);
    if (!exact) return false;
    root = r.to_string();
    return true;
}

bool ExactPolynomial::is_squarefree() const {
    // f is squarefree over Q iff Res(f, f') != 0.  For a prime p not dividing
    // n * c_n, gcd(f mod p, f' mod p) is trivial iff p does not divide Res(f, f').
    // One such prime with a trivial gcd proves squarefreeness; if f is
    // squarefree, |Res| <= ||f||^(n-1) ||f'||^n bounds how many primes above 2^60
    // can divide it, so that many nontrivial gcds prove f is not squarefree.
    const int n = degree();
    if (n < 1) return false;
    if (n == 1) return true;
    std::size_t max_bits = 0;
    for (const auto &c : coeffs_) max_bits = std::max(max_bits, c.bit_length());
    double log_f = double(max_bits) + 0.5 * std::log2(double(n + 1));
    double log_fp = log_f + std::log2(double(n));
    double bound_bits = (n - 1) * log_f + n * log_fp + 2.0;
    long long needed = (long long)(bound_bits / 60.0) + 2;
    long long tested = 0;
    for (u64 p = (u64(1) << 61) - 1; tested < needed; p -= 2) {
        if (!is_prime_u64(p)) continue;
        if (coeffs_.back().mod(p) == 0 || u64(n) % p == 0) continue;
        std::vector<u64> f(coeffs_.size()), g(coeffs_.size() - 1);
        for (std::size_t i = 0; i < coeffs_.size(); ++i) f[i] = coeffs_[i].mod(p);
        for (std::size_t i = 1; i < f.size(); ++i) g[i - 1] = mulmod(f[i], u64(i) % p, p);
        trim_poly(f);
        trim_poly(g);
        if (gcd_degree_mod(f, g, p) == 0) return true;
        ++tested;
    }
    return false;
}

int Rational::compare(const Rational &x, const Rational &y) {
    return BigInt::compare(BigInt::mul(x.num, y.den), BigInt::mul(y.num, x.den));
}

int Rational::compare_fraction(long long a, long long d) const {
    // sign(a/d - num/den) = sign(a * den - num * d), both denominators positive.
    BigInt left = den;
    left.mul_small(a);
    BigInt right = num;
    right.mul_small(d);
    return BigInt::compare(left, right);
}

namespace {

// A run of decimal digits starting at `at`; advances `at` past it.
std::string digit_run(const std::string &text, std::size_t &at) {
    const std::size_t begin = at;
    while (at < text.size() && text[at] >= '0' && text[at] <= '9') ++at;
    return text.substr(begin, at - begin);
}

}  // namespace

// Grammar: [sign] int-digits [ '.' frac-digits ] [ ('e'|'E') [sign] exp-digits ]
// with at least one int or frac digit and at least one exp digit after an 'e'.
// The exponent's magnitude is checked digit by digit as it is read (a value
// above 10000 is "exponent is too large", reported before anything after the
// exponent is looked at); every other malformed input is "must be real".
// The value is (int-digits frac-digits) x 10^(exp - #frac-digits).
bool parse_real(const std::string &input, const std::string &name, Rational &out,
                std::string &error) {
    auto reject = [&](const char *why) {
        error = name + why;
        return false;
    };
    std::size_t at = 0;
    const bool minus = at < input.size() && input[at] == '-';
    if (at < input.size() && (input[at] == '-' || input[at] == '+')) ++at;
    std::string mantissa = digit_run(input, at);
    std::size_t fraction_digits = 0;
    if (at < input.size() && input[at] == '.') {
        ++at;
        const std::string fraction = digit_run(input, at);
        fraction_digits = fraction.size();
        mantissa += fraction;
    }
    long long power_of_ten = 0;
    if (at < input.size() && (input[at] == 'e' || input[at] == 'E')) {
        ++at;
        const bool exponent_minus = at < input.size() && input[at] == '-';
        if (at < input.size() && (input[at] == '-' || input[at] == '+')) ++at;
        const std::string exponent = digit_run(input, at);
        if (exponent.empty()) return reject(" must be real");
        long long magnitude = 0;
        for (char c : exponent) {
            magnitude = magnitude * 10 + (c - '0');
            if (magnitude > 10000) return reject(" exponent is too large");
        }
        power_of_ten = exponent_minus ? -magnitude : magnitude;
    }
    if (mantissa.empty() || at != input.size()) return reject(" must be real");
    BigInt value;
    if (!BigInt::parse(mantissa, value)) return reject(" must be real");
    if (minus) value.negate();
    const long long shift = power_of_ten - (long long)fraction_digits;
    BigInt scale(1);
    for (long long k = shift < 0 ? -shift : shift; k > 0; --k) scale.mul_small(10);
    if (shift < 0) {
        out.num = value;
        out.den = scale;
    } else {
        out.num = BigInt::mul(value, scale);
        out.den = BigInt(1);
    }
    return true;
}

}  // namespace rpg
