// Exact arithmetic on the curve y^2 = f(x) for the verification stage.
//
// ExactPolynomial replaces the reference's GMP-based ExactPolynomial
// (include/exact_polynomial.hpp:9-21, src/exact_polynomial.cpp:18-71) with the
// same predicates:
//   square_root(a, b): F(a, b) = sum c_i a^i b^(n-i), times b when the
//     coefficient count is even; a point iff F >= 0 is a perfect square, and
//     the ordinate is floor(sqrt(F)) in decimal;
//   is_squarefree(): gcd(f, f') over Q is a nonzero constant.
// Rational replaces mpq_class for the -l/-u interval bounds
// (src/command_line.cpp:39-108, src/point_search.cpp:131-146).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "bigint.hpp"

namespace rpg {

class ExactPolynomial {
public:
    // Coefficients c0..cn as decimal text ([+-]digits).  Throws on bad text.
    explicit ExactPolynomial(const std::vector<std::string> &coefficients);

    // True iff F(a, b) is a square; root receives floor(sqrt(F)) in decimal.
    bool square_root(long long a, long long b, std::string &root) const;
    // Same predicate without the decimal string (used by tests and metrics).
    bool is_point(long long a, long long b) const;

    bool is_squarefree() const;
    int degree() const { return int(coeffs_.size()) - 1; }
    const std::vector<BigInt> &coefficients() const { return coeffs_; }

private:
    bool passes_residue_tests(long long a, long long b) const;
    BigInt evaluate(long long a, long long b) const;

    std::vector<BigInt> coeffs_;
    std::vector<u64> mod_wrap_;   // coefficients mod 2^64
    std::vector<u64> mod_small_;  // coefficients mod kSmallModulus
    bool fits_i64_ = false;       // every coefficient fits in a signed 64-bit word
    std::vector<long long> small_;
};

struct Rational {
    BigInt num;
    BigInt den;  // > 0
    static int compare(const Rational &x, const Rational &y);
    // Compare the fraction a/d (d > 0) with this rational.
    int compare_fraction(long long a, long long d) const;
};

// A real bound of -l / -u in the reference's accepted syntax (src/command_line.cpp:39-108):
// [+-]digits[.digits][e[+-]digits] with at least one digit and an exponent of magnitude at
// most 10000.  On failure returns false and sets error to "<name> must be real" or
// "<name> exponent is too large".
bool parse_real(const std::string &text, const std::string &name, Rational &out,
                std::string &error);

}  // namespace rpg
