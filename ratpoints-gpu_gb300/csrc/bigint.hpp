// Exact signed integers for point verification, interval tests and
// squarefreeness, written for this project (the reference uses GMP's mpz_class
// for the same roles: src/exact_polynomial.cpp:18-42, src/point_search.cpp:131-146).
//
// Sign-magnitude, 64-bit limbs, little-endian.  Only the operations the search
// needs: decimal parse/print, add, multiply, compare, floor square root,
// remainders by small moduli.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace rpg {

using u64 = std::uint64_t;
using u128 = unsigned __int128;
using i128 = __int128;

class BigInt {
public:
    BigInt() = default;
    BigInt(long long v) { assign(v); }  // NOLINT: implicit by design

    static bool parse(const std::string &text, BigInt &out);  // [+-]digits
    std::string to_string() const;

    void assign(long long v);
    bool is_zero() const { return mag_.empty(); }
    bool negative() const { return neg_; }
    int sign() const { return mag_.empty() ? 0 : (neg_ ? -1 : 1); }
    std::size_t limbs() const { return mag_.size(); }
    std::size_t bit_length() const;
    const std::vector<u64> &magnitude() const { return mag_; }

    // this = this * m  (m signed 64-bit)
    void mul_small(long long m);
    // this = this + other * m  (m signed 64-bit)
    void add_mul_small(const BigInt &other, long long m);
    void add(const BigInt &other);
    void negate() { if (!mag_.empty()) neg_ = !neg_; }

    static BigInt mul(const BigInt &a, const BigInt &b);
    static int compare(const BigInt &a, const BigInt &b);  // -1, 0, 1
    static int compare_magnitude(const std::vector<u64> &a, const std::vector<u64> &b);

    // Non-negative remainder of |this| by m (m < 2^63); sign handled by caller.
    u64 magnitude_mod(u64 m) const;
    // Remainder in [0, m) of the signed value.
    u64 mod(u64 m) const;

    // floor(sqrt(this)) for this >= 0; sets exact when the remainder is zero.
    BigInt isqrt(bool &exact) const;

private:
    void trim() {
        while (!mag_.empty() && mag_.back() == 0) mag_.pop_back();
        if (mag_.empty()) neg_ = false;
    }
    static void add_magnitude(std::vector<u64> &a, const std::vector<u64> &b);
    // a -= b, requires |a| >= |b|
    static void sub_magnitude(std::vector<u64> &a, const std::vector<u64> &b);

    std::vector<u64> mag_;
    bool neg_ = false;
};

}  // namespace rpg
