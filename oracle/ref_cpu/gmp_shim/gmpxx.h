// mpz_class and mpq_class: the part of GMP's C++ interface that the
// reference's host code uses (construction from integers, decimal strings and
// other values; + - * / and their compound forms; comparisons; get_str,
// get_mpz_t, canonicalize), written for this project over the C interface
// declared in gmp.h.  Plain value classes: every operation computes its result
// at once.  CHECKER INFRASTRUCTURE ONLY (oracle/ref_cpu/build_mock.py).
#ifndef RPG_GMPXX_SHIM_H
#define RPG_GMPXX_SHIM_H

#include <cstdlib>
#include <stdexcept>
#include <string>

#include "gmp.h"

class mpz_class {
public:
    mpz_class() { __gmpz_init(v_); }
    mpz_class(long x) { __gmpz_init_set_si(v_, x); }                // NOLINT: implicit, as in GMP
    mpz_class(int x) { __gmpz_init_set_si(v_, x); }                 // NOLINT
    mpz_class(unsigned long x) { __gmpz_init_set_si(v_, long(x)); }  // NOLINT (values below 2^63)
    mpz_class(long long x) { __gmpz_init_set_si(v_, long(x)); }     // NOLINT (LP64: long is 64-bit)
    mpz_class(const std::string &s, int base = 10) { init_str(s.c_str(), base); }
    mpz_class(const char *s, int base = 10) { init_str(s, base); }
    mpz_class(const mpz_class &o) { __gmpz_init_set(v_, o.v_); }
    mpz_class(mpz_class &&o) noexcept {
        __gmpz_init(v_);
        __gmpz_swap(v_, o.v_);
    }
    ~mpz_class() { __gmpz_clear(v_); }
    mpz_class &operator=(const mpz_class &o) {
        if (this != &o) __gmpz_set(v_, o.v_);
        return *this;
    }
    mpz_class &operator=(mpz_class &&o) noexcept {
        __gmpz_swap(v_, o.v_);
        return *this;
    }

    mpz_ptr get_mpz_t() { return v_; }
    mpz_srcptr get_mpz_t() const { return v_; }
    std::string get_str(int base = 10) const {
        char *s = __gmpz_get_str(nullptr, base, v_);
        std::string out(s);
        std::free(s);  // the library's default allocator is malloc
        return out;
    }

    mpz_class &operator+=(const mpz_class &o) {
        __gmpz_add(v_, v_, o.v_);
        return *this;
    }
    mpz_class &operator-=(const mpz_class &o) {
        __gmpz_sub(v_, v_, o.v_);
        return *this;
    }
    mpz_class &operator*=(const mpz_class &o) {
        __gmpz_mul(v_, v_, o.v_);
        return *this;
    }
    mpz_class operator-() const {
        mpz_class r;
        __gmpz_neg(r.v_, v_);
        return r;
    }
    friend mpz_class operator+(const mpz_class &a, const mpz_class &b) {
        mpz_class r;
        __gmpz_add(r.v_, a.v_, b.v_);
        return r;
    }
    friend mpz_class operator-(const mpz_class &a, const mpz_class &b) {
        mpz_class r;
        __gmpz_sub(r.v_, a.v_, b.v_);
        return r;
    }
    friend mpz_class operator*(const mpz_class &a, const mpz_class &b) {
        mpz_class r;
        __gmpz_mul(r.v_, a.v_, b.v_);
        return r;
    }
    friend int cmp(const mpz_class &a, const mpz_class &b) { return __gmpz_cmp(a.v_, b.v_); }
    friend bool operator<(const mpz_class &a, const mpz_class &b) { return cmp(a, b) < 0; }
    friend bool operator>(const mpz_class &a, const mpz_class &b) { return cmp(a, b) > 0; }
    friend bool operator<=(const mpz_class &a, const mpz_class &b) { return cmp(a, b) <= 0; }
    friend bool operator>=(const mpz_class &a, const mpz_class &b) { return cmp(a, b) >= 0; }
    friend bool operator==(const mpz_class &a, const mpz_class &b) { return cmp(a, b) == 0; }
    friend bool operator!=(const mpz_class &a, const mpz_class &b) { return cmp(a, b) != 0; }
    friend bool operator<(const mpz_class &a, long b) { return __gmpz_cmp_si(a.v_, b) < 0; }
    friend bool operator<(const mpz_class &a, int b) { return __gmpz_cmp_si(a.v_, b) < 0; }
    friend bool operator==(const mpz_class &a, int b) { return __gmpz_cmp_si(a.v_, b) == 0; }

private:
    void init_str(const char *s, int base) {
        if (__gmpz_init_set_str(v_, s, base) != 0) {
            __gmpz_clear(v_);
            throw std::invalid_argument("mpz_set_str");
        }
    }
    mpz_t v_;
};

class mpq_class {
public:
    mpq_class() { __gmpq_init(v_); }
    mpq_class(long x) {  // NOLINT: implicit, as in GMP
        __gmpq_init(v_);
        __gmpq_set_si(v_, x, 1);
    }
    mpq_class(int x) : mpq_class(long(x)) {}  // NOLINT
    mpq_class(const mpz_class &z) {            // NOLINT
        __gmpq_init(v_);
        __gmpq_set_z(v_, z.get_mpz_t());
    }
    // numerator / denominator as given (canonicalize() reduces it)
    mpq_class(const mpz_class &n, const mpz_class &d) {
        __gmpq_init(v_);
        __gmpz_set(&v_->_mp_num, n.get_mpz_t());
        __gmpz_set(&v_->_mp_den, d.get_mpz_t());
    }
    explicit mpq_class(const std::string &s, int base = 10) {
        __gmpq_init(v_);
        if (__gmpq_set_str(v_, s.c_str(), base) != 0) {
            __gmpq_clear(v_);
            throw std::invalid_argument("mpq_set_str");
        }
    }
    mpq_class(const mpq_class &o) {
        __gmpq_init(v_);
        __gmpq_set(v_, o.v_);
    }
    mpq_class(mpq_class &&o) noexcept {
        __gmpq_init(v_);
        __gmpq_swap(v_, o.v_);
    }
    ~mpq_class() { __gmpq_clear(v_); }
    mpq_class &operator=(const mpq_class &o) {
        if (this != &o) __gmpq_set(v_, o.v_);
        return *this;
    }
    mpq_class &operator=(mpq_class &&o) noexcept {
        __gmpq_swap(v_, o.v_);
        return *this;
    }

    mpq_ptr get_mpq_t() { return v_; }
    mpq_srcptr get_mpq_t() const { return v_; }
    void canonicalize() { __gmpq_canonicalize(v_); }

    mpq_class &operator+=(const mpq_class &o) {
        __gmpq_add(v_, v_, o.v_);
        return *this;
    }
    mpq_class &operator-=(const mpq_class &o) {
        __gmpq_sub(v_, v_, o.v_);
        return *this;
    }
    mpq_class &operator*=(const mpq_class &o) {
        __gmpq_mul(v_, v_, o.v_);
        return *this;
    }
    mpq_class &operator/=(const mpq_class &o) {
        __gmpq_div(v_, v_, o.v_);
        return *this;
    }
    mpq_class &operator/=(int d) { return *this /= mpq_class(long(d)); }
    friend mpq_class operator+(const mpq_class &a, const mpq_class &b) {
        mpq_class r;
        __gmpq_add(r.v_, a.v_, b.v_);
        return r;
    }
    friend mpq_class operator-(const mpq_class &a, const mpq_class &b) {
        mpq_class r;
        __gmpq_sub(r.v_, a.v_, b.v_);
        return r;
    }
    friend mpq_class operator*(const mpq_class &a, const mpq_class &b) {
        mpq_class r;
        __gmpq_mul(r.v_, a.v_, b.v_);
        return r;
    }
    friend mpq_class operator*(const mpq_class &a, unsigned long b) { return a * mpq_class(long(b)); }
    friend mpq_class operator/(const mpq_class &a, const mpq_class &b) {
        mpq_class r;
        __gmpq_div(r.v_, a.v_, b.v_);
        return r;
    }
    friend int cmp(const mpq_class &a, const mpq_class &b) { return __gmpq_cmp(a.v_, b.v_); }
    friend bool operator<(const mpq_class &a, const mpq_class &b) { return cmp(a, b) < 0; }
    friend bool operator>(const mpq_class &a, const mpq_class &b) { return cmp(a, b) > 0; }
    friend bool operator<=(const mpq_class &a, const mpq_class &b) { return cmp(a, b) <= 0; }
    friend bool operator>=(const mpq_class &a, const mpq_class &b) { return cmp(a, b) >= 0; }
    friend bool operator==(const mpq_class &a, const mpq_class &b) { return cmp(a, b) == 0; }
    friend bool operator!=(const mpq_class &a, const mpq_class &b) { return cmp(a, b) != 0; }
    friend bool operator==(const mpq_class &a, int b) { return __gmpq_cmp_si(a.v_, b, 1) == 0; }

private:
    mpq_t v_;
};

#endif
