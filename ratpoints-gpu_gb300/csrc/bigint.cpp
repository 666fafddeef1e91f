#include "bigint.hpp"

#include <algorithm>
#include <cmath>

namespace rpg {

namespace {
constexpr u64 kTen19 = 10000000000000000000ull;
}

void BigInt::assign(long long v) {
    mag_.clear();
    neg_ = v < 0;
    u64 m = neg_ ? u64(0) - u64(v) : u64(v);
    if (m) mag_.push_back(m);
    else neg_ = false;
}

bool BigInt::parse(const std::string &text, BigInt &out) {
    out = BigInt();
    std::size_t i = 0;
    bool neg = false;
    if (i < text.size() && (text[i] == '+' || text[i] == '-')) neg = text[i++] == '-';
    if (i == text.size()) return false;
    // Consume up to 19 digits at a time: out = out * 10^k + chunk.
    while (i < text.size()) {
        std::size_t take = std::min<std::size_t>(19, text.size() - i);
        u64 chunk = 0, scale = 1;
        for (std::size_t j = 0; j < take; ++j) {
            char c = text[i + j];
            if (c < '0' || c > '9') return false;
            chunk = chunk * 10 + u64(c - '0');
            scale *= 10;
        }
        i += take;
        u64 carry = chunk;
        for (auto &limb : out.mag_) {
            u128 t = u128(limb) * scale + carry;
            limb = u64(t);
            carry = u64(t >> 64);
        }
        if (carry) out.mag_.push_back(carry);
    }
    out.neg_ = neg;
    out.trim();
    return true;
}

std::string BigInt::to_string() const {
    if (mag_.empty()) return "0";
    std::vector<u64> work = mag_;
    std::vector<u64> chunks;
    while (!work.empty()) {
        u128 rem = 0;
        for (std::size_t i = work.size(); i-- > 0;) {
            u128 cur = (rem << 64) | work[i];
            work[i] = u64(cur / kTen19);
            rem = cur % kTen19;
        }
        chunks.push_back(u64(rem));
        while (!work.empty() && work.back() == 0) work.pop_back();
    }
    std::string s = neg_ ? "-" : "";
    s += std::to_string(chunks.back());
    for (std::size_t i = chunks.size() - 1; i-- > 0;) {
        std::string part = std::to_string(chunks[i]);
        s.append(19 - part.size(), '0');
        s += part;
    }
    return s;
}

std::size_t BigInt::bit_length() const {
    if (mag_.empty()) return 0;
    return 64 * (mag_.size() - 1) + (64 - std::size_t(__builtin_clzll(mag_.back())));
}

void BigInt::mul_small(long long m) {
    if (m == 0 || mag_.empty()) { mag_.clear(); neg_ = false; return; }
    bool mneg = m < 0;
    u64 mm = mneg ? u64(0) - u64(m) : u64(m);
    u64 carry = 0;
    for (auto &limb : mag_) {
        u128 t = u128(limb) * mm + carry;
        limb = u64(t);
        carry = u64(t >> 64);
    }
    if (carry) mag_.push_back(carry);
    neg_ = neg_ != mneg;
}

void BigInt::add_magnitude(std::vector<u64> &a, const std::vector<u64> &b) {
    if (a.size() < b.size()) a.resize(b.size(), 0);
    u64 carry = 0;
    std::size_t i = 0;
    for (; i < b.size(); ++i) {
        u128 t = u128(a[i]) + b[i] + carry;
        a[i] = u64(t);
        carry = u64(t >> 64);
    }
    for (; carry && i < a.size(); ++i) {
        u128 t = u128(a[i]) + carry;
        a[i] = u64(t);
        carry = u64(t >> 64);
    }
    if (carry) a.push_back(carry);
}

void BigInt::sub_magnitude(std::vector<u64> &a, const std::vector<u64> &b) {
    u64 borrow = 0;
    std::size_t i = 0;
    for (; i < b.size(); ++i) {
        u128 t = u128(a[i]) - b[i] - borrow;
        a[i] = u64(t);
        borrow = u64(t >> 64) ? 1 : 0;
    }
    for (; borrow && i < a.size(); ++i) {
        u128 t = u128(a[i]) - borrow;
        a[i] = u64(t);
        borrow = u64(t >> 64) ? 1 : 0;
    }
    while (!a.empty() && a.back() == 0) a.pop_back();
}

int BigInt::compare_magnitude(const std::vector<u64> &a, const std::vector<u64> &b) {
    if (a.size() != b.size()) return a.size() < b.size() ? -1 : 1;
    for (std::size_t i = a.size(); i-- > 0;)
        if (a[i] != b[i]) return a[i] < b[i] ? -1 : 1;
    return 0;
}

void BigInt::add(const BigInt &other) {
    if (other.mag_.empty()) return;
    if (mag_.empty()) { *this = other; return; }
    if (neg_ == other.neg_) {
        add_magnitude(mag_, other.mag_);
        return;
    }
    int c = compare_magnitude(mag_, other.mag_);
    if (c == 0) { mag_.clear(); neg_ = false; return; }
    if (c > 0) {
        sub_magnitude(mag_, other.mag_);
    } else {
        std::vector<u64> t = other.mag_;
        sub_magnitude(t, mag_);
        mag_.swap(t);
        neg_ = other.neg_;
    }
    trim();
}

void BigInt::add_mul_small(const BigInt &other, long long m) {
    if (m == 0 || other.mag_.empty()) return;
    BigInt t = other;
    t.mul_small(m);
    add(t);
}

BigInt BigInt::mul(const BigInt &a, const BigInt &b) {
    BigInt r;
    if (a.mag_.empty() || b.mag_.empty()) return r;
    r.mag_.assign(a.mag_.size() + b.mag_.size(), 0);
    for (std::size_t i = 0; i < a.mag_.size(); ++i) {
        u64 carry = 0;
        for (std::size_t j = 0; j < b.mag_.size(); ++j) {
            u128 t = u128(a.mag_[i]) * b.mag_[j] + r.mag_[i + j] + carry;
            r.mag_[i + j] = u64(t);
            carry = u64(t >> 64);
        }
        r.mag_[i + b.mag_.size()] = carry;
    }
    r.neg_ = a.neg_ != b.neg_;
    r.trim();
    return r;
}

int BigInt::compare(const BigInt &a, const BigInt &b) {
    int sa = a.sign(), sb = b.sign();
    if (sa != sb) return sa < sb ? -1 : 1;
    int c = compare_magnitude(a.mag_, b.mag_);
    return sa < 0 ? -c : c;
}

u64 BigInt::magnitude_mod(u64 m) const {
    u128 rem = 0;
    for (std::size_t i = mag_.size(); i-- > 0;) rem = ((rem << 64) | mag_[i]) % m;
    return u64(rem);
}

u64 BigInt::mod(u64 m) const {
    u64 r = magnitude_mod(m);
    return (neg_ && r) ? m - r : r;
}

BigInt BigInt::isqrt(bool &exact) const {
    exact = false;
    BigInt root;
    if (neg_) return root;
    if (mag_.empty()) { exact = true; return root; }
    if (mag_.size() <= 2) {
        // 128-bit path: floating estimate, then exact correction.
        u128 n = mag_[0] | (mag_.size() == 2 ? u128(mag_[1]) << 64 : u128(0));
        constexpr u128 kMaxRoot = ~u64(0);  // floor(sqrt(2^128 - 1))
        u128 r = u128(std::sqrt(static_cast<long double>(n)));
        if (r > kMaxRoot) r = kMaxRoot;
        while (r * r > n) --r;
        while (r < kMaxRoot && (r + 1) * (r + 1) <= n) ++r;
        exact = r * r == n;
        root.mag_.push_back(u64(r));
        if (u64(r >> 64)) root.mag_.push_back(u64(r >> 64));
        root.trim();
        return root;
    }
    // Restoring digit-by-digit square root, two bits per step:
    //   rem = 4 rem + next two bits; trial = 4 res + 1;
    //   if rem >= trial: rem -= trial, res = 2 res + 1, else res = 2 res.
    std::size_t bits = bit_length();
    std::size_t top = (bits + 1) / 2 * 2;
    std::vector<u64> rem, res, trial;
    auto shift_in = [](std::vector<u64> &v, unsigned k, u64 low) {
        u64 carry = low;
        for (auto &limb : v) {
            u64 next = limb >> (64 - k);
            limb = (limb << k) | carry;
            carry = next;
        }
        if (carry) v.push_back(carry);
    };
    for (std::size_t pos = top; pos >= 2; pos -= 2) {
        std::size_t b = pos - 2;
        u64 two = (b / 64 < mag_.size()) ? (mag_[b / 64] >> (b % 64)) & 3u : 0;
        shift_in(rem, 2, two);
        trial = res;
        shift_in(trial, 2, 1);
        if (compare_magnitude(rem, trial) >= 0) {
            sub_magnitude(rem, trial);
            shift_in(res, 1, 1);
        } else {
            shift_in(res, 1, 0);
        }
    }
    exact = rem.empty();
    root.mag_ = res;
    root.trim();
    return root;
}

}  // namespace rpg
