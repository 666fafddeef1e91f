// Link-level check of the C++ drop-in boundary: a caller written against the
// reference's include/sieve.hpp (run_modular_sieve, CandidateBatch,
// DenominatorRange), compiled against include/ratpoints_gpu/sieve.hpp and
// linked with librpgpu.  Mirrors the reference's own boundary test
// (tests/test_sieve_streaming.cpp:45-81): on y^2 = 1 + P x, with P the
// product of the 32 largest primes below 512, every site survives the
// reference plan, so the stream must deliver every (a, d) of the box exactly
// once.  Exit status 0 when every case holds; the failing case is printed.
#include <cstdio>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "ratpoints_gpu/sieve.hpp"

namespace {

// Decimal string of a product of small factors (base 10^9 limbs).
std::string decimal_product(const std::vector<int> &factors) {
    std::vector<std::uint32_t> limbs{1};
    for (int f : factors) {
        std::uint64_t carry = 0;
        for (auto &limb : limbs) {
            const std::uint64_t v = std::uint64_t(limb) * std::uint64_t(f) + carry;
            limb = std::uint32_t(v % 1000000000u);
            carry = v / 1000000000u;
        }
        if (carry) limbs.push_back(std::uint32_t(carry));
    }
    std::string out = std::to_string(limbs.back());
    for (std::size_t i = limbs.size() - 1; i-- > 0;) {
        std::string part = std::to_string(limbs[i]);
        out += std::string(9 - part.size(), '0') + part;
    }
    return out;
}

ratpoints_gpu::Coefficients dense_curve() {
    std::vector<int> primes;
    for (int v = 2; v < 512; ++v) {
        bool prime = true;
        for (int q = 2; q * q <= v; ++q) prime = prime && v % q != 0;
        if (prime) primes.push_back(v);
    }
    return {"1", decimal_product(std::vector<int>(primes.end() - 32, primes.end()))};
}

// Sieve the dense curve over [-bound, bound] x [first, last] and require every
// site exactly once, inside the box, in batches of consistent size.
bool every_site_once(long long bound, int first, int last, bool square) {
    const std::size_t width = std::size_t(2 * bound + 1);
    const std::size_t expected = width * std::size_t(last - first + 1);
    std::vector<bool> seen(expected, false);
    std::size_t delivered = 0;
    std::size_t callbacks = 0;
    const auto result = ratpoints_gpu::run_modular_sieve(
        dense_curve(), bound, ratpoints_gpu::DenominatorRange{first, last},
        [&](const ratpoints_gpu::CandidateBatch &batch) {
            if (batch.denominators.size() != batch.size())
                throw std::runtime_error("candidate batch arrays differ in length");
            ++callbacks;
            delivered += batch.size();
            for (std::size_t i = 0; i < batch.size(); ++i) {
                const long long a = batch.numerators[i];
                const int d = batch.denominators[i];
                int k = d;
                if (square) {
                    k = 0;
                    while ((long long)(k + 1) * (k + 1) <= d) ++k;
                    if ((long long)k * k != d) throw std::runtime_error("denominator is not a square");
                }
                if (a < -bound || a > bound || k < first || k > last)
                    throw std::runtime_error("candidate outside the search box");
                const std::size_t index = std::size_t(k - first) * width + std::size_t(a + bound);
                if (seen[index]) throw std::runtime_error("duplicate modular candidate");
                seen[index] = true;
            }
        },
        square);
    bool all = true;
    for (bool s : seen) all = all && s;
    if (result.survivor_count != expected || delivered != expected || !all || callbacks == 0) {
        std::fprintf(stderr, "bound=%lld range=[%d,%d] square=%d: survivors=%llu delivered=%zu expected=%zu\n",
                     bound, first, last, int(square), result.survivor_count, delivered, expected);
        return false;
    }
    if (result.metrics.word_count != (unsigned long long)((2 * bound + 32) / 32)) {
        std::fprintf(stderr, "word_count %llu\n", result.metrics.word_count);
        return false;
    }
    return true;
}

}  // namespace

int main() {
    int failures = 0;
    // the reference's case: H = 5000, d in [1, 2], 20,002 sites
    failures += !every_site_once(5000, 1, 2, false);
    // 200,020 sites: more than one survivor buffer holds, so the driver grows
    // its buffers and the stream stays complete and duplicate-free
    failures += !every_site_once(5000, 1, 20, false);
    // square denominators d = k^2, k in [3, 12]
    failures += !every_site_once(300, 3, 12, true);
    // an invalid range is rejected with std::invalid_argument, as the
    // reference's SievePlan does (src/sieve_plan.cpp:110-113)
    try {
        ratpoints_gpu::run_modular_sieve(dense_curve(), 10, ratpoints_gpu::DenominatorRange{5, 4},
                                         [](const ratpoints_gpu::CandidateBatch &) {});
        std::fprintf(stderr, "empty range accepted\n");
        ++failures;
    } catch (const std::invalid_argument &) {
    }
    if (failures == 0) std::printf("run_modular_sieve boundary: all cases hold\n");
    return failures == 0 ? 0 : 1;
}
