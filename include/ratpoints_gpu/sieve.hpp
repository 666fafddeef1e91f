// C++ drop-in declarations for the modular sieve boundary.
//
// These types and the run_modular_sieve signature are kept identical to the
// reference's include/sieve.hpp:13-47 and include/search_types.hpp:8-22, so
// its PointSearch (src/point_search.cpp) links against librpgpu in place of
// src/sieve.cu, the same way its host mock backend replaces that symbol
// (tests/mock_backend.cpp:87-135).  librpgpu's definition drives the device
// sieve with the reference plan, so the delivered candidate set is the
// reference's.
#ifndef RATPOINTS_GPU_COMPAT_SIEVE_HPP
#define RATPOINTS_GPU_COMPAT_SIEVE_HPP

#include <cstddef>
#include <functional>
#include <string>
#include <vector>

namespace ratpoints_gpu {

using Coefficients = std::vector<std::string>;

struct DenominatorRange {
    int first;
    int last;
    int count() const { return last - first + 1; }
};

struct SieveMetrics {
    float basis_ms = 0.0f;
    float sieve_ms = 0.0f;
    double plan_ms = 0.0;
    double workspace_ms = 0.0;
    double basis_wall_ms = 0.0;
    double survivor_setup_ms = 0.0;
    double verification_ms = 0.0;
    double sieve_wall_ms = 0.0;
    unsigned long long word_count = 0;
    long double initial_mask_bytes = 0.0L;
};

struct SieveResult {
    unsigned long long survivor_count = 0;
    SieveMetrics metrics;
};

struct CandidateBatch {
    std::vector<long long> numerators;
    std::vector<int> denominators;
    std::size_t size() const { return numerators.size(); }
};

using CandidateBatchCallback = std::function<void(const CandidateBatch &)>;

// Each delivered batch is consumed synchronously; device work on later
// batches may already be running while the callback executes.
SieveResult run_modular_sieve(const Coefficients &coefficients, long long numerator_bound,
                              DenominatorRange denominators,
                              const CandidateBatchCallback &callback,
                              bool square_denominators = false);

}  // namespace ratpoints_gpu

#endif
