// ratpoints_gpu::run_modular_sieve on the GB300 device sieve (reference plan),
// the C++ drop-in for the reference's src/sieve.cu:503-580.
#include "ratpoints_gpu/sieve.hpp"

#include <chrono>
#include <limits>
#include <stdexcept>

#include "plan.hpp"
#include "sieve.hpp"

namespace ratpoints_gpu {

SieveResult run_modular_sieve(const Coefficients &coefficients, long long numerator_bound,
                              DenominatorRange denominators, const CandidateBatchCallback &callback,
                              bool square_denominators) {
    using Clock = std::chrono::steady_clock;
    if (denominators.first < 1 || denominators.first > denominators.last ||
        (square_denominators && denominators.last > 46340))
        throw std::invalid_argument("invalid denominator range");  // sieve_plan.cpp:110-113
    rpg::SieveOptions options;
    options.plan = rpg::PlanKind::reference;
    options.square = square_denominators;
    rpg::Sieve sieve(coefficients, numerator_bound, options);
    const auto started = Clock::now();
    sieve.start(denominators.first, denominators.last, denominators.count());
    rpg::BatchView view;
    SieveResult result;
    double verification_ms = 0;
    CandidateBatch batch;
    while (sieve.next(view)) {
        if (view.count > std::numeric_limits<unsigned long long>::max() - result.survivor_count)
            throw std::overflow_error("total survivor count overflow");
        result.survivor_count += view.count;
        if (!view.count) continue;
        batch.numerators.assign(view.a, view.a + view.count);
        batch.denominators.assign(view.d, view.d + view.count);
        const auto v0 = Clock::now();
        callback(batch);
        verification_ms += std::chrono::duration<double, std::milli>(Clock::now() - v0).count();
    }
    const auto &t = sieve.timings();
    SieveMetrics &m = result.metrics;
    m.basis_ms = float(t.table_ms);
    m.sieve_ms = float(t.sieve_ms);
    m.plan_ms = t.plan_ms;
    m.workspace_ms = t.workspace_ms;
    m.basis_wall_ms = t.table_wall_ms;
    m.verification_ms = verification_ms;
    m.sieve_wall_ms =
        std::chrono::duration<double, std::milli>(Clock::now() - started).count() - verification_ms;
    m.word_count = (unsigned long long)rpg::word_count32(numerator_bound);
    m.initial_mask_bytes = (long double)denominators.count() * (long double)m.word_count * 14.0L * 4.0L;
    return result;
}

}  // namespace ratpoints_gpu
