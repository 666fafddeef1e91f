// Measured tuning of the single-curve fast plan's shape.
//
// The cost model of the planner (plan.hpp) picks how many stage-1 rows a
// curve gets and whether each CTA stages two or three denominators.  The tuner
// measures instead: for a curve it builds the sieve with the cost model's
// shape and with its neighbours (one and two rows fewer or more, the other
// slot count), times each on a sample of the search's denominators with CUDA
// events, and keeps the fastest.  Choices persist in a JSON file, keyed by
// the kind of curve (degree, class prime, row length, small- or large-prime
// rows), and every later sieve of a curve of that kind uses the stored shape.
// The file is named by the RPG_TUNE_CACHE environment variable; without it no
// shape is read or stored and sieves use the cost model.  No counterpart in
// the reference, whose prime set and kernel shape are fixed
// (src/sieve_plan.cpp:104-151, tests/tune_cuda.py times build variants).
#pragma once

#include <string>
#include <utility>
#include <vector>

#include "batch.hpp"
#include "sieve.hpp"

namespace rpg {

struct TuneCandidate {
    FastShape shape;                 // rows as planned (the plan may use fewer than asked)
    double bits = 0;                 // stage-1 filtering of the plan
    double ms = 0;                   // device time of the sample
    unsigned long long survivors = 0;
};

struct TuneResult {
    std::string key;
    FastShape chosen;
    std::vector<TuneCandidate> candidates;
    long long sample = 0;            // denominators timed per candidate
    bool stored = false;             // written to the cache file
};

// The kind of curve a stored shape applies to.
std::string fast_shape_key(const std::vector<std::string> &coefficients, long long bound);

// The stored shape for this kind of curve (rows 0: none, or no cache file).
FastShape tuned_fast_shape(const std::vector<std::string> &coefficients, long long bound);

// Times the candidate shapes on parameters [first, first + sample) (clipped to
// last) and stores the fastest when the cache is enabled.
TuneResult tune_fast_shape(const std::vector<std::string> &coefficients, long long bound, long long first,
                           long long last, bool square, int device, long long sample);

// The cache file (RPG_TUNE_CACHE), empty when tuning results are not kept.
std::string tune_cache_path();

// Measured tuning of the batch engine's work items.  The batched kernels take
// (curve, denominator range) items from device queues, each kernel's work cut
// into about items_per_kernel items.  The tuner runs a batch with 2,048,
// 8,192 and 32,768 items per kernel on one engine (after a warm-up run), keeps
// the one with the least batched sieve time and stores it under the kind of
// batch: its curve count, median row length and median degree (low: at most
// 6), counts and lengths in powers of two.  Later batches of that kind use it.
struct BatchTuneResult {
    std::string key;
    int items = 0;                                   // the chosen items per kernel
    std::vector<std::pair<int, double>> candidates;  // (items per kernel, batched sieve ms)
    bool stored = false;
};

std::string batch_items_key(const std::vector<BatchCurveSpec> &curves);

// The stored items per kernel for this kind of batch (0: none, or no cache file).
int tuned_batch_items(const std::vector<BatchCurveSpec> &curves);

BatchTuneResult tune_batch_items(const std::vector<BatchCurveSpec> &curves, int device);

}  // namespace rpg
