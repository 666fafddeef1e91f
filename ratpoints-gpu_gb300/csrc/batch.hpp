// Batched many-curve search: every curve's tables resident on the device at
// once and two persistent kernels over device work queues of
// (curve, denominator range) items, captured in one CUDA graph.
//
// No counterpart in the reference, which searches one curve per process
// (src/main.cpp:48-85); each curve's result here is the result of a
// single-curve PointSearch of that curve (src/point_search.cpp:171-240): same
// points, same order, the point at infinity first.
//
// Two shapes, chosen per curve by its row length W = ceil((2H + 1) / 64):
//   - wide rows (W >= kBatchWideWords): the class-strided layout of the
//     single-curve fast kernel (numerator classes mod 64 q, one CTA per
//     denominator, stage-1 rows of up to six composite moduli staged into
//     shared memory by TMA bulk copies), with per-curve descriptors;
//   - narrow rows: one warp per denominator over dense 64-site words, the
//     curve's whole stage-1 tables (moduli <= kBatchNarrowModulus, m x m
//     words each) loaded into shared memory once per work item.
// Both kernels finish with the reference's 32 selected primes tested bit by
// bit against per-curve bitmasks of f(x) mod p, then the host verifies each
// survivor exactly.
#pragma once

#include <memory>
#include <string>
#include <vector>

#include "search.hpp"

namespace rpg {

constexpr long long kBatchWideWords = 2048;
// Rows of at least this many words (numerator bounds above about 4.2e6) make
// a curve fill the device alone; a batch searches such curves one by one with
// the single-curve kernel, beside its batched kernels.
constexpr long long kBatchSoloWords = 1LL << 17;
constexpr int kBatchNarrowModulus = 34;
// Work items per batched kernel: enough that a small batch spreads over the
// device, few enough that building and fetching them stays cheap.
constexpr int kDefaultBatchItems = 8192;

struct BatchCurveSpec {
    std::vector<std::string> coefficients;
    long long bound = 0;                       // numerator bound H
    long long first = 1, last = 0;             // denominators (k in square mode)
    bool square = false;                       // denominators k^2
    bool include_infinity = true;
    std::vector<SearchInterval> intervals;     // empty: all of [-H, H]
};

struct BatchCurveResult {
    int status = 0;                    // rpg_status code (0 = ok)
    std::string error;
    std::vector<PointPair> points;     // the order of a single-curve search
    unsigned long long survivors = 0;  // modular survivors of the batched sieve
    bool wide = false;                 // which kernel swept the curve
    bool solo = false;                 // huge rows: searched alone by the single-curve kernel
    int class_prime = 1;
    std::vector<int> moduli;           // stage-1 moduli the autotuner chose
};

struct BatchStats {
    unsigned long long curves = 0, wide_curves = 0, denominators = 0, survivors = 0, points = 0;
    unsigned long long host_candidates = 0;   // survivors given to the host's exact check
    unsigned long long solo_curves = 0;       // curves with huge rows searched alone
    unsigned long long wide_items = 0, narrow_items = 0, launches = 0, words = 0;
    unsigned long long table_words = 0;
    unsigned long long swept_words = 0;       // 64-site words the sieve kernels sweep (counted by them)
    unsigned long long smem_bytes = 0;        // stage-1 shared-memory bytes those sweeps read
    long double rectangle_sites = 0;
    double plan_ms = 0, table_ms = 0, sieve_ms = 0, verify_ms = 0, wall_ms = 0;
    double wide_ms = 0, narrow_ms = 0;
    unsigned long long h2d_bytes = 0, d2h_bytes = 0;
    bool graph = false;
    int items_per_kernel = 0;                 // the work-item target the run used
    bool items_from_cache = false;            // a stored tuning result chose it
};

// Device resources of batched runs kept across runs: streams, events, the
// curve-independent tables and grow-only device buffers (tables, bitmasks,
// descriptors, work items, survivors), so that a run allocates nothing once
// the buffers are large enough.  One engine serves one thread at a time.
class BatchEngine {
public:
    explicit BatchEngine(int device);  // -1: the calling thread's current device
    ~BatchEngine();
    BatchEngine(const BatchEngine &) = delete;
    BatchEngine &operator=(const BatchEngine &) = delete;

    // Runs every valid curve in one batched pass.  Curves that fail
    // validation get a nonzero status and no points; the others are searched
    // together.  The table build and sieve launches are captured in one CUDA
    // graph when use_graph is set.  With preverify a kernel drops the
    // survivors that cannot be points before the copy to the host
    // (preverify.hpp); the points are the same either way.  Each kernel's
    // work is cut into about items_per_kernel (curve, denominator range)
    // items; 0 takes the tuned value for this kind of batch (tune.hpp), else
    // kDefaultBatchItems.
    std::vector<BatchCurveResult> run(const std::vector<BatchCurveSpec> &curves, BatchStats *stats,
                                      bool use_graph = true, bool preverify = true, int items_per_kernel = 0);
    int device() const;

    // Upper estimate of the device bytes a curve adds to a run (admission).
    static unsigned long long estimate_bytes(const BatchCurveSpec &curve);

private:
    struct Impl;
    std::unique_ptr<Impl> impl_;
};

// One batched pass on a fresh engine on `device` (-1: current).
std::vector<BatchCurveResult> batch_search(const std::vector<BatchCurveSpec> &curves, int device,
                                           BatchStats *stats, bool use_graph = true, bool preverify = true);

}  // namespace rpg
