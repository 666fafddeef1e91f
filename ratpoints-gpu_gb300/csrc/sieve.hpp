// Host driver of the device sieve: builds the per-curve tables on the GPU,
// launches the sieve over consecutive denominator batches on a CUDA stream,
// and hands each batch's survivors to the caller while later batches run.
//
// It replaces the reference's run_modular_sieve driver (src/sieve.cu:503-580):
// tables are built once per search instead of once per batch, device buffers
// are allocated once, survivor copies go through pinned memory, and up to two
// batches are in flight so host verification overlaps device work.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace rpg {

enum class PlanKind : int { reference = 0, fast = 1 };

class CudaError : public std::runtime_error {
public:
    using std::runtime_error::runtime_error;
};

// A bounded wait inside a sieve kernel ran out; the launch's output is invalid.
class DeviceTimeout : public std::runtime_error {
public:
    using std::runtime_error::runtime_error;
};

void check_cuda(cudaError_t status, const char *what);

// Shape of a fast plan: the number of stage-1 rows and the row slots (2 or 3)
// each CTA of the single-curve kernel stages.  rows 0: the cost model's choice.
struct FastShape {
    int rows = 0;
    int slots = 0;
};

struct SieveOptions {
    PlanKind plan = PlanKind::reference;
    bool square = false;            // parameters k give denominators k*k
    long long capacity = 1 << 22;   // survivors per device buffer
    int device = -1;                // -1: current device
    // Drop survivors that cannot be points on the device before the copy
    // (gcd and residue tests; see preverify.hpp).  Deliveries then hold a
    // subset of the modular survivors that still contains every point.
    bool preverify = false;
    // Fast plan only: a forced shape (rows > 0); otherwise a shape measured
    // earlier for curves of this kind (tune.hpp), when the tuning cache is
    // enabled and holds one, else the cost model's.
    FastShape fast_shape;
};

// One delivery of survivors.  Pointers stay valid until the next call to
// Sieve::next().  A batch whose survivors exceed one buffer arrives in several
// pieces; complete marks its last piece.
struct BatchView {
    long long first = 0, last = 0;   // parameter range of the batch
    const long long *a = nullptr;
    const int *d = nullptr;
    std::size_t count = 0;
    std::size_t modular = 0;         // modular survivors behind this piece (count, unless pre-verified)
    bool complete = true;
    float kernel_ms = 0.0f;          // event time of the launches behind this piece
};

struct SieveTimings {
    float table_ms = 0.0f;           // device table build (events)
    double table_wall_ms = 0.0;      // host + device table setup
    double plan_ms = 0.0;            // host plan work
    double workspace_ms = 0.0;       // allocations
    double sieve_ms = 0.0;           // sum of sieve launch event times
    unsigned long long launches = 0;
    unsigned long long reruns = 0;   // overflowed launches that were split
    unsigned long long h2d_bytes = 0;
    unsigned long long d2h_bytes = 0;
};

// Frees the idle search pipelines (streams, events, survivor buffers, pinned
// staging) that finished sieves left for reuse on `device` (-1: every
// device).  A process that resets a device must call it first.
void release_pooled_pipelines(int device);

// The fast plan a single-curve sieve uses for a curve and numerator bound
// (host only): the autotuner's choice under the fast kernel's shared-memory
// budget; *max_classes (optional) receives the most classes of one denominator.
// A shape with rows > 0 fixes the row count (the rows filtering most) and the
// row slots instead of the cost model.
struct FastPlan;
FastPlan single_curve_plan(const std::vector<std::string> &coefficients, long long bound, int *max_classes,
                           FastShape shape = FastShape{});

// The fast plan a sieve chose for its curve (empty for the reference plan).
struct FastPlanInfo {
    int class_prime = 0;           // numerator classes are taken mod 64 * class_prime
    std::vector<int> primes;       // small primes tested by the stage-1 rows
    std::vector<int> moduli;       // the stage-1 row moduli (products of those primes)
};

class Sieve {
public:
    Sieve(const std::vector<std::string> &coefficients, long long bound, const SieveOptions &options);
    ~Sieve();
    Sieve(const Sieve &) = delete;
    Sieve &operator=(const Sieve &) = delete;

    // Queue parameters [first, last] as consecutive batches of batch_size.
    void start(long long first, long long last, long long batch_size);
    // Next piece in parameter order; false when every queued batch is delivered.
    bool next(BatchView &out);
    // Drop queued and in-flight work (e.g. after a first-point stop).
    void cancel();

    const SieveTimings &timings() const;
    long long words64() const;

    // Device-resident pass for benchmarks: sieve [first, last] in batches with
    // survivors counted on the device only; returns the survivor count.  The
    // caller times it with the events it records on stream().
    unsigned long long count_only(long long first, long long last, long long batch_size);
    cudaStream_t stream() const;

    // Work of a pass over parameters [first, last]: 64-site words swept by the
    // sieve kernel and shared-memory bytes read per swept word (stage 1).
    unsigned long long swept_words(long long first, long long last) const;
    unsigned smem_bytes_per_word() const;
    FastPlanInfo fast_plan_info() const;

    // Whether a whole row (all numerators of a denominator) fits one launch:
    // false only for very large H (fast plan: more than 2^23 class words,
    // reference plan: more than 2^30 words).
    bool fits_one_launch() const;
    // Enqueue one sieve launch for parameters [first, last] (at most one batch
    // of 65536) on `stream`, writing survivors into caller-owned device arrays
    // and counting them in *out_count; `work` is a zeroed device counter the
    // launch uses for dynamic scheduling, and *error (a device word) becomes
    // nonzero if a bounded wait of the launch gives up.  Allocates nothing;
    // returns false if a row does not fit one launch or the range is invalid.
    bool launch_into(long long first, long long last, long long *out_a, int *out_d,
                     unsigned long long capacity, unsigned long long *out_count,
                     unsigned long long *work, unsigned long long *error, cudaStream_t stream);
    int device() const;

private:
    struct Impl;
    std::unique_ptr<Impl> impl_;
};

}  // namespace rpg
