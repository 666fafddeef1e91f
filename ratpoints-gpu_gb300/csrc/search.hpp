// Point search over one GPU: the reference's PointSearch
// (include/point_search.hpp:22-78, src/point_search.cpp:28-99, 101-146, 171-240)
// on a single-device batch queue.
//
// Contract kept from the reference: the point at infinity first (if requested
// and present); then batches of batch_size denominators in ascending order;
// within a batch, points sorted by (denominator, numerator); each verified
// point passes the closed-interval filter before the callback; the callback
// returns false to stop.  exact_survivors counts verified points before the
// interval filter, per completed batch.
#pragma once

#include <functional>
#include <string>
#include <vector>

#include "exact.hpp"
#include "sieve.hpp"

namespace rpg {

struct SearchInterval {
    Rational lower, upper;
    bool lower_infinite = false;
    bool upper_infinite = false;
};

struct SearchOptions {
    std::vector<std::string> coefficients;
    long long numerator_bound = 0;
    long long first = 1;             // first parameter (denominator, or k in square mode)
    long long last = 0;
    std::vector<SearchInterval> intervals;
    bool include_infinity = true;
    std::vector<int> devices;        // empty: all visible; the first listed is used
    int batch_size = 1 << 16;
    bool square = false;
    PlanKind plan = PlanKind::fast;
    int verify_threads = 0;          // 0: hardware concurrency
    long long capacity = 1 << 22;    // survivors per device buffer
    bool device_preverify = true;    // drop non-points on the device first (preverify.hpp)

    bool accepts(long long numerator, long long denominator) const;
};

struct PointPair {
    long long numerator;
    std::string ordinate;
    long long denominator;
};

struct GpuDevice {
    int id = 0;
    std::string name;
    int major = 0, minor = 0, multiprocessors = 0;
    unsigned long long memory_bytes = 0;
    std::string pci_bus_id;
};

struct DeviceMetrics {
    GpuDevice device;
    unsigned long long denominator_count = 0, batches = 0;
    double basis_ms = 0, sieve_ms = 0;
};

struct SearchMetrics {
    double wall_ms = 0;
    std::vector<DeviceMetrics> devices;
    double basis_ms = 0, sieve_ms = 0, plan_ms = 0, workspace_ms = 0, basis_wall_ms = 0;
    double survivor_setup_ms = 0, verification_ms = 0, sieve_wall_ms = 0;
    unsigned long long word_count = 0;          // 32-site words per row, as the reference reports
    unsigned long long denominator_count = 0;
    unsigned long long modular_survivors = 0;
    long double initial_mask_bytes = 0;
    unsigned long long exact_survivors = 0;
    unsigned long long host_candidates = 0;     // survivors given to the host's exact check
    unsigned long long launches = 0;
    unsigned long long h2d_bytes = 0, d2h_bytes = 0;
    double initial_mask_gbs() const;
};

using PointCallback = std::function<bool(const PointPair &)>;

// Construction validates the options (batch size, exact squarefreeness, device
// selection) and throws std::invalid_argument, before any output is written, as
// the reference's PointSearch constructor does (point_search.cpp:155-168).
// run() throws CudaError for device failures.
class PointSearch {
public:
    explicit PointSearch(SearchOptions options);
    SearchMetrics run(const PointCallback &callback);

private:
    SearchOptions options_;
    ExactPolynomial poly_;
    std::vector<GpuDevice> devices_;
};

// gpu_devices.cpp equivalents (src/gpu_devices.cpp:21-101).
std::vector<int> parse_device_selection(const std::string &text);
std::vector<GpuDevice> available_gpu_devices();
std::vector<GpuDevice> select_gpu_devices(const std::vector<int> &ids);

}  // namespace rpg
