#include "search.hpp"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <limits>
#include <stdexcept>
#include <thread>

#include "plan.hpp"

namespace rpg {

namespace {

using Clock = std::chrono::steady_clock;
double ms_since(Clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
}

long long integer_gcd(long long a, long long b) {
    // point_search.cpp:28-38
    if (a < 0) a = -a;
    while (b) {
        long long next = a % b;
        a = b;
        b = next;
    }
    return a;
}

struct Found {
    long long a;
    long long d;
    std::string y;
};

// gcd(a, d) = 1 and F(a, d) a square (point_search.cpp:48-60), over a thread pool
// for large survivor batches.
void verify(const ExactPolynomial &poly, const long long *a, const int *d, std::size_t n,
            int threads, std::vector<Found> &out) {
    auto check_range = [&](std::size_t lo, std::size_t hi, std::vector<Found> &sink) {
        std::string root;
        for (std::size_t i = lo; i < hi; ++i) {
            if (integer_gcd(a[i], d[i]) != 1) continue;
            if (poly.square_root(a[i], d[i], root)) sink.push_back(Found{a[i], d[i], root});
        }
    };
    constexpr std::size_t kChunk = 1 << 14;
    if (threads <= 1 || n < 2 * kChunk) {
        check_range(0, n, out);
        return;
    }
    const std::size_t chunks = (n + kChunk - 1) / kChunk;
    const int workers = int(std::min<std::size_t>(std::size_t(threads), chunks));
    std::vector<std::vector<Found>> parts(workers);
    std::atomic<std::size_t> next{0};
    std::vector<std::thread> pool;
    for (int t = 0; t < workers; ++t) {
        pool.emplace_back([&, t] {
            for (std::size_t c; (c = next.fetch_add(1)) < chunks;)
                check_range(c * kChunk, std::min(n, (c + 1) * kChunk), parts[t]);
        });
    }
    for (auto &th : pool) th.join();
    for (auto &p : parts) out.insert(out.end(), p.begin(), p.end());
}

void validate(const SearchOptions &options, const ExactPolynomial &poly) {
    // point_search.cpp:17-26
    if (options.batch_size < 1 || options.batch_size > (1 << 16))
        throw std::invalid_argument("denominator batch size must be in 1..65536");
    if (!poly.is_squarefree()) throw std::invalid_argument("polynomial is not squarefree");
}

void require_cuda(cudaError_t status, const char *operation) {
    if (status != cudaSuccess)
        throw CudaError(std::string(operation) + ": " + cudaGetErrorString(status));
}

}  // namespace

namespace {

// numerator/denominator inside the closed interval (an infinite end always holds).
bool inside(const SearchInterval &iv, long long numerator, long long denominator) {
    // compare_fraction gives sign(numerator/denominator - bound)
    if (!iv.lower_infinite && iv.lower.compare_fraction(numerator, denominator) < 0) return false;
    return iv.upper_infinite || iv.upper.compare_fraction(numerator, denominator) <= 0;
}

[[noreturn]] void bad_devices(const char *why) { throw std::invalid_argument(why); }

// One GPU ordinal of a --devices list: decimal digits only, at most INT_MAX.
int device_ordinal(const std::string &token) {
    long long value = 0;
    for (char c : token) {
        if (c < '0' || c > '9') bad_devices("--devices requires all or comma-separated nonnegative GPU IDs");
        value = value * 10 + (c - '0');
        if (value > std::numeric_limits<int>::max())
            bad_devices("--devices requires all or comma-separated nonnegative GPU IDs");
    }
    return int(value);
}

GpuDevice query_device(int ordinal) {
    cudaDeviceProp prop{};
    require_cuda(cudaGetDeviceProperties(&prop, ordinal), "cudaGetDeviceProperties");
    char bus[32] = {};
    require_cuda(cudaDeviceGetPCIBusId(bus, int(sizeof bus), ordinal), "cudaDeviceGetPCIBusId");
    GpuDevice g;
    g.id = ordinal;
    g.name = prop.name;
    g.major = prop.major;
    g.minor = prop.minor;
    g.multiprocessors = prop.multiProcessorCount;
    g.memory_bytes = (unsigned long long)prop.totalGlobalMem;
    g.pci_bus_id = bus;
    return g;
}

}  // namespace

bool SearchOptions::accepts(long long numerator, long long denominator) const {
    return intervals.empty() ||
           std::any_of(intervals.begin(), intervals.end(),
                       [&](const SearchInterval &iv) { return inside(iv, numerator, denominator); });
}

double SearchMetrics::initial_mask_gbs() const {
    // bytes of the reference's 14 first-stage masks per word, per millisecond of sieve time
    return sieve_ms > 0.0 ? double(initial_mask_bytes / ((long double)sieve_ms * 1.0e6L)) : 0.0;
}

// --devices: "all" (every visible GPU, returned as an empty list) or ordinals
// separated by commas.  Tokens are checked left to right: an empty token in
// the middle, a malformed or too large ordinal, or a repeated one fails where
// it is met; a list ending in a comma (or an empty text) fails after that.
std::vector<int> parse_device_selection(const std::string &text) {
    if (text == "all") return {};
    std::vector<int> ordinals;
    std::size_t begin = 0;
    for (;;) {
        const std::size_t comma = text.find(',', begin);
        const std::size_t end = comma == std::string::npos ? text.size() : comma;
        if (end == text.size() && begin == end) break;  // nothing after the last comma
        if (begin == end) bad_devices("empty GPU ID in --devices");
        const int ordinal = device_ordinal(text.substr(begin, end - begin));
        if (std::count(ordinals.begin(), ordinals.end(), ordinal))
            bad_devices("duplicate GPU ID in --devices");
        ordinals.push_back(ordinal);
        if (comma == std::string::npos) break;
        begin = comma + 1;
    }
    if (ordinals.empty() || text.back() == ',') bad_devices("--devices requires all or a nonempty GPU list");
    return ordinals;
}

std::vector<GpuDevice> available_gpu_devices() {
    int count = 0;
    const cudaError_t status = cudaGetDeviceCount(&count);
    if (status == cudaErrorNoDevice || (status == cudaSuccess && count == 0))
        throw std::runtime_error("no visible CUDA devices; check the driver and CUDA_VISIBLE_DEVICES");
    require_cuda(status, "cudaGetDeviceCount");
    std::vector<GpuDevice> devices;
    devices.reserve(std::size_t(count));
    for (int ordinal = 0; ordinal < count; ++ordinal) devices.push_back(query_device(ordinal));
    return devices;
}

// The GPUs a --devices list names, in its order (all visible ones for "all").
std::vector<GpuDevice> select_gpu_devices(const std::vector<int> &ids) {
    const std::vector<GpuDevice> visible = available_gpu_devices();
    if (ids.empty()) return visible;
    std::vector<GpuDevice> chosen;
    for (std::size_t k = 0; k < ids.size(); ++k) {
        const int id = ids[k];
        if (id < 0 || std::size_t(id) >= visible.size())
            throw std::invalid_argument("GPU ID " + std::to_string(id) +
                                        " is not visible; run --list-devices (IDs are "
                                        "CUDA-visible ordinals)");
        if (std::find(ids.begin(), ids.begin() + std::ptrdiff_t(k), id) != ids.begin() + std::ptrdiff_t(k))
            throw std::invalid_argument("duplicate GPU ID in selection");
        chosen.push_back(visible[std::size_t(id)]);
    }
    return chosen;
}

PointSearch::PointSearch(SearchOptions options)
    : options_(std::move(options)), poly_(options_.coefficients) {
    validate(options_, poly_);
    // One GPU: the first selected (or first visible) device runs every batch.
    devices_ = select_gpu_devices(options_.devices);
}

SearchMetrics PointSearch::run(const PointCallback &callback) {
    const auto started = Clock::now();
    const SearchOptions &options = options_;
    const ExactPolynomial &poly = poly_;
    const std::vector<GpuDevice> &devices = devices_;
    SearchMetrics metrics;
    DeviceMetrics entry;
    entry.device = devices.front();
    metrics.devices.push_back(entry);
    auto finish = [&]() {
        metrics.wall_ms = ms_since(started);
        return metrics;
    };
    if (options.include_infinity) {
        std::string root;
        if (poly.square_root(1, 0, root) && !callback(PointPair{1, root, 0})) return finish();
    }
    if (options.first > options.last) return finish();

    SieveOptions so;
    so.plan = options.plan;
    so.square = options.square;
    so.capacity = options.capacity;
    so.device = devices.front().id;
    so.preverify = options.device_preverify;
    Sieve sieve(options.coefficients, options.numerator_bound, so);
    const int threads = options.verify_threads > 0
                            ? options.verify_threads
                            : int(std::max(1u, std::thread::hardware_concurrency()));
    metrics.word_count = (unsigned long long)word_count32(options.numerator_bound);
    const auto sieve_started = Clock::now();
    double verification_ms = 0;
    sieve.start(options.first, options.last, options.batch_size);
    std::vector<Found> batch_points;
    unsigned long long batch_survivors = 0, batch_candidates = 0;
    BatchView view;
    bool stopped = false;
    while (!stopped && sieve.next(view)) {
        const auto v0 = Clock::now();
        verify(poly, view.a, view.d, view.count, threads, batch_points);
        batch_survivors += view.modular;
        batch_candidates += view.count;
        verification_ms += ms_since(v0);
        if (!view.complete) continue;
        std::sort(batch_points.begin(), batch_points.end(), [](const Found &l, const Found &r) {
            return l.d != r.d ? l.d < r.d : l.a < r.a;
        });
        const unsigned long long count = (unsigned long long)(view.last - view.first + 1);
        metrics.denominator_count += count;
        metrics.devices[0].denominator_count += count;
        metrics.devices[0].batches += 1;
        metrics.modular_survivors += batch_survivors;
        metrics.host_candidates += batch_candidates;
        metrics.exact_survivors += batch_points.size();
        metrics.initial_mask_bytes += (long double)count * (long double)metrics.word_count * 14.0L * 4.0L;
        for (const auto &p : batch_points) {
            if (options.accepts(p.a, p.d) && !callback(PointPair{p.a, p.y, p.d})) {
                stopped = true;
                break;
            }
        }
        batch_points.clear();
        batch_survivors = batch_candidates = 0;
    }
    if (stopped) sieve.cancel();
    const SieveTimings &t = sieve.timings();
    metrics.basis_ms = t.table_ms;
    metrics.sieve_ms = t.sieve_ms;
    metrics.plan_ms = t.plan_ms;
    metrics.workspace_ms = t.workspace_ms;
    metrics.basis_wall_ms = t.table_wall_ms;
    metrics.verification_ms = verification_ms;
    metrics.sieve_wall_ms = ms_since(sieve_started) - verification_ms;
    metrics.launches = t.launches;
    metrics.h2d_bytes = t.h2d_bytes;
    metrics.d2h_bytes = t.d2h_bytes;
    metrics.devices[0].basis_ms = t.table_ms;
    metrics.devices[0].sieve_ms = t.sieve_ms;
    return finish();
}

}  // namespace rpg
