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

bool SearchOptions::accepts(long long numerator, long long denominator) const {
    if (intervals.empty()) return true;
    for (const auto &iv : intervals) {
        // compare_fraction gives sign(numerator/denominator - bound)
        bool above = iv.lower_infinite || iv.lower.compare_fraction(numerator, denominator) >= 0;
        bool below = iv.upper_infinite || iv.upper.compare_fraction(numerator, denominator) <= 0;
        if (above && below) return true;
    }
    return false;
}

double SearchMetrics::initial_mask_gbs() const {
    if (sieve_ms == 0.0) return 0.0;
    return double(initial_mask_bytes / ((long double)sieve_ms * 1.0e6L));
}

std::vector<int> parse_device_selection(const std::string &text) {
    if (text == "all") return {};
    std::vector<int> ids;
    std::size_t start = 0;
    while (start < text.size()) {
        std::size_t end = text.find(',', start);
        if (end == std::string::npos) end = text.size();
        if (end == start) throw std::invalid_argument("empty GPU ID in --devices");
        int id = 0;
        for (std::size_t i = start; i < end; ++i) {
            if (text[i] < '0' || text[i] > '9' ||
                id > (std::numeric_limits<int>::max() - (text[i] - '0')) / 10)
                throw std::invalid_argument(
                    "--devices requires all or comma-separated nonnegative GPU IDs");
            id = id * 10 + (text[i] - '0');
        }
        if (std::find(ids.begin(), ids.end(), id) != ids.end())
            throw std::invalid_argument("duplicate GPU ID in --devices");
        ids.push_back(id);
        start = end + 1;
    }
    if (ids.empty() || text.back() == ',')
        throw std::invalid_argument("--devices requires all or a nonempty GPU list");
    return ids;
}

std::vector<GpuDevice> available_gpu_devices() {
    int count = 0;
    cudaError_t status = cudaGetDeviceCount(&count);
    if (status == cudaErrorNoDevice || (status == cudaSuccess && count == 0))
        throw std::runtime_error(
            "no visible CUDA devices; check the driver and CUDA_VISIBLE_DEVICES");
    require_cuda(status, "cudaGetDeviceCount");
    std::vector<GpuDevice> devices;
    for (int id = 0; id < count; ++id) {
        cudaDeviceProp prop{};
        require_cuda(cudaGetDeviceProperties(&prop, id), "cudaGetDeviceProperties");
        char pci[32] = {};
        require_cuda(cudaDeviceGetPCIBusId(pci, sizeof pci, id), "cudaDeviceGetPCIBusId");
        GpuDevice dev;
        dev.id = id;
        dev.name = prop.name;
        dev.major = prop.major;
        dev.minor = prop.minor;
        dev.multiprocessors = prop.multiProcessorCount;
        dev.memory_bytes = (unsigned long long)prop.totalGlobalMem;
        dev.pci_bus_id = pci;
        devices.push_back(dev);
    }
    return devices;
}

std::vector<GpuDevice> select_gpu_devices(const std::vector<int> &ids) {
    std::vector<GpuDevice> available = available_gpu_devices();
    if (ids.empty()) return available;
    std::vector<GpuDevice> selected;
    for (int id : ids) {
        if (id < 0 || std::size_t(id) >= available.size())
            throw std::invalid_argument("GPU ID " + std::to_string(id) +
                                        " is not visible; run --list-devices (IDs are "
                                        "CUDA-visible ordinals)");
        for (const auto &d : selected)
            if (d.id == id) throw std::invalid_argument("duplicate GPU ID in selection");
        selected.push_back(available[std::size_t(id)]);
    }
    return selected;
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
