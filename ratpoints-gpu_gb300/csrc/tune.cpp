#include "tune.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <stdexcept>

#include "plan.hpp"

namespace rpg {

namespace {

// ---------------------------------------------------------------------------
// The cache file: {"fast_plan_shapes": {key: {"rows": R, "slots": S,
// "sample_denominators": N, "measured_ms": {"RxS": ms, ...}}, ...},
// "batch_items": {key: {"items": N, "measured_ms": {"N": ms, ...}}, ...}}

struct Entry {
    FastShape shape;
    long long sample = 0;
    std::map<std::string, double> measured;
};

struct BatchEntry {
    int items = 0;
    std::map<std::string, double> measured;
};

struct CacheContents {
    std::map<std::string, Entry> shapes;
    std::map<std::string, BatchEntry> batches;
};

// A small JSON reader for the cache file: objects, strings, numbers (other
// values are read and ignored).  A file it cannot read counts as empty.
class JsonReader {
public:
    explicit JsonReader(const std::string &text) : t_(text) {}

    bool contents(CacheContents &out) {
        try {
            skip();
            expect('{');
            while (!take('}')) {
                const std::string name = string();
                expect(':');
                if (name == "fast_plan_shapes") {
                    expect('{');
                    while (!take('}')) {
                        const std::string key = string();
                        expect(':');
                        Entry e;
                        if (entry(e)) out.shapes[key] = e;
                        take(',');
                    }
                } else if (name == "batch_items") {
                    expect('{');
                    while (!take('}')) {
                        const std::string key = string();
                        expect(':');
                        BatchEntry e;
                        if (batch_entry(e)) out.batches[key] = e;
                        take(',');
                    }
                } else {
                    value();
                }
                take(',');
            }
            return true;
        } catch (const std::exception &) {
            out = CacheContents{};
            return false;
        }
    }

private:
    bool batch_entry(BatchEntry &e) {
        expect('{');
        while (!take('}')) {
            const std::string name = string();
            expect(':');
            if (name == "items") e.items = int(number());
            else if (name == "measured_ms") measured(e.measured);
            else value();
            take(',');
        }
        return e.items >= 64 && e.items <= (1 << 20);
    }
    void measured(std::map<std::string, double> &out) {
        expect('{');
        while (!take('}')) {
            const std::string k = string();
            expect(':');
            out[k] = number();
            take(',');
        }
    }
    bool entry(Entry &e) {
        expect('{');
        while (!take('}')) {
            const std::string name = string();
            expect(':');
            if (name == "rows") e.shape.rows = int(number());
            else if (name == "slots") e.shape.slots = int(number());
            else if (name == "sample_denominators") e.sample = (long long)number();
            else if (name == "measured_ms") {
                measured(e.measured);
            } else {
                value();
            }
            take(',');
        }
        return e.shape.rows > 0 && e.shape.rows <= kMaxFastSlots && (e.shape.slots == 2 || e.shape.slots == 3);
    }
    void skip() {
        while (i_ < t_.size() && (t_[i_] == ' ' || t_[i_] == '\n' || t_[i_] == '\t' || t_[i_] == '\r')) ++i_;
    }
    bool take(char c) {
        skip();
        if (i_ < t_.size() && t_[i_] == c) {
            ++i_;
            skip();
            return true;
        }
        return false;
    }
    void expect(char c) {
        if (!take(c)) throw std::runtime_error("malformed tuning cache");
    }
    std::string string() {
        skip();
        if (i_ >= t_.size() || t_[i_] != '"') throw std::runtime_error("malformed tuning cache");
        std::string s;
        for (++i_; i_ < t_.size() && t_[i_] != '"'; ++i_) {
            if (t_[i_] == '\\' && i_ + 1 < t_.size()) ++i_;
            s.push_back(t_[i_]);
        }
        if (i_ >= t_.size()) throw std::runtime_error("malformed tuning cache");
        ++i_;
        skip();
        return s;
    }
    double number() {
        skip();
        const char *begin = t_.c_str() + i_;
        char *end = nullptr;
        const double v = std::strtod(begin, &end);
        if (end == begin) throw std::runtime_error("malformed tuning cache");
        i_ += std::size_t(end - begin);
        skip();
        return v;
    }
    void value() {
        skip();
        if (i_ >= t_.size()) throw std::runtime_error("malformed tuning cache");
        const char c = t_[i_];
        if (c == '"') {
            string();
        } else if (c == '{' || c == '[') {
            const char close = c == '{' ? '}' : ']';
            ++i_;
            while (!take(close)) {
                if (c == '{') {
                    string();
                    expect(':');
                }
                value();
                take(',');
            }
        } else if (c == 't' || c == 'f' || c == 'n') {
            while (i_ < t_.size() && std::isalpha(static_cast<unsigned char>(t_[i_]))) ++i_;
            skip();
        } else {
            number();
        }
    }

    const std::string &t_;
    std::size_t i_ = 0;
};

std::string json_string(const std::string &s) {
    std::string out = "\"";
    for (char c : s) {
        if (c == '"' || c == '\\') out.push_back('\\');
        out.push_back(c);
    }
    return out + "\"";
}

std::string shape_name(FastShape s) { return std::to_string(s.rows) + "x" + std::to_string(s.slots); }

class ShapeCache {
public:
    bool lookup(const std::string &path, const std::string &key, FastShape &out) {
        std::lock_guard<std::mutex> lock(mutex_);
        load(path);
        auto it = contents_.shapes.find(key);
        if (it == contents_.shapes.end()) return false;
        out = it->second.shape;
        return true;
    }

    int lookup_items(const std::string &path, const std::string &key) {
        std::lock_guard<std::mutex> lock(mutex_);
        load(path);
        auto it = contents_.batches.find(key);
        return it == contents_.batches.end() ? 0 : it->second.items;
    }

    bool store(const std::string &path, const std::string &key, const Entry &e) {
        std::lock_guard<std::mutex> lock(mutex_);
        load(path);
        contents_.shapes[key] = e;
        return write(path);
    }

    bool store_items(const std::string &path, const std::string &key, const BatchEntry &e) {
        std::lock_guard<std::mutex> lock(mutex_);
        load(path);
        contents_.batches[key] = e;
        return write(path);
    }

private:
    static void write_measured(std::ostringstream &o, const std::map<std::string, double> &measured) {
        o << "\"measured_ms\": {";
        bool first = true;
        for (const auto &m : measured) {
            char buf[64];
            std::snprintf(buf, sizeof buf, "%.6f", m.second);
            o << (first ? "" : ", ") << json_string(m.first) << ": " << buf;
            first = false;
        }
        o << "}";
    }

    bool write(const std::string &path) {
        std::ostringstream o;
        o << "{\n  \"fast_plan_shapes\": {";
        bool first = true;
        for (const auto &kv : contents_.shapes) {
            o << (first ? "\n" : ",\n") << "    " << json_string(kv.first) << ": {\"rows\": "
              << kv.second.shape.rows << ", \"slots\": " << kv.second.shape.slots
              << ", \"sample_denominators\": " << kv.second.sample << ", ";
            write_measured(o, kv.second.measured);
            o << "}";
            first = false;
        }
        o << "\n  },\n  \"batch_items\": {";
        first = true;
        for (const auto &kv : contents_.batches) {
            o << (first ? "\n" : ",\n") << "    " << json_string(kv.first) << ": {\"items\": " << kv.second.items
              << ", ";
            write_measured(o, kv.second.measured);
            o << "}";
            first = false;
        }
        o << "\n  }\n}\n";
        // written to a temporary file, then renamed over the cache
        const std::string tmp = path + ".tmp";
        {
            std::ofstream f(tmp, std::ios::trunc);
            if (!f) return false;
            f << o.str();
            if (!f) return false;
        }
        return std::rename(tmp.c_str(), path.c_str()) == 0;
    }

    void load(const std::string &path) {
        if (path == loaded_path_) return;
        contents_ = CacheContents{};
        std::ifstream f(path);
        if (f) {
            std::stringstream buf;
            buf << f.rdbuf();
            const std::string text = buf.str();
            JsonReader(text).contents(contents_);
        }
        loaded_path_ = path;
    }

    std::mutex mutex_;
    std::string loaded_path_;
    CacheContents contents_;
};

ShapeCache &cache() {
    static ShapeCache c;
    return c;
}

bool same_plan(const FastPlan &a, const FastPlan &b) {
    return a.class_prime == b.class_prime && a.moduli == b.moduli && a.row_slots == b.row_slots;
}

}  // namespace

std::string tune_cache_path() {
    const char *p = std::getenv("RPG_TUNE_CACHE");
    return p && *p ? std::string(p) : std::string();
}

std::string fast_shape_key(const std::vector<std::string> &coefficients, long long bound) {
    const FastPlan p = single_curve_plan(coefficients, bound, nullptr);
    int largest = 0;
    for (const auto &f : p.slots)
        for (int q : f) largest = std::max(largest, q);
    const int degree = int(coefficients.size()) - 1;
    const int wbits = int(std::floor(std::log2(double(std::max(1LL, word_count64(bound))))));
    return "degree" + std::to_string(degree) + "-q" + std::to_string(p.class_prime) + "-words2^" +
           std::to_string(wbits) + (largest >= kFastPrimeLimit ? "-largeprimes" : "-smallprimes");
}

FastShape tuned_fast_shape(const std::vector<std::string> &coefficients, long long bound) {
    FastShape s;
    const std::string path = tune_cache_path();
    if (path.empty()) return s;
    if (!cache().lookup(path, fast_shape_key(coefficients, bound), s)) return FastShape{};
    return s;
}

TuneResult tune_fast_shape(const std::vector<std::string> &coefficients, long long bound, long long first,
                           long long last, bool square, int device, long long sample) {
    if (first < 1 || last < first || sample < 1) throw std::invalid_argument("invalid denominator range");
    TuneResult result;
    result.key = fast_shape_key(coefficients, bound);
    const long long end = std::min(last, first + sample - 1);
    result.sample = end - first + 1;
    const FastPlan automatic = single_curve_plan(coefficients, bound, nullptr);
    const int rows = int(automatic.moduli.size());
    const int slots = automatic.row_slots;
    // the cost model's shape first, then the other slot count (short rows
    // only: long rows keep two slots) and one and two rows either side
    std::vector<FastShape> shapes = {{rows, slots}};
    if (word_count64(bound) <= (1LL << 20)) shapes.push_back({rows, slots == 2 ? 3 : 2});
    for (int dr : {-1, 1, -2, 2})
        if (rows + dr >= 1 && rows + dr <= kMaxFastSlots) shapes.push_back({rows + dr, slots});
    std::vector<FastPlan> plans;
    cudaEvent_t begin = nullptr, stop = nullptr;
    check_cuda(cudaEventCreate(&begin), "cudaEventCreate");
    check_cuda(cudaEventCreate(&stop), "cudaEventCreate");
    struct Events {
        cudaEvent_t a, b;
        ~Events() {
            cudaEventDestroy(a);
            cudaEventDestroy(b);
        }
    } guard{begin, stop};
    for (const FastShape &shape : shapes) {
        const FastPlan p = single_curve_plan(coefficients, bound, nullptr, shape);
        if (std::any_of(plans.begin(), plans.end(), [&](const FastPlan &q) { return same_plan(p, q); })) continue;
        plans.push_back(p);
        SieveOptions so;
        so.plan = PlanKind::fast;
        so.square = square;
        so.device = device;
        so.fast_shape = {int(p.moduli.size()), p.row_slots};
        Sieve sieve(coefficients, bound, so);
        sieve.count_only(first, end, 1 << 16);  // warm-up: module and tables in cache
        check_cuda(cudaEventRecord(begin, sieve.stream()), "cudaEventRecord");
        const unsigned long long n = sieve.count_only(first, end, 1 << 16);
        check_cuda(cudaEventRecord(stop, sieve.stream()), "cudaEventRecord");
        check_cuda(cudaEventSynchronize(stop), "cudaEventSynchronize");
        float ms = 0;
        check_cuda(cudaEventElapsedTime(&ms, begin, stop), "cudaEventElapsedTime");
        TuneCandidate c;
        c.shape = so.fast_shape;
        c.bits = p.bits;
        c.ms = ms;
        c.survivors = n;
        result.candidates.push_back(c);
    }
    const auto best = std::min_element(result.candidates.begin(), result.candidates.end(),
                                       [](const TuneCandidate &a, const TuneCandidate &b) { return a.ms < b.ms; });
    result.chosen = best->shape;
    const std::string path = tune_cache_path();
    if (!path.empty()) {
        Entry e;
        e.shape = result.chosen;
        e.sample = result.sample;
        for (const auto &c : result.candidates) e.measured[shape_name(c.shape)] = c.ms;
        result.stored = cache().store(path, result.key, e);
    }
    return result;
}

std::string batch_items_key(const std::vector<BatchCurveSpec> &curves) {
    std::vector<long long> words, degrees;
    for (const auto &c : curves) {
        words.push_back(word_count64(std::max(1LL, c.bound)));
        degrees.push_back((long long)c.coefficients.size() - 1);
    }
    auto median = [](std::vector<long long> &v) -> long long {
        if (v.empty()) return 1;
        std::nth_element(v.begin(), v.begin() + long(v.size() / 2), v.end());
        return v[v.size() / 2];
    };
    const int cbits = int(std::floor(std::log2(double(std::max<std::size_t>(1, curves.size())))));
    const int wbits = int(std::floor(std::log2(double(std::max(1LL, median(words))))));
    return "curves2^" + std::to_string(cbits) + "-words2^" + std::to_string(wbits) +
           (median(degrees) <= 6 ? "-degree-low" : "-degree-high");
}

int tuned_batch_items(const std::vector<BatchCurveSpec> &curves) {
    const std::string path = tune_cache_path();
    if (path.empty()) return 0;
    return cache().lookup_items(path, batch_items_key(curves));
}

BatchTuneResult tune_batch_items(const std::vector<BatchCurveSpec> &curves, int device) {
    BatchTuneResult result;
    result.key = batch_items_key(curves);
    BatchEngine engine(device);
    BatchStats warm;
    engine.run(curves, &warm, true, true, kDefaultBatchItems);  // buffers sized, modules loaded
    double best = 0;
    for (int items : {2048, kDefaultBatchItems, 32768}) {
        BatchStats st;
        engine.run(curves, &st, true, true, items);
        result.candidates.push_back({items, st.sieve_ms});
        if (result.items == 0 || st.sieve_ms < best) {
            best = st.sieve_ms;
            result.items = items;
        }
    }
    const std::string path = tune_cache_path();
    if (!path.empty()) {
        BatchEntry e;
        e.items = result.items;
        for (const auto &c : result.candidates) e.measured[std::to_string(c.first)] = c.second;
        result.stored = cache().store_items(path, result.key, e);
    }
    return result;
}

}  // namespace rpg
