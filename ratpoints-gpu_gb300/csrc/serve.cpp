#include "serve.hpp"

#include <algorithm>
#include <chrono>
#include <stdexcept>

#include "exact.hpp"
#include "plan.hpp"

namespace rpg {

namespace {
using Clock = std::chrono::steady_clock;
double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}
constexpr int kStatusCuda = 2;          // rpg_status RPG_E_CUDA
constexpr int kStatusNotSquarefree = 6; // rpg_status RPG_E_NOT_SQUAREFREE
}  // namespace

struct SearchServer::Request {
    std::uint64_t id = 0;
    BatchCurveSpec spec;
    bool first_only = false;
    Clock::time_point submitted, started;
    bool has_started = false;
    long long next_first = 1;   // first-point waves: next parameter to search
    long long wave = 1;         // parameters in the next wave
    bool done = false;
    ServeResult result;
};

struct SearchServer::Lane {
    std::unique_ptr<BatchEngine> engine;
    std::thread thread;
    std::vector<std::pair<std::uint64_t, BatchCurveSpec>> batch;  // (request, entry)
    bool busy = false;
    bool has_work = false;
    bool stop = false;
    std::condition_variable cv;
};

SearchServer::SearchServer(const ServeOptions &options) : options_(options) {
    if (options_.lanes < 1 || options_.lanes > 16) throw std::invalid_argument("lanes must be 1..16");
    if (options_.max_batch_curves < 1) throw std::invalid_argument("max_batch_curves must be positive");
    for (int i = 0; i < options_.lanes; ++i) {
        auto lane = std::make_unique<Lane>();
        lane->engine = std::make_unique<BatchEngine>(options_.device);
        lanes_.push_back(std::move(lane));
    }
    for (auto &lane : lanes_) {
        Lane *l = lane.get();
        l->thread = std::thread([this, l] { lane_loop(*l); });
    }
    dispatcher_ = std::thread([this] { dispatch_loop(); });
}

SearchServer::~SearchServer() {
    {
        std::lock_guard<std::mutex> lock(mutex_);
        stopping_ = true;
    }
    work_cv_.notify_all();
    if (dispatcher_.joinable()) dispatcher_.join();
    {
        std::lock_guard<std::mutex> lock(mutex_);
        for (auto &lane : lanes_) lane->stop = true;
    }
    for (auto &lane : lanes_) {
        lane->cv.notify_all();
        if (lane->thread.joinable()) lane->thread.join();
    }
}

std::uint64_t SearchServer::submit(const BatchCurveSpec &curve, bool first_point_only) {
    auto r = std::make_unique<Request>();
    r->spec = curve;
    r->first_only = first_point_only;
    r->submitted = Clock::now();
    bool answered = false;
    if (first_point_only) {
        // the point at infinity comes first in a single search: it alone answers
        // a first-point request (after the squarefree check a search makes first)
        ExactPolynomial poly(curve.coefficients);
        if (!poly.is_squarefree()) {
            r->result.status = kStatusNotSquarefree;
            r->result.error = "polynomial is not squarefree";
            answered = true;
        } else {
            std::string root;
            if (curve.include_infinity && poly.square_root(1, 0, root)) {
                r->result.points.push_back(PointPair{1, root, 0});
                answered = true;
            } else if (curve.first > curve.last) {
                answered = true;
            }
        }
        r->spec.include_infinity = false;
        r->next_first = curve.first;
        const long long words = word_count64(std::max(1LL, curve.bound));
        r->wave = std::max(256LL, (1LL << 22) / words);
    }
    std::lock_guard<std::mutex> lock(mutex_);
    if (stopping_) throw std::logic_error("server is stopping");
    const std::uint64_t id = next_id_++;
    r->id = id;
    Request &ref = *r;
    requests_[id] = std::move(r);
    counters_.submitted += 1;
    if (answered) {
        ref.started = ref.submitted;
        ref.has_started = true;
        finish(ref);
    } else {
        pending_.push_back(id);
        work_cv_.notify_one();
    }
    return id;
}

void SearchServer::finish(Request &r) {
    const auto now = Clock::now();
    r.done = true;
    r.result.latency_ms = ms_between(r.submitted, now);
    r.result.queue_ms = r.has_started ? ms_between(r.submitted, r.started) : r.result.latency_ms;
    counters_.completed += 1;
    counters_.rectangle_sites += r.result.rectangle_sites;
    done_cv_.notify_all();
}

void SearchServer::dispatch_loop() {
    std::unique_lock<std::mutex> lock(mutex_);
    const unsigned long long budget = options_.memory_budget / (unsigned long long)options_.lanes;
    for (;;) {
        Lane *idle = nullptr;
        bool any_busy = false;
        work_cv_.wait(lock, [&] {
            idle = nullptr;
            any_busy = false;
            for (auto &lane : lanes_) {
                if (lane->busy) any_busy = true;
                else if (!idle) idle = lane.get();
            }
            return (!pending_.empty() && idle) || (stopping_ && pending_.empty() && !any_busy);
        });
        if (pending_.empty()) return;  // stopping, nothing left anywhere
        // admit waiting requests in order while their device bytes fit the budget
        std::vector<std::pair<std::uint64_t, BatchCurveSpec>> batch;
        unsigned long long used = 0;
        const auto now = Clock::now();
        while (!pending_.empty() && int(batch.size()) < options_.max_batch_curves) {
            Request &r = *requests_.at(pending_.front());
            BatchCurveSpec entry = r.spec;
            if (r.first_only) {
                entry.first = r.next_first;
                entry.last = std::min(r.spec.last, r.next_first + r.wave - 1);
            }
            const unsigned long long bytes = BatchEngine::estimate_bytes(entry);
            if (!batch.empty() && used + bytes > budget) break;
            pending_.pop_front();
            used += bytes;
            if (!r.has_started) {
                r.started = now;
                r.has_started = true;
            }
            if (r.first_only) {
                r.next_first = entry.last + 1;
                r.wave *= 16;
            }
            r.result.waves += 1;
            r.result.rectangle_sites +=
                (long double)(2 * entry.bound + 1) * (long double)std::max(0LL, entry.last - entry.first + 1);
            batch.emplace_back(r.id, std::move(entry));
        }
        counters_.batches += 1;
        counters_.entries += batch.size();
        idle->batch = std::move(batch);
        idle->busy = true;
        idle->has_work = true;
        idle->cv.notify_one();
    }
}

void SearchServer::lane_loop(Lane &lane) {
    for (;;) {
        std::vector<std::pair<std::uint64_t, BatchCurveSpec>> batch;
        {
            std::unique_lock<std::mutex> lock(mutex_);
            lane.cv.wait(lock, [&] { return lane.has_work || lane.stop; });
            if (!lane.has_work) return;
            batch = std::move(lane.batch);
            lane.has_work = false;
        }
        std::vector<BatchCurveSpec> specs;
        specs.reserve(batch.size());
        for (const auto &e : batch) specs.push_back(e.second);
        std::vector<BatchCurveResult> results;
        std::string failure;
        try {
            BatchStats stats;
            results = lane.engine->run(specs, &stats, false);
        } catch (const std::exception &e) {
            failure = e.what();
        }
        std::lock_guard<std::mutex> lock(mutex_);
        // first-point requests that go on re-enter the queue ahead of later
        // arrivals, in their order
        std::vector<std::uint64_t> again;
        for (std::size_t i = 0; i < batch.size(); ++i) {
            Request &r = *requests_.at(batch[i].first);
            if (!failure.empty()) {
                r.result.status = kStatusCuda;
                r.result.error = failure;
                finish(r);
                continue;
            }
            BatchCurveResult &br = results[i];
            r.result.survivors += br.survivors;
            if (br.status != 0) {
                r.result.status = br.status;
                r.result.error = br.error;
                finish(r);
            } else if (!r.first_only) {
                r.result.points = std::move(br.points);
                finish(r);
            } else if (!br.points.empty()) {
                r.result.points.assign(1, br.points.front());
                finish(r);
            } else if (r.next_first > r.spec.last) {
                finish(r);
            } else {
                again.push_back(r.id);
            }
        }
        for (auto it = again.rbegin(); it != again.rend(); ++it) pending_.push_front(*it);
        lane.busy = false;
        work_cv_.notify_all();
    }
}

bool SearchServer::wait(std::uint64_t id, double timeout_ms, ServeResult &out) {
    std::unique_lock<std::mutex> lock(mutex_);
    auto it = requests_.find(id);
    if (it == requests_.end()) throw std::invalid_argument("unknown request id");
    Request *r = it->second.get();
    auto ready = [&] { return r->done; };
    if (timeout_ms < 0) {
        done_cv_.wait(lock, ready);
    } else if (!done_cv_.wait_for(lock, std::chrono::duration<double, std::milli>(timeout_ms), ready)) {
        return false;
    }
    out = std::move(r->result);
    requests_.erase(id);
    return true;
}

SearchServer::Counters SearchServer::counters() const {
    std::lock_guard<std::mutex> lock(mutex_);
    return counters_;
}

}  // namespace rpg
