// Serving loop: searches arrive at any time and are answered in batches
// that overlap on the device.
//
// No counterpart in the reference, which runs one search per process
// (src/main.cpp:48-85).  Each request's answer is what a single search of it
// reports (src/point_search.cpp:171-240): all points in order, or with
// first_point_only the first point only (the -1 option, src/main.cpp:70).
//
// Continuous batching: `lanes` batch engines (each with its own CUDA streams
// and resident device buffers) take batches from one dispatcher.  Whenever a
// lane is free and requests wait, the dispatcher admits waiting requests in
// arrival order while their estimated device bytes fit the lane's share of
// the memory budget, and the lane runs them as one batched pass; requests
// that arrive meanwhile go to the next free lane, so work from several
// batches is on the device at once.  A first-point request is searched in
// denominator waves of growing size (first wave about 2^22 row words, then
// x16), each a batch entry of its own: the first wave holding an accepted
// point ends it, and since waves run in denominator order the point is the
// one a single search stops at.  A point at infinity (when requested and
// present) answers a first-point request without any device work.
#pragma once

#include <condition_variable>
#include <cstdint>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "batch.hpp"

namespace rpg {

struct ServeOptions {
    int device = -1;
    int lanes = 2;
    unsigned long long memory_budget = 8ull << 30;  // device bytes for all lanes' batches
    int max_batch_curves = 1024;
};

struct ServeResult {
    int status = 0;                  // rpg_status code
    std::string error;
    std::vector<PointPair> points;
    double latency_ms = 0;           // submit -> answer
    double queue_ms = 0;             // submit -> first batch start
    long double rectangle_sites = 0; // (2H + 1) x denominators searched
    unsigned long long survivors = 0;
    int waves = 0;                   // batch entries the request took
};

class SearchServer {
public:
    explicit SearchServer(const ServeOptions &options);
    ~SearchServer();  // finishes admitted work, then stops
    SearchServer(const SearchServer &) = delete;
    SearchServer &operator=(const SearchServer &) = delete;

    std::uint64_t submit(const BatchCurveSpec &curve, bool first_point_only);
    // Waits up to timeout_ms (< 0: no limit); true and the answer (the request
    // is then retired) once it is done.
    bool wait(std::uint64_t id, double timeout_ms, ServeResult &out);

    struct Counters {
        unsigned long long submitted = 0, completed = 0, batches = 0, entries = 0;
        long double rectangle_sites = 0;
    };
    Counters counters() const;

private:
    struct Request;
    struct Lane;
    void dispatch_loop();
    void lane_loop(Lane &lane);
    void finish(Request &r);

    ServeOptions options_;
    mutable std::mutex mutex_;
    std::condition_variable work_cv_;   // dispatcher: requests or free lanes
    std::condition_variable done_cv_;   // waiters
    std::map<std::uint64_t, std::unique_ptr<Request>> requests_;
    std::deque<std::uint64_t> pending_;
    std::vector<std::unique_ptr<Lane>> lanes_;
    std::thread dispatcher_;
    std::uint64_t next_id_ = 1;
    bool stopping_ = false;
    Counters counters_;
};

}  // namespace rpg
