// extern "C" entry points of librpgpu (include/ratpoints_gb300.h).
#include "ratpoints_gb300.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "batch.hpp"
#include "cli.hpp"
#include "exact.hpp"
#include "plan.hpp"
#include "preverify.hpp"
#include "search.hpp"
#include "serve.hpp"
#include "session.hpp"
#include "sieve.hpp"
#include "tune.hpp"

namespace {

thread_local std::string g_last_error;

rpg_status fail(rpg_status status, const std::string &message) {
    g_last_error = message;
    return status;
}

template <typename F>
rpg_status guarded(F &&body) {
    try {
        g_last_error.clear();
        return body();
    } catch (const rpg::DeviceTimeout &e) {
        return fail(RPG_E_TIMEOUT, e.what());
    } catch (const rpg::CudaError &e) {
        const std::string what = e.what();
        if (what.find("out of memory") != std::string::npos) return fail(RPG_E_OOM, what);
        return fail(RPG_E_CUDA, what);
    } catch (const std::bad_alloc &e) {
        return fail(RPG_E_OOM, e.what());
    } catch (const std::invalid_argument &e) {
        const std::string what = e.what();
        if (what == "polynomial is not squarefree") return fail(RPG_E_NOT_SQUAREFREE, what);
        return fail(RPG_E_ARG, what);
    } catch (const std::exception &e) {
        return fail(RPG_E_INTERNAL, e.what());
    }
}

bool coefficients_from(const char *const *c, int32_t n, std::vector<std::string> &out,
                       std::string &error) {
    if (!c || n < 2 || n > 101) {
        error = "supported polynomial degrees are 1 through 100";
        return false;
    }
    out.clear();
    for (int32_t i = 0; i < n; ++i) {
        if (!c[i]) {
            error = "coefficients must be decimal integers";
            return false;
        }
        std::string s(c[i]);
        if (!s.empty() && s.front() == '+') s.erase(0, 1);
        rpg::BigInt probe;
        if (!rpg::BigInt::parse(s, probe)) {
            error = "coefficients must be decimal integers";
            return false;
        }
        out.push_back(s);
    }
    rpg::BigInt lead;
    rpg::BigInt::parse(out.back(), lead);
    if (lead.is_zero()) {
        error = "leading coefficient must be nonzero";
        return false;
    }
    return true;
}

// rpg_search_options -> SearchOptions with the checks and messages of a search.
bool options_from(const rpg_search_options &o, rpg::SearchOptions &s, std::string &error) {
    if (!coefficients_from(o.coefficients, o.coefficient_count, s.coefficients, error)) return false;
    if (o.numerator_bound < 1) {
        error = "maximum height must be positive";
        return false;
    }
    if (o.first < 1 || o.first > o.last) {
        error = "empty denominator range";
        return false;
    }
    if (o.interval_count < 0 || (o.interval_count > 0 && !o.intervals)) {
        error = "invalid interval list";
        return false;
    }
    s.numerator_bound = o.numerator_bound;
    s.first = o.first;
    s.last = o.last;
    if (o.square_denominators && s.last > 46340) s.last = 46340;
    for (int32_t i = 0; i < o.interval_count; ++i) {
        rpg::SearchInterval iv;
        const rpg_interval &src = o.intervals[i];
        iv.lower_infinite = src.lower == nullptr;
        iv.upper_infinite = src.upper == nullptr;
        if (src.lower && !rpg::parse_real(src.lower, "interval lower bound", iv.lower, error))
            return false;
        if (src.upper && !rpg::parse_real(src.upper, "interval upper bound", iv.upper, error))
            return false;
        s.intervals.push_back(iv);
    }
    s.include_infinity = o.include_infinity != 0;
    s.batch_size = o.batch_size;
    s.square = o.square_denominators != 0;
    s.plan = o.plan == RPG_PLAN_REFERENCE ? rpg::PlanKind::reference : rpg::PlanKind::fast;
    if (o.device >= 0) s.devices = {o.device};
    s.verify_threads = o.verify_threads;
    s.device_preverify = (o.flags & RPG_SEARCH_HOST_VERIFY_ONLY) == 0;
    return true;
}

void fill_stats(rpg_sieve_stats *stats, const rpg::SearchMetrics &m) {
    if (!stats) return;
    std::memset(stats, 0, sizeof *stats);
    stats->survivor_count = m.modular_survivors;
    stats->host_candidates = m.host_candidates;
    stats->word_count = m.word_count;
    stats->denominator_count = m.denominator_count;
    stats->launches = m.launches;
    stats->basis_ms = m.basis_ms;
    stats->sieve_ms = m.sieve_ms;
    stats->plan_ms = m.plan_ms;
    stats->workspace_ms = m.workspace_ms;
    stats->basis_wall_ms = m.basis_wall_ms;
    stats->survivor_setup_ms = m.survivor_setup_ms;
    stats->verification_ms = m.verification_ms;
    stats->sieve_wall_ms = m.sieve_wall_ms;
    stats->initial_mask_bytes = double(m.initial_mask_bytes);
    stats->h2d_bytes = m.h2d_bytes;
    stats->d2h_bytes = m.d2h_bytes;
}

}  // namespace

namespace rpg {
// Records the message rpg_last_error() returns on this thread (for entry
// points defined outside this file).
void set_last_error(const std::string &message) { g_last_error = message; }
}  // namespace rpg

extern "C" {

rpg_status rpg_sieve_run(const char *const *coefficients, int32_t coefficient_count,
                         int64_t numerator_bound, int32_t first, int32_t last, uint32_t flags,
                         int32_t device, rpg_candidate_cb callback, void *user,
                         rpg_sieve_stats *stats) {
    return guarded([&]() -> rpg_status {
        std::vector<std::string> coeffs;
        std::string error;
        if (!coefficients_from(coefficients, coefficient_count, coeffs, error))
            return fail(RPG_E_ARG, error);
        if (numerator_bound < 1) return fail(RPG_E_ARG, "maximum height must be positive");
        if (first < 1 || first > last) return fail(RPG_E_ARG, "invalid denominator range");
        if (!callback) return fail(RPG_E_ARG, "callback must not be NULL");
        rpg::SieveOptions so;
        so.plan = (flags & RPG_SIEVE_FAST_PLAN) ? rpg::PlanKind::fast : rpg::PlanKind::reference;
        so.square = (flags & RPG_SIEVE_SQUARE_DENOMINATORS) != 0;
        so.device = device;
        if (so.square && last > 46340) return fail(RPG_E_ARG, "invalid denominator range");
        rpg::Sieve sieve(coeffs, numerator_bound, so);
        sieve.start(first, last, 1 << 16);
        rpg::BatchView view;
        unsigned long long total = 0, denominators = 0;
        std::vector<int64_t> a64;
        std::vector<int32_t> d32;
        bool stopped = false;
        while (!stopped && sieve.next(view)) {
            total += view.count;
            if (view.complete) denominators += (unsigned long long)(view.last - view.first + 1);
            if (!view.count) continue;
            a64.assign(view.a, view.a + view.count);
            d32.assign(view.d, view.d + view.count);
            if (callback(a64.data(), d32.data(), view.count, user) != 0) stopped = true;
        }
        if (stopped) sieve.cancel();
        if (stats) {
            std::memset(stats, 0, sizeof *stats);
            const auto &t = sieve.timings();
            stats->survivor_count = total;
            stats->host_candidates = total;
            stats->word_count = (uint64_t)rpg::word_count32(numerator_bound);
            stats->denominator_count = denominators;
            stats->launches = t.launches;
            stats->basis_ms = t.table_ms;
            stats->sieve_ms = t.sieve_ms;
            stats->plan_ms = t.plan_ms;
            stats->workspace_ms = t.workspace_ms;
            stats->basis_wall_ms = t.table_wall_ms;
            stats->h2d_bytes = t.h2d_bytes;
            stats->d2h_bytes = t.d2h_bytes;
        }
        return RPG_OK;
    });
}

rpg_status rpg_point_search(const rpg_search_options *o, rpg_point_cb callback, void *user,
                            rpg_sieve_stats *stats) {
    return guarded([&]() -> rpg_status {
        if (!o || !callback) return fail(RPG_E_ARG, "options and callback must not be NULL");
        rpg::SearchOptions s;
        std::string error;
        if (!options_from(*o, s, error)) return fail(RPG_E_ARG, error);
        rpg::PointSearch search(s);
        rpg::SearchMetrics m = search.run([&](const rpg::PointPair &p) {
            return callback(p.numerator, p.ordinate.c_str(), p.denominator, user) != 0;
        });
        fill_stats(stats, m);
        return RPG_OK;
    });
}

rpg_status rpg_fast_plan(const char *const *coefficients, int32_t coefficient_count, int64_t numerator_bound,
                         rpg_fast_plan_info *plan) {
    return guarded([&]() -> rpg_status {
        std::vector<std::string> coeffs;
        std::string error;
        if (!coefficients_from(coefficients, coefficient_count, coeffs, error)) return fail(RPG_E_ARG, error);
        if (!plan) return fail(RPG_E_ARG, "output must not be NULL");
        if (numerator_bound < 1) return fail(RPG_E_ARG, "maximum height must be positive");
        const rpg::FastPlan p = rpg::single_curve_plan(coeffs, numerator_bound, nullptr);
        std::memset(plan, 0, sizeof *plan);
        plan->class_prime = p.class_prime;
        plan->modulus_count = int32_t(p.moduli.size());
        for (std::size_t i = 0; i < p.moduli.size() && i < 16; ++i) {
            plan->moduli[i] = p.moduli[i];
            for (std::size_t f = 0; f < p.slots[i].size() && f < 4; ++f) plan->factors[i][f] = p.slots[i][f];
        }
        plan->bits = p.bits;
        plan->slots = p.row_slots;
        return RPG_OK;
    });
}

rpg_status rpg_tune_fast_plan(const char *const *coefficients, int32_t coefficient_count,
                              int64_t numerator_bound, int32_t first, int32_t last, uint32_t flags,
                              int32_t device, int64_t sample, rpg_tune_report *report) {
    return guarded([&]() -> rpg_status {
        std::vector<std::string> coeffs;
        std::string error;
        if (!coefficients_from(coefficients, coefficient_count, coeffs, error)) return fail(RPG_E_ARG, error);
        if (!report) return fail(RPG_E_ARG, "report must not be NULL");
        if (numerator_bound < 1) return fail(RPG_E_ARG, "maximum height must be positive");
        if (first < 1 || last < first || sample < 1) return fail(RPG_E_ARG, "invalid denominator range");
        if ((flags & RPG_SIEVE_SQUARE_DENOMINATORS) && last > 46340)
            return fail(RPG_E_ARG, "invalid denominator range");
        const rpg::TuneResult r = rpg::tune_fast_shape(coeffs, numerator_bound, first, last,
                                                       (flags & RPG_SIEVE_SQUARE_DENOMINATORS) != 0, device,
                                                       sample);
        std::memset(report, 0, sizeof *report);
        report->rows = r.chosen.rows;
        report->slots = r.chosen.slots;
        report->candidates = int32_t(std::min<std::size_t>(r.candidates.size(), RPG_TUNE_MAX_CANDIDATES));
        for (int i = 0; i < report->candidates; ++i) {
            report->candidate_rows[i] = r.candidates[i].shape.rows;
            report->candidate_slots[i] = r.candidates[i].shape.slots;
            report->candidate_ms[i] = r.candidates[i].ms;
            report->candidate_bits[i] = r.candidates[i].bits;
        }
        report->sample_denominators = r.sample;
        report->stored = r.stored ? 1 : 0;
        std::snprintf(report->key, sizeof report->key, "%s", r.key.c_str());
        return RPG_OK;
    });
}

rpg_status rpg_fast_shape(const char *const *coefficients, int32_t coefficient_count, int64_t numerator_bound,
                          int32_t *rows, int32_t *slots, int32_t *from_cache) {
    return guarded([&]() -> rpg_status {
        std::vector<std::string> coeffs;
        std::string error;
        if (!coefficients_from(coefficients, coefficient_count, coeffs, error)) return fail(RPG_E_ARG, error);
        if (!rows || !slots || !from_cache) return fail(RPG_E_ARG, "outputs must not be NULL");
        if (numerator_bound < 1) return fail(RPG_E_ARG, "maximum height must be positive");
        const rpg::FastShape stored = rpg::tuned_fast_shape(coeffs, numerator_bound);
        const rpg::FastPlan p = rpg::single_curve_plan(coeffs, numerator_bound, nullptr, stored);
        *rows = int32_t(p.moduli.size());
        *slots = p.row_slots;
        *from_cache = stored.rows > 0 ? 1 : 0;
        return RPG_OK;
    });
}

rpg_status rpg_preverify(const char *const *coefficients, int32_t coefficient_count, int64_t numerator,
                         int64_t denominator, int32_t *may_be_point) {
    return guarded([&]() -> rpg_status {
        std::vector<std::string> coeffs;
        std::string error;
        if (!coefficients_from(coefficients, coefficient_count, coeffs, error)) return fail(RPG_E_ARG, error);
        if (!may_be_point) return fail(RPG_E_ARG, "output must not be NULL");
        if (denominator < 1 || denominator > 2147483647LL) return fail(RPG_E_ARG, "denominator out of range");
        *may_be_point = rpg::preverify_host(coeffs, numerator, denominator) ? 1 : 0;
        return RPG_OK;
    });
}

rpg_status rpg_is_squarefree(const char *const *coefficients, int32_t coefficient_count,
                             int32_t *is_squarefree) {
    return guarded([&]() -> rpg_status {
        std::vector<std::string> coeffs;
        std::string error;
        if (!coefficients_from(coefficients, coefficient_count, coeffs, error))
            return fail(RPG_E_ARG, error);
        if (!is_squarefree) return fail(RPG_E_ARG, "output must not be NULL");
        *is_squarefree = rpg::ExactPolynomial(coeffs).is_squarefree() ? 1 : 0;
        return RPG_OK;
    });
}

rpg_status rpg_square_root(const char *const *coefficients, int32_t coefficient_count,
                           int64_t numerator, int64_t denominator, char *ordinate,
                           size_t ordinate_capacity, int32_t *is_point) {
    return guarded([&]() -> rpg_status {
        std::vector<std::string> coeffs;
        std::string error;
        if (!coefficients_from(coefficients, coefficient_count, coeffs, error))
            return fail(RPG_E_ARG, error);
        if (!is_point) return fail(RPG_E_ARG, "output must not be NULL");
        std::string root;
        const bool point = rpg::ExactPolynomial(coeffs).square_root(numerator, denominator, root);
        *is_point = point ? 1 : 0;
        if (point && ordinate) {
            if (root.size() + 1 > ordinate_capacity)
                return fail(RPG_E_ARG, "ordinate buffer too small");
            std::memcpy(ordinate, root.c_str(), root.size() + 1);
        }
        return RPG_OK;
    });
}

int32_t rpg_cli_main(int32_t argc, char **argv) { return rpg::run_cli(argc, argv); }

rpg_status rpg_session_create(const char *const *coefficients, int32_t coefficient_count,
                              int64_t numerator_bound, uint32_t flags, int32_t device,
                              rpg_session **session) {
    return guarded([&]() -> rpg_status {
        if (!session) return fail(RPG_E_ARG, "session must not be NULL");
        *session = nullptr;
        std::vector<std::string> coeffs;
        std::string error;
        if (!coefficients_from(coefficients, coefficient_count, coeffs, error))
            return fail(RPG_E_ARG, error);
        if (numerator_bound < 1) return fail(RPG_E_ARG, "maximum height must be positive");
        rpg::SieveOptions so;
        so.plan = (flags & RPG_SIEVE_FAST_PLAN) ? rpg::PlanKind::fast : rpg::PlanKind::reference;
        so.square = (flags & RPG_SIEVE_SQUARE_DENOMINATORS) != 0;
        so.device = device;
        std::unique_ptr<rpg_session> s(new rpg_session);
        s->sieve.reset(new rpg::Sieve(coeffs, numerator_bound, so));
        rpg::check_cuda(cudaEventCreate(&s->begin), "cudaEventCreate");
        rpg::check_cuda(cudaEventCreate(&s->end), "cudaEventCreate");
        *session = s.release();
        return RPG_OK;
    });
}

rpg_status rpg_session_count(rpg_session *session, int32_t first, int32_t last, int32_t batch_size,
                             uint64_t *survivors, double *device_ms) {
    return guarded([&]() -> rpg_status {
        if (!session) return fail(RPG_E_ARG, "session must not be NULL");
        if (first < 1 || first > last || batch_size < 1)
            return fail(RPG_E_ARG, "invalid denominator range");
        cudaStream_t st = session->sieve->stream();
        rpg::check_cuda(cudaEventRecord(session->begin, st), "cudaEventRecord");
        const unsigned long long n = session->sieve->count_only(first, last, batch_size);
        rpg::check_cuda(cudaEventRecord(session->end, st), "cudaEventRecord");
        rpg::check_cuda(cudaEventSynchronize(session->end), "cudaEventSynchronize");
        float ms = 0;
        rpg::check_cuda(cudaEventElapsedTime(&ms, session->begin, session->end),
                        "cudaEventElapsedTime");
        if (survivors) *survivors = n;
        if (device_ms) *device_ms = ms;
        return RPG_OK;
    });
}

rpg_status rpg_session_work(rpg_session *session, int32_t first, int32_t last,
                            uint64_t *words_swept, uint32_t *smem_bytes_per_word) {
    return guarded([&]() -> rpg_status {
        if (!session) return fail(RPG_E_ARG, "session must not be NULL");
        if (words_swept) *words_swept = session->sieve->swept_words(first, last);
        if (smem_bytes_per_word) *smem_bytes_per_word = session->sieve->smem_bytes_per_word();
        return RPG_OK;
    });
}

rpg_status rpg_session_plan(rpg_session *session, int32_t *class_prime, int32_t *primes,
                            int32_t capacity, int32_t *count) {
    return guarded([&]() -> rpg_status {
        if (!session || !class_prime || !count) return fail(RPG_E_ARG, "arguments must not be NULL");
        const rpg::FastPlanInfo info = session->sieve->fast_plan_info();
        *class_prime = info.class_prime;
        *count = int32_t(info.primes.size());
        if (*count > capacity || (*count && !primes)) return fail(RPG_E_ARG, "prime buffer too small");
        for (int32_t i = 0; i < *count; ++i) primes[i] = info.primes[i];
        return RPG_OK;
    });
}

void rpg_session_destroy(rpg_session *session) { delete session; }

// The batch specs of the curves that pass the option checks (their indices
// in valid); status[i] is RPG_E_ARG for the others.
void batch_specs_from(const rpg_search_options *curves, int32_t curve_count, std::vector<int32_t> &status,
                      std::vector<std::size_t> &valid, std::vector<rpg::BatchCurveSpec> &run) {
    const std::size_t count = static_cast<std::size_t>(curve_count);
    status.assign(count, RPG_OK);
    for (int32_t i = 0; i < curve_count; ++i) {
        rpg::SearchOptions s;
        std::string error;
        if (!options_from(curves[i], s, error)) {
            status[std::size_t(i)] = RPG_E_ARG;
            continue;
        }
        rpg::BatchCurveSpec b;
        b.coefficients = s.coefficients;
        b.bound = s.numerator_bound;
        b.first = s.first;
        b.last = s.last;
        b.square = s.square;
        b.include_infinity = s.include_infinity;
        b.intervals = s.intervals;
        valid.push_back(std::size_t(i));
        run.push_back(std::move(b));
    }
}

rpg_status rpg_batch_search(const rpg_search_options *curves, int32_t curve_count, int32_t device,
                            uint32_t flags, rpg_batch_point_cb callback, void *user,
                            int32_t *curve_status, uint64_t *curve_survivors,
                            rpg_batch_stats *stats) {
    return guarded([&]() -> rpg_status {
        if (curve_count < 0 || (curve_count > 0 && !curves) || !callback)
            return fail(RPG_E_ARG, "curves and callback must not be NULL");
        const std::size_t count = static_cast<std::size_t>(curve_count);
        std::vector<int32_t> status;
        std::vector<std::size_t> valid;
        std::vector<rpg::BatchCurveSpec> run;
        batch_specs_from(curves, curve_count, status, valid, run);
        rpg::BatchStats st;
        std::vector<rpg::BatchCurveResult> results =
            rpg::batch_search(run, device, &st, (flags & RPG_BATCH_NO_GRAPH) == 0,
                              (flags & RPG_BATCH_HOST_VERIFY_ONLY) == 0);
        std::vector<const rpg::BatchCurveResult *> by_index(count, nullptr);
        for (std::size_t j = 0; j < valid.size(); ++j) {
            by_index[valid[j]] = &results[j];
            if (results[j].status == RPG_E_NOT_SQUAREFREE) status[valid[j]] = RPG_E_NOT_SQUAREFREE;
            else if (results[j].status != 0) status[valid[j]] = RPG_E_ARG;
        }
        for (int32_t i = 0; i < curve_count; ++i) {
            const rpg::BatchCurveResult *r = by_index[std::size_t(i)];
            if (curve_status) curve_status[i] = status[std::size_t(i)];
            if (curve_survivors) curve_survivors[i] = r ? r->survivors : 0;
            if (!r || status[std::size_t(i)] != RPG_OK) continue;
            for (const auto &p : r->points)
                if (callback(i, p.numerator, p.ordinate.c_str(), p.denominator, user) == 0) break;
        }
        if (stats) {
            std::memset(stats, 0, sizeof *stats);
            stats->curves = st.curves;
            stats->wide_curves = st.wide_curves;
            stats->denominators = st.denominators;
            stats->survivors = st.survivors;
            stats->host_candidates = st.host_candidates;
            stats->points = st.points;
            stats->launches = st.launches;
            stats->words = st.words;
            stats->table_words = st.table_words;
            stats->swept_words = st.swept_words;
            stats->smem_bytes = st.smem_bytes;
            stats->rectangle_sites = double(st.rectangle_sites);
            stats->plan_ms = st.plan_ms;
            stats->table_ms = st.table_ms;
            stats->sieve_ms = st.sieve_ms;
            stats->wide_ms = st.wide_ms;
            stats->narrow_ms = st.narrow_ms;
            stats->verify_ms = st.verify_ms;
            stats->wall_ms = st.wall_ms;
            stats->h2d_bytes = st.h2d_bytes;
            stats->d2h_bytes = st.d2h_bytes;
            stats->graph = st.graph ? 1 : 0;
            stats->items_per_kernel = st.items_per_kernel;
            stats->items_from_cache = st.items_from_cache ? 1 : 0;
        }
        return RPG_OK;
    });
}

rpg_status rpg_tune_batch(const rpg_search_options *curves, int32_t curve_count, int32_t device,
                          rpg_batch_tune_report *report) {
    return guarded([&]() -> rpg_status {
        if (curve_count < 1 || !curves || !report) return fail(RPG_E_ARG, "curves and report must not be NULL");
        std::vector<int32_t> status;
        std::vector<std::size_t> valid;
        std::vector<rpg::BatchCurveSpec> run;
        batch_specs_from(curves, curve_count, status, valid, run);
        if (run.empty()) return fail(RPG_E_ARG, "no valid curve to tune on");
        const rpg::BatchTuneResult r = rpg::tune_batch_items(run, device);
        std::memset(report, 0, sizeof *report);
        report->items = r.items;
        report->candidates = int32_t(std::min<std::size_t>(r.candidates.size(), RPG_TUNE_MAX_CANDIDATES));
        for (int i = 0; i < report->candidates; ++i) {
            report->candidate_items[i] = r.candidates[std::size_t(i)].first;
            report->candidate_ms[i] = r.candidates[std::size_t(i)].second;
        }
        report->stored = r.stored ? 1 : 0;
        std::snprintf(report->key, sizeof report->key, "%s", r.key.c_str());
        return RPG_OK;
    });
}

rpg_status rpg_batch_items(const rpg_search_options *curves, int32_t curve_count, int32_t *items,
                           int32_t *from_cache) {
    return guarded([&]() -> rpg_status {
        if (curve_count < 0 || (curve_count > 0 && !curves) || !items || !from_cache)
            return fail(RPG_E_ARG, "curves and outputs must not be NULL");
        std::vector<int32_t> status;
        std::vector<std::size_t> valid;
        std::vector<rpg::BatchCurveSpec> run;
        batch_specs_from(curves, curve_count, status, valid, run);
        const int stored = rpg::tuned_batch_items(run);
        *items = stored > 0 ? stored : rpg::kDefaultBatchItems;
        *from_cache = stored > 0 ? 1 : 0;
        return RPG_OK;
    });
}

struct rpg_server {
    std::unique_ptr<rpg::SearchServer> server;
};

rpg_status rpg_server_create(const rpg_server_options *options, rpg_server **server) {
    return guarded([&]() -> rpg_status {
        if (!options || !server) return fail(RPG_E_ARG, "options and server must not be NULL");
        rpg::ServeOptions o;
        o.device = options->device;
        o.lanes = options->lanes;
        o.memory_budget = options->memory_budget_bytes;
        o.max_batch_curves = options->max_batch_curves;
        if (o.memory_budget == 0) return fail(RPG_E_ARG, "memory budget must be positive");
        auto s = std::make_unique<rpg_server>();
        s->server = std::make_unique<rpg::SearchServer>(o);
        *server = s.release();
        return RPG_OK;
    });
}

rpg_status rpg_server_submit(rpg_server *server, const rpg_search_options *request,
                             int32_t first_point_only, uint64_t *request_id) {
    return guarded([&]() -> rpg_status {
        if (!server || !request || !request_id)
            return fail(RPG_E_ARG, "server, request and request_id must not be NULL");
        rpg::SearchOptions s;
        std::string error;
        if (!options_from(*request, s, error)) return fail(RPG_E_ARG, error);
        rpg::BatchCurveSpec b;
        b.coefficients = s.coefficients;
        b.bound = s.numerator_bound;
        b.first = s.first;
        b.last = s.last;
        b.square = s.square;
        b.include_infinity = s.include_infinity;
        b.intervals = s.intervals;
        *request_id = server->server->submit(b, first_point_only != 0);
        return RPG_OK;
    });
}

rpg_status rpg_server_wait(rpg_server *server, uint64_t request_id, double timeout_ms,
                           rpg_point_cb callback, void *user, int32_t *done,
                           rpg_request_stats *stats) {
    return guarded([&]() -> rpg_status {
        if (!server || !done) return fail(RPG_E_ARG, "server and done must not be NULL");
        *done = 0;
        rpg::ServeResult r;
        if (!server->server->wait(request_id, timeout_ms, r)) return RPG_OK;
        *done = 1;
        if (stats) {
            std::memset(stats, 0, sizeof *stats);
            stats->latency_ms = r.latency_ms;
            stats->queue_ms = r.queue_ms;
            stats->rectangle_sites = double(r.rectangle_sites);
            stats->survivors = r.survivors;
            stats->points = r.points.size();
            stats->waves = r.waves;
        }
        if (r.status != 0) return fail(rpg_status(r.status), r.error);
        if (callback)
            for (const auto &p : r.points)
                if (callback(p.numerator, p.ordinate.c_str(), p.denominator, user) == 0) break;
        return RPG_OK;
    });
}

void rpg_server_destroy(rpg_server *server) { delete server; }

int32_t rpg_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
    return n;
}

int32_t rpg_abi_version(void) { return RPG_ABI_VERSION; }

rpg_status rpg_release_cached_resources(int32_t device) {
    return guarded([&]() -> rpg_status {
        rpg::release_pooled_pipelines(device < 0 ? -1 : device);
        return RPG_OK;
    });
}

const char *rpg_last_error(void) { return g_last_error.c_str(); }

}  // extern "C"
