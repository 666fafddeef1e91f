/*
 * ratpoints_gb300.h - C ABI of the GB300 rational-point search library (librpgpu).
 *
 * Plain C types only: pointers, sizes, fixed-width integers.  Errors cross the
 * ABI as rpg_status codes; rpg_last_error() returns the message of the last
 * failing call on the calling thread (the reference throws C++ exceptions
 * carrying the same messages: include/cuda_support.hpp:14-19,
 * src/point_search.cpp:17-26, src/sieve_plan.cpp:110-113).
 *
 * Threading: calls may run on any thread; each call binds the device it is
 * given (or the calling thread's current device) before any CUDA work, and all
 * callbacks run synchronously on the calling thread.
 */
#ifndef RATPOINTS_GB300_H
#define RATPOINTS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Raised when a structure layout or a signature changes (3: rpg_batch_stats
 * gained items_per_kernel and items_from_cache). */
#define RPG_ABI_VERSION 3

typedef enum rpg_status {
    RPG_OK = 0,
    RPG_E_ARG = 1,            /* invalid argument or option */
    RPG_E_CUDA = 2,           /* CUDA runtime failure */
    RPG_E_OOM = 3,            /* device or host allocation failed */
    RPG_E_TIMEOUT = 4,        /* a bounded device wait expired */
    RPG_E_INTERNAL = 5,       /* broken internal invariant or counter overflow */
    RPG_E_NOT_SQUAREFREE = 6  /* the polynomial is not squarefree */
} rpg_status;

/* Sieve flags. */
#define RPG_SIEVE_SQUARE_DENOMINATORS 1u /* parameters k give denominators k*k */
#define RPG_SIEVE_FAST_PLAN 2u           /* this project's plan; default is the reference plan */

/* Sieve plans for rpg_search_options.plan. */
#define RPG_PLAN_REFERENCE 0
#define RPG_PLAN_FAST 1

/* Timing and counters of one sieve or search run.  Field meanings follow the
 * reference's SieveMetrics / SearchMetrics (include/sieve.hpp:13-24,
 * include/point_search.hpp:41-60). */
typedef struct rpg_sieve_stats {
    uint64_t survivor_count;   /* modular survivors emitted */
    uint64_t word_count;       /* 32-site words per denominator row (reference metric) */
    uint64_t denominator_count;
    uint64_t launches;         /* sieve kernel launches */
    double basis_ms;           /* device table build, CUDA events */
    double sieve_ms;           /* sieve launches, CUDA events */
    double plan_ms;
    double workspace_ms;
    double basis_wall_ms;
    double survivor_setup_ms;
    double verification_ms;
    double sieve_wall_ms;
    double initial_mask_bytes;
    uint64_t h2d_bytes;        /* host-to-device bytes copied */
    uint64_t d2h_bytes;        /* device-to-host bytes copied */
    uint64_t host_candidates;  /* survivors handed to the host's exact check (after device
                                  pre-verification; survivor_count without it) */
} rpg_sieve_stats;

/* Receives one batch of modular survivors (structure of arrays).  The arrays
 * are valid only during the call.  Return 0 to continue, nonzero to stop the
 * sieve early (rpg_sieve_run then returns RPG_OK). */
typedef int (*rpg_candidate_cb)(const int64_t *numerators, const int32_t *denominators,
                                size_t count, void *user);

/*
 * Modular sieve over numerators [-numerator_bound, numerator_bound] and
 * parameters [first, last] (denominators d = k, or k*k with
 * RPG_SIEVE_SQUARE_DENOMINATORS).  Every site whose F(a, d) is a square modulo
 * each sieve modulus is delivered exactly once; order is unspecified.
 * With the reference plan the delivered set is exactly the reference's
 * survivor set (unreduced pairs included).
 *
 * Replaces: ratpoints_gpu::run_modular_sieve (include/sieve.hpp:41-47 of the
 * reference; driver at src/sieve.cu:503-580).
 */
rpg_status rpg_sieve_run(const char *const *coefficients, int32_t coefficient_count,
                         int64_t numerator_bound, int32_t first, int32_t last, uint32_t flags,
                         int32_t device, rpg_candidate_cb callback, void *user,
                         rpg_sieve_stats *stats);

/* A closed x interval; a NULL bound is unbounded.  Bounds use the -l/-u
 * syntax: [+-]digits[.digits][e[+-]digits]. */
typedef struct rpg_interval {
    const char *lower;
    const char *upper;
} rpg_interval;

typedef struct rpg_search_options {
    const char *const *coefficients;  /* c0 .. cn as decimal text */
    int32_t coefficient_count;
    int64_t numerator_bound;          /* H */
    int32_t first;                    /* parameter range (denominators, or k) */
    int32_t last;
    const rpg_interval *intervals;    /* ascending, disjoint; may be NULL */
    int32_t interval_count;
    int32_t include_infinity;         /* nonzero: report points at infinity first */
    int32_t batch_size;               /* denominators per batch, 1..65536 */
    int32_t square_denominators;
    int32_t plan;                     /* RPG_PLAN_REFERENCE or RPG_PLAN_FAST */
    int32_t device;                   /* CUDA device ordinal, -1: current */
    int32_t verify_threads;           /* host verification threads, 0: all cores */
    uint32_t flags;                   /* RPG_SEARCH_* bits */
} rpg_search_options;

/* rpg_search_options.flags.  By default a kernel drops, before the copy to the
 * host, the survivors that fail gcd(a, d) = 1 or a residue test of F(a, d)
 * (mod 2^64, the primes 3..97 and four primes below 2^31): no point fails
 * them, so the reported points are the same; the survivor count stays the
 * modular one.  This flag sends every modular survivor to the host instead,
 * as the reference does (src/point_search.cpp:48-60). */
#define RPG_SEARCH_HOST_VERIFY_ONLY 1u

/* One verified point (numerator : ordinate : denominator); the ordinate is
 * the non-negative root in decimal, valid only during the call.  Return
 * nonzero to continue, 0 to stop the search. */
typedef int (*rpg_point_cb)(int64_t numerator, const char *ordinate, int64_t denominator,
                            void *user);

/*
 * Full search: infinity first (if requested and present), then verified
 * points with gcd(a, d) = 1 in batch order, (d, a) ascending within a batch,
 * filtered by the intervals.  Fails with RPG_E_NOT_SQUAREFREE before any
 * callback if f is not squarefree.
 *
 * Replaces: ratpoints_gpu::PointSearch / PointSearch::run
 * (include/point_search.hpp:62-78, src/point_search.cpp:155-240).
 */
rpg_status rpg_point_search(const rpg_search_options *options, rpg_point_cb callback, void *user,
                            rpg_sieve_stats *stats);

/* Exact predicates.  Replace ExactPolynomial::is_squarefree and
 * ExactPolynomial::square_root (src/exact_polynomial.cpp:25-71). */
rpg_status rpg_is_squarefree(const char *const *coefficients, int32_t coefficient_count,
                             int32_t *is_squarefree);
rpg_status rpg_square_root(const char *const *coefficients, int32_t coefficient_count,
                           int64_t numerator, int64_t denominator, char *ordinate,
                           size_t ordinate_capacity, int32_t *is_point);

/* The fast plan a single-curve search uses (host only, no device needed):
 * numerator classes modulo 64 * class_prime, and the stage-1 row moduli with
 * their prime factors (factors[i][0..3], 0-padded) and filtering bits.  No
 * counterpart in the reference, whose prime set is fixed. */
typedef struct rpg_fast_plan_info {
    int32_t class_prime;
    int32_t modulus_count;
    int32_t moduli[16];
    int32_t factors[16][4];
    double bits;
    int32_t slots;             /* denominators staged per CTA by the single-curve kernel (2 or 3) */
} rpg_fast_plan_info;
rpg_status rpg_fast_plan(const char *const *coefficients, int32_t coefficient_count, int64_t numerator_bound,
                         rpg_fast_plan_info *plan);

/*
 * Measured choice of the fast plan's shape: the number of stage-1 rows and
 * the row slots (2 or 3) per CTA of the single-curve kernel.  Builds the sieve
 * with the cost model's shape and its neighbours (the other slot count, one
 * and two rows fewer or more), times each with CUDA events on parameters
 * [first, first + sample) (clipped to last; flags: RPG_SIEVE_SQUARE_DENOMINATORS),
 * and reports them with the fastest.  When the environment variable
 * RPG_TUNE_CACHE names a file, the choice is stored there as JSON, keyed by
 * the kind of curve (degree, class prime, row length, small- or large-prime
 * rows), and every later fast-plan sieve of a curve of that kind in a process
 * with that variable uses it.  No counterpart in the reference, whose kernel
 * shape is fixed (its tests/tune_cuda.py times build variants).
 */
#define RPG_TUNE_MAX_CANDIDATES 8
typedef struct rpg_tune_report {
    int32_t rows;                          /* the chosen shape */
    int32_t slots;
    int32_t candidates;                    /* shapes timed */
    int32_t candidate_rows[RPG_TUNE_MAX_CANDIDATES];
    int32_t candidate_slots[RPG_TUNE_MAX_CANDIDATES];
    double candidate_ms[RPG_TUNE_MAX_CANDIDATES];
    double candidate_bits[RPG_TUNE_MAX_CANDIDATES];
    int64_t sample_denominators;
    int32_t stored;                        /* 1: written to the RPG_TUNE_CACHE file */
    char key[96];                          /* the kind of curve, NUL-terminated */
} rpg_tune_report;
rpg_status rpg_tune_fast_plan(const char *const *coefficients, int32_t coefficient_count,
                              int64_t numerator_bound, int32_t first, int32_t last, uint32_t flags,
                              int32_t device, int64_t sample, rpg_tune_report *report);
/* The shape a fast-plan sieve of this curve would use (host only): *rows and
 * *slots of its plan, *from_cache 1 when a stored tuning result decides it
 * (see rpg_tune_fast_plan), 0 when the cost model does. */
rpg_status rpg_fast_shape(const char *const *coefficients, int32_t coefficient_count, int64_t numerator_bound,
                          int32_t *rows, int32_t *slots, int32_t *from_cache);

/* The device pre-verification test of one site, evaluated on the host:
 * *may_be_point = 0 iff gcd(a, d) != 1 or F(a, d) fails a residue test that
 * every square passes (mod 2^64, the primes 3..97, four primes below 2^31).
 * No counterpart in the reference. */
rpg_status rpg_preverify(const char *const *coefficients, int32_t coefficient_count, int64_t numerator,
                         int64_t denominator, int32_t *may_be_point);

/* The ratpoints_gpu command line in-process (src/main.cpp:48-85): writes to
 * stdout/stderr and returns the exit status. */
int32_t rpg_cli_main(int32_t argc, char **argv);

/* Benchmark session: tables resident on the device, survivors counted on the
 * device only.  rpg_session_count reports the CUDA-event time of the sieve
 * launches it issues. */
typedef struct rpg_session rpg_session;
rpg_status rpg_session_create(const char *const *coefficients, int32_t coefficient_count,
                              int64_t numerator_bound, uint32_t flags, int32_t device,
                              rpg_session **session);
rpg_status rpg_session_count(rpg_session *session, int32_t first, int32_t last,
                             int32_t batch_size, uint64_t *survivors, double *device_ms);
/* The fast plan the session chose for its curve: numerator classes are taken
 * modulo 64 * class_prime (1: 2-adic classes only) and the first-stage rows
 * test the small primes written to primes[0 .. *count).  For a reference-plan
 * session class_prime and *count are 0. */
rpg_status rpg_session_plan(rpg_session *session, int32_t *class_prime, int32_t *primes,
                            int32_t capacity, int32_t *count);

/* Work a pass over parameters [first, last] does: 64-site words the sieve
 * kernel sweeps (admissible classes only under the fast plan) and the
 * shared-memory bytes its first stage reads per swept word. */
rpg_status rpg_session_work(rpg_session *session, int32_t first, int32_t last,
                            uint64_t *words_swept, uint32_t *smem_bytes_per_word);
void rpg_session_destroy(rpg_session *session);

/*
 * Sieve [first, last] with the session's resident tables without allocating
 * any memory.  No counterpart in the reference.  It exists for callers that
 * cannot allocate when they sieve: engines that reserve all of their device
 * memory up front and hand it out from their own pool, so that a further
 * cudaMalloc would fail or bypass their accounting, and latency-bound loops
 * that cannot afford cudaMalloc/cudaFree, which may synchronize the device.
 *
 * Survivors go to the caller's device arrays (capacity entries each); the
 * caller's *device_count receives the total, which exceeds capacity when the
 * arrays were too small (entries past capacity are not written).  Work is
 * enqueued on `stream` (a cudaStream_t, NULL for the legacy default stream)
 * and the call returns without waiting; read the count after synchronizing.
 * If a bounded device wait of a launch gives up (the launch then stops early
 * and its survivor set is incomplete), *device_count is set to UINT64_MAX
 * instead: the status returned cannot report it, because the call returns
 * before the GPU runs.  The calling thread's current device is left as it was.
 *
 * Limits, each rejected with RPG_E_ARG: at most 16,777,216 denominators (256
 * launches of 65536) per call; and each row must fit one launch, which fails
 * only for very large numerator bounds (above about 1.7e10 times the class
 * prime for a fast-plan session, above about 3.4e10 for a reference-plan one;
 * rpg_sieve_run has no such limit).
 * The error word and the launches' scheduling counters live in one fixed
 * 2,056-byte device array per GPU, held until the process exits and shared by
 * all calls, which clear it first: calls that overlap on the GPU race on it,
 * so serialize them (one stream, or events).  The first call on a device
 * looks up that array's device address; make that first call before any
 * stream capture.
 */
rpg_status rpg_session_sieve_noalloc(rpg_session *session, int32_t first, int32_t last,
                                     int64_t *device_numerators, int32_t *device_denominators,
                                     uint64_t capacity, uint64_t *device_count, void *stream);

/*
 * Batched search of many curves in one pass: every curve's tables resident on
 * the device, two persistent sieve kernels over device work queues, one
 * captured CUDA graph.  No counterpart in the reference, which searches one
 * curve per process (src/main.cpp:48-85); each curve's points are exactly
 * what rpg_point_search reports for the same options, in the same order.
 *
 * Each curves[i] is read as by rpg_point_search; batch_size, plan, device
 * and verify_threads are ignored (the batch has its own plan and uses
 * `device`).  callback(i, ...) receives curve i's points in order, curves in
 * input order; returning 0 stops the delivery of curve i's remaining points
 * (as a single search stops).  curve_status[i] (optional) receives
 * RPG_OK, RPG_E_ARG or RPG_E_NOT_SQUAREFREE for curve i; a failing curve
 * gets no points and does not fail the call.  curve_survivors[i] (optional)
 * receives the modular survivors of curve i.  The call fails only for a NULL
 * argument, a negative count, or a device error.
 */
#define RPG_BATCH_NO_GRAPH 1u /* launch the batch's kernels directly, not as a CUDA graph */
#define RPG_BATCH_HOST_VERIFY_ONLY 2u /* no device pre-verification (see RPG_SEARCH_HOST_VERIFY_ONLY) */

typedef struct rpg_batch_stats {
    uint64_t curves;           /* curves searched (valid, with denominators) */
    uint64_t wide_curves;      /* of those, swept by the class-layout kernel */
    uint64_t denominators;
    uint64_t survivors;        /* modular survivors of all curves */
    uint64_t points;           /* verified points of all curves, infinity included */
    uint64_t launches;         /* kernel launches (table build and sieve) */
    uint64_t words;            /* 64-site row words of all denominators */
    uint64_t table_words;      /* stage-1 table words resident on the device */
    uint64_t swept_words;      /* 64-site words the sieve kernels sweep (counted by them) */
    uint64_t smem_bytes;       /* stage-1 shared-memory bytes those sweeps read */
    double rectangle_sites;    /* sum over curves of (2H + 1) x denominators */
    double plan_ms;            /* host: validation, plans, descriptors */
    double table_ms;           /* device table build, CUDA events */
    double sieve_ms;           /* both sieve kernels, CUDA events */
    double wide_ms;
    double narrow_ms;
    double verify_ms;          /* host exact verification */
    double wall_ms;            /* the whole call */
    uint64_t h2d_bytes;
    uint64_t d2h_bytes;
    int32_t graph;             /* nonzero if the kernels ran as a CUDA graph */
    uint64_t host_candidates;  /* survivors given to the host's exact check */
    int32_t items_per_kernel;  /* work-item target of the batched kernels */
    int32_t items_from_cache;  /* 1: a stored rpg_tune_batch result chose it */
} rpg_batch_stats;

typedef int (*rpg_batch_point_cb)(int32_t curve, int64_t numerator, const char *ordinate,
                                  int64_t denominator, void *user);

rpg_status rpg_batch_search(const rpg_search_options *curves, int32_t curve_count, int32_t device,
                            uint32_t flags, rpg_batch_point_cb callback, void *user,
                            int32_t *curve_status, uint64_t *curve_survivors,
                            rpg_batch_stats *stats);

/*
 * Measured tuning of rpg_batch_search's work items: the batched kernels take
 * (curve, denominator range) items from device queues, each kernel's work cut
 * into about N items.  rpg_tune_batch runs these curves with N = 2,048, 8,192
 * and 32,768 on one engine (after a warm-up run) and keeps the N with the
 * least batched sieve time (CUDA events) in the RPG_TUNE_CACHE file, under the
 * kind of batch (curve count, median row length, median degree; see
 * rpg_tune_fast_plan for the file).  Later batches of that kind use it; without
 * a stored value N is 8,192.  Curves that fail validation are left out.  No
 * counterpart in the reference, which searches one curve per process.
 */
typedef struct rpg_batch_tune_report {
    int32_t items;                         /* the chosen items per kernel */
    int32_t candidates;
    int32_t candidate_items[RPG_TUNE_MAX_CANDIDATES];
    double candidate_ms[RPG_TUNE_MAX_CANDIDATES];  /* batched sieve time of each */
    int32_t stored;                        /* 1: written to the RPG_TUNE_CACHE file */
    char key[96];                          /* the kind of batch, NUL-terminated */
} rpg_batch_tune_report;
rpg_status rpg_tune_batch(const rpg_search_options *curves, int32_t curve_count, int32_t device,
                          rpg_batch_tune_report *report);
/* The work items per kernel an rpg_batch_search of these curves would use
 * (host only): *from_cache 1 when a stored rpg_tune_batch result decides it. */
rpg_status rpg_batch_items(const rpg_search_options *curves, int32_t curve_count, int32_t *items,
                           int32_t *from_cache);

/*
 * Serving: searches submitted at any time, answered in batches that overlap
 * on the device (continuous batching).  No counterpart in the reference,
 * which runs one search per process (src/main.cpp:48-85).
 *
 * `lanes` batch engines, each with its own CUDA streams and device buffers
 * kept resident across batches, take batches from one dispatcher: whenever a
 * lane is free and requests wait, waiting requests are admitted in arrival
 * order while their estimated device bytes (tables, bitmasks, work items)
 * fit the lane's share of memory_budget_bytes.  Each answer is what
 * rpg_point_search reports for the same options: all points in order, or
 * with first_point_only only the first (the -1 option).  First-point
 * requests are searched in denominator waves of growing size and stop at the
 * first wave holding an accepted point.
 */
typedef struct rpg_server rpg_server;

typedef struct rpg_server_options {
    int32_t device;                 /* CUDA device ordinal, -1: current */
    int32_t lanes;                  /* concurrent batches, 1..16 */
    uint64_t memory_budget_bytes;   /* device bytes for all lanes' batches */
    int32_t max_batch_curves;       /* requests per batch */
} rpg_server_options;

typedef struct rpg_request_stats {
    double latency_ms;              /* submit -> answer */
    double queue_ms;                /* submit -> first batch start */
    double rectangle_sites;         /* (2H + 1) x denominators searched */
    uint64_t survivors;             /* modular survivors of the request */
    uint64_t points;                /* points in the answer */
    int32_t waves;                  /* batch entries the request took */
} rpg_request_stats;

rpg_status rpg_server_create(const rpg_server_options *options, rpg_server **server);
/* Fails with RPG_E_ARG for invalid options (as rpg_point_search would);
 * batch_size, plan, device and verify_threads of the request are ignored. */
rpg_status rpg_server_submit(rpg_server *server, const rpg_search_options *request,
                             int32_t first_point_only, uint64_t *request_id);
/* Waits up to timeout_ms (negative: no limit).  *done = 0 on timeout (RPG_OK).
 * When the request is done, *done = 1, its points go to callback in order
 * (returning 0 stops the delivery), the request is retired, and the call
 * returns the request's own status (RPG_OK, RPG_E_NOT_SQUAREFREE, ...).
 * One waiter per request. */
rpg_status rpg_server_wait(rpg_server *server, uint64_t request_id, double timeout_ms,
                           rpg_point_cb callback, void *user, int32_t *done,
                           rpg_request_stats *stats);
/* Finishes the admitted work, then releases the server. */
void rpg_server_destroy(rpg_server *server);

/* Self-test of the bounded mbarrier wait the pipelined sieve kernels use: one
 * thread waits up to polls (1..2^20) polls on a barrier phase that completes
 * only if arrive is non-zero.  Returns RPG_OK when the wait succeeded and
 * RPG_E_TIMEOUT when it gave up (the kernel returns normally and the context
 * stays usable), as a sieve launch reports a row copy that never landed.
 * No reference counterpart: the reference's kernels have no waits. */
rpg_status rpg_bounded_wait_selftest(int32_t device, int32_t polls, int32_t arrive);

/*
 * The shared-memory read rate of `device` (-1: the current one): every
 * resident warp issues lane-contiguous 64-bit shared loads, the access the
 * sieve kernels' first stage makes, for `iterations` x 16 loads per thread.
 * Writes the rate in GB/s (CUDA events around the launch), in bytes per SM
 * clock (that rate over the SM count and the SM clock, measured in the
 * kernel as clock64 ticks per globaltimer nanosecond) and the launch time.  The sieve's shared-memory roofline is measured against
 * it.  No counterpart in the reference.
 */
rpg_status rpg_smem_read_probe(int32_t device, int32_t iterations, double *gbs,
                               double *bytes_per_clock_per_sm, double *ms);

/* A finished rpg_sieve_run or rpg_point_search leaves its streams, events,
 * survivor buffers (up to 262,144 survivors) and pinned staging for the next
 * search on the same device (at most four such sets per process, about 16 MB
 * each).  This call frees them for `device` (-1: every device); a caller that
 * resets a device (cudaDeviceReset) calls it first.  Searches still running
 * are not affected.  No reference counterpart. */
rpg_status rpg_release_cached_resources(int32_t device);

int32_t rpg_device_count(void);
int32_t rpg_abi_version(void);
const char *rpg_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* RATPOINTS_GB300_H */
