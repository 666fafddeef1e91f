// Device sieve: table build and sieve kernels for sm_103a, and the host driver.
//
// Reference behaviour restated here (see the file:line citations per item):
//   - mask basis: bit j of word u of row r for prime p is
//     affine[((-H + 64 u + j) * r^-1) mod p], row 0 zero (src/sieve.cu:141-172,
//     with 64-site words);
//   - sieve: a site survives iff all 32 selected primes accept it; the last word
//     is clipped at +H (src/sieve.cu:221-388, 196-213, 324-330);
//   - survivors are (a, d) pairs, d = k or k*k (src/sieve.cu:179-181, 250-252).
//
// GB300 design: the tables for all 36 candidate primes are built once per search
// on the device; one persistent launch per denominator batch; each CTA stages
// the rows of its denominator's 10 largest selected primes into shared memory,
// sweeps 64-bit words (4 per thread per step, lane-contiguous, rows extended so
// no wrap test is needed inside a step), and compacts the rare stage-1
// survivors into a per-warp queue that a full warp then checks against the
// remaining 22 primes from L2-resident tables before warp-aggregated emission.
#include "sieve.hpp"
#include "tune.hpp"

#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <future>
#include <mutex>
#include <tuple>
#include <utility>

#include "plan.hpp"
#include "preverify.hpp"
#include "sieve_device.cuh"
#include "sieve_fast.cuh"

namespace rpg {

void check_cuda(cudaError_t status, const char *what) {
    if (status != cudaSuccess)
        throw CudaError(std::string(what) + ": " + cudaGetErrorString(status));
}

namespace dev {

constexpr int kK = 4;                        // words per thread per step
constexpr int kWarps = 8;
constexpr int kThreads = kWarps * kWarpSize;
constexpr int kStride = kThreads * kK;       // words per CTA step
constexpr int kExt = kWarpSize * (kK - 1);   // row extension (words)
constexpr int kRefFast = 10;                 // stage-1 primes held in shared memory
constexpr int kSlotWords = 608;              // >= 509 + kExt, even
constexpr int kQueue = 64;                   // per-warp stage-2 queue entries
constexpr long long kMaxTileWords = 1LL << 30;
constexpr std::size_t kRefSmem =
    std::size_t(kRefFast) * kSlotWords * 8 + std::size_t(kWarps) * kQueue * 12;

static_assert(kSlotWords >= kMaximumPrime + kExt, "slot must hold an extended row");
static_assert(kSlotWords % 2 == 0, "slots must keep 16-byte alignment");

struct RefTables {
    const u64 *rows;
    long long offset[kCandidatePrimes];   // word offset of (prime i, residue 0)
    int length[kCandidatePrimes];         // words per row (p + kExt rounded up to even)
    int prime[kCandidatePrimes];
    u32 magic[kCandidatePrimes];
};

__global__ void ref_table_kernel(u64 *rows, RefTables T, const unsigned char *affine,
                                 const unsigned short *inverse, const int *neg_h_mod,
                                 long long total) {
    long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (id >= total) return;
    int i = 0;
    while (i + 1 < kCandidatePrimes && T.offset[i + 1] <= id) ++i;
    const int p = T.prime[i], L = T.length[i];
    const long long rel = id - T.offset[i];
    const int r = int(rel / L);
    const int u = int(rel % L) % p;
    u64 word = 0;
    if (r != 0) {
        const int inv = inverse[i * kMaximumPrime + r];
        const int x0 = (neg_h_mod[i] + int((64LL * u) % p)) % p;
        int x = int((long long)x0 * inv % p);
        const unsigned char *aff = affine + i * kMaximumPrime;
        for (int j = 0; j < 64; ++j) {
            if (aff[x]) word |= u64(1) << j;
            x += inv;
            if (x >= p) x -= p;
        }
    }
    rows[id] = word;
}

// Stage 2 for up to 32 queued words (one per lane), then emission.
__device__ __forceinline__ void ref_drain(const u64 *qmask, const u32 *qoff, int start, int n,
                                          const RefTables &T, const SieveArgs &A, int denominator,
                                          const int *s_prime, const u32 *s_magic,
                                          const u32 *s_bmod, const long long *s_row) {
    const int lane = threadIdx.x & 31;
    u64 m = 0;
    u32 off = 0;
    if (lane < n) {
        m = qmask[start + lane];
        off = qoff[start + lane];
    }
    __syncwarp();
    const long long w = A.w_lo + off;
    if (m) {
        for (int s = kRefFast; s < kSelectedPrimes; ++s) {
            const u32 p = u32(s_prime[s]);
            u32 idx = s_bmod[s] + mod_small(off, p, s_magic[s]);
            if (idx >= p) idx -= p;
            m &= __ldg(T.rows + s_row[s] + idx);
            if (!m) break;
        }
        if (m && w == A.words - 1) {
            const int valid = int(2 * A.bound + 1 - 64 * (A.words - 1));
            if (valid < 64) m &= (u64(1) << valid) - 1;
        }
    }
    emit_survivors(m, w, A.bound, denominator, A.out_a, A.out_d, A.out_count, A.capacity);
}

__global__ void __launch_bounds__(kThreads) ref_sieve_kernel(RefTables T, SieveArgs A) {
    extern __shared__ __align__(16) u64 smem[];
    u64 *rows = smem;
    u64 *qmask = rows + kRefFast * kSlotWords;
    u32 *qoff = reinterpret_cast<u32 *>(qmask + kWarps * kQueue);

    __shared__ int s_prime[kSelectedPrimes];
    __shared__ u32 s_magic[kSelectedPrimes];
    __shared__ u32 s_bmod[kSelectedPrimes];
    __shared__ long long s_row[kSelectedPrimes];
    __shared__ int s_len[kSelectedPrimes];
    __shared__ int s_ok;

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const long long tile_words = A.w_hi - A.w_lo;
    u64 *wq_mask = qmask + warp * kQueue;
    u32 *wq_off = qoff + warp * kQueue;

    for (int item = blockIdx.x; item < A.k_count; item += gridDim.x) {
        const long long k = A.k_first + item;
        const long long d = A.square ? k * k : k;
        if (threadIdx.x == 0) {
            int n = 0;
            for (int i = kCandidatePrimes - 1; i >= 0 && n < kSelectedPrimes; --i) {
                const int p = T.prime[i];
                const int r = int(d % p);
                if (r == 0) continue;
                s_prime[n] = p;
                s_magic[n] = T.magic[i];
                s_row[n] = T.offset[i] + (long long)r * T.length[i];
                s_len[n] = T.length[i];
                s_bmod[n] = u32(A.w_lo % p);
                ++n;
            }
            s_ok = n == kSelectedPrimes;
        }
        __syncthreads();
        if (!s_ok) {  // unreachable for d < 2^31 (at most 3 candidates divide it)
            __syncthreads();
            continue;
        }
        for (int s = 0; s < kRefFast; ++s) {
            const uint4 *src = reinterpret_cast<const uint4 *>(T.rows + s_row[s]);
            uint4 *dst = reinterpret_cast<uint4 *>(rows + s * kSlotWords);
            const int n16 = s_len[s] >> 1;
            for (int t = threadIdx.x; t < n16; t += kThreads) dst[t] = __ldg(src + t);
        }
        __syncthreads();

        u32 o[kRefFast], st[kRefFast], pb[kRefFast];
        const u32 first = u32(warp * kWarpSize * kK + lane);
#pragma unroll
        for (int s = 0; s < kRefFast; ++s) {
            const u32 p = u32(s_prime[s]);
            o[s] = ((s_bmod[s] + first) % p) * 8u + u32(s * kSlotWords * 8);
            st[s] = (u32(kStride) % p) * 8u;
            pb[s] = p * 8u;
        }
        int qn = 0;
        const unsigned char *rbase = reinterpret_cast<const unsigned char *>(rows);
        for (long long off0 = 0; off0 < tile_words; off0 += kStride) {
            u64 acc[kK];
#pragma unroll
            for (int kk = 0; kk < kK; ++kk) acc[kk] = ~u64(0);
#pragma unroll
            for (int s = 0; s < kRefFast; ++s) {
                const unsigned char *rb = rbase + o[s];
#pragma unroll
                for (int kk = 0; kk < kK; ++kk)
                    acc[kk] &= *reinterpret_cast<const u64 *>(rb + 256 * kk);
                const u32 lo = u32(s * kSlotWords * 8);
                const u32 t = o[s] + st[s];
                o[s] = (t - lo >= pb[s]) ? t - pb[s] : t;
            }
#pragma unroll
            for (int kk = 0; kk < kK; ++kk) {
                const long long off = off0 + warp * kWarpSize * kK + kWarpSize * kk + lane;
                const bool live = acc[kk] != 0 && off < tile_words;
                const u32 b = __ballot_sync(kFullMask, live);
                if (b) {
                    const int pos = qn + __popc(b & lanemask_lt());
                    if (live) {
                        wq_mask[pos] = acc[kk];
                        wq_off[pos] = u32(off);
                    }
                    qn += __popc(b);
                    if (qn >= 32) {
                        __syncwarp();
                        ref_drain(wq_mask, wq_off, qn - 32, 32, T, A, int(d), s_prime, s_magic,
                                  s_bmod, s_row);
                        qn -= 32;
                    }
                }
            }
        }
        __syncwarp();
        ref_drain(wq_mask, wq_off, 0, qn, T, A, int(d), s_prime, s_magic, s_bmod, s_row);
        __syncthreads();
    }
}

}  // namespace dev

// ---------------------------------------------------------------------------

namespace {

using Clock = std::chrono::steady_clock;
double ms_since(Clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
}

template <typename T>
T *device_alloc(std::size_t count, const char *what) {
    void *p = nullptr;
    check_cuda(cudaMalloc(&p, std::max<std::size_t>(count, 1) * sizeof(T)), what);
    return static_cast<T *>(p);
}

constexpr long long kInitialSurvivors = 1 << 16;  // survivors per buffer before any growth

// The streams, events, survivor buffers and pinned staging of a finished
// search, kept for the next search on the same device so that it does not
// create and allocate them again.  Nothing in them outlives a search as
// content: every launch resets its counter words first, survivor arrays are
// written before they are read, and every table is built anew per search.
struct PooledPipeline {
    struct Buf {
        long long *a = nullptr, *pa = nullptr;
        int *d = nullptr, *pd = nullptr;
        long long cap = 0;
        unsigned long long *count = nullptr;
        cudaEvent_t begin = nullptr, end = nullptr, copied = nullptr;
    };
    int device = -1;
    cudaStream_t streams[4] = {};
    cudaEvent_t events[3] = {};
    Buf buf[2];
    unsigned long long *h_count = nullptr;
    long long *h_a = nullptr;
    int *h_d = nullptr;
    long long host_capacity = 0;
};
constexpr std::size_t kPooledPipelines = 4;                   // per process
constexpr long long kPooledSurvivors = 4 * kInitialSurvivors;  // larger buffers are freed

// Never destroyed: static destructors may run after the CUDA runtime is gone.
std::mutex &pipeline_pool_mutex() {
    static auto *m = new std::mutex();
    return *m;
}
std::vector<PooledPipeline> &pipeline_pool() {
    static auto *pool = new std::vector<PooledPipeline>();
    return *pool;
}

}  // namespace

// Most admissible numerator classes of any denominator under the fast plan:
// 2-adic classes (by d mod 64) times residues mod the class prime q (by d mod q).
int max_admissible_classes(const std::vector<std::string> &coefficients, int q) {
    const int n = int(coefficients.size()) - 1;
    std::vector<int> c64(coefficients.size());
    for (std::size_t i = 0; i < coefficients.size(); ++i) c64[i] = decimal_mod(coefficients[i], 64);
    bool square64[64] = {};
    for (int v = 0; v < 64; ++v) square64[(v * v) & 63] = true;
    int most2 = 0;
    for (int dd = 0; dd < 64; ++dd) {
        int count = 0;
        for (int r = 0; r < 64; ++r) {
            if (dd % 2 == 0 && r % 2 == 0) continue;
            int value = c64[n], power = 1;
            for (int i = n - 1; i >= 0; --i) {
                value = (value * r) & 63;
                power = (power * dd) & 63;
                value = (value + c64[i] * power) & 63;
            }
            if (n % 2 == 1) value = (value * dd) & 63;
            count += square64[value];
        }
        most2 = std::max(most2, count);
    }
    if (q <= 1) return std::max(1, most2);
    const auto aff = affine_mask(q, coefficients);
    int most_q = 0;
    for (int dq = 0; dq < q; ++dq) {
        int count = 0;
        for (int r = 0; r < q; ++r) count += dq == 0 ? (r != 0) : aff[(r * mod_inverse(dq, q)) % q];
        most_q = std::max(most_q, count);
    }
    return std::max(1, most2 * std::max(1, most_q));
}

// Dynamic shared memory of the fast kernel: `slots` staged row sets, the
// consumer queues, and the slots' class runs and item prefixes.
std::size_t fast_dynamic_smem(int row_words, int max_classes, int slots) {
    const std::size_t runs = (std::size_t(slots) * max_classes * sizeof(dev::FastRun) + 7) & ~std::size_t(7);
    return std::size_t(slots) * std::size_t(row_words) * 8 + std::size_t(dev::kFConsumers) * dev::kFQueue * 16 +
           runs + std::size_t(slots) * std::size_t(max_classes + 1) * 4;
}

// Staged row words per slot that keep a CTA within half an SM's shared
// memory (2 CTAs/SM, 1 KiB reserved each, 2 KiB of static shared memory).
long long fast_row_budget(int max_classes, int slots) {
    const long long per_cta = 228 * 1024 / 2 - 1024 - 2048;
    return (per_cta - (long long)fast_dynamic_smem(0, max_classes, slots)) / (8LL * slots);
}

FastPlan single_curve_plan(const std::vector<std::string> &coefficients, long long bound, int *max_classes,
                           FastShape shape) {
    // the staged row sets of a CTA, its queues and its slots' class runs must
    // fit shared memory at 2 CTAs/SM.  Three slots stage a denominator ahead
    // further with less shared memory per row set: they pay when sweeping a
    // denominator is short against copying its rows (rows of at most 2^20
    // words) and their plan filters within a quarter bit of the two-slot plan
    // (the C2 curve: 13.22 bits either way, 30.4 ms against 31.4 ms per step;
    // cubics with 31 M-word rows: 2 slots).
    const FastPlanner planner(coefficients, bound);
    const int classes = max_admissible_classes(coefficients, planner.class_prime());
    if (max_classes) *max_classes = classes;
    auto plan_for = [&](int slots) {
        const long long row_budget = fast_row_budget(classes, slots);
        FastPlan plan;
        for (int cap = kMaxModulus;;) {
            plan = shape.rows > 0 ? planner.plan(cap, std::min(shape.rows, kMaxFastSlots), row_budget, false)
                                  : planner.plan(cap, kMaxFastSlots, row_budget);
            int row_words = 0;
            for (int m : plan.moduli) row_words += (m + dev::kFExt + 1) & ~1;
            if (row_words <= row_budget || cap <= 64) break;
            cap = cap * 7 / 8;
        }
        plan.row_slots = slots;
        return plan;
    };
    if (shape.rows > 0) return plan_for(shape.slots == dev::kFMaxSlotCount ? dev::kFMaxSlotCount : 2);
    const FastPlan two = plan_for(2);
    if (word_count64(bound) > (1LL << 20)) return two;
    const FastPlan three = plan_for(dev::kFMaxSlotCount);
    return three.bits >= two.bits - 0.25 ? three : two;
}

struct Sieve::Impl {
    SieveOptions opt;
    long long bound = 0, words = 0;
    int device = 0, grid = 0;
    // stream: table builds and the launches into buffer 0; stream2: the
    // launches into buffer 1, so that a launch's first CTAs take the SMs that
    // the previous launch's last CTAs leave idle; copy_stream: survivor
    // downloads; count_stream: each launch's counter words, so that their
    // small copy does not sit between two launches.
    cudaStream_t stream = nullptr, stream2 = nullptr, copy_stream = nullptr, count_stream = nullptr;
    cudaEvent_t fork_event = nullptr, join_event = nullptr;  // count_only across both launch streams
    // Device time of a search: launches on the two streams overlap, so each
    // batch adds the part of its [begin, end] interval after the previous
    // batch's end, both measured from an origin recorded at start().
    cudaEvent_t origin = nullptr;
    float last_end_ms = 0;
    dev::RefTables T{};
    dev::u64 *rows = nullptr;
    // fast plan
    dev::FastTables F{};
    dev::u64 *fast_rows = nullptr;
    dev::u64 *fast_adm = nullptr;
    dev::FastClassStart *fast_starts = nullptr;
    dev::FastRun *list_runs = nullptr;     // class lists by denominator class (see FastTables)
    int *list_count = nullptr;
    long long list_words = 0;              // class words the lists cover (launches from word 0 to at least this)
    int fast_max_classes = 1;
    std::size_t fast_smem = 0;
    std::vector<dev::u64> fast_adm_host;
    std::vector<int> fast_bad_primes;      // denominator primes (see FastTables::nbad)
    FastPlan fast_plan;
    long long max_tile = dev::kMaxTileWords;
    long long capacity = 0;       // most survivors a buffer may grow to hold
    long long host_capacity = 0;  // entries of the pinned host arrays
    SieveTimings timings;

    struct Buffer {
        long long *a = nullptr;
        int *d = nullptr;
        long long *pa = nullptr;  // survivors kept by device pre-verification (same capacity)
        int *pd = nullptr;
        long long cap = 0;        // entries of a and d
        // [0] survivors, [1] work counter, [2] error word, [3] pre-verified survivors
        unsigned long long *count = nullptr;
        cudaEvent_t begin = nullptr, end = nullptr;
        cudaEvent_t copied = nullptr;  // the counter words are in pinned host memory
        long long first = 0, last = 0;
        bool busy = false;
    };
    Buffer buf[2];
    Preverifier preverifier;
    unsigned long long *h_count = nullptr;  // pinned, 4 words per buffer
    long long *h_a = nullptr;
    int *h_d = nullptr;

    // Batch queue.
    long long q_next = 0, q_last = -1, q_batch = 1;
    std::deque<int> order;  // buffers in flight, oldest first

    // Pieces of an overflowed batch still to deliver, in parameter/word order.
    struct Piece {
        long long first, last, w_lo, w_hi;
    };
    std::deque<Piece> pieces;
    long long piece_batch_first = 0, piece_batch_last = 0;

    ~Impl() { release(); }

    // Take a pooled pipeline of this device, if there is one.
    bool adopt_pipeline() {
        PooledPipeline p;
        {
            std::lock_guard<std::mutex> lock(pipeline_pool_mutex());
            auto &pool = pipeline_pool();
            auto it = std::find_if(pool.begin(), pool.end(),
                                   [&](const PooledPipeline &q) { return q.device == device; });
            if (it == pool.end()) return false;
            p = *it;
            pool.erase(it);
        }
        stream = p.streams[0];
        stream2 = p.streams[1];
        copy_stream = p.streams[2];
        count_stream = p.streams[3];
        fork_event = p.events[0];
        join_event = p.events[1];
        origin = p.events[2];
        for (int i = 0; i < 2; ++i) {
            Buffer &b = buf[i];
            const PooledPipeline::Buf &q = p.buf[i];
            b.a = q.a;
            b.d = q.d;
            b.pa = q.pa;
            b.pd = q.pd;
            b.cap = q.cap;
            b.count = q.count;
            b.begin = q.begin;
            b.end = q.end;
            b.copied = q.copied;
        }
        h_count = p.h_count;
        h_a = p.h_a;
        h_d = p.h_d;
        host_capacity = p.host_capacity;
        return true;
    }

    // Hand the pipeline to the pool if every stream finished without error
    // and the pool has room; release() then frees only what was not handed on.
    void offer_pipeline() {
        if (device < 0 || !stream || !stream2 || !copy_stream || !count_stream || !fork_event ||
            !join_event || !origin || !h_count)
            return;
        for (cudaStream_t s : {stream, stream2, copy_stream, count_stream})
            if (cudaStreamSynchronize(s) != cudaSuccess) return;
        for (const auto &b : buf)
            if (!b.count || !b.begin || !b.end || !b.copied) return;
        {
            std::lock_guard<std::mutex> lock(pipeline_pool_mutex());
            if (pipeline_pool().size() >= kPooledPipelines) return;
        }
        for (auto &b : buf)
            if (b.cap > kPooledSurvivors) {
                cudaFree(b.a);
                cudaFree(b.d);
                cudaFree(b.pa);
                cudaFree(b.pd);
                b.a = b.pa = nullptr;
                b.d = b.pd = nullptr;
                b.cap = 0;
            }
        if (host_capacity > kPooledSurvivors) {
            cudaFreeHost(h_a);
            cudaFreeHost(h_d);
            h_a = nullptr;
            h_d = nullptr;
            host_capacity = 0;
        }
        PooledPipeline p;
        p.device = device;
        p.streams[0] = stream;
        p.streams[1] = stream2;
        p.streams[2] = copy_stream;
        p.streams[3] = count_stream;
        p.events[0] = fork_event;
        p.events[1] = join_event;
        p.events[2] = origin;
        for (int i = 0; i < 2; ++i) {
            const Buffer &b = buf[i];
            PooledPipeline::Buf &q = p.buf[i];
            q.a = b.a;
            q.d = b.d;
            q.pa = b.pa;
            q.pd = b.pd;
            q.cap = b.cap;
            q.count = b.count;
            q.begin = b.begin;
            q.end = b.end;
            q.copied = b.copied;
        }
        p.h_count = h_count;
        p.h_a = h_a;
        p.h_d = h_d;
        p.host_capacity = host_capacity;
        {
            std::lock_guard<std::mutex> lock(pipeline_pool_mutex());
            if (pipeline_pool().size() >= kPooledPipelines) return;
            pipeline_pool().push_back(p);
        }
        stream = stream2 = copy_stream = count_stream = nullptr;
        fork_event = join_event = origin = nullptr;
        for (auto &b : buf) b = Buffer{};
        h_count = nullptr;
        h_a = nullptr;
        h_d = nullptr;
        host_capacity = 0;
    }

    void release() {
        offer_pipeline();
        for (auto &b : buf) {
            cudaFree(b.a);
            cudaFree(b.d);
            cudaFree(b.pa);
            cudaFree(b.pd);
            cudaFree(b.count);
            if (b.begin) cudaEventDestroy(b.begin);
            if (b.end) cudaEventDestroy(b.end);
            if (b.copied) cudaEventDestroy(b.copied);
            b = Buffer{};
        }
        cudaFree(rows);
        rows = nullptr;
        cudaFree(fast_rows);
        fast_rows = nullptr;
        cudaFree(fast_adm);
        fast_adm = nullptr;
        cudaFree(fast_starts);
        fast_starts = nullptr;
        cudaFree(list_runs);
        cudaFree(list_count);
        list_runs = nullptr;
        list_count = nullptr;
        if (h_count) cudaFreeHost(h_count);
        if (h_a) cudaFreeHost(h_a);
        if (h_d) cudaFreeHost(h_d);
        h_count = nullptr;
        h_a = nullptr;
        h_d = nullptr;
        if (stream) cudaStreamDestroy(stream);
        if (copy_stream) cudaStreamDestroy(copy_stream);
        if (count_stream) cudaStreamDestroy(count_stream);
        if (stream2) cudaStreamDestroy(stream2);
        if (fork_event) cudaEventDestroy(fork_event);
        if (join_event) cudaEventDestroy(join_event);
        if (origin) cudaEventDestroy(origin);
        origin = nullptr;
        stream = stream2 = copy_stream = count_stream = nullptr;
        fork_event = join_event = nullptr;
    }

    void build_tables(const std::vector<std::string> &coefficients) {
        auto t0 = Clock::now();
        const auto &primes = candidate_primes();
        long long total = 0;
        for (int i = 0; i < kCandidatePrimes; ++i) {
            const int p = primes[i];
            T.prime[i] = p;
            T.length[i] = (p + dev::kExt + 1) & ~1;
            T.offset[i] = total;
            T.magic[i] = dev::magic40(dev::u32(p));
            total += (long long)p * T.length[i];
        }
        std::vector<unsigned char> affine(std::size_t(kCandidatePrimes) * kMaximumPrime, 0);
        std::vector<unsigned short> inverse(std::size_t(kCandidatePrimes) * kMaximumPrime, 0);
        std::vector<int> neg_h(kCandidatePrimes);
        for (int i = 0; i < kCandidatePrimes; ++i) {
            const int p = primes[i];
            auto aff = affine_mask(p, coefficients);
            std::copy(aff.begin(), aff.end(), affine.begin() + std::size_t(i) * kMaximumPrime);
            modular_inverses(p, inverse.data() + std::size_t(i) * kMaximumPrime);
            neg_h[i] = int((p - bound % p) % p);
        }
        timings.plan_ms += ms_since(t0);
        auto t1 = Clock::now();
        rows = device_alloc<dev::u64>(std::size_t(total), "cudaMalloc(sieve tables)");
        unsigned char *d_aff = device_alloc<unsigned char>(affine.size(), "cudaMalloc(affine)");
        unsigned short *d_inv = device_alloc<unsigned short>(inverse.size(), "cudaMalloc(inverse)");
        int *d_neg = device_alloc<int>(neg_h.size(), "cudaMalloc(bound residues)");
        timings.workspace_ms += ms_since(t1);
        T.rows = rows;
        cudaEvent_t e0, e1;
        check_cuda(cudaEventCreate(&e0), "cudaEventCreate");
        check_cuda(cudaEventCreate(&e1), "cudaEventCreate");
        check_cuda(cudaEventRecord(e0, stream), "cudaEventRecord");
        check_cuda(cudaMemcpyAsync(d_aff, affine.data(), affine.size(), cudaMemcpyHostToDevice, stream),
                   "upload affine tables");
        check_cuda(cudaMemcpyAsync(d_inv, inverse.data(), inverse.size() * sizeof(unsigned short),
                                   cudaMemcpyHostToDevice, stream),
                   "upload inverses");
        check_cuda(cudaMemcpyAsync(d_neg, neg_h.data(), neg_h.size() * sizeof(int),
                                   cudaMemcpyHostToDevice, stream),
                   "upload bound residues");
        const int threads = 256;
        const long long blocks = (total + threads - 1) / threads;
        timings.h2d_bytes += affine.size() + inverse.size() * sizeof(unsigned short) +
                             neg_h.size() * sizeof(int);
        dev::ref_table_kernel<<<unsigned(blocks), threads, 0, stream>>>(rows, T, d_aff, d_inv, d_neg,
                                                                         total);
        check_cuda(cudaGetLastError(), "ref_table_kernel launch");
        check_cuda(cudaEventRecord(e1, stream), "cudaEventRecord");
        check_cuda(cudaEventSynchronize(e1), "table build");
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        timings.table_ms += ms;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaFree(d_aff);
        cudaFree(d_inv);
        cudaFree(d_neg);
        timings.table_wall_ms += ms_since(t0);
    }

    void init(const std::vector<std::string> &coefficients) {
        auto t0 = Clock::now();
        // The fast plan needs only the coefficients and the bound: choose it
        // on a host thread while the streams and buffers are created.
        PlannedRows planned;
        if (opt.plan == PlanKind::fast)
            planned = std::async(std::launch::async, [&coefficients, h = bound, forced = opt.fast_shape] {
                int max_classes = 0;
                FastShape shape = forced;
                if (shape.rows <= 0) shape = tuned_fast_shape(coefficients, h);
                FastPlan p = single_curve_plan(coefficients, h, &max_classes, shape);
                return std::make_pair(std::move(p), max_classes);
            });
        if (opt.device >= 0) check_cuda(cudaSetDevice(opt.device), "cudaSetDevice");
        check_cuda(cudaGetDevice(&device), "cudaGetDevice");
        if (!adopt_pipeline()) {
            check_cuda(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
            check_cuda(cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking), "cudaStreamCreate");
            check_cuda(cudaStreamCreateWithFlags(&count_stream, cudaStreamNonBlocking), "cudaStreamCreate");
            check_cuda(cudaStreamCreateWithFlags(&stream2, cudaStreamNonBlocking), "cudaStreamCreate");
            check_cuda(cudaEventCreateWithFlags(&fork_event, cudaEventDisableTiming), "cudaEventCreate");
            check_cuda(cudaEventCreateWithFlags(&join_event, cudaEventDisableTiming), "cudaEventCreate");
            check_cuda(cudaEventCreate(&origin), "cudaEventCreate");
        }
        check_cuda(cudaFuncSetAttribute(dev::ref_sieve_kernel,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        int(dev::kRefSmem)),
                   "cudaFuncSetAttribute");
        int sms = 0, per_sm = 0;
        check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device),
                   "cudaDeviceGetAttribute");
        check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dev::ref_sieve_kernel,
                                                                 dev::kThreads, dev::kRefSmem),
                   "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
        grid = std::max(1, sms * std::max(1, per_sm));
        // Survivor buffers start small (most searches have few survivors) and
        // grow on overflow up to the per-buffer capacity; past it a batch is
        // split.  RPG_SURVIVOR_CAPACITY fixes both at its value (at least 64,
        // one word's worth); tests use it to drive the split path.
        capacity = opt.capacity;
        long long initial = std::min<long long>(capacity, kInitialSurvivors);
        if (const char *env = std::getenv("RPG_SURVIVOR_CAPACITY")) initial = capacity = std::atoll(env);
        capacity = std::max<long long>(capacity, 64);
        initial = std::max<long long>(initial, 64);
        // A pooled buffer is kept if its capacity lies in [initial, capacity];
        // pa and pd, when present, always have the capacity of a and d.
        for (auto &b : buf) {
            if (b.cap < initial || b.cap > capacity || !b.a || !b.d) {
                cudaFree(b.a);
                cudaFree(b.d);
                cudaFree(b.pa);
                cudaFree(b.pd);
                b.a = b.pa = nullptr;
                b.d = b.pd = nullptr;
                b.cap = 0;
                b.a = device_alloc<long long>(std::size_t(initial), "cudaMalloc(survivors)");
                b.d = device_alloc<int>(std::size_t(initial), "cudaMalloc(survivors)");
                b.cap = initial;
            }
            if (opt.preverify && (!b.pa || !b.pd)) {
                cudaFree(b.pa);
                cudaFree(b.pd);
                b.pa = nullptr;
                b.pd = nullptr;
                b.pa = device_alloc<long long>(std::size_t(b.cap), "cudaMalloc(survivors)");
                b.pd = device_alloc<int>(std::size_t(b.cap), "cudaMalloc(survivors)");
            }
            if (!b.count) b.count = device_alloc<unsigned long long>(4, "cudaMalloc(count)");
            if (!b.begin) check_cuda(cudaEventCreate(&b.begin), "cudaEventCreate");
            if (!b.end) check_cuda(cudaEventCreate(&b.end), "cudaEventCreate");
            if (!b.copied)
                check_cuda(cudaEventCreateWithFlags(&b.copied, cudaEventDisableTiming), "cudaEventCreate");
            b.busy = false;
        }
        if (!h_count) check_cuda(cudaMallocHost(&h_count, 8 * sizeof(unsigned long long)), "cudaMallocHost");
        if (!h_a || !h_d || host_capacity < initial) {
            if (h_a) cudaFreeHost(h_a);
            if (h_d) cudaFreeHost(h_d);
            h_a = nullptr;
            h_d = nullptr;
            host_capacity = 0;
            check_cuda(cudaMallocHost(&h_a, std::size_t(initial) * sizeof(long long)), "cudaMallocHost");
            check_cuda(cudaMallocHost(&h_d, std::size_t(initial) * sizeof(int)), "cudaMallocHost");
            host_capacity = initial;
        }
        timings.workspace_ms += ms_since(t0);
        if (opt.plan == PlanKind::fast) build_fast_tables(coefficients, planned);
        else build_tables(coefficients);
        if (opt.preverify) {
            preverifier.prepare({&coefficients}, stream);
            timings.h2d_bytes += preverifier.upload_bytes();
        }
    }

    // Fast plan: the per-curve plan (class prime, stage-1 moduli), class-layout
    // tables for the stage-1 moduli and the 36 reference candidates, and the
    // admissible-class tables (2-adic by d mod 64, residues mod q by d mod q).
    using PlannedRows = std::future<std::pair<FastPlan, int>>;

    void build_fast_tables(const std::vector<std::string> &coefficients, PlannedRows &planned) {
        auto t0 = Clock::now();
        // the plan was started on a host thread while the buffers were set up
        std::tie(fast_plan, fast_max_classes) = planned.get();
        const int n = int(coefficients.size()) - 1;
        const int q = fast_plan.class_prime;
        const long long M = 64LL * q;
        const long long S = 64LL * M;
        std::vector<int> primes_used;
        for (const auto &f : fast_plan.slots)
            for (int p : f) primes_used.push_back(p);
        if (q > 1) primes_used.push_back(q);
        for (int p : candidate_primes()) primes_used.push_back(p);
        std::vector<unsigned char> affine;
        std::vector<unsigned short> inverse;
        std::vector<int> base(kMaximumPrime, -1), lead(kMaximumPrime, 1);
        for (int p : primes_used) {
            if (base[p] >= 0) continue;
            base[p] = int(affine.size());
            auto aff = affine_mask(p, coefficients);
            affine.insert(affine.end(), aff.begin(), aff.end());
            const std::size_t at = inverse.size();
            inverse.resize(at + std::size_t(p), 0);
            modular_inverses(p, inverse.data() + at);
            if (n % 2 == 0) {
                lead[p] = square_mod(decimal_mod(coefficients.back(), p), p) ? 1 : 0;
            }
        }
        std::vector<dev::TableSpec> specs;
        long long total = 0;
        int smem_words = 0;
        // pattern rows per (prime, rho = 0 rule): step = M mod q, window start
        // of residue x0 = x0 step^-1 mod q
        std::vector<dev::ClassPatternSpec> pspecs;
        long long pattern_total = 0;
        auto pattern_of = [&](int p, int lead_ok, dev::TableSpec &Sp, int f) {
            int found = -1;
            for (std::size_t i = 0; i < pspecs.size(); ++i)
                if (pspecs[i].q == p && pspecs[i].lead_ok == lead_ok) found = int(i);
            if (found < 0) {
                dev::ClassPatternSpec P{};
                P.out = pattern_total;
                P.q = p;
                P.words = (p + 64 + 63) / 64 + 1;
                P.factor_base = base[p];
                P.lead_ok = lead_ok;
                P.step = int(M % p);
                pattern_total += (long long)p * P.words;
                pspecs.push_back(P);
                found = int(pspecs.size()) - 1;
            }
            Sp.pattern[f] = pspecs[std::size_t(found)].out;
            Sp.pattern_words[f] = pspecs[std::size_t(found)].words;
            Sp.s_mod[f] = int(S % p);
            Sp.step_inv[f] = int(mod_inverse(M % p, p));
        };
        F = dev::FastTables{};
        F.slots = int(fast_plan.moduli.size());
        for (int sl = 0; sl < F.slots; ++sl) {
            dev::TableSpec Sp{};
            Sp.nf = int(fast_plan.slots[sl].size());
            Sp.m = fast_plan.moduli[sl];
            for (int i = 0; i < Sp.nf; ++i) {
                Sp.q[i] = fast_plan.slots[sl][i];
                pattern_of(Sp.q[i], lead[Sp.q[i]], Sp, i);
            }
            Sp.length = (Sp.m + dev::kFExt + 1) & ~1;
            Sp.offset = total;
            total += (long long)Sp.m * Sp.length;
            specs.push_back(Sp);
            dev::FastModulus &Md = F.mod[sl];
            Md.m = Sp.m;
            Md.nf = Sp.nf;
            for (int i = 0; i < Sp.nf; ++i) Md.q[i] = Sp.q[i];
            Md.length = Sp.length;
            Md.offset = Sp.offset;
            Md.smem_offset = smem_words;
            smem_words += Sp.length;
            Md.inv_stride = dev::u32(mod_inverse(S % Sp.m, Sp.m));
            Md.neg_h = dev::u32((Sp.m - bound % Sp.m) % Sp.m);
            Md.wlo_mod = 0;
            Md.step = dev::u32((dev::kWarpSize * dev::kFK) % Sp.m);
            Md.step8 = 8u * Md.step;
            Md.mod8 = 8u * dev::u32(Sp.m);
            Md.soff8 = 8u * dev::u32(Md.smem_offset);
            Md.magic = (unsigned long long)((~0ull) / (unsigned long long)Sp.m) + 1;
            F.min_modulus = sl == 0 ? Sp.m : std::min(F.min_modulus, Sp.m);
        }
        F.smem_words = smem_words;
        const auto &cands = candidate_primes();
        for (int i = 0; i < kCandidatePrimes; ++i) {
            const int p = cands[i];
            dev::TableSpec Sp{};
            Sp.nf = 1;
            Sp.m = p;
            Sp.q[0] = p;
            pattern_of(p, 0, Sp, 0);  // rows with p | d go unused: stage 2 skips such p
            Sp.length = p;
            Sp.offset = total;
            total += (long long)p * p;
            specs.push_back(Sp);
            dev::FastPrime &P = F.prime[i];
            P.offset = Sp.offset;
            P.p = p;
            P.inv_stride = dev::u32(mod_inverse(S % p, p));
            P.neg_h = dev::u32((p - bound % p) % p);
            P.magic = dev::magic40(dev::u32(p));
            P.wlo_mod = 0;
        }
        F.class_prime = q;
        F.class_mod = int(M);
        F.h_mod_m = int(bound % M);
        F.inv64_q = q > 1 ? int(mod_inverse(64 % q, q)) : 0;
        F.stride = S;
        F.count_q = (2 * bound) / M;
        F.count_r = int((2 * bound) % M);
        for (int r64 = 0; r64 < 64; ++r64) F.mod_q[r64] = (unsigned char)(q > 1 ? r64 % q : 0);
        if (q > 1)
            for (int a = 0; a < q; ++a)
                for (int rq = 0; rq < q; ++rq)
                    F.crt[a * 13 + rq] = (unsigned char)(((rq - a + q) % q) * F.inv64_q % q);
        // Admissible classes: 2-adic by d mod 64 (F(r, d) square mod 64, r odd
        // when d is even), then residues r mod q by d mod q.
        std::vector<int> c64(coefficients.size());
        for (std::size_t i = 0; i < coefficients.size(); ++i) c64[i] = decimal_mod(coefficients[i], 64);
        bool square64[64] = {};
        for (int v = 0; v < 64; ++v) square64[(v * v) & 63] = true;
        std::vector<dev::u64> adm(64 + dev::kFAdmQ, 0);
        for (int dd = 0; dd < 64; ++dd) {
            for (int r = 0; r < 64; ++r) {
                if (dd % 2 == 0 && r % 2 == 0) continue;
                int value = c64[n], power = 1;
                for (int i = n - 1; i >= 0; --i) {
                    value = (value * r) & 63;
                    power = (power * dd) & 63;
                    value = (value + c64[i] * power) & 63;
                }
                if (n % 2 == 1) value = (value * dd) & 63;
                if (square64[value]) adm[dd] |= dev::u64(1) << r;
            }
        }
        if (q > 1) {
            const auto aff = affine_mask(q, coefficients);
            for (int dq = 0; dq < q; ++dq) {
                for (int r = 0; r < q; ++r) {
                    bool ok;
                    if (dq == 0) ok = r != 0 && lead[q];
                    else ok = aff[(r * mod_inverse(dq, q)) % q] != 0;
                    if (ok) adm[64 + dq] |= dev::u64(1) << r;
                }
            }
        }
        // Denominator primes: p < 512 (p != q, which the class residues
        // already cover) with c_n not a square mod p, for even degree.  A
        // denominator divisible by one holds no points: p !| a (gcd) gives
        // F(a, d) = c_n a^n (mod p), a non-square.  The producer skips such
        // denominators (pairs p, ceil(2^64 / p) after the class residues).
        fast_bad_primes.clear();
        if (n % 2 == 0) {
            for (int p = 3; p < kMaximumPrime; p += 2) {
                bool prime = true;
                for (int f = 3; f * f <= p && prime; f += 2) prime = p % f != 0;
                if (!prime || p == q) continue;
                const int lc = decimal_mod(coefficients.back(), p);
                if (lc == 0 || square_mod(lc, p)) continue;
                fast_bad_primes.push_back(p);
                adm.push_back(dev::u64(p));
                adm.push_back((~0ull) / dev::u64(p) + 1);
            }
        }
        F.nbad = int(fast_bad_primes.size());
        fast_adm_host = adm;
        // class starts for every residue r mod M: ofs = (r + H) mod M and, per
        // modulus, the row index ((-H + ofs) S^-1) mod m of class word 0
        std::vector<dev::FastClassStart> starts(static_cast<std::size_t>(M));
        for (long long r = 0; r < M; ++r) {
            dev::FastClassStart &cs = starts[std::size_t(r)];
            const long long ofs = (r + bound % M) % M;
            cs.ofs = (unsigned short)ofs;
            for (int sl = 0; sl < F.slots; ++sl) {
                const dev::FastModulus &Md = F.mod[sl];
                cs.start[sl] = (unsigned short)((Md.neg_h + ofs) % Md.m * Md.inv_stride % Md.m);
            }
        }
        // class lists by denominator class k = (d mod 64) q + (d mod q), in the
        // order the producer would lay them out, for launches over whole rows
        const int maxc = fast_max_classes;
        const int ncombo = 64 * q;
        list_words = (F.count_q + 1 + 63) >> 6;
        std::vector<dev::FastRun> lruns;
        std::vector<int> lcount;
        int list_ipc = 1;
        if (list_words < (1LL << 23)) {
            lruns.assign(std::size_t(ncombo) * maxc, dev::FastRun{});
            lcount.assign(std::size_t(ncombo), 0);
            // every class of a whole row has the same number of sweep items:
            // that of the longest class (classes differ by one word at most)
            list_ipc = int((list_words + dev::kFItemWords - 1) / dev::kFItemWords);
            auto nth_bit = [](dev::u64 mask, int k) {
                for (int i = 0; i < k; ++i) mask &= mask - 1;
                return __builtin_ctzll(mask);
            };
            for (int dd = 0; dd < 64; ++dd)
                for (int dq = 0; dq < q; ++dq) {
                    const int k = dd * q + dq;
                    const dev::u64 classes2 = adm[std::size_t(dd)];
                    const dev::u64 classesq = q > 1 ? adm[std::size_t(64 + dq)] : dev::u64(1);
                    const int nq = __builtin_popcountll(classesq);
                    const int nclass = __builtin_popcountll(classes2) * nq;
                    if (nclass > maxc) throw std::logic_error("class list longer than the class bound");
                    for (int c = 0; c < nclass; ++c) {
                        const int i2 = c / nq;
                        const int r64 = nth_bit(classes2, i2);
                        int r = r64;
                        if (q > 1) r = r64 + 64 * int(F.crt[F.mod_q[r64] * 13 + nth_bit(classesq, c - i2 * nq)]);
                        const dev::FastClassStart &cs = starts[std::size_t(r)];
                        const long long count = F.count_q + (cs.ofs <= F.count_r ? 1 : 0);
                        const long long cw = (count + 63) >> 6;
                        const dev::u32 last_bits = cw > 0 ? dev::u32(count - 64 * (cw - 1)) : 64u;
                        dev::FastRun &run = lruns[std::size_t(k) * maxc + c];
                        run.words_last = dev::u32(cw) | (cw > 0 ? 1u << 24 : 0u) | ((last_bits - 1) << 25);
                        run.ofs = cs.ofs;
                        for (int sl = 0; sl < dev::kFastSlots; ++sl) run.start[sl] = cs.start[sl];
                        if (cw > list_words) throw std::logic_error("class longer than its row");
                    }
                    lcount[std::size_t(k)] = nclass;
                }
        }
        timings.plan_ms += ms_since(t0);
        auto t1 = Clock::now();
        if (!lruns.empty()) {
            list_runs = device_alloc<dev::FastRun>(lruns.size(), "cudaMalloc(class lists)");
            list_count = device_alloc<int>(lcount.size(), "cudaMalloc(class lists)");
            check_cuda(cudaMemcpyAsync(list_runs, lruns.data(), lruns.size() * sizeof(dev::FastRun),
                                       cudaMemcpyHostToDevice, stream),
                       "upload class lists");
            check_cuda(cudaMemcpyAsync(list_count, lcount.data(), lcount.size() * sizeof(int),
                                       cudaMemcpyHostToDevice, stream),
                       "upload class lists");
            timings.h2d_bytes += lruns.size() * sizeof(dev::FastRun) + lcount.size() * sizeof(int);
        }
        fast_rows = device_alloc<dev::u64>(std::size_t(total), "cudaMalloc(class tables)");
        fast_adm = device_alloc<dev::u64>(adm.size(), "cudaMalloc(admissible classes)");
        fast_starts = device_alloc<dev::FastClassStart>(starts.size(), "cudaMalloc(class starts)");
        unsigned char *d_aff = device_alloc<unsigned char>(affine.size(), "cudaMalloc(affine)");
        unsigned short *d_inv = device_alloc<unsigned short>(inverse.size(), "cudaMalloc(inverse)");
        dev::TableSpec *d_specs = device_alloc<dev::TableSpec>(specs.size(), "cudaMalloc(specs)");
        dev::ClassPatternSpec *d_pspecs = device_alloc<dev::ClassPatternSpec>(pspecs.size(), "cudaMalloc(specs)");
        dev::u64 *d_patterns = device_alloc<dev::u64>(std::size_t(pattern_total), "cudaMalloc(patterns)");
        timings.workspace_ms += ms_since(t1);
        cudaEvent_t e0, e1;
        check_cuda(cudaEventCreate(&e0), "cudaEventCreate");
        check_cuda(cudaEventCreate(&e1), "cudaEventCreate");
        check_cuda(cudaEventRecord(e0, stream), "cudaEventRecord");
        check_cuda(cudaMemcpyAsync(d_aff, affine.data(), affine.size(), cudaMemcpyHostToDevice, stream),
                   "upload affine tables");
        check_cuda(cudaMemcpyAsync(d_inv, inverse.data(), inverse.size() * sizeof(unsigned short),
                                   cudaMemcpyHostToDevice, stream),
                   "upload inverses");
        check_cuda(cudaMemcpyAsync(d_specs, specs.data(), specs.size() * sizeof(dev::TableSpec),
                                   cudaMemcpyHostToDevice, stream),
                   "upload table specs");
        check_cuda(cudaMemcpyAsync(d_pspecs, pspecs.data(), pspecs.size() * sizeof(dev::ClassPatternSpec),
                                   cudaMemcpyHostToDevice, stream),
                   "upload pattern specs");
        check_cuda(cudaMemcpyAsync(fast_adm, adm.data(), adm.size() * sizeof(dev::u64),
                                   cudaMemcpyHostToDevice, stream),
                   "upload admissible classes");
        check_cuda(cudaMemcpyAsync(fast_starts, starts.data(), starts.size() * sizeof(dev::FastClassStart),
                                   cudaMemcpyHostToDevice, stream),
                   "upload class starts");
        timings.h2d_bytes += affine.size() + inverse.size() * sizeof(unsigned short) +
                             specs.size() * sizeof(dev::TableSpec) + pspecs.size() * sizeof(dev::ClassPatternSpec) +
                             adm.size() * sizeof(dev::u64) + starts.size() * sizeof(dev::FastClassStart);
        const int threads = 256;
        dev::pattern_rows_kernel<<<unsigned((pattern_total + threads - 1) / threads), threads, 0, stream>>>(
            d_patterns, d_pspecs, int(pspecs.size()), d_aff, d_inv, pattern_total);
        check_cuda(cudaGetLastError(), "pattern_rows_kernel launch");
        const long long blocks = (total + threads - 1) / threads;
        dev::class_table_kernel<<<unsigned(blocks), threads, 0, stream>>>(fast_rows, d_specs, int(specs.size()),
                                                                          d_patterns, total);
        check_cuda(cudaGetLastError(), "class_table_kernel launch");
        check_cuda(cudaEventRecord(e1, stream), "cudaEventRecord");
        check_cuda(cudaEventSynchronize(e1), "class table build");
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        timings.table_ms += ms;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaFree(d_aff);
        cudaFree(d_inv);
        cudaFree(d_specs);
        cudaFree(d_pspecs);
        cudaFree(d_patterns);
        F.rows = fast_rows;
        F.prime_rows = fast_rows;
        F.admissible = fast_adm;
        F.class_starts = fast_starts;
        F.max_classes = fast_max_classes;
        F.list_runs = list_runs;
        F.list_count = list_count;
        F.list_ipc = list_ipc;
        fast_smem = fast_dynamic_smem(F.smem_words, fast_max_classes, fast_plan.row_slots);
        const void *kernel = fast_kernel_ptr(F.slots, fast_plan.row_slots);
        check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        int(fast_smem)),
                   "cudaFuncSetAttribute");
        int sms = 0, per_sm = 0;
        check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device),
                   "cudaDeviceGetAttribute");
        check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, dev::kFThreads,
                                                                 fast_smem),
                   "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
        grid = std::max(1, sms * std::max(1, per_sm));
        // Word dimension of a launch: class words (64 sites spaced M apart).
        const long long sites = 2 * bound + 1;
        words = (sites / M + 1 + 63) / 64;
        max_tile = dev::kFMaxClassWords;
        timings.table_wall_ms += ms_since(t0);
    }

    static const void *fast_kernel_ptr(int rows, int slots) {
        switch (rows * 4 + slots) {
#define RPG_FAST_PTR(n)                                                                       \
    case n * 4 + 2: return reinterpret_cast<const void *>(&dev::fast_sieve_kernel<n, 2>);   \
    case n * 4 + 3: return reinterpret_cast<const void *>(&dev::fast_sieve_kernel<n, 3>);
        RPG_FAST_PTR(1) RPG_FAST_PTR(2) RPG_FAST_PTR(3) RPG_FAST_PTR(4) RPG_FAST_PTR(5) RPG_FAST_PTR(6)
        RPG_FAST_PTR(7) RPG_FAST_PTR(8) RPG_FAST_PTR(9) RPG_FAST_PTR(10) RPG_FAST_PTR(11) RPG_FAST_PTR(12)
#undef RPG_FAST_PTR
        default: throw std::logic_error("no fast kernel for this row and slot count");
        }
    }

    void launch_fast(const dev::FastTables &Fl, const dev::SieveArgs &A, unsigned long long *work,
                     cudaStream_t st) const {
        const int blocks = int(std::min<long long>(grid, (A.k_count + dev::kFChunk - 1) / dev::kFChunk));
        const void *kernel = fast_kernel_ptr(Fl.slots, fast_plan.row_slots);
        void *params[] = {const_cast<dev::FastTables *>(&Fl), const_cast<dev::SieveArgs *>(&A), &work};
        check_cuda(cudaLaunchKernel(kernel, dim3(unsigned(blocks)), dim3(dev::kFThreads), params, fast_smem, st),
                   "fast sieve kernel launch");
    }

    dev::SieveArgs args(int which, long long first, long long last, long long w_lo, long long w_hi) {
        dev::SieveArgs A{};
        A.bound = bound;
        A.words = words;
        A.w_lo = w_lo;
        A.w_hi = w_hi;
        A.k_first = first;
        A.k_count = int(last - first + 1);
        A.square = opt.square ? 1 : 0;
        A.out_a = buf[which].a;
        A.out_d = buf[which].d;
        A.out_count = buf[which].count;
        A.capacity = (unsigned long long)buf[which].cap;
        A.error = buf[which].count + 2;
        return A;
    }

    cudaStream_t launch_stream(int which) const { return which ? stream2 : stream; }

    // Counting pass: survivors accumulate in buffer 0's counter across
    // launches; launch i runs on launch stream i mod 2 with that buffer's
    // work counter.
    void launch_counting(int which, long long first, long long last, long long w_lo, long long w_hi) {
        const dev::SieveArgs A = args(0, first, last, w_lo, w_hi);
        const cudaStream_t st = launch_stream(which);
        check_cuda(cudaMemsetAsync(buf[which].count + 1, 0, sizeof(unsigned long long), st),
                   "cudaMemsetAsync");
        launch_kernel(A, buf[which].count + 1, st);
        ++timings.launches;
    }

    void launch_kernel(const dev::SieveArgs &A, unsigned long long *work, cudaStream_t st) {
        if (opt.plan == PlanKind::fast) {
            dev::FastTables Fl = F;
            for (int i = 0; i < kCandidatePrimes; ++i)
                Fl.prime[i].wlo_mod = dev::u32(A.w_lo % Fl.prime[i].p);
            for (int i = 0; i < Fl.slots; ++i) Fl.mod[i].wlo_mod = dev::u32(A.w_lo % Fl.mod[i].m);
            if (A.w_lo != 0 || A.w_hi < list_words) {  // part of the class rows: the producer lays them out
                Fl.list_runs = nullptr;
                Fl.list_count = nullptr;
            }
            launch_fast(Fl, A, work, st);
        } else {
            const int blocks = int(std::min<long long>(grid, A.k_count));
            dev::ref_sieve_kernel<<<blocks, dev::kThreads, dev::kRefSmem, st>>>(T, A);
        }
        check_cuda(cudaGetLastError(), "sieve kernel launch");
    }

    void launch(int which, long long first, long long last, long long w_lo, long long w_hi) {
        Buffer &b = buf[which];
        b.first = first;
        b.last = last;
        b.busy = true;
        const dev::SieveArgs A = args(which, first, last, w_lo, w_hi);
        const cudaStream_t st = launch_stream(which);
        check_cuda(cudaMemsetAsync(b.count, 0, 4 * sizeof(unsigned long long), st), "cudaMemsetAsync");
        check_cuda(cudaEventRecord(b.begin, st), "cudaEventRecord");
        launch_kernel(A, b.count + 1, st);
        if (opt.preverify) {
            preverifier.launch(b.a, b.d, nullptr, b.count, (unsigned long long)b.cap, b.pa, b.pd, nullptr,
                               b.count + 3, nullptr, st);
            ++timings.launches;
        }
        check_cuda(cudaEventRecord(b.end, st), "cudaEventRecord");
        // The buffer is launched into again only after the host has waited
        // for b.copied, so this copy ends before the memset of its next launch.
        check_cuda(cudaStreamWaitEvent(count_stream, b.end, 0), "cudaStreamWaitEvent");
        check_cuda(cudaMemcpyAsync(h_count + 4 * which, b.count, 4 * sizeof(unsigned long long),
                                   cudaMemcpyDeviceToHost, count_stream),
                   "download survivor count");
        check_cuda(cudaEventRecord(b.copied, count_stream), "cudaEventRecord");
        timings.d2h_bytes += 4 * sizeof(unsigned long long);
        ++timings.launches;
    }

    // Launch queued batches into free buffers (pipelined path, rows that fit
    // one launch).  Rows longer than kMaxTileWords go through pieces instead.
    void refill() {
        if (words > max_tile || !pieces.empty()) return;
        while (order.size() < 2 && q_next <= q_last) {
            const int which = buf[0].busy ? 1 : 0;
            if (buf[which].busy) break;
            const long long first = q_next;
            const long long last = std::min(q_last, first + q_batch - 1);
            q_next = last + 1;
            launch(which, first, last, 0, words);
            order.push_back(which);
        }
    }

    // Raise if a launch into buffer `which` reported a timed-out device wait.
    void check_error_word(int which) {
        unsigned long long err = 0;
        check_cuda(cudaMemcpy(&err, buf[which].count + 2, sizeof err, cudaMemcpyDeviceToHost),
                   "download error word");
        if (err) throw DeviceTimeout("sieve kernel: bounded wait for a row copy timed out");
    }

    // Device time a completed batch adds (see origin).
    float elapsed(const Buffer &b) {
        float t0 = 0, t1 = 0;
        cudaEventElapsedTime(&t0, origin, b.begin);
        cudaEventElapsedTime(&t1, origin, b.end);
        const float ms = std::max(0.0f, t1 - std::max(t0, last_end_ms));
        last_end_ms = std::max(last_end_ms, t1);
        return ms;
    }

    void copy_out(int which, std::size_t n) {
        Buffer &b = buf[which];
        if (!n) return;
        check_cuda(cudaStreamWaitEvent(copy_stream, b.end, 0), "cudaStreamWaitEvent");
        check_cuda(cudaMemcpyAsync(h_a, opt.preverify ? b.pa : b.a, n * sizeof(long long),
                                   cudaMemcpyDeviceToHost, copy_stream),
                   "download survivors");
        check_cuda(cudaMemcpyAsync(h_d, opt.preverify ? b.pd : b.d, n * sizeof(int), cudaMemcpyDeviceToHost,
                                   copy_stream),
                   "download survivors");
        check_cuda(cudaStreamSynchronize(copy_stream), "download survivors");
        timings.d2h_bytes += n * (sizeof(long long) + sizeof(int));
    }

    // n modular survivors, of which kept (all, without pre-verification) are copied.
    void deliver(BatchView &out, int which, std::size_t n, std::size_t kept, float ms, long long first,
                 long long last, bool complete) {
        if (!opt.preverify) kept = n;
        copy_out(which, kept);
        out.first = first;
        out.last = last;
        out.a = h_a;
        out.d = h_d;
        out.count = kept;
        out.modular = n;
        out.kernel_ms = ms;
        out.complete = complete;
    }

    // Grow buffer `which` (idle) to hold n survivors if the capacity allows;
    // false if it is already as large as it may get.
    bool grow(int which, unsigned long long n) {
        Buffer &b = buf[which];
        if (b.cap >= capacity) return false;
        const long long cap = std::min<long long>(capacity, (long long)(n + n / 4 + 1024));
        const auto t0 = Clock::now();
        check_cuda(cudaStreamSynchronize(stream), "sieve stream");
        check_cuda(cudaStreamSynchronize(stream2), "sieve stream");
        cudaFree(b.a);
        cudaFree(b.d);
        cudaFree(b.pa);
        cudaFree(b.pd);
        b.a = b.pa = nullptr;
        b.d = b.pd = nullptr;
        b.cap = 0;
        b.a = device_alloc<long long>(std::size_t(cap), "cudaMalloc(survivors)");
        b.d = device_alloc<int>(std::size_t(cap), "cudaMalloc(survivors)");
        if (opt.preverify) {
            b.pa = device_alloc<long long>(std::size_t(cap), "cudaMalloc(survivors)");
            b.pd = device_alloc<int>(std::size_t(cap), "cudaMalloc(survivors)");
        }
        b.cap = cap;
        if (host_capacity < cap) {
            cudaFreeHost(h_a);
            cudaFreeHost(h_d);
            h_a = nullptr;
            h_d = nullptr;
            host_capacity = 0;
            check_cuda(cudaMallocHost(&h_a, std::size_t(cap) * sizeof(long long)), "cudaMallocHost");
            check_cuda(cudaMallocHost(&h_d, std::size_t(cap) * sizeof(int)), "cudaMallocHost");
            host_capacity = cap;
        }
        timings.workspace_ms += ms_since(t0);
        return true;
    }

    // Queue a batch as pieces: word tiles of at most kMaxTileWords.
    void queue_pieces(long long first, long long last) {
        piece_batch_first = first;
        piece_batch_last = last;
        for (long long w = 0; w < words; w += max_tile)
            pieces.push_back(Piece{first, last, w, std::min(words, w + max_tile)});
    }

    // Split a piece into two halves (by parameter, else by word range).
    void split_front(const Piece &p) {
        if (p.last > p.first) {
            const long long mid = p.first + (p.last - p.first) / 2;
            pieces.push_front(Piece{mid + 1, p.last, p.w_lo, p.w_hi});
            pieces.push_front(Piece{p.first, mid, p.w_lo, p.w_hi});
        } else if (p.w_hi - p.w_lo > 1) {
            const long long mid = p.w_lo + (p.w_hi - p.w_lo) / 2;
            pieces.push_front(Piece{p.first, p.last, mid, p.w_hi});
            pieces.push_front(Piece{p.first, p.last, p.w_lo, mid});
        } else {
            throw std::logic_error("survivor buffer cannot hold one word of survivors");
        }
    }

    // Run pieces one at a time (synchronously) until one fits a buffer.
    bool next_piece(BatchView &out) {
        while (!pieces.empty()) {
            const Piece p = pieces.front();
            pieces.pop_front();
            const int which = buf[0].busy ? 1 : 0;
            if (buf[which].busy) throw std::logic_error("no free survivor buffer");
            launch(which, p.first, p.last, p.w_lo, p.w_hi);
            check_cuda(cudaEventSynchronize(buf[which].copied), "sieve kernel");
            buf[which].busy = false;
            // the counter words came back with the launch: [2] is its error word
            if (h_count[4 * which + 2]) throw DeviceTimeout("sieve kernel: bounded wait for a row copy timed out");
            const unsigned long long n = h_count[4 * which], kept = h_count[4 * which + 3];
            const float ms = elapsed(buf[which]);
            timings.sieve_ms += ms;
            if (n > (unsigned long long)buf[which].cap) {
                ++timings.reruns;
                if (!grow(which, n)) split_front(p);
                else pieces.push_front(p);
                continue;
            }
            deliver(out, which, std::size_t(n), std::size_t(kept), ms, piece_batch_first, piece_batch_last,
                    pieces.empty());
            return true;
        }
        return false;
    }

    bool next(BatchView &out) {
        if (!pieces.empty()) return next_piece(out);
        if (order.empty() && words > max_tile && q_next <= q_last) {
            const long long first = q_next;
            const long long last = std::min(q_last, first + q_batch - 1);
            q_next = last + 1;
            queue_pieces(first, last);
            return next_piece(out);
        }
        refill();
        if (order.empty()) return false;
        const int which = order.front();
        order.pop_front();
        Buffer &b = buf[which];
        // The counter words were copied to pinned memory right after the launch.
        check_cuda(cudaEventSynchronize(b.copied), "sieve kernel");
        unsigned long long counts[4];
        for (int i = 0; i < 4; ++i) counts[i] = h_count[4 * which + i];
        if (counts[2]) throw DeviceTimeout("sieve kernel: bounded wait for a row copy timed out");
        const unsigned long long n = counts[0];
        const float ms = elapsed(b);
        timings.sieve_ms += ms;
        if (n > (unsigned long long)b.cap) {
            ++timings.reruns;
            b.busy = false;
            piece_batch_first = b.first;
            piece_batch_last = b.last;
            if (grow(which, n)) pieces.push_front(Piece{b.first, b.last, 0, words});
            else split_front(Piece{b.first, b.last, 0, words});
            return next_piece(out);
        }
        deliver(out, which, std::size_t(n), std::size_t(counts[3]), ms, b.first, b.last, true);
        b.busy = false;
        refill();
        return true;
    }
};

Sieve::Sieve(const std::vector<std::string> &coefficients, long long bound,
             const SieveOptions &options)
    : impl_(new Impl) {
    if (bound < 1) throw std::invalid_argument("numerator bound must be positive");
    // the fast kernel's queued positions a + H must stay below 2^47
    if (options.plan == PlanKind::fast && bound > (1LL << 45))
        throw std::invalid_argument("numerator bound too large for the fast plan (at most 2^45)");
    impl_->opt = options;
    impl_->bound = bound;
    impl_->words = word_count64(bound);
    try {
        impl_->init(coefficients);
    } catch (...) {
        impl_->release();
        throw;
    }
}

Sieve::~Sieve() = default;

void release_pooled_pipelines(int device) {
    std::vector<PooledPipeline> taken;
    {
        std::lock_guard<std::mutex> lock(pipeline_pool_mutex());
        auto &pool = pipeline_pool();
        for (auto it = pool.begin(); it != pool.end();) {
            if (device < 0 || it->device == device) {
                taken.push_back(*it);
                it = pool.erase(it);
            } else {
                ++it;
            }
        }
    }
    for (const auto &p : taken) {
        for (const auto &b : p.buf) {
            cudaFree(b.a);
            cudaFree(b.d);
            cudaFree(b.pa);
            cudaFree(b.pd);
            cudaFree(b.count);
            if (b.begin) cudaEventDestroy(b.begin);
            if (b.end) cudaEventDestroy(b.end);
            if (b.copied) cudaEventDestroy(b.copied);
        }
        if (p.h_count) cudaFreeHost(p.h_count);
        if (p.h_a) cudaFreeHost(p.h_a);
        if (p.h_d) cudaFreeHost(p.h_d);
        for (cudaEvent_t e : p.events)
            if (e) cudaEventDestroy(e);
        for (cudaStream_t s : p.streams)
            if (s) cudaStreamDestroy(s);
    }
}

void Sieve::start(long long first, long long last, long long batch_size) {
    if (first < 1 || last < first) throw std::invalid_argument("invalid denominator range");
    if (impl_->opt.square && last > 46340) throw std::invalid_argument("invalid denominator range");
    if (last > 2147483647LL) throw std::invalid_argument("invalid denominator range");
    cancel();
    check_cuda(cudaEventRecord(impl_->origin, impl_->stream), "cudaEventRecord");
    impl_->last_end_ms = 0;
    impl_->q_next = first;
    impl_->q_last = last;
    impl_->q_batch = std::max<long long>(1, batch_size);
}

bool Sieve::next(BatchView &out) { return impl_->next(out); }

void Sieve::cancel() {
    check_cuda(cudaStreamSynchronize(impl_->stream), "sieve stream");
    check_cuda(cudaStreamSynchronize(impl_->stream2), "sieve stream");
    for (auto &b : impl_->buf) b.busy = false;
    impl_->order.clear();
    impl_->pieces.clear();
    impl_->q_next = 0;
    impl_->q_last = -1;
}

const SieveTimings &Sieve::timings() const { return impl_->timings; }

unsigned long long Sieve::swept_words(long long first, long long last) const {
    const auto &I = *impl_;
    if (last < first) return 0;
    if (I.opt.plan != PlanKind::fast) return (unsigned long long)(last - first + 1) * I.words;
    // Denominators per residue mod M, then the words of each admissible class.
    const int q = I.F.class_prime;
    const long long M = I.F.class_mod;
    std::vector<unsigned long long> per_residue(M, 0);
    if (I.fast_bad_primes.empty()) {
        for (long long t = 0; t < M; ++t) {
            const long long lo = first + ((t - first % M) % M + M) % M;  // first k >= first, k = t (mod M)
            const unsigned long long n = lo > last ? 0 : (unsigned long long)((last - lo) / M + 1);
            const long long dres = I.opt.square ? (t * t) % M : t;
            per_residue[dres] += n;
        }
    } else {
        // parameters k without a denominator prime factor, by segments
        constexpr long long kSegment = 1LL << 22;
        std::vector<unsigned char> skip;
        for (long long lo = first; lo <= last; lo += kSegment) {
            const long long hi = std::min(last, lo + kSegment - 1);
            skip.assign(std::size_t(hi - lo + 1), 0);
            for (int p : I.fast_bad_primes)
                for (long long k = lo + ((p - lo % p) % p); k <= hi; k += p) skip[std::size_t(k - lo)] = 1;
            for (long long k = lo; k <= hi; ++k) {
                if (skip[std::size_t(k - lo)]) continue;
                const long long t = k % M;
                per_residue[I.opt.square ? (t * t) % M : t] += 1;
            }
        }
    }
    const long long sites = 2 * I.bound + 1;
    unsigned long long total = 0;
    for (long long dres = 0; dres < M; ++dres) {
        if (!per_residue[dres]) continue;
        const dev::u64 c2 = I.fast_adm_host[dres % 64];
        const dev::u64 cq = q > 1 ? I.fast_adm_host[64 + dres % q] : 1;
        unsigned long long words = 0;
        for (int r = 0; r < M; ++r) {
            if (!((c2 >> (r % 64)) & 1)) continue;
            if (q > 1 && !((cq >> (r % q)) & 1)) continue;
            const long long ofs = (r + I.bound % M) % M;
            const long long count = ofs < sites ? (sites - 1 - ofs) / M + 1 : 0;
            words += (unsigned long long)((count + 63) / 64);
        }
        total += per_residue[dres] * words;
    }
    return total;
}

FastPlanInfo Sieve::fast_plan_info() const {
    FastPlanInfo info;
    if (impl_->opt.plan != PlanKind::fast) return info;
    info.class_prime = impl_->fast_plan.class_prime;
    info.moduli = impl_->fast_plan.moduli;
    for (const auto &f : impl_->fast_plan.slots)
        for (int p : f) info.primes.push_back(p);
    return info;
}

int Sieve::device() const { return impl_->device; }

bool Sieve::fits_one_launch() const { return impl_->words <= impl_->max_tile; }

bool Sieve::launch_into(long long first, long long last, long long *out_a, int *out_d,
                        unsigned long long capacity, unsigned long long *out_count,
                        unsigned long long *work, unsigned long long *error, cudaStream_t stream) {
    const auto &I = *impl_;
    if (!fits_one_launch() || last < first || last - first + 1 > (1 << 16)) return false;
    dev::SieveArgs A{};
    A.bound = I.bound;
    A.words = I.words;
    A.w_lo = 0;
    A.w_hi = I.words;
    A.k_first = first;
    A.k_count = int(last - first + 1);
    A.square = I.opt.square ? 1 : 0;
    A.out_a = out_a;
    A.out_d = out_d;
    A.out_count = out_count;
    A.capacity = capacity;
    A.error = error;  // a bounded wait that gives up sets it
    if (I.opt.plan == PlanKind::fast) {
        I.launch_fast(I.F, A, work, stream);
    } else {
        const int blocks = int(std::min<long long>(I.grid, A.k_count));
        dev::ref_sieve_kernel<<<blocks, dev::kThreads, dev::kRefSmem, stream>>>(I.T, A);
    }
    check_cuda(cudaGetLastError(), "sieve kernel launch");
    return true;
}

unsigned Sieve::smem_bytes_per_word() const {
    return impl_->opt.plan == PlanKind::fast ? unsigned(8 * impl_->F.slots)
                                             : unsigned(8 * dev::kRefFast);
}
long long Sieve::words64() const { return impl_->words; }
cudaStream_t Sieve::stream() const { return impl_->stream; }

unsigned long long Sieve::count_only(long long first, long long last, long long batch_size) {
    if (first < 1 || last < first) throw std::invalid_argument("invalid denominator range");
    cancel();
    auto &I = *impl_;
    // Launches share buffer 0's counter: survivors past capacity are counted,
    // not stored, so the total is exact while the stores stop early.
    auto &b = I.buf[0];
    check_cuda(cudaMemsetAsync(b.count, 0, 3 * sizeof(unsigned long long), I.stream),
               "cudaMemsetAsync");
    // the second launch stream starts after the reset and joins before the read
    check_cuda(cudaEventRecord(I.fork_event, I.stream), "cudaEventRecord");
    check_cuda(cudaStreamWaitEvent(I.stream2, I.fork_event, 0), "cudaStreamWaitEvent");
    int which = 0;
    for (long long f = first; f <= last; f += batch_size) {
        const long long l = std::min(last, f + batch_size - 1);
        for (long long w = 0; w < I.words; w += I.max_tile, which ^= 1)
            I.launch_counting(which, f, l, w, std::min(I.words, w + I.max_tile));
    }
    check_cuda(cudaEventRecord(I.join_event, I.stream2), "cudaEventRecord");
    check_cuda(cudaStreamWaitEvent(I.stream, I.join_event, 0), "cudaStreamWaitEvent");
    unsigned long long total = 0;
    check_cuda(cudaMemcpyAsync(&total, b.count, sizeof total, cudaMemcpyDeviceToHost, I.stream),
               "download survivor count");
    check_cuda(cudaStreamSynchronize(I.stream), "sieve kernel");
    I.check_error_word(0);
    return total;
}

}  // namespace rpg
