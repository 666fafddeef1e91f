// rpg_session_sieve_noalloc: a sieve launch that allocates no memory.
//
// Some callers cannot allocate device memory at the moment they want to sieve:
// engines that reserve all their device memory up front and hand it out from
// their own pool (another cudaMalloc would fail or break their accounting), and
// latency-bound loops that cannot afford cudaMalloc/cudaFree, which may
// synchronize the whole device.  This entry point serves them: the per-curve
// tables were allocated earlier, when the session was created; the caller
// passes its own device arrays for the survivors and their count; and the only
// scratch the launch needs (an error word and one dynamic-scheduling counter
// per batch of 65536 denominators) lives in a fixed file-scope device array
// that every GPU loading this library holds until the process exits.
#include <cuda_runtime.h>

#include <cstdlib>
#include <mutex>
#include <string>

#include "ratpoints_gb300.h"
#include "session.hpp"
#include "sieve.hpp"

namespace rpg {
void set_last_error(const std::string &message);
}

namespace {

constexpr int kNoAllocBatch = 1 << 16;          // denominators per launch
constexpr int kNoAllocMaxBatches = 256;         // launches (work counters) per call
constexpr int kMaxDevices = 64;

// Word 0: the error word the launches set when a bounded wait gives up.
// Words 1..256: the work counters of the launches of one call.  2,056 bytes
// per device.
static __device__ __align__(256) unsigned long long g_noalloc_scratch[1 + kNoAllocMaxBatches];

std::mutex g_setup_mutex;
unsigned long long *g_scratch[kMaxDevices] = {};

rpg_status fail(rpg_status status, const std::string &message) {
    rpg::set_last_error(message);
    return status;
}

// Restores the calling thread's current device on every return path.
class CurrentDeviceGuard {
public:
    CurrentDeviceGuard() { saved_ok_ = cudaGetDevice(&saved_) == cudaSuccess; }
    ~CurrentDeviceGuard() {
        if (saved_ok_) cudaSetDevice(saved_);
    }
    CurrentDeviceGuard(const CurrentDeviceGuard &) = delete;
    CurrentDeviceGuard &operator=(const CurrentDeviceGuard &) = delete;

private:
    int saved_ = 0;
    bool saved_ok_ = false;
};

// After the call's launches: a timed-out wait in any of them turns the
// caller's survivor count into the sentinel UINT64_MAX.
__global__ void noalloc_report_kernel(const unsigned long long *error, unsigned long long *count) {
    if (threadIdx.x == 0 && *error != 0) *count = ~0ull;
}

}  // namespace

extern "C" rpg_status rpg_session_sieve_noalloc(rpg_session *session, int32_t first, int32_t last,
                                                int64_t *device_numerators,
                                                int32_t *device_denominators, uint64_t capacity,
                                                uint64_t *device_count, void *stream) {
    try {
        rpg::set_last_error("");
        if (!session || !session->sieve) return fail(RPG_E_ARG, "session must not be NULL");
        if (!device_count || (capacity && (!device_numerators || !device_denominators)))
            return fail(RPG_E_ARG, "output arrays must not be NULL");
        if (first < 1 || last < first) return fail(RPG_E_ARG, "invalid denominator range");
        const long long count = (long long)last - first + 1;
        const long long batches = (count + kNoAllocBatch - 1) / kNoAllocBatch;
        if (batches > kNoAllocMaxBatches)
            return fail(RPG_E_ARG,
                        "rpg_session_sieve_noalloc handles at most 16777216 denominators "
                        "(256 launches of 65536) per call; split the range");
        if (!session->sieve->fits_one_launch())
            return fail(RPG_E_ARG,
                        "rpg_session_sieve_noalloc needs each row in one launch: the session's "
                        "numerator bound is too large (use rpg_sieve_run)");
        const int device = session->sieve->device();
        if (device < 0 || device >= kMaxDevices) return fail(RPG_E_ARG, "unsupported device ordinal");
        CurrentDeviceGuard keep_current_device;
        rpg::check_cuda(cudaSetDevice(device), "cudaSetDevice");
        unsigned long long *scratch = nullptr;
        {
            // Once per device, with that device current: the scratch array's
            // device address (host code cannot use the symbol itself).
            std::lock_guard<std::mutex> lock(g_setup_mutex);
            if (!g_scratch[device]) {
                void *ptr = nullptr;
                cudaError_t status = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
                if (status != cudaSuccess)
                    return fail(RPG_E_CUDA, std::string("cudaGetSymbolAddress: ") +
                                                cudaGetErrorString(status));
                g_scratch[device] = static_cast<unsigned long long *>(ptr);
            }
            scratch = g_scratch[device];
        }
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        unsigned long long *error = scratch;
        unsigned long long *counters = scratch + 1;
        // The array keeps the previous call's contents: clear the error word and
        // this call's counters, and the caller's count.
        rpg::check_cuda(cudaMemsetAsync(scratch, 0, std::size_t(1 + batches) * sizeof(unsigned long long), st),
                        "cudaMemsetAsync");
        rpg::check_cuda(cudaMemsetAsync(device_count, 0, sizeof(uint64_t), st), "cudaMemsetAsync");
        // Test hook: stands in for a launch whose bounded wait gave up (a
        // timeout made on the host; no kernel is made to fail).
        if (const char *inject = std::getenv("RPG_TEST_INJECT_NOALLOC_TIMEOUT"); inject && *inject == '1')
            rpg::check_cuda(cudaMemsetAsync(error, 0xff, sizeof(unsigned long long), st), "cudaMemsetAsync");
        for (long long b = 0; b < batches; ++b) {
            const long long lo = first + b * kNoAllocBatch;
            const long long hi = lo + kNoAllocBatch - 1 < last ? lo + kNoAllocBatch - 1 : last;
            if (!session->sieve->launch_into(lo, hi, reinterpret_cast<long long *>(device_numerators),
                                             reinterpret_cast<int *>(device_denominators), capacity,
                                             reinterpret_cast<unsigned long long *>(device_count),
                                             counters + b, error, st))
                return fail(RPG_E_INTERNAL, "sieve launch rejected its parameters");
        }
        noalloc_report_kernel<<<1, 32, 0, st>>>(error, reinterpret_cast<unsigned long long *>(device_count));
        rpg::check_cuda(cudaGetLastError(), "noalloc report launch");
        return RPG_OK;
    } catch (const rpg::CudaError &e) {
        return fail(RPG_E_CUDA, e.what());
    } catch (const std::exception &e) {
        return fail(RPG_E_INTERNAL, e.what());
    }
}
