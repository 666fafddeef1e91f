// rpg_smem_read_probe: the shared-memory read rate the sieve kernels are
// bounded by, measured on the device that runs them.
//
// The stage-1 sweep of every sieve kernel reads its staged rows with
// lane-contiguous 64-bit shared loads (a warp reads 256 consecutive bytes).
// This probe issues the same loads, and nothing else but one XOR per load,
// from every resident warp of every SM, so its rate is the roofline the
// sweep is measured against: bytes per second (CUDA events around the
// launch) and bytes per SM clock (that rate over the SM count and the SM
// clock, which the first CTA measures as clock64 ticks per globaltimer
// nanosecond over its loop).
#include <cuda_runtime.h>

#include <string>

#include "ratpoints_gb300.h"
#include "sieve_device.cuh"

namespace rpg {
void set_last_error(const std::string &message);

namespace dev {
namespace {

constexpr int kProbeThreads = 512;
constexpr int kProbeWords = 4096;       // 32 KB of shared memory per CTA
constexpr int kProbeLoads = 16;         // loads per iteration, 2 KB apart

// A volatile shared load: the assembler may not merge or hoist it, so every
// iteration's loads are issued even though they read the same addresses.
__device__ __forceinline__ u64 lds64(u32 addr) {
    u64 v;
    asm volatile("ld.volatile.shared.u64 %0, [%1];" : "=l"(v) : "r"(addr) : "memory");
    return v;
}

__device__ __forceinline__ u64 global_ns() {
    u64 t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__global__ void __launch_bounds__(kProbeThreads) smem_read_probe_kernel(int iterations, u64 *sink,
                                                                        long long *clock) {
    __shared__ __align__(16) u64 buf[kProbeWords];
    for (int i = threadIdx.x; i < kProbeWords; i += blockDim.x) buf[i] = u64(i) * 0x9E3779B97F4A7C15ull;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    // warp w reads bytes [256 (w mod 8), +256) of each 2 KB stripe
    const u32 base = smem_addr(buf) + u32(lane) * 8u + u32(warp & 7) * 256u;
    u64 a0 = 0, a1 = 0, a2 = 0, a3 = 0;
    const u64 n0 = global_ns();
    const long long t0 = clock64();
    for (int it = 0; it < iterations; ++it) {
#pragma unroll
        for (int k = 0; k < kProbeLoads; k += 4) {
            a0 ^= lds64(base + u32(k + 0) * 2048u);
            a1 ^= lds64(base + u32(k + 1) * 2048u);
            a2 ^= lds64(base + u32(k + 2) * 2048u);
            a3 ^= lds64(base + u32(k + 3) * 2048u);
        }
    }
    const long long t1 = clock64();
    const u64 n1 = global_ns();
    __syncthreads();
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        clock[0] = t1 - t0;         // SM clock ticks
        clock[1] = (long long)(n1 - n0);  // nanoseconds
    }
    const u64 acc = a0 ^ a1 ^ a2 ^ a3;
    if (acc == 0x5A5A5A5A5A5A5A5Aull) sink[0] = acc;  // keeps the loads live
}

}  // namespace
}  // namespace dev
}  // namespace rpg

extern "C" rpg_status rpg_smem_read_probe(int32_t device, int32_t iterations, double *gbs,
                                          double *bytes_per_clock_per_sm, double *ms) {
    using namespace rpg::dev;
    if (iterations < 1 || iterations > (1 << 20) || !gbs || !bytes_per_clock_per_sm || !ms) {
        rpg::set_last_error("iterations must be in [1, 2^20] and the outputs non-NULL");
        return RPG_E_ARG;
    }
    auto cuda_fail = [](cudaError_t e, const char *what) {
        rpg::set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? RPG_E_OOM : RPG_E_CUDA;
    };
    cudaError_t e = device >= 0 ? cudaSetDevice(device) : cudaSuccess;
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    int dev_id = 0, sms = 0, per_sm = 0;
    if ((e = cudaGetDevice(&dev_id)) != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev_id)) != cudaSuccess)
        return cuda_fail(e, "cudaDeviceGetAttribute");
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, smem_read_probe_kernel, kProbeThreads,
                                                           0)) != cudaSuccess)
        return cuda_fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    const int blocks = sms * (per_sm > 0 ? per_sm : 1);
    void *scratch = nullptr;
    if ((e = cudaMalloc(&scratch, 64)) != cudaSuccess) return cuda_fail(e, "cudaMalloc");
    cudaEvent_t start = nullptr, stop = nullptr;
    long long clock[2] = {0, 0};
    float elapsed = 0.0f;
    e = cudaEventCreate(&start);
    if (e == cudaSuccess) e = cudaEventCreate(&stop);
    if (e == cudaSuccess) {
        auto *sink = static_cast<u64 *>(scratch);
        auto *cyc = reinterpret_cast<long long *>(static_cast<char *>(scratch) + 32);
        smem_read_probe_kernel<<<blocks, kProbeThreads>>>(iterations / 8 + 1, sink, cyc);  // warm-up
        cudaEventRecord(start);
        smem_read_probe_kernel<<<blocks, kProbeThreads>>>(iterations, sink, cyc);
        cudaEventRecord(stop);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventSynchronize(stop);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&elapsed, start, stop);
        if (e == cudaSuccess) e = cudaMemcpy(clock, cyc, sizeof clock, cudaMemcpyDeviceToHost);
    }
    if (start) cudaEventDestroy(start);
    if (stop) cudaEventDestroy(stop);
    cudaFree(scratch);
    if (e != cudaSuccess) return cuda_fail(e, "shared-memory probe");
    const double per_block = double(kProbeThreads) * iterations * kProbeLoads * 8.0;
    *ms = elapsed;
    *gbs = per_block * blocks / (elapsed * 1e-3) / 1e9;
    const double ghz = clock[1] > 0 ? double(clock[0]) / double(clock[1]) : 0.0;
    *bytes_per_clock_per_sm = ghz > 0 ? *gbs / (double(sms) * ghz) : 0.0;
    return RPG_OK;
}
