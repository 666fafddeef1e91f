// rpg_bounded_wait_selftest: the failure path of the bounded mbarrier wait
// that every pipelined sieve kernel uses, exercised without a fault.
//
// One thread initialises an mbarrier for one arrival and waits on its first
// phase with a short poll limit.  When nothing arrives the wait gives up, the
// kernel records it in its status word and returns, and the host reports
// RPG_E_TIMEOUT as it does for a sieve launch whose row copy never landed;
// the context stays usable.  When the thread arrives first the wait succeeds.
#include <cuda_runtime.h>

#include <string>

#include "ratpoints_gb300.h"
#include "sieve_device.cuh"

namespace rpg {
void set_last_error(const std::string &message);

namespace dev {
namespace {

__global__ void bounded_wait_kernel(int polls, int arrive, int *status) {
    __shared__ __align__(8) unsigned long long bar;
    if (threadIdx.x != 0) return;
    const u32 b = smem_addr(&bar);
    mbar_init(b, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    if (arrive) mbar_arrive(b);
    *status = mbar_wait(b, 0, polls) ? 0 : 1;
}

}  // namespace
}  // namespace dev
}  // namespace rpg

extern "C" rpg_status rpg_bounded_wait_selftest(int32_t device, int32_t polls, int32_t arrive) {
    if (polls < 1 || polls > (1 << 20)) {
        rpg::set_last_error("polls must be in [1, 2^20]");
        return RPG_E_ARG;
    }
    auto cuda_fail = [](cudaError_t e, const char *what) {
        rpg::set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? RPG_E_OOM : RPG_E_CUDA;
    };
    cudaError_t e = device >= 0 ? cudaSetDevice(device) : cudaSuccess;
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    int *d_status = nullptr;
    if ((e = cudaMalloc(&d_status, sizeof(int))) != cudaSuccess) return cuda_fail(e, "cudaMalloc");
    int status = -1;
    e = cudaMemset(d_status, 0xff, sizeof(int));
    if (e == cudaSuccess) {
        rpg::dev::bounded_wait_kernel<<<1, 32>>>(polls, arrive ? 1 : 0, d_status);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(&status, d_status, sizeof status, cudaMemcpyDeviceToHost);
    cudaFree(d_status);
    if (e != cudaSuccess) return cuda_fail(e, "bounded wait self-test");
    if (status == 1) {
        rpg::set_last_error("self-test: bounded mbarrier wait gave up after " + std::to_string(polls) +
                            " polls");
        return RPG_E_TIMEOUT;
    }
    if (status != 0) {
        rpg::set_last_error("self-test: the kernel wrote no status");
        return RPG_E_INTERNAL;
    }
    return RPG_OK;
}
