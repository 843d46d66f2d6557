// Bounded device waits: the run-time poll limit of the tensor-core kernels'
// mbarrier waits, a grid barrier whose spin gives up, and self-tests that
// make each kind of wait run out on purpose (an mbarrier nothing arrives at,
// a barrier count no grid reaches), so that callers can see the status come
// back instead of a hang.  Nothing here faults or traps: an expired wait
// sets ERR_TIMEOUT in a status word and the kernel returns.
#include <atomic>

#include "device_common.cuh"
#include "tc_common.cuh"

namespace omdg {

static std::atomic<int> g_wait_polls{TC_WAIT_LIMIT};

int tc_wait_polls() { return g_wait_polls.load(std::memory_order_relaxed); }

// One CTA: allocates TMEM as the MLP kernel does, waits on an mbarrier that
// nothing arrives at (bounded by `polls`), then releases TMEM and returns.
__global__ void __launch_bounds__(128) k_selftest_mbar(int polls, unsigned* status) {
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem;
    __shared__ volatile int abort;
    const int warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        abort = 0;
        mbar_fence_init();
    }
    if (warp == 0) {
        tmem_alloc(&tmem, 32);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    // nothing was issued on the barrier: there is nothing in flight to drain
    if (!mbar_wait_n(&bar, 0, polls)) abort = 1;
    __syncthreads();
    if (abort && threadIdx.x == 0) atomicOr(status, ERR_TIMEOUT);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, 32);
}

// One CTA at a grid barrier that waits for `target` arrivals.
__global__ void k_selftest_grid(unsigned* counter, unsigned target, int polls, unsigned* status) {
    grid_barrier(counter, target, polls, status);
}

}  // namespace omdg

extern "C" {

int omdg_set_wait_polls(int polls) {
    if (polls < 0) return OMDG_EINVAL;
    omdg::g_wait_polls.store(polls == 0 ? omdg::TC_WAIT_LIMIT : polls, std::memory_order_relaxed);
    return OMDG_OK;
}

int omdg_selftest_wait(int which, int polls, unsigned* status_out) {
    if (!status_out || polls < 1 || (which != 0 && which != 1)) return OMDG_EINVAL;
    unsigned* d = nullptr;  // [0] status, [1] barrier counter
    if (cudaMalloc(&d, 2 * sizeof(unsigned)) != cudaSuccess) return OMDG_ENOMEM;
    cudaError_t e = cudaMemset(d, 0, 2 * sizeof(unsigned));
    if (e == cudaSuccess) {
        if (which == 0) omdg::k_selftest_mbar<<<1, 128>>>(polls, d);
        else omdg::k_selftest_grid<<<1, 32>>>(d + 1, 2u, polls, d);  // one CTA waits for two
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(status_out, d, sizeof(unsigned), cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e == cudaSuccess ? OMDG_OK : OMDG_ECUDA;
}

}  // extern "C"
