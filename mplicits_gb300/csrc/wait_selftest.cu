// Self-test of the bounded-wait contract that every pipelined kernel of the
// library follows: a wait that cannot complete gives up after a wall-clock
// limit, records MPL_ERR_DEVICE_TIMEOUT in the device status word, raises
// its CTA's abort flag, and the CTA's other waits leave through that flag,
// so the launch returns and the context stays usable.  The test kernel runs
// the same wait routine as the level kernels (bf16::mbar_wait_abort) on
// barriers that nothing arrives at, with no bulk copy or MMA in flight.
#include "level_bf16.cuh"

namespace mpl {

namespace {

// One CTA of two warps.  Warp 0 waits with the given limit on barrier 0 and
// must give up; warp 1 waits with the kernels' own limit (kWaitLimitNs) on
// barrier 1 and must leave early, through the abort flag warp 0 raised.
// result[0], [1]: whether each warp's wait succeeded (lane 0); result[2],
// [3]: the nanoseconds each warp waited.
__global__ void wait_selftest_kernel(uint64_t limit_ns, int* status,
                                     long long* __restrict__ result) {
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ int abort_flag;
  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    abort_flag = 0;
    fence_barrier_init();
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5;
  const uint64_t t0 = global_timer_ns();
  const bool ok = warp == 0
                      ? bf16::mbar_wait_abort(&bars[0], 0u, status, &abort_flag, limit_ns)
                      : bf16::mbar_wait_abort(&bars[1], 0u, status, &abort_flag);
  const uint64_t dt = global_timer_ns() - t0;
  if ((threadIdx.x & 31) == 0) {
    result[warp] = ok ? 1 : 0;
    result[2 + warp] = (long long)dt;
  }
}

}  // namespace

}  // namespace mpl

using namespace mpl;

extern "C" int mpl_wait_selftest(int64_t limit_ns, int64_t* result_dev, void* stream) {
  if (!result_dev || limit_ns < 1000000 || limit_ns > (int64_t)kWaitLimitNs)
    return MPL_ERR_INVALID_ARG;
  int* status = device_status_ptr();
  if (!status) return MPL_ERR_CUDA;
  wait_selftest_kernel<<<1, 64, 0, (cudaStream_t)stream>>>(
      (uint64_t)limit_ns, status, reinterpret_cast<long long*>(result_dev));
  MPL_LAUNCH_CHECK();
  return MPL_OK;
}
