// Bounded waits that nothing completes: the timeout path of the kernels, exercised
// without faulting or hanging a GPU.
//
// Every wait in the stepping kernels is bounded: a tile whose TMA copies do not
// land (mbar_wait) or whose neighbouring tile rows do not finish the previous step
// (wait_counters, the persistent wavefront kernel) gives up after a poll limit,
// ORs FDS_STATUS_TMA_TIMEOUT into the caller's status word and returns, and the
// host raises. This kernel runs the same two wait helpers on an mbarrier that no
// arrival or copy targets and on a counter that nothing increments, with a small
// poll limit, so a test can check the whole path: the waits end, the status word
// is set, the context stays usable. No asynchronous copy is ever issued, so none is
// in flight when the CTA exits.
#include "fds_capi.h"
#include "fds_internal.h"
#include "tma.cuh"

namespace {

__global__ void __launch_bounds__(128) bounded_wait_selftest(int mode, int32_t* status,
                                                             const uint32_t* counter,
                                                             long long limit) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) fds::mbar_init(&bar, 1);  // one arrival expected; none comes
  __syncthreads();
  bool ok = true;
  if (mode == 0) {
    ok = fds::mbar_wait(&bar, 0, limit);
  } else if (threadIdx.x == 0) {
    ok = fds::wait_counters(counter, 0, 0, 1u, limit);  // the counter stays 0
  }
  if (__syncthreads_or(!ok) && threadIdx.x == 0) atomicOr(status, fds::kStatusTmaTimeout);
}

}  // namespace

extern "C" int32_t fds_selftest_bounded_wait(int32_t mode, int32_t* status,
                                             const uint32_t* counter, int64_t poll_limit,
                                             void* stream) {
  if (mode != 0 && mode != 1) return fds::set_error(FDS_E_ARG, "mode must be 0 or 1");
  if (!status || (mode == 1 && !counter)) return fds::set_error(FDS_E_ARG, "null argument");
  if (poll_limit < 1 || poll_limit > (1 << 20))
    return fds::set_error(FDS_E_ARG, "poll limit must lie in [1, 2^20]");
  bounded_wait_selftest<<<1, 128, 0, static_cast<cudaStream_t>(stream)>>>(mode, status, counter,
                                                                          poll_limit);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return fds::set_error(FDS_E_LAUNCH, "self-test launch: %s", cudaGetErrorString(e));
  return FDS_OK;
}
