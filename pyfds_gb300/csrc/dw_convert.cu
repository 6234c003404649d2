// float64 <-> double-word conversion on the device (fds_dw_split / fds_dw_join):
// the same roundings as the host conversion of pyfds_gb300 (numpy float32 casts and
// a float64 sum), so either side produces the same bits.
#include <cuda_runtime.h>
#include <stdint.h>

#include "fds_capi.h"
#include "fds_internal.h"

namespace fds {
namespace {

__global__ void __launch_bounds__(256) dw_split_kernel(const double* __restrict__ in,
                                                       float2* __restrict__ out, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double x = in[i];
    const float hi = __double2float_rn(x);
    out[i] = make_float2(hi, __double2float_rn(__dsub_rn(x, (double)hi)));
  }
}

__global__ void __launch_bounds__(256) dw_join_kernel(const float2* __restrict__ in,
                                                      double* __restrict__ out, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float2 v = in[i];
    out[i] = __dadd_rn((double)v.x, (double)v.y);
  }
}

int grid_for(int64_t n) {
  // SM count of the first device used (any value gives correct grid-stride loops)
  static const int nsm = []() {
    int dev = 0, count = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      return 1;
    return count < 1 ? 1 : count;
  }();
  const int64_t blocks = (n + 255) / 256;
  return (int)(blocks < (int64_t)nsm * 8 ? blocks : (int64_t)nsm * 8);
}

}  // namespace
}  // namespace fds

extern "C" {

int32_t fds_dw_split(const double* in, void* out, int64_t n, void* stream) {
  using namespace fds;
  if (n < 0 || (n > 0 && (!in || !out))) return set_error(FDS_E_ARG, "dw_split: bad arguments");
  if (((uintptr_t)out & 7) != 0) return set_error(FDS_E_ARG, "dw_split: output not 8-byte aligned");
  if (n == 0) return FDS_OK;
  dw_split_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(in, (float2*)out, n);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? FDS_OK : set_error(FDS_E_LAUNCH, "dw_split: %s", cudaGetErrorString(e));
}

int32_t fds_dw_join(const void* in, double* out, int64_t n, void* stream) {
  using namespace fds;
  if (n < 0 || (n > 0 && (!in || !out))) return set_error(FDS_E_ARG, "dw_join: bad arguments");
  if (((uintptr_t)in & 7) != 0) return set_error(FDS_E_ARG, "dw_join: input not 8-byte aligned");
  if (n == 0) return FDS_OK;
  dw_join_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>((const float2*)in, out, n);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? FDS_OK : set_error(FDS_E_LAUNCH, "dw_join: %s", cudaGetErrorString(e));
}

}  // extern "C"
