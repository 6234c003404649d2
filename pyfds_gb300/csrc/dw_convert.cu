// float64 <-> double-word conversion on the device (fds_dw_split / fds_dw_join):
// the same roundings as the host conversion of pyfds_gb300 (numpy float32 casts and
// a float64 sum), so either side produces the same bits. And the host gather
// (fds_host_gather): on a host whose pageable memory the GPU reads coherently
// (Grace: NVLink-C2C with address translation), one kernel reads the caller's arrays
// where they are and writes them to the device, converted, instead of one copy per
// array (each of which first waits for the stream).
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

// Blocks (blockIdx.y) take items; blockIdx.x strides over one item's values. The item
// table and the arrays are host memory, read through the GPU's address translation.
__global__ void __launch_bounds__(256) host_gather_kernel(const FdsGatherItem* items, int32_t count) {
  for (int32_t it = blockIdx.y; it < count; it += gridDim.y) {
    const FdsGatherItem g = items[it];
    const double* __restrict__ src = g.src;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < g.n;
         i += (int64_t)gridDim.x * blockDim.x) {
      const double x = src[i];
      if (g.kind == FDS_GATHER_F64) {
        static_cast<double*>(g.dst)[i] = x;
      } else if (g.kind == FDS_GATHER_F32) {
        static_cast<float*>(g.dst)[i] = __double2float_rn(x);
      } else {
        const float hi = __double2float_rn(x);
        static_cast<float2*>(g.dst)[i] =
            make_float2(hi, __double2float_rn(__dsub_rn(x, (double)hi)));
      }
    }
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

int32_t fds_host_access(void) {
  int dev = 0, pageable = 0, host_pt = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&host_pt, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) !=
          cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  return pageable == 1 && host_pt == 1 ? 1 : 0;
}

int32_t fds_host_gather(const FdsGatherItem* items, int32_t count, void* stream) {
  using namespace fds;
  if (count < 0 || (count > 0 && !items)) return set_error(FDS_E_ARG, "host_gather: bad arguments");
  if (count == 0) return FDS_OK;
  if (!fds_host_access())
    return set_error(FDS_E_ARG, "host_gather: the device does not read pageable host memory");
  int64_t most = 0;
  for (int32_t k = 0; k < count; ++k) {
    const FdsGatherItem& g = items[k];
    if (g.n < 0 || (g.n > 0 && (!g.src || !g.dst)) || g.kind < FDS_GATHER_F64 ||
        g.kind > FDS_GATHER_DW)
      return set_error(FDS_E_ARG, "host_gather: item %d malformed", k);
    if (((uintptr_t)g.src & 7) != 0 || ((uintptr_t)g.dst & (g.kind == FDS_GATHER_F32 ? 3 : 7)) != 0)
      return set_error(FDS_E_ARG, "host_gather: item %d misaligned", k);
    most = g.n > most ? g.n : most;
  }
  if (most == 0) return FDS_OK;
  const int64_t bx = (most + 255) / 256;
  const dim3 grid((unsigned)(bx < 64 ? bx : 64), (unsigned)(count < 65535 ? count : 65535));
  host_gather_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(items, count);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? FDS_OK : set_error(FDS_E_LAUNCH, "host_gather: %s", cudaGetErrorString(e));
}

}  // extern "C"
