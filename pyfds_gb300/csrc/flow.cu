// Moving-medium shift of AcousticFlow2D (pyfds/acoustic_flow.py:49-57): after a
// step, every row y whose period f = flow_period[y] divides the step (numpy's
// `step % f == 0`; f == 0 counts as dividing) moves one cell in +x in p, vx and vy,
// and its first cell becomes 0.
//
// One CTA per row, in place: the row is processed in chunks of blockDim.x cells
// from its right end to its left; within a chunk every thread reads its source
// cell (one to the left) before a barrier and writes after it, and the cells a
// chunk reads lie left of it, so nothing is read after it was overwritten.
#include "fds_capi.h"
#include "fds_internal.h"

namespace fds {
namespace {

__device__ __forceinline__ bool row_due(const int64_t* period, int y, int64_t step) {
  const int64_t f = period[y];
  return f == 0 || step % f == 0;
}

template <typename T>
__device__ __forceinline__ void shift_row(T* row, int nx) {
  const int nb = blockDim.x;
  for (int x0 = ((nx - 1) / nb) * nb; x0 >= 0; x0 -= nb) {
    const int x = x0 + (int)threadIdx.x;
    T v = T(0);
    if (x < nx && x >= 1) v = row[x - 1];
    __syncthreads();
    if (x < nx) row[x] = v;
    __syncthreads();
  }
}

template <typename TP, typename TF>
__global__ void __launch_bounds__(256) flow_shift_kernel(TP* p, TF* u, TF* v, int nx, int ny,
                                                         const int64_t* period, int64_t step) {
  const int y = blockIdx.x;
  if (y >= ny || !row_due(period, y, step)) return;
  const size_t base = (size_t)y * nx;
  shift_row(p + base, nx);
  shift_row(u + base, nx);
  shift_row(v + base, nx);
}

}  // namespace

int32_t launch_flow_shift(const FdsStagProblem* prob, void* const* cur, int64_t step,
                          cudaStream_t stream) {
  if (!(prob->flags & FDS_FLAG_FLOW) || !prob->flow_period)
    return set_error(FDS_E_ARG, "flow shift needs FDS_FLAG_FLOW and flow_period");
  if (prob->family != FDS_FAMILY_ACOUSTIC || !(prob->flags & FDS_FLAG_HAS_V) ||
      (prob->flags & FDS_FLAG_AXI))
    return set_error(FDS_E_ARG, "flow applies to 2-D Cartesian acoustic fields");
  if (!cur[0] || !cur[1] || !cur[2]) return set_error(FDS_E_ARG, "missing state buffer");
  switch (prob->precision) {
    case FDS_PREC_F64:
      flow_shift_kernel<double, double><<<prob->ny, 256, 0, stream>>>(
          (double*)cur[0], (double*)cur[1], (double*)cur[2], prob->nx, prob->ny,
          prob->flow_period, step);
      break;
    case FDS_PREC_F32:
      flow_shift_kernel<float, float><<<prob->ny, 256, 0, stream>>>(
          (float*)cur[0], (float*)cur[1], (float*)cur[2], prob->nx, prob->ny, prob->flow_period,
          step);
      break;
    case FDS_PREC_DW:  // double words move as 8-byte units (zero bits are 0 + 0)
      flow_shift_kernel<unsigned long long, unsigned long long><<<prob->ny, 256, 0, stream>>>(
          (unsigned long long*)cur[0], (unsigned long long*)cur[1], (unsigned long long*)cur[2],
          prob->nx, prob->ny, prob->flow_period, step);
      break;
    default:
      return set_error(FDS_E_ARG, "flow shift: precision %d not built", prob->precision);
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(FDS_E_LAUNCH, "flow shift launch: %s", cudaGetErrorString(e));
  return FDS_OK;
}

}  // namespace fds

extern "C" int32_t fds_stag_flow_shift(const FdsStagProblem* prob, FdsStagState* state,
                                       int64_t step, void* stream) {
  if (!prob || !state) return fds::set_error(FDS_E_ARG, "null argument");
  if (prob->nx < 1 || prob->ny < 1 || step < 0) return fds::set_error(FDS_E_ARG, "bad arguments");
  return fds::launch_flow_shift(prob, state->cur, step, (cudaStream_t)stream);
}
