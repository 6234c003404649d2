// Float32 instantiations of the fused staggered-grid step.
#include "stag_run.cuh"

namespace fds {
int32_t run_stag_f32(const FdsStagProblem* p, FdsStagState* s, const FdsStagTables* t,
                     int64_t step0, int32_t nsteps, int32_t store_flux, cudaStream_t st) {
  return run_stag_typed<float, float, float, false, true>(p, s, t, step0, nsteps, store_flux, st);
}
int32_t run_batch_f32(const FdsStagProblem* p, FdsStagState* s, const FdsStagTables* t,
                       int32_t count, void* ws, size_t wsb, int64_t step0, int32_t nsteps,
                       int32_t store_flux, uint32_t mode, cudaStream_t st) {
  return run_batch_typed<float, float, float, true>(p, s, t, count, ws, wsb, step0, nsteps, store_flux, mode,
                                                  st);
}
}  // namespace fds
