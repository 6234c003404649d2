// Double-word instantiations of the fused staggered-grid step: state and
// coefficients as float32 (hi, lo) pairs, arithmetic on the FP32 pipe with
// float64-class accuracy (dw.cuh). Default and tile-menu variants; no
// register-marching variants (they shuffle scalar values between lanes).
#include "stag_run.cuh"

namespace fds {
int32_t run_stag_dw(const FdsStagProblem* p, FdsStagState* s, const FdsStagTables* t,
                    int64_t step0, int32_t nsteps, int32_t store_flux, cudaStream_t st) {
  return run_stag_typed<dw, dw, dw, false, true>(p, s, t, step0, nsteps, store_flux, st);
}
int32_t run_batch_dw(const FdsStagProblem* p, FdsStagState* s, const FdsStagTables* t,
                     int32_t count, void* ws, size_t wsb, int64_t step0, int32_t nsteps,
                     int32_t store_flux, uint32_t mode, cudaStream_t st) {
  return run_batch_typed<dw, dw, dw, true>(p, s, t, count, ws, wsb, step0, nsteps, store_flux,
                                           mode, st);
}
}  // namespace fds
