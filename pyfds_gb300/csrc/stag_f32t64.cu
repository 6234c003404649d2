// Thermal fields with float32 fluxes and coefficients and a float64 temperature:
// per-step temperature increments far from the heated edge fall below the float32
// spacing near 300 K (2^-15 K), so the temperature itself accumulates in float64.
#include "stag_run.cuh"

namespace fds {
int32_t run_stag_f32t64(const FdsStagProblem* p, FdsStagState* s, const FdsStagTables* t,
                        int64_t step0, int32_t nsteps, int32_t store_flux, cudaStream_t st) {
  return run_stag_typed<double, float, float, false, false>(p, s, t, step0, nsteps, store_flux,
                                                            st);
}
int32_t run_batch_f32t64(const FdsStagProblem* p, FdsStagState* s, const FdsStagTables* t,
                       int32_t count, void* ws, size_t wsb, int64_t step0, int32_t nsteps,
                       int32_t store_flux, uint32_t mode, cudaStream_t st) {
  return run_batch_typed<double, float, float, false>(p, s, t, count, ws, wsb, step0, nsteps, store_flux, mode,
                                                  st);
}
}  // namespace fds
