// ThermoAcoustic1D in one library call (pyfds/coupled_fields.py:10-65): the acoustic
// and the thermal 1-D steps alternate with the loss coupling of the acoustic velocity
// into the temperature (BoundaryCoupling with ThermoAcoustic1D._loss_coupling).
//
// The loss kernel forms a_v_p (v * rho) in scipy's DIA order (y = 0, diagonal -1 then
// 0) and the product chain of the reference's expression
// ((mu / rho_th / c_th) * vd^2) * dt with unfused operations, so an exact-mode run is
// the reference's bit for bit.
#include "fds_capi.h"
#include "fds_internal.h"

namespace fds {
namespace {

// mode 0: T += loss; 1: acc = loss (empty accumulator); 2: acc += loss;
// 3: acc = loss, then T += acc; 4: acc += loss, then T += acc
__global__ void __launch_bounds__(256)
    loss_kernel(int n, const double* __restrict__ v, const double* __restrict__ rho,
                const double* __restrict__ bx, const double* __restrict__ g, double dt,
                double* __restrict__ T, double* __restrict__ acc, int mode) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double vd = 0.0;
  if (i >= 1) vd = __dadd_rn(vd, __dmul_rn(-bx[i - 1], __dmul_rn(v[i - 1], rho[i - 1])));
  vd = __dadd_rn(vd, __dmul_rn(bx[i], __dmul_rn(v[i], rho[i])));
  const double loss = __dmul_rn(__dmul_rn(g[i], __dmul_rn(vd, vd)), dt);
  if (mode == 0) {
    T[i] = __dadd_rn(T[i], loss);
    return;
  }
  const double a = (mode == 1 || mode == 3) ? loss : __dadd_rn(acc[i], loss);
  if (mode >= 3) {
    T[i] = __dadd_rn(T[i], a);
  } else {
    acc[i] = a;
  }
}

// The tables of one step of a multi-step plan: output row s of each component
FdsStagTables step_tables(const FdsStagTables& t, int32_t s) {
  FdsStagTables o = t;
  for (int k = 0; k < 3; ++k)
    if (o.comp[k].probe_tile_start && o.comp[k].out) {
      o.comp[k].out += (int64_t)s * o.comp[k].ncols;
      o.comp[k].out_rows = t.comp[k].out_rows - s;
    }
  return o;
}

}  // namespace
}  // namespace fds

extern "C" int32_t fds_thermoacoustic_run(
    const FdsStagProblem* ac, FdsStagState* acs, const FdsStagTables* act,
    const FdsStagProblem* th, FdsStagState* ths, const FdsStagTables* tht, const double* g,
    const double* rho_ac, double* acc, int32_t* acc_empty, double dt, int32_t stepping,
    int32_t accumulate, int64_t step0, int32_t nsteps, void* stream) {
  using namespace fds;
  if (!ac || !acs || !act || !th || !ths || !tht || !g || !rho_ac || !acc || !acc_empty)
    return set_error(FDS_E_ARG, "null argument");
  if (ac->family != FDS_FAMILY_ACOUSTIC || th->family != FDS_FAMILY_THERMAL ||
      ac->precision != FDS_PREC_F64 || th->precision != FDS_PREC_F64 || ac->ny != 1 ||
      th->ny != 1 || ac->nx != th->nx || (ac->flags & FDS_FLAG_HAS_V) || (th->flags & FDS_FLAG_HAS_V))
    return set_error(FDS_E_ARG, "need a float64 Acoustic1D and Thermal1D of the same size");
  if (stepping < 1 || nsteps < 0 || step0 < 0) return set_error(FDS_E_ARG, "bad stepping or steps");
  if (!ac->coefs.bx) return set_error(FDS_E_ARG, "acoustic coefficients missing");
  const int n = ac->nx;
  cudaStream_t s = (cudaStream_t)stream;
  // one step per field and call, between the coupling launches: the tile kernel
  // (stages 1), not the kernels that keep a 1-D field in shared memory for a whole call
  FdsStagProblem ac1 = *ac, th1 = *th;
  ac1.stages = 1;
  th1.stages = 1;
  for (int32_t k = 0; k < nsteps; ++k) {
    const int64_t step = step0 + k;
    FdsStagTables ta = step_tables(*act, k), tt = step_tables(*tht, k);
    int32_t rc = fds_stag_run(&ac1, acs, &ta, step, 1, 1, stream);
    if (rc != FDS_OK) return rc;
    rc = fds_stag_run(&th1, ths, &tt, step, 1, 0, stream);
    if (rc != FDS_OK) return rc;
    const bool due = step % stepping == 0;
    int mode;
    if (!accumulate) {
      if (!due) continue;
      mode = 0;
    } else if (due) {
      mode = *acc_empty ? 3 : 4;
      *acc_empty = 1;
    } else {
      mode = *acc_empty ? 1 : 2;
      *acc_empty = 0;
    }
    loss_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, (const double*)acs->cur[1], rho_ac,
                                                (const double*)ac->coefs.bx, g, dt,
                                                (double*)ths->cur[0], acc, mode);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(FDS_E_LAUNCH, "loss coupling: %s", cudaGetErrorString(e));
  }
  return FDS_OK;
}
