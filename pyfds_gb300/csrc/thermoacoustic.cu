// ThermoAcoustic1D in one library call (pyfds/coupled_fields.py:10-65): the acoustic
// and the thermal 1-D steps alternate with the loss coupling of the acoustic velocity
// into the temperature (BoundaryCoupling with ThermoAcoustic1D._loss_coupling).
//
// The loss kernel forms a_v_p (v * rho) in scipy's DIA order (y = 0, diagonal -1 then
// 0) and the product chain of the reference's expression
// ((mu / rho_th / c_th) * vd^2) * dt with unfused operations, so an exact-mode run is
// the reference's bit for bit.
#include <cstdlib>
#include <utility>

#include "fds_capi.h"
#include "fds_internal.h"
#include "stag_run.cuh"
#include "ta_warp.cuh"

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

// A 1-D float64 field's kernel arguments: size, tiling (the 1-D tile the tables are
// bucketed for), coefficients, tables and its current state.
StagArgs<double, double, double> args_1d(const FdsStagProblem* prob, const FdsStagState* st,
                                         const FdsStagTables* tabs, int64_t step0) {
  StagArgs<double, double, double> a{};
  a.nx = prob->nx;
  a.ny = 1;
  a.n = prob->nx;
  a.tiles_x = (prob->nx + prob->tile_x - 1) / prob->tile_x;
  a.ntiles = a.tiles_x;
  const FdsCoefs& c = prob->coefs;
  a.bx = (const double*)c.bx;
  a.by = a.bx;
  a.kx = (const double*)c.kx;
  a.ky = a.kx;
  a.axm = (const double*)c.axm;
  a.ad = (const double*)c.ad;
  a.axp = (const double*)c.axp;
  a.offset = prob->offset;
  for (int k = 0; k < 3; ++k) a.tab[k] = tabs->comp[k];
  a.pool = tabs->pool;
  a.status = tabs->status;
  a.step0 = step0;
  a.p_in = (const double*)st->cur[0];
  a.u_in = (const double*)st->cur[1];
  a.step = step0;
  return a;
}

// Every step of the call in one cluster launch (ta_warp_kernel): the first step's
// pressure and temperature bounds and probes (the prologues), then the launch.
// kWaveUnsupported where the field needs more warps than a cluster holds.
template <class CA, class CT>
int32_t run_ta_warp(const FdsStagProblem* ac, FdsStagState* acs, const FdsStagTables* act,
                    const FdsStagProblem* th, FdsStagState* ths, const FdsStagTables* tht,
                    TaWarpArgs t, cudaStream_t s) {
  const int n = ac->nx;
  const char* env = std::getenv("FDS_CLUSTER_BLOCK_STEPS");
  const int want = env ? std::atoi(env) : 0;
  t.K = std::min(8, std::max(1, want > 0 ? want : 6));  // window edges G = K + 2 <= m
  const int G = t.K + 2, m = kWarpLanes - 2 * G;
  const int nw = (n + m - 1) / m;
  const auto kernel = ta_warp_kernel<CA, CT>;
  int ncta = 0, nwc = 0;
  size_t smem = 0;
  auto shape = [&](int ctas) {
    ncta = std::min(ctas, nw);
    nwc = (nw + ncta - 1) / ncta;
    ncta = (nw + nwc - 1) / nwc;
    smem = ta_inbox_bytes(nwc, G) + 2 * warp_slot_bytes((nwc - 1) * m + kWarpLanes);
    return nwc <= kTaWarpsPerCta && smem <= kResidentMaxSmem;
  };
  if (!shape(kClusterMaxCta)) return kWaveUnsupported;
  LaunchShape ls;
  int32_t rc = kernel_shape<ta_warp_kernel<CA, CT>>(smem, nwc * 32, false, &ls);
  if (rc != FDS_OK) return rc;
  if (!cluster_fits(kernel, ncta, nwc * 32, smem)) {
    if (!shape(kClusterPortableCta)) return kWaveUnsupported;
    rc = kernel_shape<ta_warp_kernel<CA, CT>>(smem, nwc * 32, false, &ls);
    if (rc != FDS_OK) return rc;
  }
  StagArgs<double, double, double> A = args_1d(ac, acs, act, t.step0);
  StagArgs<double, double, double> H = args_1d(th, ths, tht, t.step0);
  rc = resident_prologue(A, acs, act, t.step0, s);
  if (rc != FDS_OK) return rc;
  rc = resident_prologue(H, ths, tht, t.step0, s);
  if (rc != FDS_OK) return rc;
  const bool odd = (t.nsteps & 1) != 0;  // the states end where nsteps swaps leave them
  t.fin[0] = (double*)(odd ? acs->nxt[0] : acs->cur[0]);
  t.fin[1] = (double*)(odd ? acs->nxt[1] : acs->cur[1]);
  t.fin[2] = (double*)(odd ? ths->nxt[0] : ths->cur[0]);
  t.fin[3] = (double*)(odd ? ths->nxt[1] : ths->cur[1]);
  const cudaError_t e = launch_cluster(kernel, ncta, nwc * 32, smem, s, A, H, t);
  if (e != cudaSuccess)
    return set_error(FDS_E_LAUNCH, "thermo-acoustic launch: %s", cudaGetErrorString(e));
  if (odd)
    for (int k = 0; k < 3; ++k) {
      std::swap(acs->cur[k], acs->nxt[k]);
      std::swap(ths->cur[k], ths->nxt[k]);
    }
  return FDS_OK;
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
  if (nsteps == 0) return FDS_OK;
  if (!(ac->flags & FDS_FLAG_FLOW) && !(th->flags & FDS_FLAG_FLOW) &&
      ((ac->flags & FDS_FLAG_EXACT) != 0) == ((th->flags & FDS_FLAG_EXACT) != 0) &&
      !(th->flags & FDS_FLAG_ABSORB)) {
    // every step in one launch on the warps of a cluster
    TaWarpArgs t{};
    t.rho = rho_ac;
    t.g = g;
    t.acc = acc;
    t.dt = dt;
    t.step0 = step0;
    t.nsteps = nsteps;
    t.stepping = stepping;
    t.accumulate = accumulate ? 1 : 0;
    t.acc_empty = *acc_empty ? 1 : 0;
    const bool absorb = (ac->flags & FDS_FLAG_ABSORB) != 0;
    const bool exact = (ac->flags & FDS_FLAG_EXACT) != 0;
    int32_t rw;
#define FDS_TA(ABS, EX)                                                                      \
  run_ta_warp<StagCfg<kTile1dX, 1, kThreads, false, true, ABS, false, EX>,                  \
              StagCfg<kTile1dX, 1, kThreads, false, false, false, false, EX>>(               \
      ac, acs, act, th, ths, tht, t, s)
    if (exact)
      rw = absorb ? FDS_TA(true, true) : FDS_TA(false, true);
    else
      rw = absorb ? FDS_TA(true, false) : FDS_TA(false, false);
#undef FDS_TA
    if (rw != kWaveUnsupported) {
      if (rw == FDS_OK && accumulate) *acc_empty = ((step0 + nsteps - 1) % stepping == 0) ? 1 : 0;
      return rw;
    }
  }
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
