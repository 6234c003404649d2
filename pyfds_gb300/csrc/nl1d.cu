// Nonlinear 1-D acoustics (IdealGas1D, Acoustic2ndOrder1D; pyfds/nonlinear_acoustics.py).
//
// The grids of these fields are small (hundreds to thousands of cells) and the steps
// many, so one CTA runs every step of a call in one launch: the phases of a step
// (pressure bounds/outputs, velocity update, velocity bounds/outputs, density update,
// density bounds/outputs, state equation) are separated by block barriers, and the
// state stays in L1/L2. Each DIA product is formed in scipy's accumulation order
// (y = 0, then one diagonal after the other); with FDS_FLAG_EXACT every operation is
// an unfused IEEE operation, so the result is the reference's bit for bit except
// where the ideal-gas state equation calls pow (the device pow and the host's libm
// may differ in the last bit).
#include "fds_capi.h"
#include "fds_internal.h"

namespace fds {
namespace {

constexpr int kNlThreads = 1024;

template <bool EXACT>
struct Ops {
  __device__ static double mul(double a, double b) { return EXACT ? __dmul_rn(a, b) : a * b; }
  __device__ static double add(double a, double b) { return EXACT ? __dadd_rn(a, b) : a + b; }
  __device__ static double sub(double a, double b) { return EXACT ? __dsub_rn(a, b) : a - b; }
  __device__ static double div(double a, double b) { return __ddiv_rn(a, b); }
};

struct NlArgs {
  double* p;
  double* v[2];
  double* r[2];
  const double* a;
  const double* rho0;
  const double* e1;
  const double* e2;
  double f1, fc;
  FdsCompTables tab[3];
  const double* pool;
  int n, ntiles;
  int64_t step0;
  int32_t nsteps;
};

// values[idx] = additive * old + value, in list order (pyfds/regions.py:125-145)
template <bool EXACT>
__device__ void apply_bounds(const FdsCompTables& tb, int ntiles, double* x, const double* pool,
                             int64_t step) {
  if (!tb.bound_tile_start) return;
  const int e = tb.bound_tile_start[ntiles];
  for (int g = threadIdx.x; g < e; g += blockDim.x) {
    const FdsBoundGroup grp = tb.groups[g];
    double val = x[grp.cell];
    for (int o = grp.op_begin; o < grp.op_end; ++o) {
      const FdsBoundOp op = tb.ops[o];
      const double add = (op.flags & FDS_BOP_SIGNAL)
                             ? pool[op.off + step * (int64_t)op.stride] + op.scalar
                             : op.scalar;
      val = Ops<EXACT>::add(Ops<EXACT>::mul(op.mul, val), add);
    }
    x[grp.cell] = val;
  }
}

__device__ void write_probes(const FdsCompTables& tb, int ntiles, const double* x, int64_t row) {
  if (!tb.probe_tile_start || tb.out_rows <= 0) return;
  const int e = tb.probe_tile_start[ntiles];
  double* out = tb.out + row * (int64_t)tb.ncols;
  for (int q = threadIdx.x; q < e; q += blockDim.x) {
    const FdsProbe pr = tb.probes[q];
    out[pr.col] = x[pr.cell];
  }
}

template <bool EXACT, int KIND, bool CONV, bool NLS>
__global__ void __launch_bounds__(kNlThreads) nl1d_kernel(const NlArgs a) {
  using O = Ops<EXACT>;
  const int n = a.n;
  const double f1 = a.f1, fc = a.fc;
  double* p = a.p;
  for (int32_t s = 0; s < a.nsteps; ++s) {
    const int64_t step = a.step0 + s;
    const double* v = a.v[s & 1];
    double* vn = a.v[(s & 1) ^ 1];
    const double* r = a.r[s & 1];
    double* rn = a.r[(s & 1) ^ 1];
    apply_bounds<EXACT>(a.tab[0], a.ntiles, p, a.pool, step);
    __syncthreads();
    write_probes(a.tab[0], a.ntiles, p, s);
    // velocity: v - ((a_v_p p) / B [+ a_v_v2 v] - (a_v_v v) / B), B = rho0 + d
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      double t1 = 0.0;  // backward difference: diagonals -1 (-f1) then 0 (f1)
      if (i >= 1) t1 = O::add(t1, O::mul(-f1, p[i - 1]));
      t1 = O::add(t1, O::mul(f1, p[i]));
      double t3 = 0.0;  // second difference: diagonals -1 (a), 0 (-2a), +1 (a)
      if (i >= 1) t3 = O::add(t3, O::mul(a.a[i - 1], v[i - 1]));
      t3 = O::add(t3, O::mul(O::mul(-2.0, a.a[i]), v[i]));
      if (i + 1 < n) t3 = O::add(t3, O::mul(a.a[i + 1], v[i + 1]));
      const double B = O::add(a.rho0[i], r[i]);
      double term = O::div(t1, B);
      if (CONV) {
        double t2 = 0.0;  // central difference: diagonals -1 (-fc) then +1 (fc)
        if (i >= 1) t2 = O::add(t2, O::mul(-fc, v[i - 1]));
        if (i + 1 < n) t2 = O::add(t2, O::mul(fc, v[i + 1]));
        term = O::add(term, t2);
      }
      term = O::sub(term, O::div(t3, B));
      vn[i] = O::sub(v[i], term);
    }
    __syncthreads();
    apply_bounds<EXACT>(a.tab[1], a.ntiles, vn, a.pool, step);
    __syncthreads();
    write_probes(a.tab[1], a.ntiles, vn, s);
    // density: d - a_d_v ((d + rho0) v), forward difference: diagonals 0 (-f1), +1 (f1)
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const double w0 = O::mul(O::add(r[i], a.rho0[i]), vn[i]);
      double t = O::add(0.0, O::mul(-f1, w0));
      if (i + 1 < n) t = O::add(t, O::mul(f1, O::mul(O::add(r[i + 1], a.rho0[i + 1]), vn[i + 1])));
      rn[i] = O::sub(r[i], t);
    }
    __syncthreads();
    apply_bounds<EXACT>(a.tab[2], a.ntiles, rn, a.pool, step);
    __syncthreads();
    write_probes(a.tab[2], a.ntiles, rn, s);
    // state equation
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const double d = rn[i];
      double pv;
      if (KIND == FDS_NL1D_IDEAL_GAS) {
        if (NLS) {
          const double x = O::div(O::add(a.rho0[i], d), a.rho0[i]);
          pv = O::mul(a.e1[i], O::sub(pow(x, a.e2[i]), 1.0));
        } else {
          pv = O::mul(a.e1[i], d);
        }
      } else {
        pv = O::add(O::mul(a.e1[i], d), O::mul(a.e2[i], O::mul(d, d)));
      }
      p[i] = pv;
    }
    __syncthreads();
  }
}

template <bool EXACT>
void launch(const NlArgs& a, int kind, bool conv, bool nls, cudaStream_t s) {
  if (kind == FDS_NL1D_IDEAL_GAS) {
    if (conv && nls) nl1d_kernel<EXACT, FDS_NL1D_IDEAL_GAS, true, true><<<1, kNlThreads, 0, s>>>(a);
    else if (conv) nl1d_kernel<EXACT, FDS_NL1D_IDEAL_GAS, true, false><<<1, kNlThreads, 0, s>>>(a);
    else if (nls) nl1d_kernel<EXACT, FDS_NL1D_IDEAL_GAS, false, true><<<1, kNlThreads, 0, s>>>(a);
    else nl1d_kernel<EXACT, FDS_NL1D_IDEAL_GAS, false, false><<<1, kNlThreads, 0, s>>>(a);
  } else {
    nl1d_kernel<EXACT, FDS_NL1D_SECOND_ORDER, true, false><<<1, kNlThreads, 0, s>>>(a);
  }
}

}  // namespace
}  // namespace fds

extern "C" int32_t fds_nl1d_run(const FdsNl1dProblem* prob, FdsStagState* st,
                                const FdsStagTables* tables, int64_t step0, int32_t nsteps,
                                void* stream) {
  using namespace fds;
  if (!prob || !st || !tables) return set_error(FDS_E_ARG, "null argument");
  if (prob->n < 1 || prob->tile_x < 1 || nsteps < 0 || step0 < 0)
    return set_error(FDS_E_ARG, "bad grid, tiling or step range");
  if (prob->kind != FDS_NL1D_IDEAL_GAS && prob->kind != FDS_NL1D_SECOND_ORDER)
    return set_error(FDS_E_ARG, "unknown nonlinear kind %d", prob->kind);
  if (!prob->a || !prob->rho0 || !prob->e1 || !prob->e2)
    return set_error(FDS_E_ARG, "missing coefficient arrays");
  for (int k = 0; k < 3; ++k) {
    if (!st->cur[k] || (k > 0 && !st->nxt[k])) return set_error(FDS_E_ARG, "missing state buffer %d", k);
    const FdsCompTables& t = tables->comp[k];
    if (t.probe_tile_start && (!t.out || t.out_rows < nsteps))
      return set_error(FDS_E_ARG, "output buffer of component %d too small", k);
  }
  if (nsteps == 0) return FDS_OK;
  NlArgs a{};
  a.p = (double*)st->cur[0];
  a.v[0] = (double*)st->cur[1];
  a.v[1] = (double*)st->nxt[1];
  a.r[0] = (double*)st->cur[2];
  a.r[1] = (double*)st->nxt[2];
  a.a = prob->a;
  a.rho0 = prob->rho0;
  a.e1 = prob->e1;
  a.e2 = prob->e2;
  a.f1 = prob->f1;
  a.fc = prob->fc;
  for (int k = 0; k < 3; ++k) a.tab[k] = tables->comp[k];
  a.pool = tables->pool;
  a.n = prob->n;
  a.ntiles = (prob->n + prob->tile_x - 1) / prob->tile_x;
  a.step0 = step0;
  a.nsteps = nsteps;
  const bool conv = prob->kind == FDS_NL1D_SECOND_ORDER || (prob->flags & FDS_NL1D_CONVECTIVE);
  const bool nls = (prob->flags & FDS_NL1D_NL_STATE) != 0;
  cudaStream_t s = (cudaStream_t)stream;
  if (prob->flags & FDS_FLAG_EXACT)
    launch<true>(a, prob->kind, conv, nls, s);
  else
    launch<false>(a, prob->kind, conv, nls, s);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(FDS_E_LAUNCH, "nonlinear 1-D launch: %s", cudaGetErrorString(e));
  // velocity and density were ping-ponged once per step
  if (nsteps & 1)
    for (int k = 1; k < 3; ++k) std::swap(st->cur[k], st->nxt[k]);
  return FDS_OK;
}
