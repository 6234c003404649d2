// Nonlinear 1-D acoustics (IdealGas1D, Acoustic2ndOrder1D; pyfds/nonlinear_acoustics.py).
//
// These grids are small (hundreds to thousands of cells) and the steps many, so every
// step of a call runs in one launch: CTA b owns tile b (tile_x cells) and loops over
// the steps; grids of up to 16 tiles as one thread-block cluster with hardware
// barriers, larger ones as a cooperative launch with global-memory grid barriers. A step's phases (pressure bounds/outputs, velocity update and
// bounds/outputs, density update and bounds/outputs, state equation) touch a
// neighbour's cell in two places only: the velocity update reads p[i-1], the density
// update reads v[i+1] and d[i+1]. So two grid-wide barriers per step suffice: after
// the pressure bounds and after the velocity bounds. (Ping-pong buffers for v and d
// keep every other read ahead of the next overwrite by at least one barrier.) Each
// CTA applies the boundary groups and probes of its own tile, which the host tables
// bucket per tile. Spreading the cells over many SMs matters on GB300: the state
// equation's pow and the divisions run on the FP64 pipe, about 2 FMAs per clock per SM.
//
// Each DIA product is formed in scipy's accumulation order (y = 0, then one diagonal
// after the other); with FDS_FLAG_EXACT every operation is an unfused IEEE operation,
// so the result is the reference's bit for bit except where the ideal-gas state
// equation calls pow (the device pow and the host's libm may differ in the last bit).
#include <algorithm>
#include <utility>

#include "fds_capi.h"
#include "fds_internal.h"

namespace fds {
namespace {

constexpr long long kBarrierLimit = 1ll << 22;
// arrivals one launch may count on its 32-bit barrier counter
constexpr int64_t kMaxBarrierArrivals = 0xfffffff0ll;

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
  unsigned* sync;
  int32_t* status;
  int n, tile, ntiles;
  int64_t step0;
  int64_t row0;  // output row of this launch's first step (calls run in several launches)
  int32_t nsteps;
};

// values[idx] = additive * old + value, in list order (pyfds/regions.py:125-145), for
// the boundary groups of tile `t`
template <bool EXACT>
__device__ void apply_bounds(const FdsCompTables& tb, int t, double* x, const double* pool,
                             int64_t step) {
  if (!tb.bound_tile_start) return;
  const int e = tb.bound_tile_start[t + 1];
  for (int g = tb.bound_tile_start[t] + threadIdx.x; g < e; g += blockDim.x) {
    const FdsBoundGroup grp = tb.groups[g];
    if (!grp.primary) continue;  // the global array: once per cell (not halo copies)
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

__device__ void write_probes(const FdsCompTables& tb, int t, const double* x, int64_t row) {
  if (!tb.probe_tile_start || tb.out_rows <= 0) return;
  const int e = tb.probe_tile_start[t + 1];
  double* out = tb.out + row * (int64_t)tb.ncols;
  for (int q = tb.probe_tile_start[t] + threadIdx.x; q < e; q += blockDim.x) {
    const FdsProbe pr = tb.probes[q];
    out[pr.col] = x[pr.cell];
  }
}

// Grid-wide barrier number k (0-based) of this launch: every CTA adds one to the
// counter and waits until it reaches (k + 1) * gridDim.x. The counter is zeroed before
// each launch and a launch runs at most kMaxBarrierArrivals / gridDim.x barriers (the
// host splits longer calls), so neither the counter nor the target wraps. Bounded:
// false if the wait gave up.
__device__ bool grid_barrier(unsigned* count, unsigned k) {
  __syncthreads();
  int ok = 1;
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(count, 1u);
    const unsigned target = (k + 1) * gridDim.x;
    long long i = 0;
    const volatile unsigned* c = count;
    while (*c < target) {
      if (++i > kBarrierLimit) {
        ok = 0;
        break;
      }
      __nanosleep(16);
    }
    __threadfence();
  }
  return __syncthreads_and(ok) != 0;
}

// Every thread of every CTA of the cluster arrives; the release / acquire pair at
// cluster scope orders each CTA's global-memory writes before the barrier with the
// other CTAs' reads after it.
__device__ __forceinline__ void nl_cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n"
               "barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

// CLUSTER: the grid is one thread-block cluster (up to 16 CTAs) and the step's two
// barriers are the hardware cluster barrier (about a tenth of the global-memory grid
// barrier's cost); else a cooperative launch with bounded grid barriers.
template <bool EXACT, int KIND, bool CONV, bool NLS, bool CLUSTER>
__global__ void __launch_bounds__(256) nl1d_kernel(const NlArgs a) {
  using O = Ops<EXACT>;
  const int n = a.n;
  const int t = blockIdx.x;
  const int c0 = t * a.tile;
  const int c1 = min(n, c0 + a.tile);
  const double f1 = a.f1, fc = a.fc;
  double* p = a.p;
  unsigned k = 0;
  for (int32_t s = 0; s < a.nsteps; ++s) {
    const int64_t step = a.step0 + s;
    const double* v = a.v[s & 1];
    double* vn = a.v[(s & 1) ^ 1];
    const double* r = a.r[s & 1];
    double* rn = a.r[(s & 1) ^ 1];
    apply_bounds<EXACT>(a.tab[0], t, p, a.pool, step);
    __syncthreads();
    write_probes(a.tab[0], t, p, a.row0 + s);
    if constexpr (CLUSTER) {
      nl_cluster_sync();
      ++k;
    } else if (!grid_barrier(a.sync, k++)) {
      break;
    }
    // velocity: v - ((a_v_p p) / B [+ a_v_v2 v] - (a_v_v v) / B), B = rho0 + d
    for (int i = c0 + threadIdx.x; i < c1; i += blockDim.x) {
      double t1 = 0.0;  // backward difference: diagonals -1 (-f1) then 0 (f1)
      if (i >= 1) t1 = O::add(t1, O::mul(-f1, p[i - 1]));
      t1 = O::add(t1, O::mul(f1, p[i]));
      double t3 = 0.0;  // second difference: diagonals -1 (a), 0 (-2a), +1 (a)
      if (i >= 1) t3 = O::add(t3, O::mul(a.a[i - 1], v[i - 1]));
      t3 = O::add(t3, O::mul(O::mul(-2.0, a.a[i]), v[i]));
      if (i + 1 < n) t3 = O::add(t3, O::mul(a.a[i + 1], v[i + 1]));
      const double B = O::add(a.rho0[i], r[i]);
      // exact: the reference's two divisions; otherwise one reciprocal of B (each
      // quotient within an ulp or so of the division's, inside the 1e-12 bar)
      const double rB = EXACT ? 0.0 : __drcp_rn(B);
      double term = EXACT ? O::div(t1, B) : t1 * rB;
      if (CONV) {
        double t2 = 0.0;  // central difference: diagonals -1 (-fc) then +1 (fc)
        if (i >= 1) t2 = O::add(t2, O::mul(-fc, v[i - 1]));
        if (i + 1 < n) t2 = O::add(t2, O::mul(fc, v[i + 1]));
        term = O::add(term, t2);
      }
      term = O::sub(term, EXACT ? O::div(t3, B) : t3 * rB);
      vn[i] = O::sub(v[i], term);
    }
    __syncthreads();
    apply_bounds<EXACT>(a.tab[1], t, vn, a.pool, step);
    __syncthreads();
    write_probes(a.tab[1], t, vn, a.row0 + s);
    if constexpr (CLUSTER) {
      nl_cluster_sync();
      ++k;
    } else if (!grid_barrier(a.sync, k++)) {
      break;
    }
    // density: d - a_d_v ((d + rho0) v), forward difference: diagonals 0 (-f1), +1 (f1)
    for (int i = c0 + threadIdx.x; i < c1; i += blockDim.x) {
      const double w0 = O::mul(O::add(r[i], a.rho0[i]), vn[i]);
      double tt = O::add(0.0, O::mul(-f1, w0));
      if (i + 1 < n)
        tt = O::add(tt, O::mul(f1, O::mul(O::add(r[i + 1], a.rho0[i + 1]), vn[i + 1])));
      rn[i] = O::sub(r[i], tt);
    }
    __syncthreads();
    apply_bounds<EXACT>(a.tab[2], t, rn, a.pool, step);
    __syncthreads();
    write_probes(a.tab[2], t, rn, a.row0 + s);
    // state equation (own cells)
    for (int i = c0 + threadIdx.x; i < c1; i += blockDim.x) {
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
  if (k < 2u * (unsigned)a.nsteps && threadIdx.x == 0 && a.status)
    atomicOr(a.status, FDS_STATUS_TMA_TIMEOUT);
}

using NlKernel = void (*)(NlArgs);

template <bool EXACT, bool CLUSTER>
NlKernel pick(int kind, bool conv, bool nls) {
  if (kind == FDS_NL1D_IDEAL_GAS) {
    if (conv && nls) return nl1d_kernel<EXACT, FDS_NL1D_IDEAL_GAS, true, true, CLUSTER>;
    if (conv) return nl1d_kernel<EXACT, FDS_NL1D_IDEAL_GAS, true, false, CLUSTER>;
    if (nls) return nl1d_kernel<EXACT, FDS_NL1D_IDEAL_GAS, false, true, CLUSTER>;
    return nl1d_kernel<EXACT, FDS_NL1D_IDEAL_GAS, false, false, CLUSTER>;
  }
  return nl1d_kernel<EXACT, FDS_NL1D_SECOND_ORDER, true, false, CLUSTER>;
}

constexpr int kNlMaxClusterCta = 16;  // with the non-portable cluster size allowed

// Whether one cluster of `ctas` CTAs of `fn` (threads each, no dynamic shared memory)
// can be scheduled: the portable size always, up to 16 where the device allows it.
bool nl_cluster_fits(NlKernel fn, int ctas, int threads) {
  if (ctas > kNlMaxClusterCta) return false;
  if (ctas <= 8) return true;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)ctas;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3((unsigned)ctas, 1, 1);
  cfg.blockDim = dim3((unsigned)threads, 1, 1);
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int clusters = 0;
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess ||
      cudaOccupancyMaxActiveClusters(&clusters, fn, &cfg) != cudaSuccess || clusters < 1) {
    (void)cudaGetLastError();
    return false;
  }
  return true;
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
  if (!prob->a || !prob->rho0 || !prob->e1 || !prob->e2 || !prob->sync)
    return set_error(FDS_E_ARG, "missing coefficient arrays or barrier counter");
  for (int k = 0; k < 3; ++k) {
    if (!st->cur[k] || (k > 0 && !st->nxt[k])) return set_error(FDS_E_ARG, "missing state buffer %d", k);
    const FdsCompTables& t = tables->comp[k];
    if (t.probe_tile_start && (!t.out || t.out_rows < nsteps))
      return set_error(FDS_E_ARG, "output buffer of component %d too small", k);
  }
  if (nsteps == 0) return FDS_OK;
  const int ntiles = (prob->n + prob->tile_x - 1) / prob->tile_x;
  // steps per launch: two barriers per step, kMaxBarrierArrivals per launch
  const int64_t per_launch = kMaxBarrierArrivals / (2 * (int64_t)ntiles);
  if (per_launch < 1) return set_error(FDS_E_SIZE, "too many tiles (%d)", ntiles);
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
  a.sync = prob->sync;
  a.status = prob->status;
  a.n = prob->n;
  a.tile = prob->tile_x;
  a.ntiles = ntiles;
  a.step0 = step0;
  a.nsteps = nsteps;
  const bool conv = prob->kind == FDS_NL1D_SECOND_ORDER || (prob->flags & FDS_NL1D_CONVECTIVE);
  const bool nls = (prob->flags & FDS_NL1D_NL_STATE) != 0;
  const bool exact = (prob->flags & FDS_FLAG_EXACT) != 0;
  const int threads = prob->tile_x < 256 ? ((prob->tile_x + 31) / 32) * 32 : 256;
  cudaStream_t s = (cudaStream_t)stream;
  // a grid of at most 16 tiles: one cluster, every step in one launch with hardware
  // barriers (no barrier counter, no per-launch step limit)
  NlKernel fc = exact ? pick<true, true>(prob->kind, conv, nls) : pick<false, true>(prob->kind, conv, nls);
  if (nl_cluster_fits(fc, ntiles, threads)) {
    a.step0 = step0;
    a.row0 = 0;
    a.nsteps = nsteps;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)ntiles;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3((unsigned)ntiles, 1, 1);
    cfg.blockDim = dim3((unsigned)threads, 1, 1);
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, fc, a);
    if (e != cudaSuccess)
      return set_error(FDS_E_LAUNCH, "nonlinear 1-D cluster launch: %s", cudaGetErrorString(e));
    if (nsteps & 1)
      for (int k = 1; k < 3; ++k) std::swap(st->cur[k], st->nxt[k]);
    return FDS_OK;
  }
  NlKernel fn = exact ? pick<true, false>(prob->kind, conv, nls) : pick<false, false>(prob->kind, conv, nls);
  // every CTA waits for the others at the grid barriers: all must be resident
  int dev = 0, sms = 0, per_sm = 0, coop = 0;
  cudaError_t q = cudaGetDevice(&dev);
  if (q == cudaSuccess) q = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  if (q == cudaSuccess) q = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (q == cudaSuccess)
    q = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)fn, threads, 0);
  if (q != cudaSuccess)
    return set_error(FDS_E_LAUNCH, "nonlinear 1-D residency query: %s", cudaGetErrorString(q));
  if (!coop || (int64_t)per_sm * sms < ntiles)
    return set_error(FDS_E_SIZE, "%d tiles cannot all be resident (%d per SM x %d SMs)", ntiles,
                     per_sm, sms);
  for (int64_t done = 0; done < nsteps;) {
    const int32_t m = (int32_t)std::min<int64_t>(per_launch, nsteps - done);
    a.step0 = step0 + done;
    a.row0 = done;
    a.nsteps = m;
    cudaError_t e = cudaMemsetAsync(prob->sync, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess) return set_error(FDS_E_LAUNCH, "barrier reset: %s", cudaGetErrorString(e));
    void* params[] = {&a};
    e = cudaLaunchCooperativeKernel((const void*)fn, dim3(ntiles), dim3(threads), params, 0, s);
    if (e != cudaSuccess)
      return set_error(FDS_E_LAUNCH, "nonlinear 1-D launch: %s", cudaGetErrorString(e));
    // velocity and density were ping-ponged once per step
    if (m & 1) {
      std::swap(a.v[0], a.v[1]);
      std::swap(a.r[0], a.r[1]);
      for (int k = 1; k < 3; ++k) std::swap(st->cur[k], st->nxt[k]);
    }
    done += m;
  }
  return FDS_OK;
}
