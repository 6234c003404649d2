// Every step of a ThermoAcoustic1D call in one launch (pyfds/coupled_fields.py:10-65):
// the acoustic step, the thermal step and the loss coupling of the acoustic velocity
// into the temperature (BoundaryCoupling, pyfds/coupling.py, with
// ThermoAcoustic1D._loss_coupling) on the warps of one thread-block cluster, one cell
// of both fields per lane in registers (the scheme of warp_1d.cuh).
//
// A step, in the reference's order: the acoustic flux (its boundary chain and probes),
// the acoustic pressure (the next step's chain and probes), the thermal flux and
// temperature, then the loss from the new acoustic velocity of the cell and the cell
// before it, added to the temperature (or accumulated, every `stepping`-th step added
// with the accumulator), and only then the temperature's next-step chain and probes.
// The loss reads one more cell to the left than the fields' own updates, so a warp's
// window holds G = K + 2 cells past its owned ones on each side; after each block of
// K steps the pressure, velocity, temperature and accumulator of the window edges go
// to the neighbour warps' inboxes. Every value runs the one-field kernels' arithmetic
// (flux_1d, potential_regs, the boundary chains) and the loss kernel's unfused
// product chain, so the results are the per-step launches' bit for bit.
#pragma once

#include "warp_1d.cuh"

namespace fds {

struct TaWarpArgs {
  double* fin[4];     // where the acoustic pressure, velocity, temperature, heat flux end
  const double* rho;  // acoustic density per cell
  const double* g;    // loss factor per cell (viscosity / thermal density / heat capacity)
  double* acc;        // accumulated loss per cell (read at the start, written at the end)
  double dt;
  int64_t step0;
  int32_t nsteps, K, stepping, accumulate, acc_empty;
};

constexpr int kTaArrays = 4;  // exchanged per edge cell: pressure, velocity, temperature, loss
constexpr int kTaWarpsPerCta = 8;  // (256 threads: the registers of two fields per lane)

__host__ __device__ constexpr size_t ta_inbox_bytes(int nwc, int g) {
  return round128((size_t)nwc * 2 * 2 * kTaArrays * g * sizeof(double));
}

// Tables of a field's two components read where they are (global memory).
__device__ __forceinline__ void tables_in_place(const FdsCompTables* tab, int ntiles,
                                                ResidentTables* out) {
  for (int c = 0; c < 2; ++c) {
    out[c].ngroups = tab[c].bound_tile_start ? tab[c].bound_tile_start[ntiles] : 0;
    out[c].nprobes = tab[c].probe_tile_start ? tab[c].probe_tile_start[ntiles] : 0;
    out[c].groups = tab[c].groups;
    out[c].ops = tab[c].ops;
    out[c].probes = tab[c].probes;
    out[c].group_count = nullptr;
  }
}

// One component's per-lane boundary chain and probe of a lane's cell.
struct TaLane {
  LaneBound b;
  int code;        // probe code (-1 none, a column, -2 several)
  double* out;     // the single probe's column pointer (row 0)
  int64_t stride;  // output row stride
  int32_t rows;
};

__device__ __forceinline__ TaLane ta_lane(const ResidentTables& rt, const FdsCompTables& tb,
                                          int2 range, int code, const double* pool,
                                          const double* zero) {
  TaLane l;
  l.b = lane_bound_of<double>(rt, range, pool, zero);
  l.code = code;
  l.out = code >= 0 ? tb.out + code : nullptr;
  l.stride = tb.ncols;
  l.rows = tb.out_rows;
  return l;
}

// The chain and probe of one component for step `step` / output row `row`: MODE 0 none,
// 1 one-operation chains and single probes, 2 any (table chains, several probes on a
// cell).
template <int MODE>
__device__ __forceinline__ double ta_apply(const TaLane& l, const WarpBounds& w,
                                           const ResidentTables& rt, const FdsCompTables& tb,
                                           const double* pool, double v, int64_t step,
                                           int64_t row, int cell) {
  if constexpr (MODE == 1) {
    // a uniform branch skips the components without chains in this warp (running the
    // chain code on every lane would cost more than the branch)
    if (w.fast) v = lane_bound<true>(l.b, v, step);
    if (l.out && row < l.rows) l.out[row * l.stride] = v;
  } else if constexpr (MODE == 2) {
    if (w.fast) v = lane_bound<true>(l.b, v, step);
    if (w.table && l.b.kind == 1) v = bound_chain(rt, l.b.range, v, pool, step);
    if (l.code != -1) probe_cell(rt, tb, l.code, cell, row, v);
  }
  return v;
}

template <class CA, class CT>
__global__ void __launch_bounds__(kTaWarpsPerCta * 32, 1)
    ta_warp_kernel(const __grid_constant__ StagArgs<double, double, double> A,
                   const __grid_constant__ StagArgs<double, double, double> H,
                   const __grid_constant__ TaWarpArgs t) {
  static_assert(!CA::HAS_V && !CT::HAS_V && CA::MEMORY && !CT::MEMORY, "1-D acoustic + thermal");
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int n = (int)A.n;
  const int rank = (int)blockIdx.x;  // the grid is one cluster
  const int nwc = (int)blockDim.x / 32;
  const int wid = (int)threadIdx.x / 32;
  const int lane = (int)threadIdx.x & 31;
  const int K = t.K;
  const int G = K + 2;
  const int m = kWarpLanes - 2 * G;
  const int gw = rank * nwc + wid;
  const int c0 = min(n, gw * m);
  const int c1 = min(n, c0 + m);
  const bool idle = c0 >= c1;
  const int cell = c0 - G + lane;
  const bool in = !idle && cell >= 0 && cell < n;
  const bool own = cell >= c0 && cell < c1;
  const int t0 = min(n, rank * nwc * m);
  const int tbase = t0 - G;
  const int tw = (nwc - 1) * m + kWarpLanes;
  double* inbox = reinterpret_cast<double*>(smem_raw);  // [warp][parity][side][array][G]
  unsigned char* q = smem_raw + ta_inbox_bytes(nwc, G);
  int2* grA = reinterpret_cast<int2*>(q);
  int* pcA = reinterpret_cast<int*>(q + 2 * round128((size_t)(tw + 2) * sizeof(int2)));
  q += warp_slot_bytes(tw);
  int2* grH = reinterpret_cast<int2*>(q);
  int* pcH = reinterpret_cast<int*>(q + 2 * round128((size_t)(tw + 2) * sizeof(int2)));
  __shared__ double s_zero;
  if (threadIdx.x == 0) s_zero = 0.0;
  ResidentTables rA[2], rH[2];
  tables_in_place(A.tab, A.ntiles, rA);
  tables_in_place(H.tab, H.ntiles, rH);
  const int lo = max(tbase, 0), hi = min(tbase + tw, n), t1 = min(n, t0 + nwc * m);
  cluster_slot_tables(rA, grA, pcA, tw, tbase, lo, hi, t0, t1);  // ends with a barrier
  cluster_slot_tables(rH, grH, pcH, tw, tbase, lo, hi, t0, t1);
  TaLane lPa, lFa, lPh, lFh;
  {
    const int slot = in ? cell - tbase + 1 : 0;  // in [1, tw] for lanes in the field
    const int2 none = make_int2(0, 0);
    const bool ok = in;
    lPa = ta_lane(rA[0], A.tab[0], ok ? grA[slot] : none, ok && own ? pcA[slot] : -1, A.pool, &s_zero);
    lFa = ta_lane(rA[1], A.tab[1], ok ? grA[(tw + 2) + slot] : none,
                  ok && own ? pcA[(tw + 2) + slot] : -1, A.pool, &s_zero);
    lPh = ta_lane(rH[0], H.tab[0], ok ? grH[slot] : none, ok && own ? pcH[slot] : -1, H.pool, &s_zero);
    lFh = ta_lane(rH[1], H.tab[1], ok ? grH[(tw + 2) + slot] : none,
                  ok && own ? pcH[(tw + 2) + slot] : -1, H.pool, &s_zero);
  }
  // state and coefficients of the lane's cell (zeros outside the field)
  double p = 0.0, u = 0.0, T = 0.0, qh = 0.0, acc = 0.0;
  double b = 0.0, bm = 0.0, k = 0.0, kn = 0.0, am = 0.0, a0 = 0.0, ap = 0.0;
  double bt = 0.0, btm = 0.0, kt = 0.0, ktn = 0.0, rho = 0.0, rhom = 0.0, gl = 0.0;
  if (in) {
    p = A.p_in[cell];
    u = A.u_in[cell];
    T = H.p_in[cell];
    acc = t.acc[cell];
    b = A.bx[cell];
    k = A.kx[cell];
    bt = H.bx[cell];
    kt = H.kx[cell];
    rho = t.rho[cell];
    gl = t.g[cell];
    if (cell > 0) {
      bm = A.bx[cell - 1];
      btm = H.bx[cell - 1];
      rhom = t.rho[cell - 1];
    }
    if (cell + 1 < n) {
      kn = A.kx[cell + 1];
      ktn = H.kx[cell + 1];
    }
    if constexpr (CA::ABSORB) {
      am = ldg0(A.axm, cell - 1, A.n);
      a0 = ldg0(A.ad, cell, A.n);
      ap = ldg0(A.axp, cell + 1, A.n);
    }
  }
  const unsigned full = 0xffffffffu;
  const WarpBounds wPa = warp_bounds(lPa.b), wFa = warp_bounds(lFa.b);
  const WarpBounds wPh = warp_bounds(lPh.b), wFh = warp_bounds(lFh.b);
  const bool special = __any_sync(full, lPa.b.kind || lFa.b.kind || lPh.b.kind || lFh.b.kind ||
                                             lPa.code != -1 || lFa.code != -1 ||
                                             lPh.code != -1 || lFh.code != -1);
  const bool general = wPa.table || wFa.table || wPh.table || wFh.table ||
                       __any_sync(full, lPa.code == -2 || lFa.code == -2 || lPh.code == -2 ||
                                            lFh.code == -2);
  // the coupling's phase within `stepping` and whether the accumulator is empty (the
  // host's per-step bookkeeping, the same for every thread)
  int phase = (int)(t.step0 % t.stepping);
  int acc_empty = t.acc_empty;
  // every CTA of the cluster runs before a neighbour writes into its shared memory
  cluster_sync();
  int blk = 0;
  for (int32_t s0 = 0; s0 < t.nsteps; s0 += K, ++blk) {
    const int ke = min(K, t.nsteps - s0);
    if (!idle && blk > 0) {
      // the edge lanes from the neighbour warps' last block
      const int par = (blk - 1) & 1;
      const double* bx0 = inbox + (size_t)((wid * 2 + par) * 2 + 0) * kTaArrays * G;
      const double* bx1 = inbox + (size_t)((wid * 2 + par) * 2 + 1) * kTaArrays * G;
      if (gw > 0 && lane < G) {
        p = bx0[lane];
        u = bx0[G + lane];
        T = bx0[2 * G + lane];
        acc = bx0[3 * G + lane];
      }
      const int r = cell - c1;
      if (r >= 0 && r < G && cell < n) {
        p = bx1[r];
        u = bx1[G + r];
        T = bx1[2 * G + r];
        acc = bx1[3 * G + r];
      }
    }
    // each step's coupling mode: 0 add the loss; 1 / 2 start / add to the accumulator;
    // 3 / 4 the same, then add the accumulator; -1 none
#define FDS_TA_STEPS(MODE)                                                                 \
  for (int kk = 0; kk < ke; ++kk) {                                                        \
    const int32_t s = s0 + kk;                                                             \
    const int64_t step = t.step0 + s;                                                      \
    const bool next = s + 1 < t.nsteps;                                                    \
    const bool due = phase == 0;                                                           \
    phase = phase + 1 == t.stepping ? 0 : phase + 1;                                       \
    int mode;                                                                              \
    if (!t.accumulate) {                                                                   \
      mode = due ? 0 : -1;                                                                 \
    } else if (due) {                                                                      \
      mode = acc_empty ? 3 : 4;                                                            \
      acc_empty = 1;                                                                       \
    } else {                                                                               \
      mode = acc_empty ? 1 : 2;                                                            \
      acc_empty = 0;                                                                       \
    }                                                                                      \
    /* acoustic */                                                                         \
    const double pm = shfl_up1(p);                                                         \
    double ul = 0.0, ur = 0.0;                                                             \
    if constexpr (CA::ABSORB) {                                                            \
      ul = shfl_up1(u);                                                                    \
      ur = shfl_down1(u);                                                                  \
    }                                                                                      \
    double un = flux_1d<CA>(A, p, pm, b, bm, u, ul, ur, am, a0, ap);                       \
    un = ta_apply<MODE>(lFa, wFa, rA[1], A.tab[1], A.pool, un, step, s, cell);             \
    if (in) u = un;                                                                        \
    const double un1 = shfl_down1(u);                                                      \
    double pn = potential_regs<CA>(A, p, u, un1, 0.0, 0.0, k, kn, 0.0, 0.0, cell);         \
    if (next) pn = ta_apply<MODE>(lPa, wPa, rA[0], A.tab[0], A.pool, pn, step + 1, s + 1, cell); \
    if (in) p = pn;                                                                        \
    /* thermal */                                                                          \
    const double Tm = shfl_up1(T);                                                         \
    double qn = flux_1d<CT>(H, T, Tm, bt, btm, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0);              \
    qn = ta_apply<MODE>(lFh, wFh, rH[1], H.tab[1], H.pool, qn, step, s, cell);             \
    if (in) qh = qn;                                                                       \
    const double qn1 = shfl_down1(qh);                                                     \
    double Tn = potential_regs<CT>(H, T, qh, qn1, 0.0, 0.0, kt, ktn, 0.0, 0.0, cell);      \
    /* the loss of this step's acoustic velocity (the loss kernel's product chain) */      \
    const double vm = shfl_up1(u);                                                         \
    const double vd0 = cell >= 1 ? xadd(0.0, xmul(-bm, xmul(vm, rhom))) : 0.0;            \
    const double vd = xadd(vd0, xmul(b, xmul(u, rho)));                                    \
    const double loss = xmul(xmul(gl, xmul(vd, vd)), t.dt);                                \
    const double an = (mode == 1 || mode == 3) ? loss : xadd(acc, loss);                   \
    const double tc = xadd(Tn, mode == 0 ? loss : an);                                     \
    Tn = (mode == 0 || mode >= 3) ? tc : Tn;                                               \
    if (in && mode >= 1) acc = an;                                                         \
    if (next) Tn = ta_apply<MODE>(lPh, wPh, rH[0], H.tab[0], H.pool, Tn, step + 1, s + 1, cell); \
    if (in) T = Tn;                                                                        \
  }
    if (!idle) {
      if (!special) {
        FDS_TA_STEPS(0)
      } else if (general) {
        FDS_TA_STEPS(2)
      } else {
        FDS_TA_STEPS(1)
      }
    } else {
      // (the coupling's bookkeeping advances for every warp alike)
      for (int kk = 0; kk < ke; ++kk) {
        const bool due = phase == 0;
        phase = phase + 1 == t.stepping ? 0 : phase + 1;
        if (t.accumulate) acc_empty = due ? 1 : 0;
      }
    }
#undef FDS_TA_STEPS
    if (s0 + K < t.nsteps) {
      if (!idle) {
        // the first G owned cells to the left warp's right edge, the last G to the
        // right warp's left edge
        const int par = blk & 1;
        if (gw > 0 && own && cell < c0 + G) {
          const int tgt = gw - 1;
          double* dst = inbox + (size_t)(((tgt % nwc) * 2 + par) * 2 + 1) * kTaArrays * G;
          const int o = cell - c0;
          const uint32_t r = (uint32_t)(tgt / nwc);
          st_cluster(&dst[o], r, p);
          st_cluster(&dst[G + o], r, u);
          st_cluster(&dst[2 * G + o], r, T);
          st_cluster(&dst[3 * G + o], r, acc);
        }
        if (c1 < n && own && cell >= c1 - G) {
          const int tgt = gw + 1;
          double* dst = inbox + (size_t)(((tgt % nwc) * 2 + par) * 2 + 0) * kTaArrays * G;
          const int o = cell - (c1 - G);
          const uint32_t r = (uint32_t)(tgt / nwc);
          st_cluster(&dst[o], r, p);
          st_cluster(&dst[G + o], r, u);
          st_cluster(&dst[2 * G + o], r, T);
          st_cluster(&dst[3 * G + o], r, acc);
        }
      }
      cluster_sync();
    }
  }
  bool bad_a = false, bad_h = false;
  if (own) {
    t.fin[0][cell] = p;
    t.fin[1][cell] = u;
    t.fin[2][cell] = T;
    t.fin[3][cell] = qh;
    t.acc[cell] = acc;
    bad_a = nonfinite(p);
    bad_h = nonfinite(T);
  }
  // each field's own status word
  if (A.status && __any_sync(full, bad_a) && lane == 0) atomicOr(A.status, kStatusNonFinite);
  if (H.status && __any_sync(full, bad_h) && lane == 0) atomicOr(H.status, kStatusNonFinite);
}

}  // namespace fds
