// Register-marching staggered step for lossless 2-D fields (the hot path).
//
// One warp owns a strip of W = 32*CX - 2 columns and TY rows. Lane L holds the
// CX consecutive cells x0 + L*CX + k (k < CX) of a row, x0 = c0 - 1: cell j = 0 is
// the left halo column c0 - 1 and cell j = 32*CX - 1 the right halo column c0 + W,
// so every x-neighbour is in the warp (register or shuffle) and all lanes run the
// same instructions. The warp walks down its rows keeping three rows in registers:
// the current row y, row y + 1 (whose new fluxes the potential update of row y
// needs) and row y + 2 (loads in flight, prefetched one iteration ahead).
//
// Per row the order is the reference's sim_step order (pyfds/acoustics.py:111-128):
// new fluxes of row y+1 -> their boundaries and outputs -> new potential of row y
// -> next step's potential boundaries and outputs of row y -> stores. Boundaries
// and outputs come from the per-task tables sorted by slot (row-major), consumed by
// a cursor per component. Cells are addressed by flat index x + y*nx, so the
// reference's row-end wrap and the dropping of out-of-range neighbours need no
// special case; slots of out-of-range cells hold exact zeros.
//
// No shared memory and no CTA barrier: warps of a CTA are independent.
#pragma once

#include "stag_kernel.cuh"

namespace fds {

template <int CX_, int TY_, int NW_, bool MEMORY_>
struct MarchCfg {
  static constexpr int CX = CX_;
  static constexpr int TY = TY_;
  static constexpr int NW = NW_;  // warps per CTA
  static constexpr int NT = NW * 32;
  static constexpr int WW = 32 * CX;  // cells per warp row (slot stride)
  static constexpr int W = WW - 2;    // owned columns per warp
  static constexpr bool MEMORY = MEMORY_;
};

template <typename T>
__device__ __forceinline__ T shfl_up1(T v) {
  return __shfl_up_sync(0xffffffffu, v, 1);
}
template <typename T>
__device__ __forceinline__ T shfl_down1(T v) {
  return __shfl_down_sync(0xffffffffu, v, 1);
}

// Loads one row of a lane's CX cells (out-of-range cells read as zero).
#define FDS_MARCH_ROW(S)                                                   \
  TP S##p[CX];                                                             \
  TF S##uo[CX], S##vo[CX];                                                 \
  TC S##bx[CX], S##by[CX], S##kx[CX], S##ky[CX];

#define FDS_MARCH_LOAD(S, Y)                                               \
  _Pragma("unroll") for (int k = 0; k < CX; ++k) {                         \
    const int64_t f_ = (int64_t)(Y) * a.nx + xl + k;                       \
    const bool ok_ = (f_ >= 0 && f_ < a.n);                                \
    const int64_t g_ = ok_ ? f_ : 0;                                       \
    S##p[k] = ok_ ? a.p_in[g_] : TP(0);                                    \
    if constexpr (C::MEMORY) {                                             \
      S##uo[k] = ok_ ? a.u_in[g_] : TF(0);                                 \
      S##vo[k] = ok_ ? a.v_in[g_] : TF(0);                                 \
    } else {                                                               \
      S##uo[k] = TF(0);                                                    \
      S##vo[k] = TF(0);                                                    \
    }                                                                      \
    S##bx[k] = ok_ ? __ldg(a.bx + g_) : TC(0);                             \
    S##kx[k] = ok_ ? __ldg(a.kx + g_) : TC(0);                             \
    if (!iso) {                                                            \
      S##by[k] = ok_ ? __ldg(a.by + g_) : TC(0);                           \
      S##ky[k] = ok_ ? __ldg(a.ky + g_) : TC(0);                           \
    } else {                                                               \
      S##by[k] = S##bx[k];                                                 \
      S##ky[k] = S##kx[k];                                                 \
    }                                                                      \
  }

#define FDS_MARCH_COPY(D, S)                                               \
  _Pragma("unroll") for (int k = 0; k < CX; ++k) {                         \
    D##p[k] = S##p[k];                                                     \
    D##uo[k] = S##uo[k];                                                   \
    D##vo[k] = S##vo[k];                                                   \
    D##bx[k] = S##bx[k];                                                   \
    D##by[k] = S##by[k];                                                   \
    D##kx[k] = S##kx[k];                                                   \
    D##ky[k] = S##ky[k];                                                   \
  }

// New fluxes of one row (cur*) from that row and the row above (up*).
template <class C, typename TP, typename TF, typename TC>
__device__ __forceinline__ void march_flux_row(const StagCore<TP, TF, TC>& a, int y, int xl,
                                               bool want_x, const TP (&up_p)[C::CX],
                                               const TC (&up_by)[C::CX], const TP (&cp)[C::CX],
                                               const TF (&cuo)[C::CX], const TF (&cvo)[C::CX],
                                               const TC (&cbx)[C::CX], const TC (&cby)[C::CX],
                                               TF (&uo)[C::CX], TF (&vo)[C::CX]) {
  constexpr int CX = C::CX;
  // x-neighbour (left) of this lane's first cell comes from the previous lane
  const TP pl = shfl_up1(cp[CX - 1]);
  const TC bl = shfl_up1(cbx[CX - 1]);
#pragma unroll
  for (int k = 0; k < CX; ++k) {
    const int64_t f = (int64_t)y * a.nx + xl + k;
    const bool ok = (f >= 0 && f < a.n);
    const TF p = (TF)cp[k];
    const TF pm = (TF)(k == 0 ? pl : cp[k - 1]);
    const TF b = (TF)cbx[k];
    const TF bm = (TF)(k == 0 ? bl : cbx[k - 1]);
    const TF by = (TF)cby[k];
    const TF bym = (TF)up_by[k];
    const TF pym = (TF)up_p[k];
    TF u = TF(0), v;
    if constexpr (C::MEMORY) {
      if (want_x) u = fma(bm, pm, fma(-b, p, cuo[k]));
      v = fma(bym, pym, fma(-by, p, cvo[k]));
    } else if constexpr (sizeof(TP) > sizeof(TF)) {
      // float64 potential: form the flux difference in float64 (see flux_new)
      const TP pk = cp[k];
      if (want_x) u = (TF)fma((TP)bm, (TP)(k == 0 ? pl : cp[k - 1]), -((TP)b * pk));
      v = (TF)fma((TP)bym, (TP)up_p[k], -((TP)by * pk));
    } else {
      // float32 temperature stored as T - offset (see flux_new)
      const TF off = (TF)a.offset;
      if (want_x) u = fma(-(b - bm), off, fma(bm, pm, -(b * p)));
      v = fma(-(by - bym), off, fma(bym, pym, -(by * p)));
    }
    uo[k] = ok ? u : TF(0);
    vo[k] = ok ? v : TF(0);
  }
}

// Boundary groups of the current row for one component: groups are sorted by
// slot, so the cursor advances through the rows of the task in order.
template <int CX, int WW, typename T>
__device__ __forceinline__ void march_bounds(const FdsCompTables& tb, int& cur, int end, int row,
                                             int lane, T (&v)[CX], const double* pool,
                                             int64_t step) {
  while (cur < end) {
    const FdsBoundGroup g = tb.groups[cur];
    if (g.pos / WW != row) break;
    const int j = g.pos % WW;
    if (lane == j / CX) {
      const int kk = j % CX;
#pragma unroll
      for (int k = 0; k < CX; ++k) {
        if (k == kk) {
          T x = v[k];
          for (int o = g.op_begin; o < g.op_end; ++o) {
            const FdsBoundOp op = tb.ops[o];
            const double val = (op.flags & FDS_BOP_SIGNAL)
                                   ? pool[op.off + step * (int64_t)op.stride] + op.scalar
                                   : op.scalar;
            x = xadd(xmul((T)op.mul, x), (T)val);
          }
          v[k] = x;
        }
      }
    }
    ++cur;
  }
}

template <int CX, int WW, typename T>
__device__ __forceinline__ void march_probes(const FdsCompTables& tb, int& cur, int end, int row,
                                             int lane, const T (&v)[CX], int64_t out_row) {
  while (cur < end) {
    const FdsProbe pr = tb.probes[cur];
    if (pr.pos / WW != row) break;
    const int j = pr.pos % WW;
    if (lane == j / CX && out_row >= 0 && out_row < tb.out_rows) {
      const int kk = j % CX;
      T x = v[0];
#pragma unroll
      for (int k = 1; k < CX; ++k)
        if (k == kk) x = v[k];
      tb.out[out_row * (int64_t)tb.ncols + pr.col] = (double)x;
    }
    ++cur;
  }
}

template <class C, typename TP, typename TF, typename TC>
__global__ void __launch_bounds__(C::NT, 4)
    march_step_kernel(const __grid_constant__ StagArgs<TP, TF, TC> a) {
  constexpr int CX = C::CX, TY = C::TY, WW = C::WW, W = C::W;
  const int lane = threadIdx.x & 31;
  const int task = blockIdx.x * C::NW + (threadIdx.x >> 5);
  if (task >= a.ntiles) return;  // the whole warp leaves together
  const bool iso = a.iso != 0;
  const int ty = tile_row(a, task);
  const int tx = task - ty * a.tiles_x;
  const int c0 = tx * W;
  const int y0 = ty * TY;
  const int cend = min(c0 + W, a.nx);  // owned columns [c0, cend)
  const int yend = min(y0 + TY, a.ny);  // owned rows [y0, yend)
  const int xl = c0 - 1 + lane * CX;    // column of this lane's first cell

  // table cursors (groups and probes of this task, sorted by slot)
  const FdsCompTables& T0 = a.tab[0];
  const FdsCompTables& T1 = a.tab[1];
  const FdsCompTables& T2 = a.tab[2];
  int b0 = 0, e0 = 0, b1 = 0, e1 = 0, b2 = 0, e2 = 0;
  int q0 = 0, f0 = 0, q1 = 0, f1 = 0, q2 = 0, f2 = 0;
  if (T0.bound_tile_start) { b0 = T0.bound_tile_start[task]; e0 = T0.bound_tile_start[task + 1]; }
  if (T1.bound_tile_start) { b1 = T1.bound_tile_start[task]; e1 = T1.bound_tile_start[task + 1]; }
  if (T2.bound_tile_start) { b2 = T2.bound_tile_start[task]; e2 = T2.bound_tile_start[task + 1]; }
  if (T0.probe_tile_start) { q0 = T0.probe_tile_start[task]; f0 = T0.probe_tile_start[task + 1]; }
  if (T1.probe_tile_start) { q1 = T1.probe_tile_start[task]; f1 = T1.probe_tile_start[task + 1]; }
  if (T2.probe_tile_start) { q2 = T2.probe_tile_start[task]; f2 = T2.probe_tile_start[task + 1]; }

  // which of my cells this task owns
  bool own_x[CX];
#pragma unroll
  for (int k = 0; k < CX; ++k) own_x[k] = (xl + k >= c0 && xl + k < cend);

  // rows in registers: R = current row, N = next row, F = prefetched row
  FDS_MARCH_ROW(R)
  FDS_MARCH_ROW(N)
  FDS_MARCH_ROW(F)
  FDS_MARCH_LOAD(R, y0 - 1)  // only its potential and y factor are used
  FDS_MARCH_LOAD(N, y0)
  FDS_MARCH_LOAD(F, y0 + 1)

  TF ux[CX], vy[CX];  // new fluxes of the current row
  TF uxn[CX], vyn[CX];

  // fluxes of row y0 (the y flux needs row y0 - 1)
  march_flux_row<C>(a, y0, xl, true, Rp, Rby, Np, Nuo, Nvo, Nbx, Nby, ux, vy);
  march_bounds<CX, WW>(T1, b1, e1, 0, lane, ux, a.pool, a.step);
  march_bounds<CX, WW>(T2, b2, e2, 0, lane, vy, a.pool, a.step);
  march_probes<CX, WW>(T1, q1, f1, 0, lane, ux, a.step - a.step0);
  march_probes<CX, WW>(T2, q2, f2, 0, lane, vy, a.step - a.step0);
  FDS_MARCH_COPY(R, N)
  FDS_MARCH_COPY(N, F)

#pragma unroll 1
  for (int ly = 0; ly < TY; ++ly) {
    const int y = y0 + ly;
    if (y >= a.ny) break;
    FDS_MARCH_LOAD(F, y + 2)  // prefetch
    // fluxes of row y + 1 (the x flux only where row y + 1 is owned)
    const bool next_owned = (ly + 1 < TY) && (y + 1 < yend);
    march_flux_row<C>(a, y + 1, xl, next_owned, Rp, Rby, Np, Nuo, Nvo, Nbx, Nby, uxn, vyn);
    if (next_owned) march_bounds<CX, WW>(T1, b1, e1, ly + 1, lane, uxn, a.pool, a.step);
    march_bounds<CX, WW>(T2, b2, e2, ly + 1, lane, vyn, a.pool, a.step);
    if (next_owned) {
      march_probes<CX, WW>(T1, q1, f1, ly + 1, lane, uxn, a.step - a.step0);
      march_probes<CX, WW>(T2, q2, f2, ly + 1, lane, vyn, a.step - a.step0);
    }
    // potential of row y
    const TF uxr = shfl_down1(ux[0]);
    const TC kxr = shfl_down1(Rkx[0]);
    TP pn[CX];
#pragma unroll
    for (int k = 0; k < CX; ++k) {
      const TF un1 = (k == CX - 1) ? uxr : ux[k + 1];
      const TF kxn = (TF)((k == CX - 1) ? kxr : Rkx[k + 1]);
      const TF kxi = (TF)Rkx[k];
      const TF kyi = (TF)Rky[k];
      const TF kyn = (TF)Nky[k];
      if constexpr (sizeof(TP) == sizeof(TF)) {
        TF acc = (TF)Rp[k];
        acc = fma(kxi, ux[k], acc);
        acc = fma(-kxn, un1, acc);
        acc = fma(kyi, vy[k], acc);
        acc = fma(-kyn, vyn[k], acc);
        pn[k] = (TP)acc;
      } else {
        TF inc = kxi * ux[k];
        inc = fma(-kxn, un1, inc);
        inc = fma(kyi, vy[k], inc);
        inc = fma(-kyn, vyn[k], inc);
        pn[k] = Rp[k] + (TP)inc;
      }
    }
    if (a.apply_next) {
      march_bounds<CX, WW>(T0, b0, e0, ly, lane, pn, a.pool, a.step + 1);
      march_probes<CX, WW>(T0, q0, f0, ly, lane, pn, a.step + 1 - a.step0);
    }
    // stores of the owned cells of row y
#pragma unroll
    for (int k = 0; k < CX; ++k) {
      if (own_x[k] && y < yend) {
        const int64_t f = (int64_t)y * a.nx + xl + k;
        a.p_out[f] = pn[k];
        if (a.store_flux) {
          a.u_out[f] = ux[k];
          a.v_out[f] = vy[k];
        }
      }
    }
    FDS_MARCH_COPY(R, N)
    FDS_MARCH_COPY(N, F)
#pragma unroll
    for (int k = 0; k < CX; ++k) {
      ux[k] = uxn[k];
      vy[k] = vyn[k];
    }
  }
}

#undef FDS_MARCH_ROW
#undef FDS_MARCH_LOAD
#undef FDS_MARCH_COPY

}  // namespace fds
