// Every step of a call for a 1-D field on the warps of one thread-block cluster, one
// cell per lane in registers (pyfds/acoustics.py:40-52, pyfds/thermal.py:46-51,
// repeated by Field.simulate, pyfds/fields.py:87-93).
//
// Warp w owns the cells [c0, c1) = [w m, min(n, (w + 1) m)); lane l holds cell
// c0 - G + l (G = K + 1), so a warp's 32 lanes cover its cells and G more on each
// side (m + 2 G <= 32). A step is two register updates with no barrier and no
// shared-memory access: the flux of cell i needs the potential of cell i - 1 (a
// shuffle up; with absorption the old fluxes of cells i - 1 and i + 1, a shuffle
// each), its potential the new flux of cell i + 1 (a shuffle down). Lane 0 has no
// left neighbour and lane 31 no right one, so their values go wrong, and the error
// moves inwards by one cell per step: after K steps the owned lanes (G to G + m - 1)
// are still exact, as in the shared-memory window kernel (cluster_1d.cuh). After each
// block of K steps, each warp writes the potential and flux of its first G owned
// cells into the left neighbour warp's inbox and of its last G into the right one's
// (in this CTA's shared memory or, for the first and last warp of a CTA, the
// neighbouring CTA's, through distributed shared memory); one cluster barrier, and
// the next block starts by reading the inbox into the edge lanes. The inboxes are
// double-buffered by block parity (the argument of cluster_1d.cuh).
//
// Each lane's boundary chain and probe code are looked up once (cluster_slot_tables
// over the CTA's cells, the chain then held in registers, LaneBound); every value runs
// flux_1d / potential_regs and the chain's arithmetic, the tile kernel's, so the owned
// cells are the tile kernel's bit for bit. Warps without a boundary cell or a probe
// (most of them) step through a loop without either, warps with one-operation chains
// and single probes through straight-line code (a branch inside the step loop costs
// tens of cycles of a step's few hundred), others through a loop with the table chains.
// Lanes of cells outside the field keep zeros (the neighbours the reference's
// operators drop); a warp past the field's end only takes part in the barriers.
#pragma once

#include "cluster_1d.cuh"
#include "march_kernel.cuh"

namespace fds {

constexpr int kWarpLanes = 32;           // cells of a warp's window: one per lane
constexpr int kWarpMaxPerCta = 16;       // warps per CTA (512 threads, 128 registers each)
constexpr int kWarpDefaultBlockSteps = 7;
constexpr int kWarpMaxBlockSteps = 9;    // m = 32 - 2 (K + 1) >= K + 1

// Owned cells per warp with K steps per block.
__host__ __device__ constexpr int warp_owned_cells(int k) { return kWarpLanes - 2 * (k + 1); }

// Shared memory of the inboxes of nwc warps with window edges of g cells: potential and
// flux, two block parities, two sides.
template <typename TP, typename TF>
__host__ __device__ constexpr size_t warp_inbox_bytes(int nwc, int g) {
  return round128((size_t)nwc * 4 * g * sizeof(TP)) + round128((size_t)nwc * 4 * g * sizeof(TF));
}

// Shared memory of the per-cell boundary ranges and probe codes of w cells.
__host__ __device__ constexpr size_t warp_slot_bytes(int w) {
  return 2 * round128((size_t)(w + 2) * sizeof(int2)) + 2 * round128((size_t)(w + 2) * sizeof(int));
}

__device__ __forceinline__ dw shfl_up1(dw v) {
  return dw(__shfl_up_sync(0xffffffffu, v.hi, 1), __shfl_up_sync(0xffffffffu, v.lo, 1));
}
__device__ __forceinline__ dw shfl_down1(dw v) {
  return dw(__shfl_down_sync(0xffffffffu, v.hi, 1), __shfl_down_sync(0xffffffffu, v.lo, 1));
}

// A cell's boundary chain held in registers. A chain of one operation whose factor is
// exactly +1 (an additive boundary) or +0 (a held value) and whose value is a constant
// or a signal sample (with no constant added), the forms pyfds's boundaries take on a
// float64 field, is applied by lane_bound without the multiplication: 1 * v is v, and
// 0 * v is a zero with v's sign (NaN for a non-finite v), so the one addition left
// has the table chain's operands and gives its result bit for bit. Other chains run
// bound_chain from the tables.
struct LaneBound {
  int32_t kind;         // 0 none, 1 the table chain, 2 factor +1, 3 factor +0
  int32_t signal;       // the value is the signal sample src[off + step * stride]
  int32_t stride;       // (0 without a signal: src[0] is then a readable zero)
  int32_t pad;
  int64_t off;
  const double* src;    // the signal pool, or a zero in shared memory
  double value;         // the constant value (no signal)
  int2 range;           // the table chain's operations
};

template <typename T>
__device__ __forceinline__ LaneBound lane_bound_of(const ResidentTables& t, int2 r,
                                                   const double* pool, const double* zero) {
  LaneBound lb{0, 0, 0, 0, 0, zero, 0.0, r};
  if (r.y <= r.x) return lb;
  lb.kind = 1;
  if constexpr (std::is_same<T, double>::value) {
    if (r.y - r.x == 1) {
      const FdsBoundOp op = t.ops[r.x];
      const long long mb = __double_as_longlong(op.mul);
      const bool signal = (op.flags & FDS_BOP_SIGNAL) != 0;
      if ((mb == 0x3FF0000000000000ll || mb == 0) &&
          (!signal || __double_as_longlong(op.scalar) == 0)) {
        lb.kind = mb ? 2 : 3;
        lb.signal = signal;
        if (signal) {
          lb.src = pool;
          lb.off = op.off;
          lb.stride = op.stride;
        }
        lb.value = op.scalar;
      }
    }
  }
  return lb;
}

// The fast chain of each lane applied to its new value v (lanes without one keep v),
// in straight-line code: ADD (compile-time for the warp: some lane has factor +1 or a
// signal value) runs the one addition for the warp; without it, chains of held
// constants take integer operations only.
template <bool ADD>
__device__ __forceinline__ double lane_bound(const LaneBound& lb, double v, int64_t step) {
  constexpr long long kSign = (long long)0x8000000000000000ull;
  constexpr long long kNaN = 0x7FF8000000000000ll;
  const long long vb = __double_as_longlong(v);
  const bool nf = nonfinite(v);
  // xmul(mul, v): v for factor +1; for factor +0 a zero with v's sign, NaN past finite
  const long long zb = lb.kind == 3 ? (nf ? kNaN : (vb & kSign)) : vb;
  long long wb = __double_as_longlong(lb.value);
  double r;
  if constexpr (ADD) {
    // the sample + 0.0: the sample with a negative zero made positive
    long long xb = __double_as_longlong(lb.src[lb.off + step * (int64_t)lb.stride]);
    xb = xb == kSign ? 0 : xb;
    wb = lb.signal ? xb : wb;
    r = xadd(__longlong_as_double(zb), __longlong_as_double(wb));
  } else {
    // held constants: zb + value is the value, or for a zero value a zero that is
    // negative only when both are (NaN for a non-finite v)
    r = nf ? __longlong_as_double(kNaN)
           : (((unsigned long long)wb << 1) != 0) ? __longlong_as_double(wb)
           : (zb < 0 && wb < 0) ? -0.0 : 0.0;
  }
  return lb.kind >= 2 ? r : v;
}

// Warp-uniform summary of the lanes' chains of one component: any fast chain, any that
// needs the addition (factor +1, or a signal value), any table chain.
struct WarpBounds {
  bool fast, add, table;
};

__device__ __forceinline__ WarpBounds warp_bounds(const LaneBound& lb) {
  const unsigned full = 0xffffffffu;
  return {__any_sync(full, lb.kind >= 2) != 0,
          __any_sync(full, lb.kind == 2 || (lb.kind == 3 && lb.signal)) != 0,
          __any_sync(full, lb.kind == 1) != 0};
}

// Dynamic shared memory: the inboxes of the CTA's warps (at offset 0, the same in every
// CTA of the cluster), the per-cell tables of the CTA's cells, the boundary and probe
// tables, the signal pool when it fits.
template <class C, typename TP, typename TF, typename TC>
__global__ void __launch_bounds__(kWarpMaxPerCta * 32, 1)
    stag_1d_warp_kernel(const __grid_constant__ StagArgs<TP, TF, TC> a, int32_t nsteps,
                        TP* p_fin, TF* u_fin, int64_t pool_cached, int32_t K) {
  static_assert(!C::HAS_V, "1-D fields");
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int n = (int)a.n;
  const int rank = (int)blockIdx.x;  // the grid is one cluster
  const int nwc = (int)blockDim.x / 32;
  const int wid = (int)threadIdx.x / 32;
  const int lane = (int)threadIdx.x & 31;
  const int G = K + 1;
  const int m = warp_owned_cells(K);
  const int gw = rank * nwc + wid;
  const int c0 = min(n, gw * m);
  const int c1 = min(n, c0 + m);
  const bool idle = c0 >= c1;  // (warp-uniform)
  const int cell = c0 - G + lane;
  const bool in = !idle && cell >= 0 && cell < n;
  const bool own = cell >= c0 && cell < c1;
  // the CTA's cells, as far as its lanes reach: [tbase, tbase + tw)
  const int t0 = min(n, rank * nwc * m);
  const int tbase = t0 - G;
  const int tw = (nwc - 1) * m + kWarpLanes;
  TP* inP = reinterpret_cast<TP*>(smem_raw);  // [warp][parity][side: 0 left, 1 right][G]
  TF* inU = reinterpret_cast<TF*>(smem_raw + round128((size_t)nwc * 4 * G * sizeof(TP)));
  unsigned char* q = smem_raw + warp_inbox_bytes<TP, TF>(nwc, G);
  int2* gr = reinterpret_cast<int2*>(q);
  int* pc = reinterpret_cast<int*>(q + 2 * round128((size_t)(tw + 2) * sizeof(int2)));
  unsigned char* area = q + warp_slot_bytes(tw);
  ResidentTables rt[2];
  stage_tables(a.tab, a.ntiles, area, rt);  // ends with a barrier
  const double* pool = a.pool;
  if (pool_cached > 0) {
    double* sp = reinterpret_cast<double*>(area + kResidentTableBytes);
    for (int64_t i = threadIdx.x; i < pool_cached; i += blockDim.x) sp[i] = a.pool[i];
    pool = sp;
  }
  cluster_slot_tables(rt, gr, pc, tw, tbase, max(tbase, 0), min(tbase + tw, n), t0,
                      min(n, t0 + nwc * m));  // ends with a barrier
  __shared__ double s_zero;  // the signal source of lanes without a signal
  if (threadIdx.x == 0) s_zero = 0.0;
  LaneBound bP = lane_bound_of<TP>(rt[0], make_int2(0, 0), pool, &s_zero);
  LaneBound bF = lane_bound_of<TF>(rt[1], make_int2(0, 0), pool, &s_zero);
  int cP = -1, cF = -1;  // probe codes (-1: none, a column, -2: several)
  TP p = TP(0);
  TF u = TF(0), k = TF(0), kn = TF(0), am = TF(0), a0 = TF(0), ap = TF(0);
  TC b = TC(0), bm = TC(0);
  if (in) {
    const int slot = cell - tbase + 1;  // in [1, tw]
    bP = lane_bound_of<TP>(rt[0], gr[slot], pool, &s_zero);
    bF = lane_bound_of<TF>(rt[1], gr[(tw + 2) + slot], pool, &s_zero);
    if (own) {
      cP = pc[slot];
      cF = pc[(tw + 2) + slot];
    }
    p = a.p_in[cell];
    if constexpr (C::MEMORY) u = a.u_in[cell];
    b = a.bx[cell];
    if (cell > 0) bm = a.bx[cell - 1];
    k = (TF)a.kx[cell];
    if (cell + 1 < n) kn = (TF)a.kx[cell + 1];
    if constexpr (C::MEMORY && C::ABSORB) {
      am = (TF)ldg0(a.axm, cell - 1, a.n);
      a0 = (TF)ldg0(a.ad, cell, a.n);
      ap = (TF)ldg0(a.axp, cell + 1, a.n);
    }
  }
  // a lane's single probe as an output column pointer (row 0) and the row stride
  double* const oP = (cP >= 0) ? a.tab[0].out + cP : nullptr;
  double* const oF = (cF >= 0) ? a.tab[1].out + cF : nullptr;
  const int64_t sP = a.tab[0].ncols, sF = a.tab[1].ncols;
  const int32_t rP = a.tab[0].out_rows, rF = a.tab[1].out_rows;
  // the step loop of a warp: without boundary cells or probes; with the potential's
  // one-operation chains and single probes, in straight-line code holding only the
  // parts the warp has (a branch, or code run for lanes that need none of it, costs
  // tens of cycles of the step's few hundred on the dependent chain); or any other
  // case (the general loop)
  const bool special =
      __any_sync(0xffffffffu, bP.kind != 0 || bF.kind != 0 || cP != -1 || cF != -1);
  const WarpBounds wP = warp_bounds(bP), wF = warp_bounds(bF);
  // straight-line loops cover the potential's one-operation chains and single
  // probes; the flux's chains or probes, table chains and several probes on a cell
  // take the general loop
  const bool general = wP.table || wF.table || wF.fast ||
                       __any_sync(0xffffffffu, cP == -2 || cF != -1);
  const bool pprobe = __any_sync(0xffffffffu, cP != -1);
  // every CTA of the cluster runs before a neighbour writes into its shared memory
  cluster_sync();
  int blk = 0;
  for (int32_t s0 = 0; s0 < nsteps; s0 += K, ++blk) {
    if (!idle) {
      if (blk > 0) {
        // the edge lanes from the neighbour warps' last block
        const int par = (blk - 1) & 1;
        const TP* bp = inP + (wid * 2 + par) * 2 * G;
        const TF* bu = inU + (wid * 2 + par) * 2 * G;
        if (gw > 0 && lane < G) {
          p = bp[lane];
          if constexpr (C::MEMORY) u = bu[lane];
        }
        const int t = cell - c1;
        if (t >= 0 && t < G && cell < n) {
          p = bp[G + t];
          if constexpr (C::MEMORY) u = bu[G + t];
        }
      }
      const int ke = min(K, nsteps - s0);
      // one step: new flux (its boundary chain and probes), new potential (the next
      // step's boundary chain and probes; the last step's are the next call's prologue)
#define FDS_WARP_STEPS(MODE, PB, PP, ADDP)                                             \
  for (int kk = 0; kk < ke; ++kk) {                                                    \
    const int32_t s = s0 + kk;                                                         \
    const TP pm = shfl_up1(p);                                                         \
    TF ul = TF(0), ur = TF(0);                                                         \
    if constexpr (C::MEMORY && C::ABSORB) {                                            \
      ul = shfl_up1(u);                                                                \
      ur = shfl_down1(u);                                                              \
    }                                                                                  \
    TF un = flux_1d<C>(a, p, pm, b, bm, u, ul, ur, am, a0, ap);                        \
    if constexpr (MODE == 2) {                                                         \
      if constexpr (std::is_same<TF, double>::value)                                   \
        if (wF.fast) un = lane_bound<true>(bF, un, a.step + s);                        \
      if (wF.table && bF.kind == 1) un = bound_chain(rt[1], bF.range, un, pool, a.step + s); \
      if (cF != -1) probe_cell(rt[1], a.tab[1], cF, cell, s, un);                      \
    }                                                                                  \
    if (in) u = un;                                                                    \
    const TF un1 = shfl_down1(u);                                                      \
    TP pn = potential_regs<C>(a, p, u, un1, TF(0), TF(0), k, kn, TF(0), TF(0), cell);  \
    if constexpr (MODE == 1) {                                                         \
      const bool next = s + 1 < nsteps;                                                \
      if constexpr (PB && std::is_same<TP, double>::value)                             \
        pn = next ? lane_bound<ADDP>(bP, pn, a.step + s + 1) : pn;                     \
      if constexpr (PP)                                                                \
        if (oP && next && s + 1 < rP) oP[(s + 1) * sP] = (double)pn;                   \
    } else if constexpr (MODE == 2) {                                                  \
      if (s + 1 < nsteps) {                                                            \
        if constexpr (std::is_same<TP, double>::value)                                 \
          if (wP.fast) pn = lane_bound<true>(bP, pn, a.step + s + 1);                  \
        if (wP.table && bP.kind == 1)                                                  \
          pn = bound_chain(rt[0], bP.range, pn, pool, a.step + s + 1);                 \
        if (cP != -1) probe_cell(rt[0], a.tab[0], cP, cell, s + 1, pn);                \
      }                                                                                \
    }                                                                                  \
    if (in) p = pn;                                                                    \
  }
      if (!special) {
        FDS_WARP_STEPS(0, false, false, false)
      } else if (general) {
        FDS_WARP_STEPS(2, false, false, false)
      } else if (!wP.fast) {
        FDS_WARP_STEPS(1, false, true, false)
      } else if (!pprobe) {
        if (wP.add) {
          FDS_WARP_STEPS(1, true, false, true)
        } else {
          FDS_WARP_STEPS(1, true, false, false)
        }
      } else if (wP.add) {
        FDS_WARP_STEPS(1, true, true, true)
      } else {
        FDS_WARP_STEPS(1, true, true, false)
      }
#undef FDS_WARP_STEPS
    }
    if (s0 + K < nsteps) {
      if (!idle) {
        // the first G owned cells to the left warp's right edge, the last G to the
        // right warp's left edge (a neighbour's edge lies within this warp's cells)
        const int par = blk & 1;
        if (gw > 0 && own && cell < c0 + G) {
          const int tgt = gw - 1;
          const int o = (((tgt % nwc) * 2 + par) * 2 + 1) * G + (cell - c0);
          st_cluster(&inP[o], (uint32_t)(tgt / nwc), p);
          if constexpr (C::MEMORY) st_cluster(&inU[o], (uint32_t)(tgt / nwc), u);
        }
        if (c1 < n && own && cell >= c1 - G) {
          const int tgt = gw + 1;
          const int o = (((tgt % nwc) * 2 + par) * 2 + 0) * G + (cell - (c1 - G));
          st_cluster(&inP[o], (uint32_t)(tgt / nwc), p);
          if constexpr (C::MEMORY) st_cluster(&inU[o], (uint32_t)(tgt / nwc), u);
        }
      }
      cluster_sync();
    }
  }
  // (no CTA writes into another's shared memory after the barrier that ends the
  // second-to-last block, so each CTA may leave as soon as it is done)
  bool bad = false;
  if (own) {
    p_fin[cell] = p;
    u_fin[cell] = u;
    bad = nonfinite(p);
  }
  if (a.status && __any_sync(0xffffffffu, bad) && lane == 0)
    atomicOr(a.status, kStatusNonFinite);
}

}  // namespace fds
