// Fused staggered-grid time step for the pyfds field families on sm_103a.
//
// One launch advances one field by one step (pyfds/acoustics.py:111-128 and its
// 1-D / axisymmetric / thermal siblings). A CTA owns a TX x TY tile of cells and
// stages in shared memory everything the step needs around it:
//
//   region  : columns x0-4 .. x0+TX+3, rows y0-1 .. y0+TY+1 (1-D: one row); the
//             4-column left margin keeps every row start 16-byte aligned for TMA
//   sP      : potential (pressure / temperature) after this step's bounds
//   sU, sV  : old flux, then the new flux over the "extended" regions
//             U-ext = [x0, x1] x [y0, y1)   (one column right of the tile)
//             V-ext = [x0, x1) x [y0, y1]   (one row below the tile)
//             which the potential update of the owned cells reads.
//   sBx, sKx (and sBy, sKy unless they equal the x factors): the coefficient
//             tiles, staged with the state so that the FP64 phases read shared
//             memory only (no global-load latency between fused multiply-adds).
//
// Every slot is addressed by the flat index i = x + y*nx of its (x, y), so the
// reference's row-end wrap (cell (nx-1, y) couples to (0, y+1)) and the dropping
// of out-of-range neighbours fall out of the indexing: a slot whose flat index is
// outside [0, n) holds 0 and contributes an exact zero.
//
// Order inside the launch (the reference's sim_step order):
//   flux update (U-ext, V-ext) -> x-flux bounds -> x-flux probes -> y-flux bounds
//   -> y-flux probes -> potential update (owned cells) -> [potential bounds and
//   probes of the NEXT step, unless this is the last step of the call].
// The potential bounds/probes of the first step of a call are applied by a
// separate prologue launch.
//
// Arithmetic: the default F64 form uses fused multiply-adds only (8 DFMA per cell
// and step for a 2-D lossless field, the minimum for this stencil: GB300 issues
// about 2 FP64 lanes per clock per SM, so FP64 instructions, not bytes, bound the
// F64 step). FDS_FLAG_EXACT instead evaluates each DIA product and sum in the
// reference's order with correctly rounded __dmul_rn/__dadd_rn, which reproduces
// scipy's non-fused x86-64 results bit for bit.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "dw.cuh"
#include "fds_capi.h"
#include "tma.cuh"

namespace fds {

// Arguments of one field's step, without the tensor maps (the part the tile code
// reads; a batched CTA keeps a copy of it in shared memory).
template <typename TP, typename TF, typename TC>
struct StagCore {
  int32_t nx, ny;
  int64_t n;
  int32_t tiles_x;
  int32_t tx_shift;  // tile row = (tile * tx_mul) >> tx_shift (division by tiles_x)
  uint64_t tx_mul;
  const TP* p_in;
  TP* p_out;
  const TF* u_in;
  TF* u_out;
  const TF* v_in;
  TF* v_out;
  const TC* bx;
  const TC* by;
  const TC* kx;
  const TC* ky;
  const TC* aym;
  const TC* axm;
  const TC* ad;
  const TC* axp;
  const TC* ayp;
  const TC* ex;
  const TC* rx;
  FdsCompTables tab[3];
  const double* pool;
  int64_t step;
  int64_t step0;
  int32_t apply_next;
  int32_t store_flux;
  int32_t iso;  // by == bx and ky == kx: the y factors are not staged separately
  int32_t ntiles;
  int32_t use_tma;  // stage the region with TMA boxes (tm[]) instead of cp.async
  int32_t prefetch; // TMA path: also prefetch into L2 the region of tile + prefetch (0: off)
  int32_t substeps; // two-step kernel: steps this launch advances (1 or 2)
  int32_t* status;  // OR-ed with kStatus* bits; may be null
  double offset;    // potential stored as value - offset (thermal float32), else 0
};

template <typename TP, typename TF, typename TC>
struct StagArgs : StagCore<TP, TF, TC> {
  // tensor maps of the arrays staged per tile: P, U, V, Bx, Kx, By, Ky
  CUtensorMap tm[7];
};

// Per-launch step fields (shared by every instance of a batched launch).
struct StepInfo {
  int64_t step;
  int64_t step0;
  int32_t apply_next;
  int32_t store_flux;
  int32_t substeps;  // two-step kernels: steps of this launch (1 or 2)
};

template <typename TP, typename TF, typename TC>
__device__ __forceinline__ StepInfo step_of(const StagCore<TP, TF, TC>& a) {
  return StepInfo{a.step, a.step0, a.apply_next, a.store_flux, a.substeps};
}

// Tile row and column of a tile index without an integer division (which the
// compiler builds from float conversions, per thread): the host sets tx_mul =
// ceil(2^(32+l) / tiles_x) and tx_shift = 32 + l with l = ceil(log2(tiles_x)); for
// tile < 2^31 the product stays below 2^64 and the quotient is exact (the rounding
// error of tx_mul adds less than 1 / tiles_x to tile / tiles_x).
template <typename TP, typename TF, typename TC>
__device__ __forceinline__ int tile_row(const StagCore<TP, TF, TC>& a, int tile) {
  return (int)(((uint64_t)(uint32_t)tile * a.tx_mul) >> a.tx_shift);
}

// Cell origin (x0, y0) of a tile.
template <class C, typename TP, typename TF, typename TC>
__device__ __forceinline__ void tile_origin(const StagCore<TP, TF, TC>& a, int tile, int& x0,
                                            int& y0) {
  const int ty = tile_row(a, tile);
  x0 = (tile - ty * a.tiles_x) * C::TX;
  y0 = ty * C::TY;
}

// Host side of tile_row: the multiplier and shift for `tiles_x` columns of tiles.
inline void tile_divider(int32_t tiles_x, uint64_t* mul, int32_t* shift) {
  int l = 0;
  while ((1ll << l) < (long long)tiles_x) ++l;
  *shift = 32 + l;
  *mul = ((1ull << (32 + l)) + (uint64_t)tiles_x - 1) / (uint64_t)tiles_x;
}

// Resident CTAs per SM the 256-thread 2-D tile kernels are compiled for (the
// register budget per thread follows: 65536 / (256 x blocks)). Measured on the
// 2048^2 acoustic step: float64 potential 5 (4: -2 %, 6 spills and loses 6 %),
// float32 potential 6 (4: -8 %). Double words: 5 (the absorbing variants, 4, spill
// at 5).
#ifndef FDS_STAG_BLOCKS_256_F64
#define FDS_STAG_BLOCKS_256_F64 5
#endif
#ifndef FDS_STAG_BLOCKS_256_F32
#define FDS_STAG_BLOCKS_256_F32 6
#endif
#ifndef FDS_STAG_BLOCKS_256_DW
#define FDS_STAG_BLOCKS_256_DW 5
#endif
#ifndef FDS_BATCH_BLOCKS_256
#define FDS_BATCH_BLOCKS_256 4
#endif
// two steps per tile in the batched kernel, 4-byte values: 5 (128.6 -> 136.2
// Gcell/s against 4 on 256 layered instances); 8-byte values keep 4 (at 5 float64
// spills, and their staging holds four CTAs anyway)
#ifndef FDS_BATCH_TB2_BLOCKS_256_F32
#define FDS_BATCH_TB2_BLOCKS_256_F32 5
#endif

// Variant switches of the tile kernel.
template <int TX_, int TY_, int NT_, bool HAS_V_, bool MEMORY_, bool ABSORB_, bool AXI_,
          bool EXACT_, int STAGES_ = 1>
struct StagCfg {
  static constexpr bool TWO_STEP = false;  // two steps per tile (Tb2Cfg)
  static constexpr int STAGES = STAGES_;  // staging buffers (2: persistent, prefetching)
  static constexpr int TX = TX_;
  static constexpr int TY = TY_;
  static constexpr int NT = NT_;
  static constexpr bool HAS_V = HAS_V_;
  static constexpr bool MEMORY = MEMORY_;  // acoustic flux keeps its old value
  static constexpr bool ABSORB = ABSORB_;
  static constexpr bool AXI = AXI_;
  static constexpr bool EXACT = EXACT_;
  static constexpr int OY = HAS_V ? 1 : 0;  // region row of y0
  static constexpr int OX = 4;               // region column of x0 (16-byte aligned start)
  static constexpr int RX = TX + 8;          // region columns x0-4 .. x0+TX+3
  static constexpr int RY = HAS_V ? TY + 3 : TY;
  static constexpr int RN = RX * RY;
  // CTAs per SM of the batched kernel (more registers per thread than the
  // single-field kernel: a tighter budget spills)
  static constexpr int MIN_BLOCKS =
      STAGES == 2 ? 1 : (HAS_V ? (NT >= 512 ? 2 : FDS_BATCH_BLOCKS_256) : 2);
  // CTAs per SM of the single-field kernel for a potential of `psize` bytes per value
  // (`dword`: double-word float32 pairs)
  // CTAs per SM of the batched kernel for values of `psize` bytes
  static constexpr int batch_blocks(int psize) { return MIN_BLOCKS; }
  static constexpr int min_blocks(int psize, bool dword = false) {
    return STAGES == 2 ? 1
                       : (HAS_V ? (NT >= 512 ? 2
                                             : (dword ? (ABSORB ? 4 : FDS_STAG_BLOCKS_256_DW)
                                                      : psize == 4 ? FDS_STAG_BLOCKS_256_F32
                                                                   : FDS_STAG_BLOCKS_256_F64))
                                : 2);
  }
};

template <typename T>
__device__ __forceinline__ T ldg0(const T* p, int64_t i, int64_t n) {
  return (i >= 0 && i < n) ? ldg_t(p + i) : T(0);
}

// Exact (reference-order) arithmetic: correctly rounded, never contracted.
__device__ __forceinline__ double xmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double xadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double xsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float xmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float xadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float xsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ dw xmul(const dw& a, const dw& b) { return a * b; }
__device__ __forceinline__ dw xadd(const dw& a, const dw& b) { return a + b; }
__device__ __forceinline__ dw xsub(const dw& a, const dw& b) { return a - b; }

// NaN or infinity, from the exponent bits (integer instructions only: the FP64 pipe
// stays free for the step's arithmetic).
__device__ __forceinline__ bool nonfinite(double x) {
  return ((__double2hiint(x) >> 20) & 0x7ff) == 0x7ff;
}
__device__ __forceinline__ bool nonfinite(float x) {
  return ((__float_as_uint(x) >> 23) & 0xff) == 0xff;
}
__device__ __forceinline__ bool nonfinite(const dw& x) { return nonfinite(x.hi); }

// Boundary chains of one component for this tile, applied to shared slots.
// new = additive * old + value, additive as a number (pyfds/regions.py:125-145)
template <int NT, typename T>
__device__ __forceinline__ void apply_bound_groups(const FdsCompTables& tb, int tile, T* s,
                                                   const double* pool, int64_t step) {
  if (tb.bound_tile_start == nullptr) return;
  const int b = tb.bound_tile_start[tile];
  const int e = tb.bound_tile_start[tile + 1];
  for (int g = b + (int)threadIdx.x; g < e; g += NT) {
    const FdsBoundGroup grp = tb.groups[g];
    T v = s[grp.pos];
    for (int o = grp.op_begin; o < grp.op_end; ++o) {
      const FdsBoundOp op = tb.ops[o];
      const double val = (op.flags & FDS_BOP_SIGNAL)
                             ? pool[op.off + step * (int64_t)op.stride] + op.scalar
                             : op.scalar;
      v = xadd(xmul((T)op.mul, v), (T)val);
    }
    s[grp.pos] = v;
  }
}

// True if the tile has entries in a per-tile table (tile_start[tile] <
// tile_start[tile + 1]); false for a missing table. The same for every thread.
__device__ __forceinline__ bool tile_has(const int32_t* tile_start, int tile) {
  return tile_start != nullptr && tile_start[tile] < tile_start[tile + 1];
}

template <int NT, typename T>
__device__ __forceinline__ void write_probes(const FdsCompTables& tb, int tile, const T* s,
                                             int64_t row) {
  if (tb.probe_tile_start == nullptr) return;
  if (row < 0 || row >= tb.out_rows) return;
  const int b = tb.probe_tile_start[tile];
  const int e = tb.probe_tile_start[tile + 1];
  double* out = tb.out + row * (int64_t)tb.ncols;
  for (int q = b + (int)threadIdx.x; q < e; q += NT) {
    const FdsProbe pr = tb.probes[q];
    out[pr.col] = (double)s[pr.pos];
  }
}

// Absorption operator a_vx_vx applied at flat index i (slot pos) to the old flux
// held in s: diagonals sorted by offset, as scipy's todia() stores them.
template <class C, typename TP, typename TF, typename TC>
__device__ __forceinline__ TF absorb_term(const StagCore<TP, TF, TC>& a, const TF* s, int pos,
                                          int64_t i) {
  TF acc = TF(0);
  if (C::HAS_V) acc = xadd(acc, xmul((TF)ldg0(a.aym, i - a.nx, a.n), s[pos - C::RX]));
  acc = xadd(acc, xmul((TF)ldg0(a.axm, i - 1, a.n), s[pos - 1]));
  acc = xadd(acc, xmul((TF)ldg0(a.ad, i, a.n), s[pos]));
  acc = xadd(acc, xmul((TF)ldg0(a.axp, i + 1, a.n), s[pos + 1]));
  if (C::HAS_V) acc = xadd(acc, xmul((TF)ldg0(a.ayp, i + a.nx, a.n), s[pos + C::RX]));
  return acc;
}

template <class C, typename TP, typename TF, typename TC>
__device__ __forceinline__ TF absorb_fma(const StagCore<TP, TF, TC>& a, const TF* s, int pos,
                                         int64_t i, TF acc) {
  if (C::HAS_V) acc = fma((TF)ldg0(a.aym, i - a.nx, a.n), s[pos - C::RX], acc);
  acc = fma((TF)ldg0(a.axm, i - 1, a.n), s[pos - 1], acc);
  acc = fma((TF)ldg0(a.ad, i, a.n), s[pos], acc);
  acc = fma((TF)ldg0(a.axp, i + 1, a.n), s[pos + 1], acc);
  if (C::HAS_V) acc = fma((TF)ldg0(a.ayp, i + a.nx, a.n), s[pos + C::RX], acc);
  return acc;
}

// The new flux of a cell of a 1-D field from register operands: the potentials p_ of
// the cell and pm_ of the cell before it, their factors b_ and bm_, the old flux u
// and, with absorption, the old fluxes ul / ur of the neighbour cells and the
// absorption diagonals am / a0 / ap at them (absorb_term's order). flux_new's
// arithmetic, which calls it for 1-D fields.
template <class C, typename TP, typename TF, typename TC>
__device__ __forceinline__ TF flux_1d(const StagCore<TP, TF, TC>& a, TP p_, TP pm_, TC b_,
                                      TC bm_, TF u, TF ul, TF ur, TF am, TF a0, TF ap) {
  static_assert(!C::HAS_V && !C::AXI, "1-D fields");
  const TF b = (TF)b_;
  const TF bm = (TF)bm_;
  const TF p = (TF)p_;
  const TF pm = (TF)pm_;
  if constexpr (C::EXACT) {
    // a_v_p.dot(p): offsets [-1, 0] -> (0 + (-bm)*pm) + b*p
    const TF t = xadd(-xmul(bm, pm), xmul(b, p));
    if constexpr (!C::MEMORY) {
      return -t;  // heat flux: q = -a_q_t.dot(T)
    } else {
      TF r = t;
      if constexpr (C::ABSORB) {
        TF acc = TF(0);
        acc = xadd(acc, xmul(am, ul));
        acc = xadd(acc, xmul(a0, u));
        acc = xadd(acc, xmul(ap, ur));
        r = xsub(r, acc);
      }
      return xsub(u, r);
    }
  } else {
    if constexpr (!C::MEMORY) {
      if constexpr (sizeof(TP) > sizeof(TF)) {
        const TP bp = (TP)b_ * p_;
        return (TF)fma((TP)bm_, pm_, -bp);
      } else if constexpr (sizeof(TF) == 4 || std::is_same<TF, dw>::value) {
        return settle(fma(-(b - bm), (TF)a.offset, fma(bm, pm, -(b * p))));
      } else {
        return settle(fma(bm, pm, -(b * p)));
      }
    } else {
      TF acc = u;
      acc = fma(-b, p, acc);
      acc = fma(bm, pm, acc);
      if constexpr (C::ABSORB) {
        acc = fma(am, ul, acc);
        acc = fma(a0, u, acc);
        acc = fma(ap, ur, acc);
      }
      return settle(acc);
    }
  }
}

// New flux at flat index i from the potential slots (pos, pos - back) and the
// old flux; sB holds this direction's factors (slots of out-of-range cells hold 0).
template <class C, bool IS_X, typename TP, typename TF, typename TC>
__device__ __forceinline__ TF flux_new(const StagCore<TP, TF, TC>& a, const TP* sP, const TF* sF,
                                       const TC* sB, int pos, int64_t i, int x) {
  if constexpr (!C::HAS_V) {
    // 1-D fields: the same arithmetic as the warp kernel's register form
    static_assert(IS_X, "1-D fields have x fluxes only");
    TF u = TF(0), ul = TF(0), ur = TF(0), am = TF(0), a0 = TF(0), ap = TF(0);
    if constexpr (C::MEMORY) u = sF[pos];
    if constexpr (C::MEMORY && C::ABSORB) {
      ul = sF[pos - 1];
      ur = sF[pos + 1];
      am = (TF)ldg0(a.axm, i - 1, a.n);
      a0 = (TF)ldg0(a.ad, i, a.n);
      ap = (TF)ldg0(a.axp, i + 1, a.n);
    }
    return flux_1d<C>(a, sP[pos], sP[pos - 1], sB[pos], sB[pos - 1], u, ul, ur, am, a0, ap);
  } else {
    const int back = IS_X ? 1 : C::RX;
    const TF b = (TF)sB[pos];
    const TF bm = (TF)sB[pos - back];
    const TF p = (TF)sP[pos];
    const TF pm = (TF)sP[pos - back];
    if constexpr (C::EXACT) {
      // a_v_p.dot(p): offsets [-s, 0] -> (0 + (-bm)*pm) + b*p
      const TF t = xadd(-xmul(bm, pm), xmul(b, p));
      if constexpr (!C::MEMORY) {
        return -t;  // heat flux: q = -a_q_t.dot(T)
      } else {
        const TF u = sF[pos];
        TF r = t;
        if constexpr (C::ABSORB) r = xsub(r, absorb_term<C>(a, sF, pos, i));
        if constexpr (C::AXI && C::ABSORB && IS_X) {
          // + dt*mu/rho * vx / r**2   (pyfds/acoustics.py:213-215)
          const TF rad = (TF)ldg_t(a.rx + x);
          const TF e = xmul((TF)ldg_t(a.ex + i), u);
          r = xadd(r, e / xmul(rad, rad));
        }
        return xsub(u, r);
      }
    } else {
      if constexpr (!C::MEMORY) {
        if constexpr (sizeof(TP) > sizeof(TF)) {
          // float64 potential, float32 flux: the difference of the two products is
          // formed in float64 (near 300 K the float32 spacing, 2^-15 K, would swamp
          // small gradients) and only the flux is rounded to float32
          const TP bp = (TP)sB[pos] * sP[pos];
          return (TF)fma((TP)sB[pos - back], sP[pos - back], -bp);
        } else if constexpr (sizeof(TF) == 4 || std::is_same<TF, dw>::value) {
          // float32 / double-word temperature stored as T - offset: add the reference's
          // interface term -(b - bm) * offset (zero inside a material, and when offset
          // is 0)
          return settle(fma(-(b - bm), (TF)a.offset, fma(bm, pm, -(b * p))));
        } else {
          return settle(fma(bm, pm, -(b * p)));
        }
      } else {
        TF acc = sF[pos];
        acc = fma(-b, p, acc);
        acc = fma(bm, pm, acc);
        if constexpr (C::ABSORB) acc = absorb_fma<C>(a, sF, pos, i, acc);
        if constexpr (C::AXI && C::ABSORB && IS_X) {
          const TF rad = (TF)ldg_t(a.rx + x);
          acc = acc - ((TF)ldg_t(a.ex + i) * sF[pos]) / (rad * rad);
        }
        return settle(acc);
      }
    }
  }
}

// flux_new for the lossless, non-exact variants with the neighbour offset `back` as a
// runtime value (1: x flux, RX: y flux); the same arithmetic as flux_new.
template <class C, typename TP, typename TF, typename TC>
__device__ __forceinline__ TF flux_lossless(const TP* sP, const TF* sF, const TC* sB, int pos,
                                            int back, double offset) {
  static_assert(!C::EXACT && !C::ABSORB, "lossless, non-exact variants only");
  const TF b = (TF)sB[pos];
  const TF bm = (TF)sB[pos - back];
  const TF p = (TF)sP[pos];
  const TF pm = (TF)sP[pos - back];
  if constexpr (!C::MEMORY) {
    if constexpr (sizeof(TP) > sizeof(TF)) {
      const TP bp = (TP)sB[pos] * sP[pos];
      return (TF)fma((TP)sB[pos - back], sP[pos - back], -bp);
    } else if constexpr (sizeof(TF) == 4 || std::is_same<TF, dw>::value) {
      return settle(fma(-(b - bm), (TF)offset, fma(bm, pm, -(b * p))));
    } else {
      return settle(fma(bm, pm, -(b * p)));
    }
  } else {
    TF acc = sF[pos];
    acc = fma(-b, p, acc);
    acc = fma(bm, pm, acc);
    return settle(acc);
  }
}

// Shared memory of one staging buffer of this variant; every array starts on a
// 128-byte boundary (TMA destinations).
__host__ __device__ constexpr size_t round128(size_t b) { return (b + 127) / 128 * 128; }

template <class C, typename TP, typename TF, typename TC>
__host__ __device__ constexpr size_t stag_buffer_bytes(bool iso) {
  return round128((size_t)C::RN * sizeof(TP)) +
         (C::HAS_V ? 2 : 1) * round128((size_t)C::RN * sizeof(TF)) +
         (iso || !C::HAS_V ? 2 : 4) * round128((size_t)C::RN * sizeof(TC));
}

// The arrays of one staging buffer (see the region layout above).
template <typename TP, typename TF, typename TC>
struct StagBuf {
  TP* P;
  TF* U;
  TF* V;
  TC* Bx;
  TC* Kx;
  TC* By;
  TC* Ky;
};

template <class C, typename TP, typename TF, typename TC>
__device__ __forceinline__ StagBuf<TP, TF, TC> carve_buffer(unsigned char* base, bool iso) {
  constexpr size_t RN = C::RN;
  StagBuf<TP, TF, TC> b;
  unsigned char* q = base;
  b.P = reinterpret_cast<TP*>(q);
  q += round128(RN * sizeof(TP));
  b.U = reinterpret_cast<TF*>(q);
  q += round128(RN * sizeof(TF));
  b.V = C::HAS_V ? reinterpret_cast<TF*>(q) : b.U;
  if (C::HAS_V) q += round128(RN * sizeof(TF));
  b.Bx = reinterpret_cast<TC*>(q);
  q += round128(RN * sizeof(TC));
  b.Kx = reinterpret_cast<TC*>(q);
  q += round128(RN * sizeof(TC));
  if (iso || !C::HAS_V) {
    b.By = b.Bx;
    b.Ky = b.Kx;
  } else {
    b.By = reinterpret_cast<TC*>(q);
    q += round128(RN * sizeof(TC));
    b.Ky = reinterpret_cast<TC*>(q);
  }
  return b;
}

// Asynchronous global -> shared copy of one element (4 or 8 bytes); a slot whose
// cell is out of range is zero-filled (source size 0, no bytes are read).
template <typename T>
__device__ __forceinline__ void cp_async_elem(T* dst, const T* base, int64_t f, bool ok) {
  static_assert(sizeof(T) == 4 || sizeof(T) == 8, "4- or 8-byte elements");
  const unsigned saddr = (unsigned)__cvta_generic_to_shared(dst);
  const T* src = base + (ok ? f : 0);
  const int n = ok ? (int)sizeof(T) : 0;
  // no "memory" clobber: shared memory written here is only read after
  // cp_async_wait (which carries the clobber) and a barrier
  if constexpr (sizeof(T) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(saddr), "l"(src), "r"(n));
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(saddr), "l"(src), "r"(n));
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Issue the copies of the potential, old flux and coefficients of one tile's region.
// Slots are walked with incremental (column, row, flat index) updates.
template <class C, typename TP, typename TF, typename TC>
__device__ __forceinline__ void stage_tile(const StagCore<TP, TF, TC>& a, int tile,
                                           const StagBuf<TP, TF, TC>& b, bool iso) {
  constexpr int NT = C::NT, RX = C::RX, RN = C::RN, OY = C::OY;
  constexpr int DC = NT % RX, DR = NT / RX;
  const int nx = a.nx;
  const int64_t n = a.n;
  const TP* p_in = a.p_in;
  const TF* u_in = a.u_in;
  const TF* v_in = a.v_in;
  const TC* bx = a.bx;
  const TC* kx = a.kx;
  const TC* by = a.by;
  const TC* ky = a.ky;
  int x0, y0;
  tile_origin<C>(a, tile, x0, y0);
  int c = threadIdx.x % RX;
  int64_t f = (int64_t)(y0 + (int)threadIdx.x / RX - OY) * nx + (x0 + c - C::OX);
  const int64_t df = (int64_t)DR * nx + DC;
  const int64_t wrap = (int64_t)nx - RX;
  for (int e = threadIdx.x; e < RN; e += NT) {
    const bool ok = (f >= 0 && f < n);
    cp_async_elem(b.P + e, p_in, f, ok);
    if constexpr (C::MEMORY) {
      cp_async_elem(b.U + e, u_in, f, ok);
      if constexpr (C::HAS_V) cp_async_elem(b.V + e, v_in, f, ok);
    }
    cp_async_elem(b.Bx + e, bx, f, ok);
    cp_async_elem(b.Kx + e, kx, f, ok);
    if (!iso) {
      cp_async_elem(b.By + e, by, f, ok);
      cp_async_elem(b.Ky + e, ky, f, ok);
    }
    c += DC;
    f += df;
    if (c >= RX) {
      c -= RX;
      f += wrap;
    }
  }
}

// TMA staging of one tile's region: thread 0 issues one box per array into the
// buffer, completing on `bar` (an mbarrier initialised for one arrival).
template <class C, typename TP, typename TF, typename TC>
__device__ __forceinline__ void tma_issue_tile(const StagCore<TP, TF, TC>& a, const CUtensorMap* tm,
                                               int tile, const StagBuf<TP, TF, TC>& b, bool iso,
                                               uint64_t* bar) {
  constexpr int RN = C::RN;
  int gx, gy;
  tile_origin<C>(a, tile, gx, gy);
  gx -= C::OX;
  gy -= C::OY;
  uint32_t bytes = RN * (uint32_t)(sizeof(TP) + 2 * sizeof(TC));
  if constexpr (C::MEMORY) bytes += (C::HAS_V ? 2 : 1) * RN * (uint32_t)sizeof(TF);
  if (!iso) bytes += 2 * RN * (uint32_t)sizeof(TC);
  // order the CTA's earlier generic accesses to this buffer (made visible to this
  // thread by the preceding barrier) before the asynchronous-proxy writes
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
  mbar_arrive_expect_tx(bar, bytes);
  tma_load_2d(b.P, &tm[0], gx, gy, bar);
  if constexpr (C::MEMORY) {
    tma_load_2d(b.U, &tm[1], gx, gy, bar);
    if constexpr (C::HAS_V) tma_load_2d(b.V, &tm[2], gx, gy, bar);
  }
  tma_load_2d(b.Bx, &tm[3], gx, gy, bar);
  tma_load_2d(b.Kx, &tm[4], gx, gy, bar);
  if (!iso) {
    tma_load_2d(b.By, &tm[5], gx, gy, bar);
    tma_load_2d(b.Ky, &tm[6], gx, gy, bar);
  }
}

// L2 prefetch of the boxes of a later tile (one thread), when they lie inside the
// arrays: the CTA that stages that tile then reads L2 instead of waiting on DRAM.
template <class C, typename TP, typename TF, typename TC>
__device__ __forceinline__ void tma_prefetch_tile(const StagCore<TP, TF, TC>& a,
                                                  const CUtensorMap* tm, int tile, bool iso) {
  int gx, gy;
  tile_origin<C>(a, tile, gx, gy);
  gx -= C::OX;
  gy -= C::OY;
  if (gx < 0 || gy < 0 || gx + C::RX > a.nx || gy + C::RY > a.ny) return;
  tma_prefetch_2d(&tm[0], gx, gy);
  if constexpr (C::MEMORY) {
    tma_prefetch_2d(&tm[1], gx, gy);
    if constexpr (C::HAS_V) tma_prefetch_2d(&tm[2], gx, gy);
  }
  tma_prefetch_2d(&tm[3], gx, gy);
  tma_prefetch_2d(&tm[4], gx, gy);
  if (!iso) {
    tma_prefetch_2d(&tm[5], gx, gy);
    tma_prefetch_2d(&tm[6], gx, gy);
  }
}

// Waits (bounded) for a tile's boxes, then patches the slots whose column lies
// outside [0, nx): the box reads them as zeros, the flat-index semantics want the
// cells of the neighbouring row. Returns false for every thread on a timeout.
template <class C, typename TP, typename TF, typename TC>
__device__ __forceinline__ bool tma_finish_tile(const StagCore<TP, TF, TC>& a, int tile,
                                                const StagBuf<TP, TF, TC>& b, bool iso,
                                                uint64_t* bar, uint32_t parity) {
  constexpr int RX = C::RX, RN = C::RN, OX = C::OX, OY = C::OY, NT = C::NT;
  constexpr long long kWaitLimit = 1ll << 22;
  int x0, y0;
  tile_origin<C>(a, tile, x0, y0);
  bool ok = mbar_wait(bar, parity, kWaitLimit);
  if (__syncthreads_or(!ok)) {
    // give the copies in flight a second bounded chance to land before leaving
    if (!ok) mbar_wait(bar, parity, kWaitLimit);
    if (threadIdx.x == 0 && a.status) atomicOr(a.status, kStatusTmaTimeout);
    return false;
  }
  // box columns outside [0, nx): c in [0, clo) on the left, [chi, RX) on the right
  const int clo = max(0, OX - x0);
  const int chi = min(RX, a.nx - (x0 - OX));
  const int wl = clo, wr = RX - chi;
  if (wl + wr > 0) {
    constexpr int RY = RN / RX;
    for (int q = threadIdx.x; q < (wl + wr) * RY; q += NT) {
      const int r = q / (wl + wr);
      const int j = q - r * (wl + wr);
      const int cc = j < wl ? j : chi + (j - wl);
      const int e = r * RX + cc;
      const int x = x0 - OX + cc;
      const int64_t f = (int64_t)(y0 - OY + r) * a.nx + x;
      const bool in = (f >= 0 && f < a.n);
      // state through L2: in the persistent wavefront kernel other CTAs wrote it
      // during this launch
      b.P[e] = in ? ldcg_t(a.p_in + f) : TP(0);
      if constexpr (C::MEMORY) {
        b.U[e] = in ? ldcg_t(a.u_in + f) : TF(0);
        if constexpr (C::HAS_V) b.V[e] = in ? ldcg_t(a.v_in + f) : TF(0);
      }
      b.Bx[e] = in ? a.bx[f] : TC(0);
      b.Kx[e] = in ? a.kx[f] : TC(0);
      if (!iso) {
        b.By[e] = in ? a.by[f] : TC(0);
        b.Ky[e] = in ? a.ky[f] : TC(0);
      }
    }
  }
  __syncthreads();
  return true;
}

// New potential of a cell from its old potential p, the new fluxes around it (x: u
// at the cell, un1 at its right neighbour; y: v at the cell, vn1 at the cell below)
// and the potential update factors; x is the cell's column (the radius of the exact
// axisymmetric scaling). The reference's operation order in exact mode; fused
// multiply-adds otherwise.
template <class C, typename TP, typename TF, typename TC>
__device__ __forceinline__ TP potential_regs(const StagCore<TP, TF, TC>& a, TP p, TF u, TF un1,
                                             TF v, TF vn1, TF kxi, TF kxn, TF kyi, TF kyn,
                                             int x) {
  if constexpr (C::EXACT) {
    TF w = u, wn = un1;
    if constexpr (C::AXI) {
      // a_p_vx.dot(vx * r): the flux is scaled by the radius of its column
      const int xn = (x + 1 == a.nx) ? 0 : x + 1;
      w = xmul(u, (TF)ldg_t(a.rx + x));
      wn = xmul(un1, (TF)ldg_t(a.rx + xn));
    }
    // forward difference, offsets [0, s]: (0 + (-k)*w) + kn*wn
    TF sx = xadd(-xmul(kxi, w), xmul(kxn, wn));
    if constexpr (C::HAS_V) {
      const TF sy = xadd(-xmul(kyi, v), xmul(kyn, vn1));
      sx = xadd(sx, sy);
    }
    return (TP)xsub((TF)p, sx);
  } else if constexpr (sizeof(TP) == sizeof(TF)) {
    TF acc = (TF)p;
    acc = fma(kxi, u, acc);
    acc = fma(-kxn, un1, acc);
    if constexpr (C::HAS_V) {
      acc = fma(kyi, v, acc);
      acc = fma(-kyn, vn1, acc);
    }
    return (TP)settle(acc);
  } else {
    // float increment accumulated into a float64 potential
    TF inc = kxi * u;
    inc = fma(-kxn, un1, inc);
    if constexpr (C::HAS_V) {
      inc = fma(kyi, v, inc);
      inc = fma(-kyn, vn1, inc);
    }
    return p + (TP)inc;
  }
}

// potential_regs with every operand read from the staged slots around slot ps.
template <class C, typename TP, typename TF, typename TC>
__device__ __forceinline__ TP potential_cell(const StagCore<TP, TF, TC>& a, const TP* sP,
                                             const TF* sU, const TF* sV, const TC* sKx,
                                             const TC* sKy, int ps, int x) {
  TF v = TF(0), vn1 = TF(0), kyi = TF(0), kyn = TF(0);
  if constexpr (C::HAS_V) {
    v = sV[ps];
    vn1 = sV[ps + C::RX];
    kyi = (TF)sKy[ps];
    kyn = (TF)sKy[ps + C::RX];
  }
  return potential_regs<C>(a, sP[ps], sU[ps], sU[ps + 1], v, vn1, (TF)sKx[ps], (TF)sKx[ps + 1],
                           kyi, kyn, x);
}

// Everything after the region has landed: flux update, flux bounds and probes,
// potential update, next step's potential bounds and probes, stores.
//
// Thread t owns the cells t + NT*k (k < OIT) of the TX x TY tile, TX a power of
// two, and keeps their slot and flat index in registers through all phases. The
// extended flux regions reach one column right (U) and one row down (V) of the
// tile: inside a partial tile the owner of that slot computes it; past a full tile
// the first TY threads compute the U column and the next TX threads the V row.
template <class C, typename TP, typename TF, typename TC>
__device__ __forceinline__ void compute_tile(const StagCore<TP, TF, TC>& a, const StepInfo si,
                                             int tile, const StagBuf<TP, TF, TC>& b) {
  constexpr int TX = C::TX, TY = C::TY, NT = C::NT, RX = C::RX, OY = C::OY;
  constexpr int OIT = TX * TY / NT;
  static_assert((TX & (TX - 1)) == 0, "tile width must be a power of two");
  static_assert((TX * TY) % NT == 0, "the tile's cells must divide evenly among threads");
  // float64 (bound by the FP64 pipe) keeps the cells' potential and new fluxes in
  // registers for the potential update instead of reloading them from shared memory,
  // and on 2-D tiles gives each thread OIT consecutive rows of one column, so that
  // the flux below a cell is mostly the thread's own register. The other precisions
  // (bound by instruction issue) keep cells NT apart and reload: the registers would
  // spill (double-word two-step kernel: 8 -> 56 bytes)
  constexpr bool REGS = std::is_same<TF, double>::value && std::is_same<TP, double>::value;
  constexpr bool ROWS = REGS && C::HAS_V && NT % TX == 0;
  static_assert(!C::HAS_V || TX + TY <= NT, "halo threads: TX + TY must not exceed NT");
  TP* sP = b.P;
  TF* sU = b.U;
  TF* sV = b.V;
  const TC* sBx = b.Bx;
  const TC* sKx = b.Kx;
  const TC* sBy = b.By;
  const TC* sKy = b.Ky;
  int x0, y0;
  tile_origin<C>(a, tile, x0, y0);
  const int x1 = min(x0 + TX, a.nx);  // end of owned columns
  const int y1 = min(y0 + TY, a.ny);
  const int tid = threadIdx.x;

  int pos[OIT];
  int64_t fo[OIT];
  int xo[OIT];
  bool own[OIT], inu[OIT], inv[OIT];
  // ROWS: thread t owns column t % TX, rows (t / TX) * OIT .. + OIT - 1; else cells
  // t, t + NT, ...
#pragma unroll
  for (int k = 0; k < OIT; ++k) {
    const int lx = ROWS ? tid % TX : (tid + NT * k) % TX;
    const int ly = ROWS ? (tid / TX) * OIT + k : (tid + NT * k) / TX;
    const int x = x0 + lx;
    const int y = y0 + ly;
    pos[k] = (ly + OY) * RX + lx + C::OX;
    fo[k] = (int64_t)y * a.nx + x;
    xo[k] = x;
    own[k] = (x < x1 && y < y1);
    inu[k] = (x <= x1 && y < y1 && fo[k] < a.n);  // U-ext, incl. a partial tile's edge
    inv[k] = (x < x1 && y <= y1 && fo[k] < a.n);  // V-ext, incl. a partial tile's edge
  }
  // halo threads past a full tile
  const bool hu = (tid < TY) && (x1 == x0 + TX);
  const bool hv = C::HAS_V && (tid >= TY) && (tid < TY + TX) && (y1 == y0 + TY);
  const int hu_pos = (tid + OY) * RX + TX + C::OX;
  const int64_t hu_f = (int64_t)(y0 + tid) * a.nx + x1;
  const int hv_lx = tid - TY;
  const int hv_pos = (TY + OY) * RX + hv_lx + C::OX;
  const int64_t hv_f = (int64_t)y1 * a.nx + x0 + hv_lx;

  // ---- new fluxes over U-ext and V-ext ----
  TP po[OIT];  // (REGS) the cells' potential after this step's bounds
  if constexpr (REGS) {
#pragma unroll
    for (int k = 0; k < OIT; ++k) po[k] = sP[pos[k]];
  }
  TF un[OIT], vn[OIT];
#pragma unroll
  for (int k = 0; k < OIT; ++k) {
    un[k] = inu[k] ? flux_new<C, true>(a, sP, sU, sBx, pos[k], fo[k],
                                       xo[k] == a.nx ? 0 : xo[k])
                   : TF(0);
    if constexpr (C::HAS_V)
      vn[k] = inv[k] ? flux_new<C, false>(a, sP, sV, sBy, pos[k], fo[k], xo[k]) : TF(0);
  }
  TF uh = TF(0), vh = TF(0);
  const bool hu_ok = hu && (y0 + tid < y1) && hu_f < a.n;
  const bool hv_ok = hv && (x0 + hv_lx < x1) && hv_f < a.n;
  if constexpr (C::HAS_V && !C::EXACT && !C::ABSORB) {
    // both halo strips through one code path: the warp holding the U column and the
    // start of the V row issues its flux arithmetic once, with every lane busy
    // (the x and y flux differ only in the neighbour offset and the arrays)
    const bool isx = tid < TY;
    const TF h = (isx ? hu_ok : hv_ok)
                     ? flux_lossless<C>(sP, isx ? sU : sV, isx ? sBx : sBy,
                                        isx ? hu_pos : hv_pos, isx ? 1 : RX, a.offset)
                     : TF(0);
    uh = h;
    vh = h;
  } else {
    if (hu_ok) uh = flux_new<C, true>(a, sP, sU, sBx, hu_pos, hu_f, x1 == a.nx ? 0 : x1);
    if constexpr (C::HAS_V)
      if (hv_ok) vh = flux_new<C, false>(a, sP, sV, sBy, hv_pos, hv_f, x0 + hv_lx);
  }
  if constexpr (C::MEMORY && C::ABSORB) __syncthreads();  // neighbours read the old flux
#pragma unroll
  for (int k = 0; k < OIT; ++k) {
    sU[pos[k]] = un[k];
    if constexpr (C::HAS_V) sV[pos[k]] = vn[k];
  }
  if (hu) sU[hu_pos] = uh;
  if constexpr (C::HAS_V)
    if (hv) sV[hv_pos] = vh;
  __syncthreads();

  // ---- flux bounds and probes (this step) ----
  // (tiles without flux bounds, most of them, skip the barrier: the potential update
  // and the probes read the fluxes as the barrier above left them)
  if (tile_has(a.tab[1].bound_tile_start, tile) ||
      (C::HAS_V && tile_has(a.tab[2].bound_tile_start, tile))) {
    apply_bound_groups<NT>(a.tab[1], tile, sU, a.pool, si.step);
    if constexpr (C::HAS_V) apply_bound_groups<NT>(a.tab[2], tile, sV, a.pool, si.step);
    __syncthreads();
    // the bounds may have changed the fluxes held in registers
    if constexpr (REGS) {
#pragma unroll
      for (int k = 0; k < OIT; ++k) {
        un[k] = sU[pos[k]];
        if constexpr (C::HAS_V) vn[k] = sV[pos[k]];
      }
    }
  }
  write_probes<NT>(a.tab[1], tile, sU, si.step - si.step0);
  if constexpr (C::HAS_V) write_probes<NT>(a.tab[2], tile, sV, si.step - si.step0);

  // ---- potential update of the owned cells ----
  TP pn[OIT];
#pragma unroll
  for (int k = 0; k < OIT; ++k) {
    const int ps = pos[k];
    pn[k] = TP(0);
    if (own[k]) {
      if constexpr (REGS) {
        if (si.store_flux) {
          a.u_out[fo[k]] = un[k];
          if constexpr (C::HAS_V) a.v_out[fo[k]] = vn[k];
        }
        // the flux below the cell: this thread's next row, or the slot past its rows
        TF vb = TF(0), kyi = TF(0), kyn = TF(0);
        if constexpr (C::HAS_V) {
          vb = (ROWS && k + 1 < OIT) ? vn[(k + 1) % OIT] : sV[ps + RX];
          kyi = (TF)sKy[ps];
          kyn = (TF)sKy[ps + RX];
        }
        pn[k] = potential_regs<C>(a, po[k], un[k], sU[ps + 1], vn[k], vb, (TF)sKx[ps],
                                  (TF)sKx[ps + 1], kyi, kyn, xo[k]);
      } else {
        if (si.store_flux) {
          a.u_out[fo[k]] = sU[ps];
          if constexpr (C::HAS_V) a.v_out[fo[k]] = sV[ps];
        }
        pn[k] = potential_cell<C>(a, sP, sU, sV, sKx, sKy, ps, xo[k]);
      }
    }
  }
  // the next step's potential bounds and probes go through shared memory; a tile
  // without them (most tiles) keeps the new potential in registers. No barrier is
  // needed before the write: in the update above each thread read only the potential
  // of its own cells.
  if (si.apply_next && (tile_has(a.tab[0].bound_tile_start, tile) ||
                        tile_has(a.tab[0].probe_tile_start, tile))) {
#pragma unroll
    for (int k = 0; k < OIT; ++k)
      if (own[k]) sP[pos[k]] = pn[k];
    __syncthreads();
    apply_bound_groups<NT>(a.tab[0], tile, sP, a.pool, si.step + 1);
    __syncthreads();
    write_probes<NT>(a.tab[0], tile, sP, si.step + 1 - si.step0);
#pragma unroll
    for (int k = 0; k < OIT; ++k)
      if (own[k]) pn[k] = sP[pos[k]];
  }
  // ---- store the owned potential ----
#pragma unroll
  for (int k = 0; k < OIT; ++k)
    if (own[k]) a.p_out[fo[k]] = pn[k];
  // the last step of a call reports a diverged field (NaN and infinity spread, so
  // the final potential shows any earlier blow-up)
  if (!si.apply_next && a.status) {
    bool bad = false;
#pragma unroll
    for (int k = 0; k < OIT; ++k) bad = bad || (own[k] && nonfinite(pn[k]));
    if (__any_sync(0xffffffffu, bad) && (tid & 31) == 0) atomicOr(a.status, kStatusNonFinite);
  }
}

// Grid-stride over tiles. STAGES == 1: one tile per CTA, staged then computed.
// STAGES == 2 (persistent CTAs): the copies of the next tile are in flight while
// the current tile is computed from the other buffer. Staging is TMA when the
// launch provides tensor maps (use_tma) and cp.async otherwise.
template <class C, typename TP, typename TF, typename TC>
__global__ void __launch_bounds__(C::NT, C::min_blocks(sizeof(TP), std::is_same<TP, dw>::value))
    stag_step_kernel(const __grid_constant__ StagArgs<TP, TF, TC> a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const bool iso = a.iso || !C::HAS_V;
  const size_t bytes = stag_buffer_bytes<C, TP, TF, TC>(iso);
  // the TMA barriers follow the buffers; TMA needs 128-byte aligned destinations
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + C::STAGES * bytes);
  const bool tma = a.use_tma && (smem_addr(smem_raw) & 127u) == 0;
  const StagBuf<TP, TF, TC> buf0 = carve_buffer<C, TP, TF, TC>(smem_raw, iso);
  int t = blockIdx.x;
  if (tma && threadIdx.x == 0)
    for (int k = 0; k < C::STAGES; ++k) mbar_init(bars + k, 1);
  __syncthreads();
  if constexpr (C::STAGES == 1) {
    if (tma) {
      if (threadIdx.x == 0) {
        tma_issue_tile<C>(a, a.tm, t, buf0, iso, bars);
        if (a.prefetch > 0 && t + a.prefetch < a.ntiles)
          tma_prefetch_tile<C>(a, a.tm, t + a.prefetch, iso);
      }
      if (!tma_finish_tile<C>(a, t, buf0, iso, bars, 0)) return;
    } else {
      stage_tile<C>(a, t, buf0, iso);
      cp_async_commit();
      cp_async_wait<0>();
      __syncthreads();
    }
    compute_tile<C>(a, step_of(a), t, buf0);
  } else {
    const StagBuf<TP, TF, TC> buf1 = carve_buffer<C, TP, TF, TC>(smem_raw + bytes, iso);
    const int stride = gridDim.x;
    if (t < a.ntiles) {
      if (tma) {
        if (threadIdx.x == 0) tma_issue_tile<C>(a, a.tm, t, buf0, iso, bars);
      } else {
        stage_tile<C>(a, t, buf0, iso);
      }
    }
    if (!tma) cp_async_commit();
    for (int k = 0; t < a.ntiles; ++k, t += stride) {
      const int tn = t + stride;
      const int cur = k & 1;
      __syncthreads();  // every thread is done with the buffer the next copies fill
      if (tn < a.ntiles) {
        if (tma) {
          if (threadIdx.x == 0) tma_issue_tile<C>(a, a.tm, tn, cur ? buf0 : buf1, iso, bars + (cur ^ 1));
        } else {
          stage_tile<C>(a, tn, cur ? buf0 : buf1, iso);
        }
      }
      if (tma) {
        // buffer `cur` completes once per use: its (k >> 1)-th use has parity (k >> 1) & 1
        if (!tma_finish_tile<C>(a, t, cur ? buf1 : buf0, iso, bars + cur, (k >> 1) & 1)) {
          // let a prefetch in flight into the other buffer land before leaving
          if (tn < a.ntiles) mbar_wait(bars + (cur ^ 1), ((k + 1) >> 1) & 1, 1ll << 22);
          return;
        }
      } else {
        cp_async_commit();
        cp_async_wait<1>();  // this thread's copies of tile t have landed
        __syncthreads();     // ... and every other thread's
      }
      compute_tile<C>(a, step_of(a), t, cur ? buf1 : buf0);
    }
  }
}

// ------------------------------------------------------- every step in one launch
//
// Persistent wavefront over a whole call (stages 4): each CTA takes work items
// (step s, tile t) from a queue in the order item = s * ntiles + t, waits until the
// tile rows around t finished step s - 1, stages its region with TMA, computes it
// with compute_tile and publishes one more finished tile of its row. A tile's region
// (rows y0 - 1 .. y0 + TY + 1, and through the flat-index wrap the neighbouring
// rows' edge cells) lies in tile rows ty - 1 .. ty + 1 for TY >= 3, and those rows
// also cover every tile that reads the cells this tile overwrites (ping-pong
// buffers: step s writes what step s - 2 read). So the per-row counters order every
// read after the write it needs and every overwrite after the reads of the old
// values. Consecutive steps overlap and no launch boundary separates them: the
// one-launch-per-step kernel spends about a tenth of each launch with SMs idle in
// the wave tail and ramp.
//
// No deadlock: items are handed out in order, so the smallest unfinished item is
// held by a running CTA and every item it waits for has a smaller index and is
// finished. Every wait is bounded (status bit kStatusTmaTimeout, the CTA returns).
template <typename TP, typename TF, typename TC>
struct StagWaveArgs {
  StagArgs<TP, TF, TC> par[2];  // step parity 0 reads the cur buffers, 1 the nxt ones
  uint32_t* sync;    // [0]: next work item; [1 + r]: tiles of row r done, summed over steps
  int32_t tiles_y;
  int32_t nsteps;    // steps of this launch
  int64_t step;      // global step of the launch's first step
  int32_t flux_all;  // store the fluxes on every step (else on the call's last only)
  int32_t more;      // steps of the same call follow this launch
  int32_t prefetch;  // L2 prefetch distance in work items (0: off)
};

constexpr long long kWaveWaitLimit = 1ll << 22;

// True if tile rows ty - 1 .. ty + 1 have finished `s` steps (one acquire load each).
template <typename TP, typename TF, typename TC>
__device__ __forceinline__ bool wave_rows_ready(const StagWaveArgs<TP, TF, TC>& w, int ty, int s) {
  const uint32_t need = (uint32_t)s * (uint32_t)w.par[0].tiles_x;
  const int r0 = ty > 0 ? ty - 1 : 0;
  const int r1 = ty + 1 < w.tiles_y ? ty + 1 : w.tiles_y - 1;
  bool ok = true;
  for (int r = r0; r <= r1; ++r) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(w.sync + 1 + r) : "memory");
    ok = ok && v >= need;
  }
  return ok;
}

// Thread 0: wait (bounded) until tile rows ty - 1 .. ty + 1 have finished `s` steps.
template <typename TP, typename TF, typename TC>
__device__ __forceinline__ bool wave_wait_rows(const StagWaveArgs<TP, TF, TC>& w, int ty, int s) {
  const int r0 = ty > 0 ? ty - 1 : 0;
  const int r1 = ty + 1 < w.tiles_y ? ty + 1 : w.tiles_y - 1;
  return wait_counters(w.sync + 1, r0, r1, (uint32_t)s * (uint32_t)w.par[0].tiles_x,
                       kWaveWaitLimit);
}

// Resident CTAs per SM the wavefront kernel is compiled for: the one-stage kernel's
// figure, or fewer where its staging buffer fits fewer CTAs into the SM's 228 KB
// (1 KB reserved per CTA), so that the register budget is not cut for CTAs that
// could never be resident (float64 64 x 16: 4, 64 registers instead of 48 and
// spills).
template <class C, typename TP, typename TF, typename TC>
__host__ __device__ constexpr int wave_blocks() {
  constexpr int by_regs = C::min_blocks(sizeof(TP), std::is_same<TP, dw>::value);
  constexpr int by_smem =
      (int)((228u * 1024u) / (stag_buffer_bytes<C, TP, TF, TC>(true) + 16u + 1024u));
  return by_smem < by_regs ? (by_smem > 0 ? by_smem : 1) : by_regs;
}

template <class C, typename TP, typename TF, typename TC>
__global__ void __launch_bounds__(C::NT, (wave_blocks<C, TP, TF, TC>()))
    stag_wave_kernel(const __grid_constant__ StagWaveArgs<TP, TF, TC> w) {
  static_assert(C::STAGES == 1 && C::HAS_V && !C::TWO_STEP && C::TY >= 3,
                "one-stage 2-D tiles at least three rows high");
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ int s_item[2];
  const bool iso = w.par[0].iso != 0;
  const size_t bytes = stag_buffer_bytes<C, TP, TF, TC>(iso);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw + bytes);
  const StagBuf<TP, TF, TC> buf = carve_buffer<C, TP, TF, TC>(smem_raw, iso);
  const int ntiles = w.par[0].ntiles;
  const uint32_t total = (uint32_t)w.nsteps * (uint32_t)ntiles;
  int32_t* status = w.par[0].status;
  if (threadIdx.x == 0) mbar_init(bar, 1);
  __syncthreads();
  uint32_t uses = 0;  // completed phases of the mbarrier
  // Thread 0 takes each next item from the queue as soon as the current tile's copies
  // are issued and checks its dependencies right away (the loads' round trips
  // overlap the copies and the compute); only an item whose rows were not ready then
  // is checked again, with the bounded wait, when its turn comes.
  uint32_t next = 0;
  bool next_ready = false;
  if (threadIdx.x == 0) next = atomicAdd(w.sync, 1u);
  for (;;) {
    if (threadIdx.x == 0) {
      const uint32_t item = next;
      int s = -1, tile = 0;
      if (item < total) {
        s = (int)(item / (uint32_t)ntiles);
        tile = (int)(item - (uint32_t)s * (uint32_t)ntiles);
        const StagArgs<TP, TF, TC>& a = w.par[s & 1];
        if (s > 0 && !next_ready && !wave_wait_rows(w, tile_row(a, tile), s)) {
          if (status) atomicOr(status, kStatusTmaTimeout);
          s = -2;
        } else {
          // the tensor copies (async proxy) read what other CTAs stored (generic proxy)
          asm volatile("fence.proxy.async.global;\n" ::: "memory");
          tma_issue_tile<C>(a, a.tm, tile, buf, iso, bar);
          next = atomicAdd(w.sync, 1u);
          next_ready = false;
          if (next < total) {
            const int s1 = (int)(next / (uint32_t)ntiles);
            const int t1 = (int)(next - (uint32_t)s1 * (uint32_t)ntiles);
            next_ready = s1 == 0 || wave_rows_ready(w, tile_row(w.par[0], t1), s1);
          }
          const uint32_t ahead = item + (uint32_t)w.prefetch;
          if (w.prefetch > 0 && ahead < total) {
            const int s2 = (int)(ahead / (uint32_t)ntiles);
            tma_prefetch_tile<C>(w.par[s2 & 1], w.par[s2 & 1].tm,
                                 (int)(ahead - (uint32_t)s2 * (uint32_t)ntiles), iso);
          }
        }
      }
      s_item[0] = s;
      s_item[1] = tile;
    }
    __syncthreads();
    const int s = s_item[0], tile = s_item[1];
    if (s < 0) break;  // queue empty, or a wait gave up (nothing in flight)
    const StagArgs<TP, TF, TC>& a = w.par[s & 1];
    if (!tma_finish_tile<C>(a, tile, buf, iso, bar, uses & 1u)) return;
    ++uses;
    const bool last = s + 1 == w.nsteps;
    compute_tile<C>(a,
                    StepInfo{w.step + s, a.step0, (!last || w.more) ? 1 : 0,
                             (w.flux_all || (last && !w.more)) ? 1 : 0, 1},
                    tile, buf);
    __syncthreads();  // every thread's stores are issued and the buffer is free
    if (threadIdx.x == 0) {
      // publish the tile (release: the CTA's stores, ordered before by the barrier)
      asm volatile("red.release.gpu.global.add.u32 [%0], 1;\n" ::"l"(w.sync + 1 + tile_row(a, tile))
                   : "memory");
    }
  }
}

// ------------------------------------------------------------ two steps per tile
//
// Temporal blocking for the lossless 2-D variants (memory-bound precisions): a
// CTA stages a region two rows taller than the one-step kernel's (rows y0-2 ..
// y0+TY+1, columns x0-4 .. x0+TX+3; slot layout 2), computes step n on a ring one
// cell wider than the tile (fluxes on U: x0-1 .. x0+TX+1 x y0-1 .. y0+TY, V: x0-1
// .. x0+TX x y0-1 .. y0+TY+1, potential on x0-1 .. x0+TX x y0-1 .. y0+TY), then
// step n+1 on the tile exactly as the one-step kernel does, and stores the owned
// cells once: the state crosses HBM once per two steps. Every cell is computed in
// the one-step kernel's operation order, so the results are the same bit for bit.
// The bound tables of layout 2 hold every slot of the ring where a bound cell is
// computed; applying step n+1's bounds to ring slots that step n+1 does not
// recompute is harmless (they are neither read nor stored). Probes belong to the
// owning tile only.
template <int TX_, int TY_, int NT_, bool MEMORY_>
struct Tb2Cfg : StagCfg<TX_, TY_, NT_, true, MEMORY_, false, false, false, 1> {
  static constexpr bool TWO_STEP = true;
  static constexpr int batch_blocks(int psize) {
    return psize == 4 ? FDS_BATCH_TB2_BLOCKS_256_F32 : FDS_BATCH_BLOCKS_256;
  }
  static constexpr int OY = 2;
  static constexpr int RY = TY_ + 4;
  static constexpr int RN = (TX_ + 8) * RY;
};

// New potential at slot ps (lossless, float64 / float32 / double words): the
// one-stage kernel's expression, term by term.
template <class C, typename TP, typename TF, typename TC>
__device__ __forceinline__ TP potential_new(const StagBuf<TP, TF, TC>& b, int ps) {
  TF acc = (TF)b.P[ps];
  acc = fma((TF)b.Kx[ps], b.U[ps], acc);
  acc = fma(-(TF)b.Kx[ps + 1], b.U[ps + 1], acc);
  acc = fma((TF)b.Ky[ps], b.V[ps], acc);
  acc = fma(-(TF)b.Ky[ps + C::RX], b.V[ps + C::RX], acc);
  return (TP)settle(acc);
}

// Calls f(pos, flat) for the slots of a W x H block of the region whose first cell is
// (x0 + dx0, y0 + dy0), thread t taking slots t, t + NT, ...; the slot and flat index
// advance incrementally (no division per slot).
template <class C, int W, int H, typename F>
__device__ __forceinline__ void for_block(int x0, int y0, int dx0, int dy0, int nx, F&& f) {
  constexpr int NT = C::NT, RX = C::RX, DC = NT % W, DR = NT / W;
  int col = (int)threadIdx.x % W;
  const int row = (int)threadIdx.x / W;
  int pos = (row + dy0 + C::OY) * RX + col + dx0 + C::OX;
  int64_t flat = (int64_t)(y0 + dy0 + row) * nx + (x0 + dx0 + col);
  for (int c = threadIdx.x; c < W * H; c += NT) {
    f(pos, flat);
    col += DC;
    pos += DR * RX + DC;
    flat += (int64_t)DR * nx + DC;
    if (col >= W) {
      col -= W;
      pos += RX - W;
      flat += nx - W;
    }
  }
}

// Step si.step on the ring around the tile, in place in the staged region.
template <class C, typename TP, typename TF, typename TC>
__device__ __forceinline__ void compute_ring(const StagCore<TP, TF, TC>& a, const StepInfo si,
                                             int tile, const StagBuf<TP, TF, TC>& b) {
  constexpr int TX = C::TX, TY = C::TY, NT = C::NT, RX = C::RX, OX = C::OX, OY = C::OY;
  int x0, y0;
  tile_origin<C>(a, tile, x0, y0);
  // fluxes: each slot reads only its own old flux and the potential. Slots of
  // cells outside the field get 0, as in the one-step kernel (thermal fluxes are
  // not staged, so those slots would otherwise hold stale shared memory, which the
  // potential update multiplies by a zero coefficient)
  constexpr int UW = TX + 3, UH = TY + 2, VW = TX + 2, VH = TY + 3;
  const int64_t n = a.n;
  for_block<C, UW, UH>(x0, y0, -1, -1, a.nx, [&](int pos, int64_t f) {
    b.U[pos] = (f >= 0 && f < n) ? flux_new<C, true>(a, b.P, b.U, b.Bx, pos, f, 0) : TF(0);
  });
  for_block<C, VW, VH>(x0, y0, -1, -1, a.nx, [&](int pos, int64_t f) {
    b.V[pos] = (f >= 0 && f < n) ? flux_new<C, false>(a, b.P, b.V, b.By, pos, f, 0) : TF(0);
  });
  __syncthreads();
  apply_bound_groups<NT>(a.tab[1], tile, b.U, a.pool, si.step);
  apply_bound_groups<NT>(a.tab[2], tile, b.V, a.pool, si.step);
  __syncthreads();
  write_probes<NT>(a.tab[1], tile, b.U, si.step - si.step0);
  write_probes<NT>(a.tab[2], tile, b.V, si.step - si.step0);
  // potential of step si.step + 1: each slot reads only its own old value
  constexpr int PW = TX + 2, PH = TY + 2;
  for_block<C, PW, PH>(x0, y0, -1, -1, a.nx, [&](int pos, int64_t f) {
    if (f >= 0 && f < n) b.P[pos] = potential_new<C>(b, pos);
  });
  __syncthreads();
  apply_bound_groups<NT>(a.tab[0], tile, b.P, a.pool, si.step + 1);
  __syncthreads();
  write_probes<NT>(a.tab[0], tile, b.P, si.step + 1 - si.step0);
}

// One tile, one or two steps (a.substeps), one CTA per tile, TMA or cp.async
// staging, L2 prefetch of a later tile as in the one-step kernel.
template <class C, typename TP, typename TF, typename TC>
__global__ void __launch_bounds__(C::NT, C::min_blocks(sizeof(TP), std::is_same<TP, dw>::value))
    stag_tb2_kernel(const __grid_constant__ StagArgs<TP, TF, TC> a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const bool iso = a.iso != 0;
  const size_t bytes = stag_buffer_bytes<C, TP, TF, TC>(iso);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + bytes);
  const bool tma = a.use_tma && (smem_addr(smem_raw) & 127u) == 0;
  const StagBuf<TP, TF, TC> buf = carve_buffer<C, TP, TF, TC>(smem_raw, iso);
  const int t = blockIdx.x;
  if (tma && threadIdx.x == 0) mbar_init(bars, 1);
  __syncthreads();
  if (tma) {
    if (threadIdx.x == 0) {
      tma_issue_tile<C>(a, a.tm, t, buf, iso, bars);
      if (a.prefetch > 0 && t + a.prefetch < a.ntiles)
        tma_prefetch_tile<C>(a, a.tm, t + a.prefetch, iso);
    }
    if (!tma_finish_tile<C>(a, t, buf, iso, bars, 0)) return;
  } else {
    stage_tile<C>(a, t, buf, iso);
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
  }
  const StepInfo si = step_of(a);
  if (a.substeps == 2) {
    compute_ring<C>(a, si, t, buf);
    __syncthreads();
    compute_tile<C>(a, StepInfo{si.step + 1, si.step0, si.apply_next, si.store_flux, 1}, t, buf);
  } else {
    compute_tile<C>(a, si, t, buf);
  }
}

// Potential bounds and probes of the first step of a call, in place on the
// global potential (one CTA: bounds, barrier, probes).
template <typename TP>
__global__ void __launch_bounds__(1024) stag_prologue_kernel(TP* p, FdsCompTables tb,
                                                             const double* pool, int64_t step,
                                                             int32_t ntiles, int64_t row) {
  if (tb.bound_tile_start != nullptr) {
    const int e = tb.bound_tile_start[ntiles];
    for (int g = threadIdx.x; g < e; g += blockDim.x) {
      const FdsBoundGroup grp = tb.groups[g];
      if (!grp.primary) continue;  // the global array: once per cell (not halo copies)
      TP v = p[grp.cell];
      for (int o = grp.op_begin; o < grp.op_end; ++o) {
        const FdsBoundOp op = tb.ops[o];
        const double val = (op.flags & FDS_BOP_SIGNAL)
                               ? pool[op.off + step * (int64_t)op.stride] + op.scalar
                               : op.scalar;
        v = xadd(xmul((TP)op.mul, v), (TP)val);
      }
      p[grp.cell] = v;
    }
  }
  __syncthreads();
  if (tb.probe_tile_start != nullptr && tb.out_rows > 0) {
    const int e = tb.probe_tile_start[ntiles];
    for (int q = threadIdx.x; q < e; q += blockDim.x) {
      const FdsProbe pr = tb.probes[q];
      tb.out[row * (int64_t)tb.ncols + pr.col] = (double)p[pr.cell];
    }
  }
}

}  // namespace fds
