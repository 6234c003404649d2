// Fused staggered-grid time step for the pyfds field families on sm_103a.
//
// One launch advances one field by one step (pyfds/acoustics.py:111-128 and its
// 1-D / axisymmetric / thermal siblings). A CTA owns a TX x TY tile of cells and
// stages in shared memory everything the step needs around it:
//
//   region  : columns x0-1 .. x0+TX+1, rows y0-1 .. y0+TY+1 (1-D: one row)
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

#include "fds_capi.h"

namespace fds {

template <typename TP, typename TF, typename TC>
struct StagArgs {
  int32_t nx, ny;
  int64_t n;
  int32_t tiles_x;
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
};

// Variant switches of the tile kernel.
template <int TX_, int TY_, int NT_, bool HAS_V_, bool MEMORY_, bool ABSORB_, bool AXI_,
          bool EXACT_>
struct StagCfg {
  static constexpr int TX = TX_;
  static constexpr int TY = TY_;
  static constexpr int NT = NT_;
  static constexpr bool HAS_V = HAS_V_;
  static constexpr bool MEMORY = MEMORY_;  // acoustic flux keeps its old value
  static constexpr bool ABSORB = ABSORB_;
  static constexpr bool AXI = AXI_;
  static constexpr bool EXACT = EXACT_;
  static constexpr int OY = HAS_V ? 1 : 0;  // region row of y0
  static constexpr int RX = TX + 3;
  static constexpr int RY = HAS_V ? TY + 3 : TY;
  static constexpr int RN = RX * RY;
  static constexpr int MIN_BLOCKS = HAS_V ? (NT >= 512 ? 2 : 4) : 2;
};

template <typename T>
__device__ __forceinline__ T ldg0(const T* p, int64_t i, int64_t n) {
  return (i >= 0 && i < n) ? __ldg(p + i) : T(0);
}

// Exact (reference-order) arithmetic: correctly rounded, never contracted.
__device__ __forceinline__ double xmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double xadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double xsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float xmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float xadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float xsub(float a, float b) { return __fsub_rn(a, b); }

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
      const double val = (op.flags & FDS_BOP_SIGNAL) ? pool[op.off + step * (int64_t)op.stride]
                                                     : op.scalar;
      v = xadd(xmul((T)op.mul, v), (T)val);
    }
    s[grp.pos] = v;
  }
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
__device__ __forceinline__ TF absorb_term(const StagArgs<TP, TF, TC>& a, const TF* s, int pos,
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
__device__ __forceinline__ TF absorb_fma(const StagArgs<TP, TF, TC>& a, const TF* s, int pos,
                                         int64_t i, TF acc) {
  if (C::HAS_V) acc = fma((TF)ldg0(a.aym, i - a.nx, a.n), s[pos - C::RX], acc);
  acc = fma((TF)ldg0(a.axm, i - 1, a.n), s[pos - 1], acc);
  acc = fma((TF)ldg0(a.ad, i, a.n), s[pos], acc);
  acc = fma((TF)ldg0(a.axp, i + 1, a.n), s[pos + 1], acc);
  if (C::HAS_V) acc = fma((TF)ldg0(a.ayp, i + a.nx, a.n), s[pos + C::RX], acc);
  return acc;
}

// New flux at flat index i from the potential slots (pos, pos - back) and the
// old flux; sB holds this direction's factors (slots of out-of-range cells hold 0).
template <class C, bool IS_X, typename TP, typename TF, typename TC>
__device__ __forceinline__ TF flux_new(const StagArgs<TP, TF, TC>& a, const TP* sP, const TF* sF,
                                       const TC* sB, int pos, int64_t i, int x) {
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
        const TF rad = (TF)__ldg(a.rx + x);
        const TF e = xmul((TF)__ldg(a.ex + i), u);
        r = xadd(r, e / xmul(rad, rad));
      }
      return xsub(u, r);
    }
  } else {
    if constexpr (!C::MEMORY) {
      return fma(bm, pm, -(b * p));
    } else {
      TF acc = sF[pos];
      acc = fma(-b, p, acc);
      acc = fma(bm, pm, acc);
      if constexpr (C::ABSORB) acc = absorb_fma<C>(a, sF, pos, i, acc);
      if constexpr (C::AXI && C::ABSORB && IS_X) {
        const TF rad = (TF)__ldg(a.rx + x);
        acc = acc - ((TF)__ldg(a.ex + i) * sF[pos]) / (rad * rad);
      }
      return acc;
    }
  }
}

// Dynamic shared memory of one CTA of this variant.
template <class C, typename TP, typename TF, typename TC>
constexpr size_t stag_smem_bytes(bool iso) {
  return (size_t)C::RN * (sizeof(TP) + (C::HAS_V ? 2 : 1) * sizeof(TF) +
                          (iso || !C::HAS_V ? 2 : 4) * sizeof(TC));
}

template <class C, typename TP, typename TF, typename TC>
__global__ void __launch_bounds__(C::NT, C::MIN_BLOCKS)
    stag_step_kernel(const StagArgs<TP, TF, TC> a) {
  constexpr int TX = C::TX, TY = C::TY, NT = C::NT, RX = C::RX, RN = C::RN, OY = C::OY;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TP* sP = reinterpret_cast<TP*>(smem_raw);
  TF* sU = reinterpret_cast<TF*>(sP + RN);
  TF* sV = sU + (C::HAS_V ? RN : 0);
  TC* sBx = reinterpret_cast<TC*>(sV + RN);
  TC* sKx = sBx + RN;
  const bool iso = a.iso || !C::HAS_V;
  TC* sBy = iso ? sBx : sKx + RN;
  TC* sKy = iso ? sKx : sBy + RN;

  const int tile = blockIdx.x;
  const int tx = tile % a.tiles_x;
  const int ty = tile / a.tiles_x;
  const int x0 = tx * TX;
  const int y0 = ty * TY;
  const int x1 = min(x0 + TX, a.nx);  // end of owned columns
  const int y1 = min(y0 + TY, a.ny);
  const int tid = threadIdx.x;

  // ---- stage the potential, old flux and coefficients over the region ----
  for (int e = tid; e < RN; e += NT) {
    const int lx = e % RX - 1;
    const int ly = e / RX - OY;
    const int64_t f = (int64_t)(y0 + ly) * a.nx + (x0 + lx);
    const bool ok = (f >= 0 && f < a.n);
    sP[e] = ok ? a.p_in[f] : TP(0);
    if constexpr (C::MEMORY) {
      sU[e] = ok ? a.u_in[f] : TF(0);
      if constexpr (C::HAS_V) sV[e] = ok ? a.v_in[f] : TF(0);
    }
    sBx[e] = ok ? __ldg(a.bx + f) : TC(0);
    sKx[e] = ok ? __ldg(a.kx + f) : TC(0);
    if (!iso) {
      sBy[e] = ok ? __ldg(a.by + f) : TC(0);
      sKy[e] = ok ? __ldg(a.ky + f) : TC(0);
    }
  }
  __syncthreads();

  // ---- flux update over U-ext and V-ext, kept in registers ----
  constexpr int UC = (TX + 1) * TY;
  constexpr int UIT = (UC + NT - 1) / NT;
  constexpr int VC = C::HAS_V ? TX * (TY + 1) : 0;
  constexpr int VIT = C::HAS_V ? (VC + NT - 1) / NT : 0;
  TF un[UIT];
  TF vn[VIT > 0 ? VIT : 1];
#pragma unroll
  for (int k = 0; k < UIT; ++k) {
    const int e = tid + k * NT;
    un[k] = TF(0);
    if (e < UC) {
      const int lx = e % (TX + 1);
      const int ly = e / (TX + 1);
      const int x = x0 + lx;
      const int y = y0 + ly;
      const int64_t f = (int64_t)y * a.nx + x;
      if (x <= x1 && y < y1 && f < a.n) {
        const int pos = (ly + OY) * RX + lx + 1;
        const int xr = (x == a.nx) ? 0 : x;  // column of the wrapped halo cell
        un[k] = flux_new<C, true>(a, sP, sU, sBx, pos, f, xr);
      }
    }
  }
  if constexpr (C::HAS_V) {
#pragma unroll
    for (int k = 0; k < VIT; ++k) {
      const int e = tid + k * NT;
      vn[k] = TF(0);
      if (e < VC) {
        const int lx = e % TX;
        const int ly = e / TX;
        const int x = x0 + lx;
        const int y = y0 + ly;
        const int64_t f = (int64_t)y * a.nx + x;
        if (x < x1 && y <= y1 && f < a.n) {
          const int pos = (ly + OY) * RX + lx + 1;
          vn[k] = flux_new<C, false>(a, sP, sV, sBy, pos, f, x);
        }
      }
    }
  }
  if constexpr (C::MEMORY && C::ABSORB) __syncthreads();  // neighbours read old flux
#pragma unroll
  for (int k = 0; k < UIT; ++k) {
    const int e = tid + k * NT;
    if (e < UC) sU[(e / (TX + 1) + OY) * RX + e % (TX + 1) + 1] = un[k];
  }
  if constexpr (C::HAS_V) {
#pragma unroll
    for (int k = 0; k < VIT; ++k) {
      const int e = tid + k * NT;
      if (e < VC) sV[(e / TX + OY) * RX + e % TX + 1] = vn[k];
    }
  }
  __syncthreads();

  // ---- flux bounds and probes (this step) ----
  apply_bound_groups<NT>(a.tab[1], tile, sU, a.pool, a.step);
  if constexpr (C::HAS_V) apply_bound_groups<NT>(a.tab[2], tile, sV, a.pool, a.step);
  __syncthreads();
  write_probes<NT>(a.tab[1], tile, sU, a.step - a.step0);
  if constexpr (C::HAS_V) write_probes<NT>(a.tab[2], tile, sV, a.step - a.step0);

  // ---- potential update of the owned cells ----
  constexpr int OC = TX * TY;
  constexpr int OIT = (OC + NT - 1) / NT;
  TP pn[OIT];
#pragma unroll
  for (int k = 0; k < OIT; ++k) {
    const int e = tid + k * NT;
    const int lx = e % TX;
    const int ly = e / TX;
    const int x = x0 + lx;
    const int y = y0 + ly;
    const int64_t f = (int64_t)y * a.nx + x;
    pn[k] = TP(0);
    if (e < OC && x < x1 && y < y1) {
      const int pos = (ly + OY) * RX + lx + 1;
      if (a.store_flux) {
        a.u_out[f] = sU[pos];
        if constexpr (C::HAS_V) a.v_out[f] = sV[pos];
      }
      const TF kxi = (TF)sKx[pos];
      const TF kxn = (TF)sKx[pos + 1];
      const TF u = sU[pos];
      const TF un1 = sU[pos + 1];
      TF kyi = TF(0), kyn = TF(0), v = TF(0), vn1 = TF(0);
      if constexpr (C::HAS_V) {
        kyi = (TF)sKy[pos];
        kyn = (TF)sKy[pos + RX];
        v = sV[pos];
        vn1 = sV[pos + RX];
      }
      if constexpr (C::EXACT) {
        TF w = u, wn = un1;
        if constexpr (C::AXI) {
          // a_p_vx.dot(vx * r): the flux is scaled by the radius of its column
          const int xn = (x + 1 == a.nx) ? 0 : x + 1;
          w = xmul(u, (TF)__ldg(a.rx + x));
          wn = xmul(un1, (TF)__ldg(a.rx + xn));
        }
        // forward difference, offsets [0, s]: (0 + (-k)*w) + kn*wn
        TF sx = xadd(-xmul(kxi, w), xmul(kxn, wn));
        if constexpr (C::HAS_V) {
          const TF sy = xadd(-xmul(kyi, v), xmul(kyn, vn1));
          sx = xadd(sx, sy);
        }
        pn[k] = (TP)xsub((TF)sP[pos], sx);
      } else if constexpr (sizeof(TP) == sizeof(TF)) {
        TF acc = (TF)sP[pos];
        acc = fma(kxi, u, acc);
        acc = fma(-kxn, un1, acc);
        if constexpr (C::HAS_V) {
          acc = fma(kyi, v, acc);
          acc = fma(-kyn, vn1, acc);
        }
        pn[k] = (TP)acc;
      } else {
        // float increment accumulated into a float64 potential
        TF inc = kxi * u;
        inc = fma(-kxn, un1, inc);
        if constexpr (C::HAS_V) {
          inc = fma(kyi, v, inc);
          inc = fma(-kyn, vn1, inc);
        }
        pn[k] = sP[pos] + (TP)inc;
      }
    }
  }
  __syncthreads();  // all reads of sP done
#pragma unroll
  for (int k = 0; k < OIT; ++k) {
    const int e = tid + k * NT;
    if (e < OC) sP[(e / TX + OY) * RX + e % TX + 1] = pn[k];
  }
  if (a.apply_next) {
    __syncthreads();
    apply_bound_groups<NT>(a.tab[0], tile, sP, a.pool, a.step + 1);
    __syncthreads();
    write_probes<NT>(a.tab[0], tile, sP, a.step + 1 - a.step0);
  }
  // ---- store the owned potential ----
#pragma unroll
  for (int k = 0; k < OIT; ++k) {
    const int e = tid + k * NT;
    const int lx = e % TX;
    const int ly = e / TX;
    const int x = x0 + lx;
    const int y = y0 + ly;
    if (e < OC && x < x1 && y < y1) {
      a.p_out[(int64_t)y * a.nx + x] = sP[(ly + OY) * RX + lx + 1];
    }
  }
}

// Potential bounds and probes of the first step of a call, in place on the
// global potential (one CTA: bounds, barrier, probes).
template <typename TP>
__global__ void __launch_bounds__(1024) stag_prologue_kernel(TP* p, FdsCompTables tb,
                                                             const double* pool, int64_t step,
                                                             int32_t ntiles) {
  if (tb.bound_tile_start != nullptr) {
    const int e = tb.bound_tile_start[ntiles];
    for (int g = threadIdx.x; g < e; g += blockDim.x) {
      const FdsBoundGroup grp = tb.groups[g];
      TP v = p[grp.cell];
      for (int o = grp.op_begin; o < grp.op_end; ++o) {
        const FdsBoundOp op = tb.ops[o];
        const double val = (op.flags & FDS_BOP_SIGNAL) ? pool[op.off + step * (int64_t)op.stride]
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
      tb.out[pr.col] = (double)p[pr.cell];
    }
  }
}

}  // namespace fds
