// Every step of a call for a 1-D field spread over the CTAs of one thread-block
// cluster (pyfds/acoustics.py:40-52, pyfds/thermal.py:46-51, repeated by
// Field.simulate, pyfds/fields.py:87-93).
//
// One CTA holds a field of a few thousand cells in shared memory, but then the step
// runs on one SM: four DFMA per cell and step at two per clock, about 1 us per step
// for 1000 cells. Here CTA r of a cluster of CL CTAs owns the cells [c0, c1) =
// [r m, min(n, (r + 1) m)) and keeps a window of G = K + 1 further cells on each side:
// slot j of its shared arrays holds cell c0 - G - 1 + j, for j in [0, W + 2) with
// W = m + 2 G (slots 0 and W + 1 pad the window; slots of cells outside the field hold
// zeros, the neighbours the reference's operators drop, and are never updated).
//
// A block of K steps updates every window cell that lies in the field without any
// exchange. The flux of cell i reads the potentials of cells i - 1 and i (with
// absorption also the old fluxes of cells i - 1 and i + 1) and the potential of cell i
// the new fluxes of cells i and i + 1, so values that depend on the stale cells past
// the window's edges spread by one cell per step: after k steps of a block the cells
// [c0 - G, c0 - G + k) and, on the right, the potentials from c1 + G - k - 1 on
// (the fluxes from c1 + G - k on) may be wrong, and after K steps the owned cells
// are still exact. Then each CTA writes the potential and flux of its first G cells
// into the left neighbour's inbox and of its last G cells into the right neighbour's,
// through distributed shared memory; one cluster barrier makes them visible, and the
// next block starts by copying the inbox into the window's edge cells. The inboxes
// are double-buffered by block parity: a neighbour writes inbox[b & 1] at the end of
// block b, this CTA reads it at the start of block b + 1, and the next write into it
// (end of block b + 2) comes after the barrier that ends block b + 1, which this CTA
// reaches only after that read. A call takes ceil(nsteps / K) - 1 cluster barriers
// instead of one per step, for 2 G / m more cell updates.
//
// Every window cell runs the tile kernel's arithmetic (flux_new, potential_regs) and
// the boundary chain of its cell (the tables by cell, as the owner applies them), in
// the thread that computed the value and before it is stored, as are the probes of
// the owned cells; so a step takes two CTA barriers (three with absorption), and the
// owned cells are the tile kernel's bit for bit.
#pragma once

#include <algorithm>

#include "resident_1d.cuh"

namespace fds {

constexpr int kClusterThreads = 128;
constexpr int kClusterCellsPerThread = 9;  // window slots per thread
constexpr int kClusterPortableCta = 8;     // the portable cluster size
constexpr int kClusterMaxCta = 16;         // with the non-portable size allowed
constexpr int kClusterMaxCellsPerCta = 1024;
constexpr int kClusterWindow = kClusterThreads * kClusterCellsPerThread;
constexpr int kClusterMaxBlockSteps = 64;

// Steps per exchange block for m owned cells (`want`: the requested count, 0 for the
// default): by default the window m + 2 (K + 1) fills the slots of the fewest
// thread passes that hold m + 4 cells (the flux and potential updates of a step take
// one dependent chain per pass), at most kClusterMaxBlockSteps; always the window fits
// the slots of one CTA, each window edge (K + 1 cells) lies within the one
// neighbouring CTA (K + 1 <= m), and K >= 1.
inline int cluster_block_steps(int m, int want) {
  const int passes = (m + 4 + kClusterThreads - 1) / kClusterThreads;
  int k = want > 0 ? want
                   : std::min(kClusterMaxBlockSteps, (passes * kClusterThreads - m) / 2 - 1);
  k = std::min(k, (kClusterWindow - m) / 2 - 1);
  k = std::min(k, m - 1);
  return std::max(k, 1);
}

// Shared memory of the inboxes of a window edge of g cells: potential and flux, two
// sides, two block parities.
template <typename TP, typename TF>
__host__ __device__ constexpr size_t cluster_inbox_bytes(int g) {
  return round128((size_t)4 * g * sizeof(TP)) + round128((size_t)4 * g * sizeof(TF));
}

// Shared memory of a window of w cells: potential, flux, the two coefficient arrays,
// and per slot and component (potential, flux) the boundary chain's operation range
// and the probe code (cluster_slot_tables).
template <typename TP, typename TF, typename TC>
__host__ __device__ constexpr size_t cluster_window_bytes(int w) {
  return resident_smem<TP, TF, TC>(w) + 2 * round128((size_t)(w + 2) * sizeof(int2)) +
         2 * round128((size_t)(w + 2) * sizeof(int));
}

// The boundary chain ops[r.x, r.y) applied to the new value v of a cell (the step's
// signal samples from pool): the tile kernel's chain, in the thread that computed v.
template <typename T>
__device__ __forceinline__ T bound_chain(const ResidentTables& t, int2 r, T v,
                                         const double* pool, int64_t step) {
  for (int o = r.x; o < r.y; ++o) {
    const FdsBoundOp op = t.ops[o];
    const double val = (op.flags & FDS_BOP_SIGNAL)
                           ? pool[op.off + step * (int64_t)op.stride] + op.scalar
                           : op.scalar;
    v = xadd(xmul((T)op.mul, v), (T)val);
  }
  return v;
}

// Output row `row` of the probes of one cell: `code` is the column of its only probe,
// or -2 when it has several (found in the probe list).
template <typename T>
__device__ __forceinline__ void probe_cell(const ResidentTables& t, const FdsCompTables& tb,
                                           int code, int cell, int64_t row, T v) {
  if (row >= tb.out_rows) return;
  double* out = tb.out + row * (int64_t)tb.ncols;
  if (code >= 0) {
    out[code] = (double)v;
    return;
  }
  for (int q = 0; q < t.nprobes; ++q)
    if (t.probes[q].cell == cell) out[t.probes[q].col] = (double)v;
}

// Per window slot: the operation range of the cell's boundary chain ({0, 0}: none)
// for the cells [lo, hi), one primary placement per cell as the table compiler
// merges them; the probe code of the owned cells [c0, c1) (-1: none, a column, -2:
// several). Called by every thread; ends with a barrier.
__device__ __forceinline__ void cluster_slot_tables(const ResidentTables* rt, int2* gr,
                                                    int* pc, int w, int base, int lo, int hi,
                                                    int c0, int c1) {
  for (int j = threadIdx.x; j < 2 * (w + 2); j += blockDim.x) {
    gr[j] = make_int2(0, 0);
    pc[j] = -1;
  }
  __syncthreads();
  for (int c = 0; c < 2; ++c) {
    for (int g = threadIdx.x; g < rt[c].ngroups; g += blockDim.x) {
      const FdsBoundGroup grp = rt[c].groups[g];
      if (grp.primary && grp.cell >= lo && grp.cell < hi)
        gr[c * (w + 2) + (int)grp.cell - base + 1] = make_int2(grp.op_begin, grp.op_end);
    }
    for (int q = threadIdx.x; q < rt[c].nprobes; q += blockDim.x) {
      const FdsProbe pr = rt[c].probes[q];
      if (pr.cell >= c0 && pr.cell < c1) {
        int* code = &pc[c * (w + 2) + (int)pr.cell - base + 1];
        if (atomicCAS(code, -1, pr.col) != -1) atomicExch(code, -2);
      }
    }
  }
  __syncthreads();
}

// Store v into the shared-memory word `local` of cluster CTA `rank` (the same
// offset in that CTA's shared memory).
template <typename T>
__device__ __forceinline__ void st_cluster(T* local, uint32_t rank, const T& v) {
  static_assert(sizeof(T) == 4 || sizeof(T) == 8, "4- or 8-byte values");
  uint32_t remote;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;\n"
               : "=r"(remote)
               : "r"(smem_addr(local)), "r"(rank));
  if constexpr (sizeof(T) == 8) {
    uint64_t bits;
    memcpy(&bits, &v, 8);
    asm volatile("st.shared::cluster.u64 [%0], %1;\n" ::"r"(remote), "l"(bits) : "memory");
  } else {
    uint32_t bits;
    memcpy(&bits, &v, 4);
    asm volatile("st.shared::cluster.u32 [%0], %1;\n" ::"r"(remote), "r"(bits) : "memory");
  }
}

// Every thread of every CTA of the cluster arrives; the release / acquire pair orders
// the distributed-shared-memory stores before the barrier with the loads after it.
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n"
               "barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

// Dynamic shared memory: the inboxes (at offset 0, the same in every CTA of the
// cluster), the window (cluster_window_bytes), the boundary and probe tables, the
// signal pool when it fits.
template <class C, typename TP, typename TF, typename TC>
__global__ void __launch_bounds__(kClusterThreads, 1)
    stag_1d_cluster_kernel(const __grid_constant__ StagArgs<TP, TF, TC> a, int32_t nsteps,
                           TP* p_fin, TF* u_fin, int64_t pool_cached, int32_t m, int32_t K) {
  static_assert(!C::HAS_V, "1-D fields");
  constexpr int CPT = kClusterCellsPerThread;
  constexpr int NT = kClusterThreads;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int n = (int)a.n;
  const int rank = (int)blockIdx.x;  // the grid is one cluster
  const int ncta = (int)gridDim.x;
  const int G = K + 1;
  const int W = m + 2 * G;
  const int c0 = rank * m;
  const int c1 = min(n, c0 + m);
  const int base = c0 - G;      // the cell of slot 1
  const int lo = max(base, 0);  // the window's cells in the field: [lo, hi)
  const int hi = min(base + W, n);
  const int jl = lo - base + 1;  // their first slot
  const int cnt = hi - lo;
  TP* inP = reinterpret_cast<TP*>(smem_raw);  // [parity][side: 0 left, 1 right][G]
  TF* inU = reinterpret_cast<TF*>(smem_raw + round128((size_t)4 * G * sizeof(TP)));
  unsigned char* win = smem_raw + cluster_inbox_bytes<TP, TF>(G);
  TP* sP = reinterpret_cast<TP*>(win);
  TF* sU = reinterpret_cast<TF*>(win + resident_bytes<TP>(W));
  TC* sB = reinterpret_cast<TC*>(win + resident_bytes<TP>(W) + resident_bytes<TF>(W));
  TC* sK = reinterpret_cast<TC*>(win + resident_bytes<TP>(W) + resident_bytes<TF>(W) +
                                 resident_bytes<TC>(W));
  const int tid = threadIdx.x;
  for (int j = tid; j < W + 2; j += NT) {
    const int i = base - 1 + j;
    const bool in = i >= 0 && i < n;
    sP[j] = in ? a.p_in[i] : TP(0);
    sU[j] = (in && C::MEMORY) ? a.u_in[i] : TF(0);
    sB[j] = in ? a.bx[i] : TC(0);
    sK[j] = in ? a.kx[i] : TC(0);
  }
  int2* gr = reinterpret_cast<int2*>(win + resident_smem<TP, TF, TC>(W));  // [2][W + 2]
  int* pc = reinterpret_cast<int*>(win + resident_smem<TP, TF, TC>(W) +
                                   2 * round128((size_t)(W + 2) * sizeof(int2)));
  unsigned char* area = win + cluster_window_bytes<TP, TF, TC>(W);
  ResidentTables rt[2];
  stage_tables(a.tab, a.ntiles, area, rt);  // ends with a barrier
  const double* pool = a.pool;
  if (pool_cached > 0) {
    double* sp = reinterpret_cast<double*>(area + kResidentTableBytes);
    for (int64_t i = tid; i < pool_cached; i += NT) sp[i] = a.pool[i];
    pool = sp;
  }
  cluster_slot_tables(rt, gr, pc, W, base, lo, hi, c0, c1);  // ends with a barrier
  const int2* grP = gr;  // potential (component 0)
  const int2* grF = gr + (W + 2);
  const int* pcP = pc;
  const int* pcF = pc + (W + 2);
  // every CTA of the cluster runs (and has staged its pool) before a neighbour writes
  // into its shared memory
  cluster_sync();
  int blk = 0;
  for (int32_t s0 = 0; s0 < nsteps; s0 += K, ++blk) {
    if (blk > 0) {
      // the window's edge cells from the neighbours' last block
      const int par = (blk - 1) & 1;
      for (int t = tid; t < G; t += NT) {
        if (rank > 0) {
          sP[1 + t] = inP[(par * 2 + 0) * G + t];
          if constexpr (C::MEMORY) sU[1 + t] = inU[(par * 2 + 0) * G + t];
        }
        if (c1 + t < n) {
          const int j = c1 + t - base + 1;
          sP[j] = inP[(par * 2 + 1) * G + t];
          if constexpr (C::MEMORY) sU[j] = inU[(par * 2 + 1) * G + t];
        }
      }
      __syncthreads();
    }
    const int ke = min(K, nsteps - s0);
    for (int k = 0; k < ke; ++k) {
      const int32_t s = s0 + k;
      const int64_t step = a.step + s;
      // ---- new flux of every window cell in the field, its boundary chain and probes
      // in the same thread ----
      TF un[CPT];
#pragma unroll
      for (int q = 0; q < CPT; ++q) {
        if (q * NT >= cnt) break;
        const int j = tid + q * NT;
        if (j < cnt) {
          const int ps = jl + j;
          TF v = flux_new<C, true>(a, sP, sU, sB, ps, (int64_t)(lo + j), lo + j);
          const int2 r = grF[ps];
          if (r.y > r.x) v = bound_chain(rt[1], r, v, pool, step);
          const int code = pcF[ps];
          if (code != -1) probe_cell(rt[1], a.tab[1], code, lo + j, s, v);
          un[q] = v;
        } else {
          un[q] = TF(0);
        }
      }
      if constexpr (C::MEMORY && C::ABSORB) __syncthreads();  // neighbours read the old flux
#pragma unroll
      for (int q = 0; q < CPT; ++q) {
        if (q * NT >= cnt) break;
        const int j = tid + q * NT;
        if (j < cnt) sU[jl + j] = un[q];
      }
      __syncthreads();
      // ---- new potential of every window cell in the field; the next step's
      // boundary chain and probes (the last step's are the next call's prologue) ----
      const bool next = s + 1 < nsteps;
      TP pn[CPT];
#pragma unroll
      for (int q = 0; q < CPT; ++q) {
        if (q * NT >= cnt) break;
        const int j = tid + q * NT;
        if (j < cnt) {
          const int ps = jl + j;
          TP v = potential_regs<C>(a, sP[ps], sU[ps], sU[ps + 1], TF(0), TF(0), (TF)sK[ps],
                                   (TF)sK[ps + 1], TF(0), TF(0), lo + j);
          if (next) {
            const int2 r = grP[ps];
            if (r.y > r.x) v = bound_chain(rt[0], r, v, pool, step + 1);
            const int code = pcP[ps];
            if (code != -1) probe_cell(rt[0], a.tab[0], code, lo + j, s + 1, v);
          }
          pn[q] = v;
        } else {
          pn[q] = TP(0);
        }
      }
#pragma unroll
      for (int q = 0; q < CPT; ++q) {
        if (q * NT >= cnt) break;
        const int j = tid + q * NT;
        if (j < cnt) sP[jl + j] = pn[q];
      }
      __syncthreads();
    }
    if (s0 + K < nsteps) {
      // the first G owned cells to the left neighbour's right edge, the last G to the
      // right neighbour's left edge (a neighbour's window edge lies within this CTA's
      // cells, or past the field)
      const int par = blk & 1;
      for (int t = tid; t < G; t += NT) {
        if (rank > 0 && c0 + t < c1) {
          const int j = c0 + t - base + 1;
          st_cluster(&inP[(par * 2 + 1) * G + t], (uint32_t)(rank - 1), sP[j]);
          if constexpr (C::MEMORY)
            st_cluster(&inU[(par * 2 + 1) * G + t], (uint32_t)(rank - 1), sU[j]);
        }
        if (rank + 1 < ncta) {
          const int j = c1 - G + t - base + 1;
          st_cluster(&inP[(par * 2 + 0) * G + t], (uint32_t)(rank + 1), sP[j]);
          if constexpr (C::MEMORY)
            st_cluster(&inU[(par * 2 + 0) * G + t], (uint32_t)(rank + 1), sU[j]);
        }
      }
      cluster_sync();
    }
  }
  // (no CTA writes into another's shared memory after the barrier that ends the
  // second-to-last block, so each CTA may leave as soon as it is done)
  bool bad = false;
  for (int c = c0 + tid; c < c1; c += NT) {
    const int j = c - base + 1;
    const TP v = sP[j];
    p_fin[c] = v;
    u_fin[c] = sU[j];
    bad = bad || nonfinite(v);
  }
  if (a.status && __any_sync(0xffffffffu, bad) && (tid & 31) == 0)
    atomicOr(a.status, kStatusNonFinite);
}

}  // namespace fds
