// Every step of a call for a 1-D field that fits one CTA's shared memory, in one
// launch (pyfds/acoustics.py:40-52 for Acoustic1D, pyfds/thermal.py:46-51 for
// Thermal1D, repeated by Field.simulate, pyfds/fields.py:87-93).
//
// A 1-D field of a few thousand cells is far too small to fill a GPU: one launch per
// step costs a few microseconds of launch and wave overhead for well under a
// microsecond of arithmetic. Here one CTA loads the potential, the flux and their
// coefficients into shared memory once, runs every step with barriers between the
// phases, and stores the state once. Slot i + 1 holds cell i; slots 0 and n + 1 hold
// zeros, the neighbours the reference's operators drop. Each cell is computed by
// flux_new and potential_cell, the arithmetic of the tile kernel, so the results are
// the tile kernel's bit for bit (and, in exact mode, the reference's).
//
// Boundaries and outputs come from the same per-tile tables: every boundary group
// flagged primary (one per cell) and every probe, addressed by its flat cell index.
// The first step's potential bounds and probes are applied by the prologue kernel,
// as for the tile kernel.
#pragma once

#include "stag_kernel.cuh"

namespace fds {

constexpr int kResidentThreads = 1024;
constexpr int kResidentCellsPerThread = 4;
constexpr int kResidentMaxCells = kResidentThreads * kResidentCellsPerThread;

// Boundary chains of one component on every primary placement, applied to the
// field-wide slot array s (slot = cell + 1).
template <typename T>
__device__ __forceinline__ void apply_bound_cells(const FdsCompTables& tb, int ntiles, T* s,
                                                  const double* pool, int64_t step) {
  if (tb.bound_tile_start == nullptr) return;
  const int e = tb.bound_tile_start[ntiles];
  for (int g = threadIdx.x; g < e; g += blockDim.x) {
    const FdsBoundGroup grp = tb.groups[g];
    if (!grp.primary) continue;
    T v = s[grp.cell + 1];
    for (int o = grp.op_begin; o < grp.op_end; ++o) {
      const FdsBoundOp op = tb.ops[o];
      const double val = (op.flags & FDS_BOP_SIGNAL)
                             ? pool[op.off + step * (int64_t)op.stride] + op.scalar
                             : op.scalar;
      v = xadd(xmul((T)op.mul, v), (T)val);
    }
    s[grp.cell + 1] = v;
  }
}

template <typename T>
__device__ __forceinline__ void write_probe_cells(const FdsCompTables& tb, int ntiles,
                                                  const T* s, int64_t row) {
  if (tb.probe_tile_start == nullptr) return;
  if (row < 0 || row >= tb.out_rows) return;
  const int e = tb.probe_tile_start[ntiles];
  double* out = tb.out + row * (int64_t)tb.ncols;
  for (int q = threadIdx.x; q < e; q += blockDim.x) {
    const FdsProbe pr = tb.probes[q];
    out[pr.col] = (double)s[pr.cell + 1];
  }
}

__device__ __forceinline__ bool has_bounds(const FdsCompTables& tb, int ntiles) {
  return tb.bound_tile_start != nullptr && tb.bound_tile_start[ntiles] > 0;
}

__device__ __forceinline__ bool has_probes(const FdsCompTables& tb, int ntiles) {
  return tb.probe_tile_start != nullptr && tb.probe_tile_start[ntiles] > 0;
}

template <typename T>
__host__ __device__ constexpr size_t resident_bytes(int n) {
  return round128((size_t)(n + 2) * sizeof(T));
}

// Shared memory of a resident run of n cells.
template <typename TP, typename TF, typename TC>
__host__ __device__ constexpr size_t resident_smem(int n) {
  return resident_bytes<TP>(n) + resident_bytes<TF>(n) + 2 * resident_bytes<TC>(n);
}

template <class C, typename TP, typename TF, typename TC>
__global__ void __launch_bounds__(kResidentThreads, 1)
    stag_1d_resident_kernel(const __grid_constant__ StagArgs<TP, TF, TC> a, int32_t nsteps,
                            TP* p_fin, TF* u_fin) {
  static_assert(!C::HAS_V, "1-D fields");
  constexpr int CPT = kResidentCellsPerThread;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int n = (int)a.n;
  const int ntiles = a.ntiles;
  TP* sP = reinterpret_cast<TP*>(smem_raw);
  TF* sU = reinterpret_cast<TF*>(smem_raw + resident_bytes<TP>(n));
  TC* sB = reinterpret_cast<TC*>(smem_raw + resident_bytes<TP>(n) + resident_bytes<TF>(n));
  TC* sK = reinterpret_cast<TC*>(smem_raw + resident_bytes<TP>(n) + resident_bytes<TF>(n) +
                                 resident_bytes<TC>(n));
  const int tid = threadIdx.x;
  for (int j = tid; j < n + 2; j += kResidentThreads) {
    const int i = j - 1;
    const bool in = i >= 0 && i < n;
    sP[j] = in ? a.p_in[i] : TP(0);
    sU[j] = (in && C::MEMORY) ? a.u_in[i] : TF(0);
    sB[j] = in ? a.bx[i] : TC(0);
    sK[j] = in ? a.kx[i] : TC(0);
  }
  const bool fb = has_bounds(a.tab[1], ntiles);
  const bool fp = has_probes(a.tab[1], ntiles);
  const bool pb = has_bounds(a.tab[0], ntiles);
  const bool pp = has_probes(a.tab[0], ntiles);
  __syncthreads();
  for (int32_t s = 0; s < nsteps; ++s) {
    const int64_t step = a.step + s;
    // ---- new flux of every cell ----
    TF un[CPT];
#pragma unroll
    for (int k = 0; k < CPT; ++k) {
      const int i = tid + k * kResidentThreads;
      un[k] = i < n ? flux_new<C, true>(a, sP, sU, sB, i + 1, (int64_t)i, i) : TF(0);
    }
    if constexpr (C::MEMORY && C::ABSORB) __syncthreads();  // neighbours read the old flux
#pragma unroll
    for (int k = 0; k < CPT; ++k) {
      const int i = tid + k * kResidentThreads;
      if (i < n) sU[i + 1] = un[k];
    }
    __syncthreads();
    if (fb) {
      apply_bound_cells(a.tab[1], ntiles, sU, a.pool, step);
      __syncthreads();
    }
    if (fp) write_probe_cells(a.tab[1], ntiles, sU, s);
    // ---- new potential of every cell (each thread reads its own cells' potential) ----
    TP pn[CPT];
#pragma unroll
    for (int k = 0; k < CPT; ++k) {
      const int i = tid + k * kResidentThreads;
      pn[k] = i < n ? potential_cell<C>(a, sP, sU, sU, sK, sK, i + 1, i) : TP(0);
    }
#pragma unroll
    for (int k = 0; k < CPT; ++k) {
      const int i = tid + k * kResidentThreads;
      if (i < n) sP[i + 1] = pn[k];
    }
    __syncthreads();
    if (s + 1 < nsteps) {
      // the next step's potential bounds and probes
      if (pb) {
        apply_bound_cells(a.tab[0], ntiles, sP, a.pool, step + 1);
        __syncthreads();
      }
      if (pp) write_probe_cells(a.tab[0], ntiles, sP, s + 1);
    }
  }
  // the call's last potential reports a diverged field
  bool bad = false;
  for (int j = tid; j < n; j += kResidentThreads) {
    const TP v = sP[j + 1];
    p_fin[j] = v;
    u_fin[j] = sU[j + 1];
    bad = bad || nonfinite(v);
  }
  if (a.status && __any_sync(0xffffffffu, bad) && (tid & 31) == 0)
    atomicOr(a.status, kStatusNonFinite);
}

}  // namespace fds
