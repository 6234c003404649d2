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
// They are copied into shared memory when they fit, and so is the boundary signal
// pool, so that a step reads no global memory except the absorption diagonals. The
// first step's potential bounds and probes are applied by the prologue kernel, as
// for the tile kernel.
#pragma once

#include "stag_kernel.cuh"

namespace fds {

constexpr int kResidentThreads = 1024;
constexpr int kResidentCellsPerThread = 4;
constexpr int kResidentMaxCells = kResidentThreads * kResidentCellsPerThread;

// Shared memory for the boundary groups, operations and probes of the potential and
// the flux (used when they fit; a few boundary cells and probes, as 1-D fields have).
constexpr size_t kResidentTableBytes = 32 * 1024;
constexpr size_t kResidentMaxSmem = 227 * 1024;  // opt-in shared memory of one CTA

// One component's boundary groups, operations and probes (shared or global memory).
struct ResidentTables {
  int ngroups, nprobes;
  const FdsBoundGroup* groups;
  const FdsBoundOp* ops;
  const FdsProbe* probes;
  const int32_t* group_count;  // non-null: ngroups as read from the table
};

// Boundary chains on every primary placement (one per cell), applied to the
// field-wide slot array s (slot = cell + 1).
template <typename T>
__device__ __forceinline__ void apply_bound_cells(const ResidentTables& t, T* s,
                                                  const double* pool, int64_t step) {
  for (int g = threadIdx.x; g < t.ngroups; g += blockDim.x) {
    const FdsBoundGroup grp = t.groups[g];
    if (!grp.primary) continue;
    T v = s[grp.cell + 1];
    for (int o = grp.op_begin; o < grp.op_end; ++o) {
      const FdsBoundOp op = t.ops[o];
      const double val = (op.flags & FDS_BOP_SIGNAL)
                             ? pool[op.off + step * (int64_t)op.stride] + op.scalar
                             : op.scalar;
      v = xadd(xmul((T)op.mul, v), (T)val);
    }
    s[grp.cell + 1] = v;
  }
}

template <typename T>
__device__ __forceinline__ void write_probe_cells(const ResidentTables& t, const FdsCompTables& tb,
                                                  const T* s, int64_t row) {
  if (row < 0 || row >= tb.out_rows) return;
  double* out = tb.out + row * (int64_t)tb.ncols;
  for (int q = threadIdx.x; q < t.nprobes; q += blockDim.x) {
    const FdsProbe pr = t.probes[q];
    out[pr.col] = (double)s[pr.cell + 1];
  }
}

// The tables of components 0 and 1, copied into `area` (kResidentTableBytes) when
// they fit, else read where they are. Called by every thread; ends with a barrier.
__device__ __forceinline__ void stage_tables(const FdsCompTables* tab, int ntiles,
                                             unsigned char* area, ResidentTables* out) {
  __shared__ int s_nops[2];
  int ng[2], np[2];
  for (int c = 0; c < 2; ++c) {
    ng[c] = tab[c].bound_tile_start ? tab[c].bound_tile_start[ntiles] : 0;
    np[c] = tab[c].probe_tile_start ? tab[c].probe_tile_start[ntiles] : 0;
  }
  if (threadIdx.x < 2) s_nops[threadIdx.x] = 0;
  __syncthreads();
  for (int c = 0; c < 2; ++c)
    for (int g = threadIdx.x; g < ng[c]; g += blockDim.x)
      atomicMax(&s_nops[c], tab[c].groups[g].op_end);
  __syncthreads();
  size_t need = 0;
  for (int c = 0; c < 2; ++c)
    need += round128((size_t)ng[c] * sizeof(FdsBoundGroup)) +
            round128((size_t)s_nops[c] * sizeof(FdsBoundOp)) +
            round128((size_t)np[c] * sizeof(FdsProbe));
  const bool fit = need <= kResidentTableBytes;
  unsigned char* q = area;
  for (int c = 0; c < 2; ++c) {
    ResidentTables t{ng[c], np[c], tab[c].groups, tab[c].ops, tab[c].probes, nullptr};
    if (fit) {
      FdsBoundGroup* g = reinterpret_cast<FdsBoundGroup*>(q);
      q += round128((size_t)ng[c] * sizeof(FdsBoundGroup));
      FdsBoundOp* o = reinterpret_cast<FdsBoundOp*>(q);
      q += round128((size_t)s_nops[c] * sizeof(FdsBoundOp));
      FdsProbe* p = reinterpret_cast<FdsProbe*>(q);
      q += round128((size_t)np[c] * sizeof(FdsProbe));
      for (int i = threadIdx.x; i < ng[c]; i += blockDim.x) g[i] = tab[c].groups[i];
      for (int i = threadIdx.x; i < s_nops[c]; i += blockDim.x) o[i] = tab[c].ops[i];
      for (int i = threadIdx.x; i < np[c]; i += blockDim.x) p[i] = tab[c].probes[i];
      t.groups = g;
      t.ops = o;
      t.probes = p;
    }
    out[c] = t;
  }
  __syncthreads();
}

template <typename T>
__host__ __device__ constexpr size_t resident_bytes(int n) {
  return round128((size_t)(n + 2) * sizeof(T));
}

// Shared memory of the state and coefficients of a resident run of n cells.
template <typename TP, typename TF, typename TC>
__host__ __device__ constexpr size_t resident_smem(int n) {
  return resident_bytes<TP>(n) + resident_bytes<TF>(n) + 2 * resident_bytes<TC>(n);
}

template <class C, typename TP, typename TF, typename TC>
__global__ void __launch_bounds__(kResidentThreads, 1)
    stag_1d_resident_kernel(const __grid_constant__ StagArgs<TP, TF, TC> a, int32_t nsteps,
                            TP* p_fin, TF* u_fin, int64_t pool_cached) {
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
  // boundary tables and probes in shared memory when they fit; the signal pool too
  // when the host reserved room for it (pool_cached values)
  unsigned char* area = smem_raw + resident_smem<TP, TF, TC>(n);
  ResidentTables rt[2];
  stage_tables(a.tab, ntiles, area, rt);
  const double* pool = a.pool;
  if (pool_cached > 0) {
    double* sp = reinterpret_cast<double*>(area + kResidentTableBytes);
    for (int64_t i = tid; i < pool_cached; i += kResidentThreads) sp[i] = a.pool[i];
    pool = sp;
  }
  const bool fb = rt[1].ngroups > 0;
  const bool fp = rt[1].nprobes > 0;
  const bool pb = rt[0].ngroups > 0;
  const bool pp = rt[0].nprobes > 0;
  __syncthreads();
  for (int32_t s = 0; s < nsteps; ++s) {
    const int64_t step = a.step + s;
    // ---- new flux of every cell ----
    // (slots k past the field are skipped as a whole: the same branch for every
    // thread, so no predicated-off FP64 instructions occupy the pipe)
    TF un[CPT];
#pragma unroll
    for (int k = 0; k < CPT; ++k) {
      if (k * kResidentThreads >= n) break;
      const int i = tid + k * kResidentThreads;
      un[k] = i < n ? flux_new<C, true>(a, sP, sU, sB, i + 1, (int64_t)i, i) : TF(0);
    }
    if constexpr (C::MEMORY && C::ABSORB) __syncthreads();  // neighbours read the old flux
#pragma unroll
    for (int k = 0; k < CPT; ++k) {
      if (k * kResidentThreads >= n) break;
      const int i = tid + k * kResidentThreads;
      if (i < n) sU[i + 1] = un[k];
    }
    __syncthreads();
    if (fb) {
      apply_bound_cells(rt[1], sU, pool, step);
      __syncthreads();
    }
    if (fp) write_probe_cells(rt[1], a.tab[1], sU, s);
    // ---- new potential of every cell (each thread reads its own cells' potential) ----
    TP pn[CPT];
#pragma unroll
    for (int k = 0; k < CPT; ++k) {
      if (k * kResidentThreads >= n) break;
      const int i = tid + k * kResidentThreads;
      pn[k] = i < n ? potential_cell<C>(a, sP, sU, sU, sK, sK, i + 1, i) : TP(0);
    }
#pragma unroll
    for (int k = 0; k < CPT; ++k) {
      if (k * kResidentThreads >= n) break;
      const int i = tid + k * kResidentThreads;
      if (i < n) sP[i + 1] = pn[k];
    }
    __syncthreads();
    if (s + 1 < nsteps) {
      // the next step's potential bounds and probes
      if (pb) {
        apply_bound_cells(rt[0], sP, pool, step + 1);
        __syncthreads();
      }
      if (pp) write_probe_cells(rt[0], a.tab[0], sP, s + 1);
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
