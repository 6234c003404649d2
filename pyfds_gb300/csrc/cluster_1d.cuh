// Every step of a call for a 1-D field spread over the CTAs of one thread-block
// cluster (pyfds/acoustics.py:40-52, pyfds/thermal.py:46-51, repeated by
// Field.simulate, pyfds/fields.py:87-93).
//
// One CTA holds a field of a few thousand cells in shared memory, but then the step
// runs on one SM: four DFMA per cell and step at two per clock, about 1 us per step
// for 1000 cells. Here CTA r of a cluster of CL CTAs owns the cells [r m, (r + 1) m)
// and one halo cell on each side (slot 0: the cell left of its first, slot m_r + 1:
// the cell right of its last; slots past the field hold zeros, the neighbours the
// reference's operators drop). A step needs two values from the neighbours:
//   - the flux update of the first owned cell reads the potential of the cell to
//     its left (after that cell's potential update and bounds): the left CTA writes
//     it into this CTA's slot 0 through distributed shared memory;
//   - the potential update of the last owned cell reads the flux of the cell to its
//     right (after that cell's flux update and bounds): the right CTA writes it into
//     this CTA's hr[parity].
// (With absorption the flux update also reads the old fluxes of both neighbours:
// hl[] / hr[] hold them, double-buffered by step parity so that a neighbour can
// write this step's flux while this CTA still reads the last one.) Two cluster
// barriers per step order these writes after the reads they replace and before the
// reads that need them.
//
// Without absorption one cluster barrier per step suffices: each CTA also computes
// the flux of the cell right of its block (slot m_r + 1), from that cell's potential
// (a halo value) and its own previous flux (which this CTA computed the step before),
// with the same arithmetic and bounds as the owner does, so the potential update of
// its last cell needs nothing from the neighbour. Only potentials cross CTAs: after
// its potential update and bounds, a CTA writes its first and last potential into
// the neighbours' halo slots pl[parity] / pr[parity], double-buffered so that a
// neighbour still reading the last step's values is not overwritten.
//
// Every cell is computed by flux_new and potential_regs, the tile kernel's
// arithmetic, so results are the tile kernel's bit for bit.
#pragma once

#include "resident_1d.cuh"

namespace fds {

constexpr int kClusterThreads = 128;
constexpr int kClusterCellsPerThread = 8;
constexpr int kClusterMaxCta = 8;  // the portable cluster size
constexpr int kClusterMaxCellsPerCta = kClusterThreads * kClusterCellsPerThread;

// Boundary chains on the primary placements of the cells [c0, c1), applied to the
// slot array s (slot = cell - c0 + 1).
template <typename T>
__device__ __forceinline__ void apply_bound_range(const ResidentTables& t, T* s,
                                                  const double* pool, int64_t step, int c0,
                                                  int c1) {
  for (int g = threadIdx.x; g < t.ngroups; g += blockDim.x) {
    const FdsBoundGroup grp = t.groups[g];
    if (!grp.primary || grp.cell < c0 || grp.cell >= c1) continue;
    const int j = (int)grp.cell - c0 + 1;
    T v = s[j];
    for (int o = grp.op_begin; o < grp.op_end; ++o) {
      const FdsBoundOp op = t.ops[o];
      const double val = (op.flags & FDS_BOP_SIGNAL)
                             ? pool[op.off + step * (int64_t)op.stride] + op.scalar
                             : op.scalar;
      v = xadd(xmul((T)op.mul, v), (T)val);
    }
    s[j] = v;
  }
}

template <typename T>
__device__ __forceinline__ void write_probe_range(const ResidentTables& t,
                                                  const FdsCompTables& tb, const T* s,
                                                  int64_t row, int c0, int c1) {
  if (row < 0 || row >= tb.out_rows) return;
  double* out = tb.out + row * (int64_t)tb.ncols;
  for (int q = threadIdx.x; q < t.nprobes; q += blockDim.x) {
    const FdsProbe pr = t.probes[q];
    if (pr.cell >= c0 && pr.cell < c1) out[pr.col] = (double)s[pr.cell - c0 + 1];
  }
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

template <class C, typename TP, typename TF, typename TC>
__global__ void __launch_bounds__(kClusterThreads, 1)
    stag_1d_cluster_kernel(const __grid_constant__ StagArgs<TP, TF, TC> a, int32_t nsteps,
                           TP* p_fin, TF* u_fin, int64_t pool_cached, int32_t m) {
  static_assert(!C::HAS_V, "1-D fields");
  constexpr int CPT = kClusterCellsPerThread;
  constexpr int NT = kClusterThreads;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ TF hl[2], hr[2];  // old / new flux of the neighbour cells, by step parity
  __shared__ TP pl[2], pr[2];  // potential of the neighbour cells, by step parity
  constexpr bool ONE = !(C::MEMORY && C::ABSORB);  // one cluster barrier per step
  const int n = (int)a.n;
  const int ntiles = a.ntiles;
  const int rank = (int)blockIdx.x;  // the grid is one cluster
  const int ncta = (int)gridDim.x;
  const int c0 = rank * m;
  const int c1 = min(n, c0 + m);
  const int mr = c1 - c0;  // cells owned here
  TP* sP = reinterpret_cast<TP*>(smem_raw);
  TF* sU = reinterpret_cast<TF*>(smem_raw + resident_bytes<TP>(m));
  TC* sB = reinterpret_cast<TC*>(smem_raw + resident_bytes<TP>(m) + resident_bytes<TF>(m));
  TC* sK = reinterpret_cast<TC*>(smem_raw + resident_bytes<TP>(m) + resident_bytes<TF>(m) +
                                 resident_bytes<TC>(m));
  const int tid = threadIdx.x;
  for (int j = tid; j < mr + 2; j += NT) {
    const int i = c0 - 1 + j;
    const bool in = i >= 0 && i < n;
    sP[j] = in ? a.p_in[i] : TP(0);
    sU[j] = (in && C::MEMORY) ? a.u_in[i] : TF(0);
    sB[j] = in ? a.bx[i] : TC(0);
    sK[j] = in ? a.kx[i] : TC(0);
  }
  unsigned char* area = smem_raw + resident_smem<TP, TF, TC>(m);
  ResidentTables rt[2];
  stage_tables(a.tab, ntiles, area, rt);  // ends with a barrier
  const double* pool = a.pool;
  if (pool_cached > 0) {
    double* sp = reinterpret_cast<double*>(area + kResidentTableBytes);
    for (int64_t i = tid; i < pool_cached; i += NT) sp[i] = a.pool[i];
    pool = sp;
  }
  if (tid == 0) {
    // the neighbours' fluxes and potentials before the first step (parity of step -1)
    hl[1] = sU[0];
    hr[1] = sU[mr + 1];
    hl[0] = hr[0] = TF(0);
    pl[1] = sP[0];
    pr[1] = sP[mr + 1];
    pl[0] = pr[0] = TP(0);
  }
  // ONE: this CTA also computes the flux of cell c1 (slot mr + 1) when it exists
  const int nf = (ONE && c1 < n) ? mr + 1 : mr;
  const bool fb = rt[1].ngroups > 0;
  const bool fp = rt[1].nprobes > 0;
  const bool pb = rt[0].ngroups > 0;
  const bool pp = rt[0].nprobes > 0;
  // every CTA has loaded its halo before any neighbour writes into it
  cluster_sync();
  for (int32_t s = 0; s < nsteps; ++s) {
    const int64_t step = a.step + s;
    const int cur = s & 1, old = cur ^ 1;
    if constexpr (ONE) {
      // the neighbours' potentials of the last step into the halo slots; each is read
      // only by the thread that writes it here (cells c0 and c1 below)
      if (tid == 0) sP[0] = pl[old];
      if (nf > mr && tid == mr % NT) sP[mr + 1] = pr[old];
    }
    if constexpr (C::MEMORY && C::ABSORB) {
      // the neighbours' fluxes of the last step, where the absorption term reads them
      if (tid == 0) {
        sU[0] = hl[old];
        sU[mr + 1] = hr[old];
      }
      __syncthreads();
    }
    // ---- new flux of every owned cell ----
    // (CPT + 1 slots per thread: with ONE a CTA of the maximal block computes one flux
    // past its cells)
    TF un[CPT + 1];
#pragma unroll
    for (int k = 0; k < CPT + 1; ++k) {
      if (k * NT >= nf) break;
      const int j = tid + k * NT;  // owned index (mr: the cell right of the block); slot j + 1
      un[k] = j < nf ? flux_new<C, true>(a, sP, sU, sB, j + 1, (int64_t)(c0 + j), c0 + j)
                     : TF(0);
    }
    if constexpr (C::MEMORY && C::ABSORB) __syncthreads();  // neighbours read the old flux
#pragma unroll
    for (int k = 0; k < CPT + 1; ++k) {
      if (k * NT >= nf) break;
      const int j = tid + k * NT;
      if (j < nf) sU[j + 1] = un[k];
    }
    __syncthreads();
    if (fb) {
      // ONE: the bounds of cell c1 too, where this CTA computed its flux
      apply_bound_range(rt[1], sU, pool, step, c0, c0 + nf);
      __syncthreads();
    }
    if (fp) write_probe_range(rt[1], a.tab[1], sU, s, c0, c1);
    if constexpr (!ONE) {
      // this step's flux of the first and last owned cells to the neighbours
      if (tid == 0) {
        if (rank > 0) st_cluster(&hr[cur], (uint32_t)(rank - 1), sU[1]);
        if (rank + 1 < ncta) st_cluster(&hl[cur], (uint32_t)(rank + 1), sU[mr]);
      }
      cluster_sync();
    }
    // ---- new potential of every owned cell (the last one reads the right
    // neighbour's new flux from hr[cur]; outside the field it stays 0) ----
    TP pn[CPT];
#pragma unroll
    for (int k = 0; k < CPT; ++k) {
      if (k * NT >= mr) break;
      const int j = tid + k * NT;
      if (j < mr) {
        const int ps = j + 1;
        const TF un1 = (!ONE && j + 1 == mr) ? hr[cur] : sU[ps + 1];
        pn[k] = potential_regs<C>(a, sP[ps], sU[ps], un1, TF(0), TF(0), (TF)sK[ps],
                                  (TF)sK[ps + 1], TF(0), TF(0), c0 + j);
      } else {
        pn[k] = TP(0);
      }
    }
#pragma unroll
    for (int k = 0; k < CPT; ++k) {
      if (k * NT >= mr) break;
      const int j = tid + k * NT;
      if (j < mr) sP[j + 1] = pn[k];
    }
    __syncthreads();
    if (s + 1 < nsteps) {
      if (pb) {
        apply_bound_range(rt[0], sP, pool, step + 1, c0, c1);
        __syncthreads();
      }
      if (pp) write_probe_range(rt[0], a.tab[0], sP, s + 1, c0, c1);
    }
    if constexpr (ONE) {
      // the first and last owned potentials to the neighbours' halo slots
      if (tid == 0) {
        if (rank > 0) st_cluster(&pr[cur], (uint32_t)(rank - 1), sP[1]);
        if (rank + 1 < ncta) st_cluster(&pl[cur], (uint32_t)(rank + 1), sP[mr]);
      }
    } else {
      // the last owned cell's potential to the right neighbour's left halo
      if (tid == 0 && rank + 1 < ncta) st_cluster(&sP[0], (uint32_t)(rank + 1), sP[mr]);
    }
    cluster_sync();
  }
  bool bad = false;
  for (int j = tid; j < mr; j += NT) {
    const TP v = sP[j + 1];
    p_fin[c0 + j] = v;
    u_fin[c0 + j] = sU[j + 1];
    bad = bad || nonfinite(v);
  }
  if (a.status && __any_sync(0xffffffffu, bad) && (tid & 31) == 0)
    atomicOr(a.status, kStatusNonFinite);
}

}  // namespace fds
