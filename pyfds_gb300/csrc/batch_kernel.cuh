// Batched staggered step: many independent fields (instances of uneven size and
// media, same variant) advanced by one launch per step.
//
// Each instance has two descriptors (StagArgs in global memory, one per
// ping-pong parity: parity 0 reads `cur` and writes `nxt`, parity 1 the reverse),
// holding its grid, coefficient pointers, tables and the TMA tensor maps of the
// arrays it reads. A work list of (instance, tile) pairs covers every tile of
// every instance (a two-step configuration advances it two steps when the launch's
// StepInfo says so). STAGES == 1: one CTA per work item, which also prefetches into
// L2 the region of the item `prefetch` places ahead. STAGES == 2: persistent
// CTAs walk the work list, prefetching the next item's region (possibly another
// instance's) while computing the current one.
#pragma once

#include "stag_kernel.cuh"

namespace fds {

// Copies the core arguments of a descriptor into shared memory (a CTA reads
// them there: stores of the tile code to global memory cannot alias them).
template <typename TP, typename TF, typename TC>
__device__ __forceinline__ void load_core(StagCore<TP, TF, TC>* dst,
                                          const StagArgs<TP, TF, TC>* src) {
  constexpr int W = sizeof(StagCore<TP, TF, TC>) / 4;
  const uint32_t* s = reinterpret_cast<const uint32_t*>(static_cast<const StagCore<TP, TF, TC>*>(src));
  uint32_t* d = reinterpret_cast<uint32_t*>(dst);
  for (int i = threadIdx.x; i < W; i += blockDim.x) d[i] = s[i];
}

// Dynamic shared memory of the batched kernel: staging buffers, one mbarrier per
// stage, one core copy. The buffers are carved for the isotropic layout (five
// arrays) when every instance of the batch is isotropic, else for the anisotropic
// one (seven): for 8-byte values that is the difference between two and four CTAs
// per SM.
template <class C, typename TP, typename TF, typename TC>
__host__ __device__ constexpr size_t batch_smem_bytes(bool all_iso) {
  return C::STAGES * stag_buffer_bytes<C, TP, TF, TC>(all_iso) + 16 * C::STAGES +
         round128(sizeof(StagCore<TP, TF, TC>));
}

template <class C, typename TP, typename TF, typename TC>
__global__ void __launch_bounds__(C::NT, C::batch_blocks(sizeof(TP)))
    stag_batch_kernel(const StagArgs<TP, TF, TC>* __restrict__ descs, const int2* __restrict__ work,
                      int nwork, const StepInfo si, int parity, int prefetch, int all_iso) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const size_t bytes = stag_buffer_bytes<C, TP, TF, TC>(all_iso != 0);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + C::STAGES * bytes);
  StagCore<TP, TF, TC>* core =
      reinterpret_cast<StagCore<TP, TF, TC>*>(smem_raw + C::STAGES * bytes + 16 * C::STAGES);
  const bool aligned = (smem_addr(smem_raw) & 127u) == 0;
  if (threadIdx.x == 0)
    for (int k = 0; k < C::STAGES; ++k) mbar_init(bars + k, 1);
  int w = blockIdx.x;
  if constexpr (C::STAGES == 1) {
    if (w >= nwork) return;
    const int2 it = work[w];
    const StagArgs<TP, TF, TC>* d = descs + 2 * it.x + parity;
    load_core(core, d);
    __syncthreads();
    const StagCore<TP, TF, TC>& a = *core;
    const bool iso = a.iso || !C::HAS_V;
    const StagBuf<TP, TF, TC> buf = carve_buffer<C, TP, TF, TC>(smem_raw, iso);
    if (a.use_tma && aligned) {
      if (threadIdx.x == 0) {
        tma_issue_tile<C>(a, d->tm, it.y, buf, iso, bars);
        // L2 prefetch of the work item `prefetch` ahead (possibly another instance)
        if (prefetch > 0 && w + prefetch < nwork) {
          const int2 ip = work[w + prefetch];
          const StagArgs<TP, TF, TC>* dp = descs + 2 * ip.x + parity;
          if (dp->use_tma) tma_prefetch_tile<C>(*dp, dp->tm, ip.y, dp->iso || !C::HAS_V);
        }
      }
      if (!tma_finish_tile<C>(a, it.y, buf, iso, bars, 0)) return;
    } else {
      stage_tile<C>(a, it.y, buf, iso);
      cp_async_commit();
      cp_async_wait<0>();
      __syncthreads();
    }
    if constexpr (C::TWO_STEP) {
      if (si.substeps == 2) {  // steps si.step and si.step + 1 of this tile
        compute_ring<C>(a, si, it.y, buf);
        __syncthreads();
        compute_tile<C>(a, StepInfo{si.step + 1, si.step0, si.apply_next, si.store_flux, 1},
                        it.y, buf);
        return;
      }
    }
    compute_tile<C>(a, si, it.y, buf);
  } else {
    __syncthreads();
    const int stride = gridDim.x;
    uint32_t uses[2] = {0u, 0u};  // completed TMA uses of each buffer's barrier
    if (w < nwork) {
      const int2 it = work[w];
      const StagArgs<TP, TF, TC>* d = descs + 2 * it.x + parity;
      const bool iso = d->iso || !C::HAS_V;
      const StagBuf<TP, TF, TC> b0 = carve_buffer<C, TP, TF, TC>(smem_raw, iso);
      if (d->use_tma && aligned) {
        if (threadIdx.x == 0) tma_issue_tile<C>(*d, d->tm, it.y, b0, iso, bars);
      } else {
        stage_tile<C>(*d, it.y, b0, iso);
      }
    }
    cp_async_commit();
    for (int k = 0; w < nwork; ++k, w += stride) {
      const int cur = k & 1;
      const int2 it = work[w];
      const int wn = w + stride;
      __syncthreads();  // every thread is done with the buffer the next copies fill
      load_core(core, descs + 2 * it.x + parity);
      __syncthreads();  // the whole core copy is visible before anyone reads it
      if (wn < nwork) {
        const int2 itn = work[wn];
        const StagArgs<TP, TF, TC>* dn = descs + 2 * itn.x + parity;
        const bool ison = dn->iso || !C::HAS_V;
        const StagBuf<TP, TF, TC> bn =
            carve_buffer<C, TP, TF, TC>(smem_raw + (cur ^ 1) * bytes, ison);
        if (dn->use_tma && aligned) {
          if (threadIdx.x == 0) tma_issue_tile<C>(*dn, dn->tm, itn.y, bn, ison, bars + (cur ^ 1));
        } else {
          stage_tile<C>(*dn, itn.y, bn, ison);
        }
      }
      cp_async_commit();
      const bool tma = descs[2 * it.x + parity].use_tma && aligned;
      const bool iso = descs[2 * it.x + parity].iso || !C::HAS_V;
      const StagBuf<TP, TF, TC> bc = carve_buffer<C, TP, TF, TC>(smem_raw + cur * bytes, iso);
      if (tma) {
        // barrier `cur` completes once per TMA use of its buffer (items may mix
        // TMA and cp.async staging, so the uses are counted, not derived from k)
        if (!tma_finish_tile<C>(*core, it.y, bc, iso, bars + cur, uses[cur] & 1u)) {
          // let a prefetch in flight into the other buffer land before leaving
          if (wn < nwork && descs[2 * work[wn].x + parity].use_tma)
            mbar_wait(bars + (cur ^ 1), uses[cur ^ 1] & 1u, 1ll << 22);
          return;
        }
        ++uses[cur];
      } else {
        cp_async_wait<1>();
        __syncthreads();
      }
      compute_tile<C>(*core, si, it.y, bc);
    }
  }
}

// Potential bounds and probes of the first step of a batched call: one CTA per
// instance, in place on that instance's current potential.
template <typename TP, typename TF, typename TC>
__global__ void __launch_bounds__(256) stag_batch_prologue_kernel(
    const StagArgs<TP, TF, TC>* descs, int count, int64_t step) {
  const int inst = blockIdx.x;
  if (inst >= count) return;
  const StagArgs<TP, TF, TC>& a = descs[2 * inst];  // parity 0 reads `cur`
  const FdsCompTables& tb = a.tab[0];
  TP* p = const_cast<TP*>(a.p_in);
  if (tb.bound_tile_start != nullptr) {
    const int e = tb.bound_tile_start[a.ntiles];
    for (int g = threadIdx.x; g < e; g += blockDim.x) {
      const FdsBoundGroup grp = tb.groups[g];
      if (!grp.primary) continue;  // the global array: once per cell
      TP v = p[grp.cell];
      for (int o = grp.op_begin; o < grp.op_end; ++o) {
        const FdsBoundOp op = tb.ops[o];
        const double val = (op.flags & FDS_BOP_SIGNAL)
                               ? a.pool[op.off + step * (int64_t)op.stride] + op.scalar
                               : op.scalar;
        v = xadd(xmul((TP)op.mul, v), (TP)val);
      }
      p[grp.cell] = v;
    }
  }
  __syncthreads();
  if (tb.probe_tile_start != nullptr && tb.out_rows > 0) {
    const int e = tb.probe_tile_start[a.ntiles];
    for (int q = threadIdx.x; q < e; q += blockDim.x) {
      const FdsProbe pr = tb.probes[q];
      tb.out[pr.col] = (double)p[pr.cell];
    }
  }
}

}  // namespace fds
