// Batched staggered step: many independent fields (instances of uneven size and
// media, same variant) advanced by one launch per step.
//
// Each instance has two descriptors (StagArgs in global memory, one per
// ping-pong parity: parity 0 reads `cur` and writes `nxt`, parity 1 the reverse),
// holding its grid, coefficient pointers, tables and the TMA tensor maps of the
// arrays it reads. A work list of (instance, tile) pairs covers every tile of
// every instance. STAGES == 1: one CTA per work item. STAGES == 2: persistent
// CTAs walk the work list, prefetching the next item's region (possibly another
// instance's) while computing the current one.
#pragma once

#include "stag_kernel.cuh"

namespace fds {

template <class C, typename TP, typename TF, typename TC>
__global__ void __launch_bounds__(C::NT, C::MIN_BLOCKS)
    stag_batch_kernel(const StagArgs<TP, TF, TC>* __restrict__ descs, const int2* __restrict__ work,
                      int nwork, const StepInfo si, int parity) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  // every instance of one launch shares the variant; iso may differ per instance,
  // so buffers are carved for the anisotropic (larger) layout
  const size_t bytes = stag_buffer_bytes<C, TP, TF, TC>(false);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + C::STAGES * bytes);
  const bool aligned = (smem_addr(smem_raw) & 127u) == 0;
  if (threadIdx.x == 0)
    for (int k = 0; k < C::STAGES; ++k) mbar_init(bars + k, 1);
  __syncthreads();
  int w = blockIdx.x;
  if constexpr (C::STAGES == 1) {
    if (w >= nwork) return;
    const int2 it = work[w];
    const StagArgs<TP, TF, TC>& a = descs[2 * it.x + parity];
    const bool iso = a.iso || !C::HAS_V;
    const StagBuf<TP, TF, TC> buf = carve_buffer<C, TP, TF, TC>(smem_raw, iso);
    if (a.use_tma && aligned) {
      if (threadIdx.x == 0) tma_issue_tile<C>(a, it.y, buf, iso, bars);
      if (!tma_finish_tile<C>(a, it.y, buf, iso, bars, 0)) return;
    } else {
      stage_tile<C>(a, it.y, buf, iso);
      cp_async_commit();
      cp_async_wait<0>();
      __syncthreads();
    }
    compute_tile<C>(a, si, it.y, buf);
  } else {
    const int stride = gridDim.x;
    uint32_t uses[2] = {0u, 0u};  // completed TMA uses of each buffer's barrier
    if (w < nwork) {
      const int2 it = work[w];
      const StagArgs<TP, TF, TC>& a = descs[2 * it.x + parity];
      const bool iso = a.iso || !C::HAS_V;
      const StagBuf<TP, TF, TC> b0 = carve_buffer<C, TP, TF, TC>(smem_raw, iso);
      if (a.use_tma && aligned) {
        if (threadIdx.x == 0) tma_issue_tile<C>(a, it.y, b0, iso, bars);
      } else {
        stage_tile<C>(a, it.y, b0, iso);
      }
    }
    cp_async_commit();
    for (int k = 0; w < nwork; ++k, w += stride) {
      const int cur = k & 1;
      const int2 it = work[w];
      const StagArgs<TP, TF, TC>& a = descs[2 * it.x + parity];
      const bool iso = a.iso || !C::HAS_V;
      const StagBuf<TP, TF, TC> bc = carve_buffer<C, TP, TF, TC>(smem_raw + cur * bytes, iso);
      const int wn = w + stride;
      __syncthreads();  // every thread is done with the buffer the next copies fill
      if (wn < nwork) {
        const int2 itn = work[wn];
        const StagArgs<TP, TF, TC>& an = descs[2 * itn.x + parity];
        const bool ison = an.iso || !C::HAS_V;
        const StagBuf<TP, TF, TC> bn =
            carve_buffer<C, TP, TF, TC>(smem_raw + (cur ^ 1) * bytes, ison);
        if (an.use_tma && aligned) {
          if (threadIdx.x == 0) tma_issue_tile<C>(an, itn.y, bn, ison, bars + (cur ^ 1));
        } else {
          stage_tile<C>(an, itn.y, bn, ison);
        }
      }
      cp_async_commit();
      if (a.use_tma && aligned) {
        // barrier `cur` completes once per TMA use of its buffer (items may mix
        // TMA and cp.async staging, so the uses are counted, not derived from k)
        if (!tma_finish_tile<C>(a, it.y, bc, iso, bars + cur, uses[cur] & 1u)) {
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
      compute_tile<C>(a, si, it.y, bc);
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
      TP v = p[grp.cell];
      for (int o = grp.op_begin; o < grp.op_end; ++o) {
        const FdsBoundOp op = tb.ops[o];
        const double val = (op.flags & FDS_BOP_SIGNAL) ? a.pool[op.off + step * (int64_t)op.stride]
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
