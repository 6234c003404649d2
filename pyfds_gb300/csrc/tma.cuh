// Tensor-memory-accelerator (TMA) helpers: 2-D tile loads into shared memory that
// complete on an mbarrier, a bounded wait on that barrier, and host-side encoding
// of the tensor maps (through the driver entry point, so the library links only
// the CUDA runtime).
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace fds {

// Status bits a kernel ORs into FdsStagTables.status.
constexpr int32_t kStatusTmaTimeout = 1;
constexpr int32_t kStatusNonFinite = 2;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
  // make the initialised barrier visible to the asynchronous (TMA) proxy
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

// One 2-D box of `map` at element coordinates (x, y) -> shared memory `dst`.
// x * element size must be a multiple of 16 bytes; out-of-range elements read 0.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];\n" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
      : "memory");
}

// L2 prefetch of one 2-D box of `map` at (x, y): a hint, with no shared-memory
// destination and no completion. Callers pass boxes inside the array.
__device__ __forceinline__ void tma_prefetch_2d(const CUtensorMap* map, int x, int y) {
  asm volatile("cp.async.bulk.prefetch.tensor.2d.L2.global.tile [%0, {%1, %2}];\n" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(x), "r"(y)
               : "memory");
}

// Waits for phase `parity` of the barrier to complete; gives up after `limit`
// polls (each poll may suspend the thread for a short hardware-defined time).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long limit) {
  const uint32_t a = smem_addr(bar);
  for (long long i = 0; i < limit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Waits until counters c[r0 .. r1] (global memory, written by other CTAs) have each
// reached `need`, reading them with acquire semantics; gives up after `limit` polls
// of one counter (a short sleep between polls).
__device__ __forceinline__ bool wait_counters(const uint32_t* c, int r0, int r1, uint32_t need,
                                              long long limit) {
  for (int r = r0; r <= r1; ++r) {
    long long i = 0;
    for (;;) {
      uint32_t v;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(c + r) : "memory");
      if (v >= need) break;
      if (++i > limit) return false;
      __nanosleep(64);
    }
  }
  return true;
}

// ---------------------------------------------------------------- host side

// The driver's tensor-map encoder, looked up once (a static initialised under the
// language's once-only guarantee, so concurrent first calls see the same result).
inline PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = []() {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
  }();
  return fn;
}

// Row-major [ny][nx] array of 4- or 8-byte floats, boxes of bx x by elements.
inline bool encode_tile_map(CUtensorMap* m, const void* base, size_t esize, int nx, int ny, int bx,
                            int by) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc || !base) return false;
  if (((uintptr_t)base & 15) != 0 || ((size_t)nx * esize) % 16 != 0) return false;
  if (bx > 256 || by > 256 || (bx * esize) % 16 != 0) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)nx, (cuuint64_t)ny};
  const cuuint64_t strides[1] = {(cuuint64_t)nx * esize};
  const cuuint32_t box[2] = {(cuuint32_t)bx, (cuuint32_t)by};
  const cuuint32_t estr[2] = {1, 1};
  const CUtensorMapDataType dt =
      esize == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
  CUresult r = enc(m, dt, 2, const_cast<void*>(base), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

}  // namespace fds
