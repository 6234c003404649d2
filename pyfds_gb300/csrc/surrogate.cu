// Learned-surrogate kernels: BF16 3x3 (dilated) convolutions as implicit GEMMs on
// the fifth-generation tensor cores, their weight gradients, a fused AdamW step,
// and the packing of solver states into network inputs.
//
// Activations are stored channel-group blocked, [B][C/8][H][W][8] (bf16): the 8
// channels of a pixel are one 16-byte row, and a row segment of one channel group
// is contiguous in memory.
//
// Convolution (forward and data gradient), per CTA tile of kRows output rows x 128
// pixels of one image:
//   * TMA copies, per group of 8 input channels, kRows + 2 input rows of 128 + 2d
//     pixels (zero-filled outside the image: the convolution's padding) into a
//     "slab" [row][pixel][8 channels] of shared memory. A slab row of 8 pixels is
//     one 8 x 16-byte core matrix, so the A operand (128 pixels x 16 channels,
//     K-major) of any tap (dy, dx) is the same slab pair at a start address moved
//     by ((r + dy) * pitch + dx * d) * 16 bytes: no im2col copy.
//   * The packed weights of the layer stay in shared memory for the whole kernel.
//   * Warp-specialised: a producer warp stages tiles, one thread of the MMA warp
//     issues 9 taps x cin/16 MMAs (M = 128, N = cout, K = 16) per output row into
//     a tensor-memory accumulator, 16 epilogue warps (one per tensor-memory lane
//     quarter and output row) add bias / residual, apply GELU or its derivative
//     and store bf16 (or float32). Two staging buffers and two accumulator sets
//     let copies, MMAs and epilogues of consecutive tiles overlap; the roles hand
//     off through mbarriers only.
// Weight gradient: D[co][ci] (M = 64 >= cout, N = cin) summed over pixels per tap,
// with both operands MN-major (channel-contiguous activations used as they are).
//
// Every wait on an mbarrier is bounded; a CTA that gives up records
// FDS_SURR_STATUS_TIMEOUT, waits (bounded) for its copies and MMAs in flight,
// frees its tensor memory and returns.
#include <cuda_bf16.h>

#include "fds_internal.h"
#include "fds_surrogate.h"
#include "umma.cuh"

namespace fds {
namespace surr {

constexpr int kTilePx = 128;   // pixels per tile row (M of the forward MMA)
constexpr int kRows = 4;       // output rows per forward tile
constexpr int kWRows = 2;      // output rows per weight-gradient tile
constexpr int kConvThreads = 32 * (2 + 4 * kRows);  // producer, MMA, 16 epilogue warps
constexpr int kBiasWarps = 8;                         // weight gradient: one pixel per thread
constexpr int kWgradThreads = 32 * (2 + kBiasWarps);
constexpr int kTmemCols = 512;
constexpr int kAccStride = 64;  // tensor-memory columns per forward accumulator
constexpr long long kWaitLimit = 1ll << 22;
constexpr int kMaxSmem = 232448;  // 227 KB opt-in per CTA
// Every launch requests all of it: one CTA holds an SM (and its 512 tensor-memory
// columns) alone, and every operand address an MMA can form from a descriptor of
// this kernel stays inside the CTA's shared memory.
constexpr int kMinSmem = kMaxSmem;

__host__ __device__ constexpr int round_up(int v, int m) { return (v + m - 1) / m * m; }

// GELU, tanh form: 0.5 v (1 + tanh(sqrt(2/pi) (v + 0.044715 v^3))).
__device__ __forceinline__ float tanh_approx(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
constexpr float kGeluA = 0.7978845608028654f;  // sqrt(2 / pi)
constexpr float kGeluB = 0.044715f;
__device__ __forceinline__ float gelu(float v) {
  const float t = tanh_approx(kGeluA * fmaf(kGeluB * v * v, v, v));
  return 0.5f * v * (1.0f + t);
}
__device__ __forceinline__ float gelu_grad(float v) {
  const float t = tanh_approx(kGeluA * fmaf(kGeluB * v * v, v, v));
  return 0.5f * (1.0f + t) + 0.5f * v * (1.0f - t * t) * kGeluA * fmaf(3.0f * kGeluB, v * v, 1.0f);
}

__device__ __forceinline__ void unpack8(const uint4& u, float (&f)[8]) {
  const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float2 v = __bfloat1622float2(h[i]);
    f[2 * i] = v.x;
    f[2 * i + 1] = v.y;
  }
}
__device__ __forceinline__ uint4 pack8(const float (&f)[8]) {
  uint4 u;
  __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&u);
#pragma unroll
  for (int i = 0; i < 4; ++i) h[i] = __floats2bfloat162_rn(f[2 * i], f[2 * i + 1]);
  return u;
}

// Packed operand index of weight (tap, co, ci): per (tap, 16-channel chunk of ci)
// a K-major N x 16 block [ci half][co][8].
__host__ __device__ __forceinline__ int64_t packed_index(int tap, int co, int ci, int cin,
                                                         int cout) {
  const int kc = ci >> 4, kh = (ci >> 3) & 1;
  return ((int64_t)((tap * (cin >> 4) + kc) * 2 + kh) * cout + co) * 8 + (ci & 7);
}

struct Tile {
  int b, y0, x0;  // output row r is y0 + r * dil; staged row k is y0 + (k - 1) * dil
};

// Tiles: images x row blocks of rows * dil rows x dil phases x 128-pixel columns.
__device__ __forceinline__ Tile decode_tile(int t, int H, int W, int dil, int rows) {
  const int nxq = W / kTilePx;
  const int xq = t % nxq;
  t /= nxq;
  const int j = t % dil;
  t /= dil;
  const int nyb = H / (rows * dil);
  const int yb = t % nyb;
  return {t / nyb, yb * rows * dil + j, xq * kTilePx};
}

// Stages `nrows` rows (spaced dil, starting row_shift rows above output row 0) of
// `ngroups` 8-channel groups, rx pixels each; row k of group g lands at
// dst + g * gstride + k * rstride.
__device__ __forceinline__ void issue_rows(const CUtensorMap* map, const Tile& tl, int dil,
                                           int ngroups, int nrows, int rx, int gstride,
                                           int rstride, int row_shift, unsigned char* dst,
                                           uint64_t* bar) {
  for (int g = 0; g < ngroups; ++g)
    for (int k = 0; k < nrows; ++k)
      tma_load_4d(dst + g * gstride + k * rstride, map, 0, tl.x0 - (rx - kTilePx) / 2,
                  tl.y0 + (k - row_shift) * dil, tl.b * ngroups + g, bar);
}

struct ConvDev {
  const __nv_bfloat16* w;
  const float* bias;
  const __nv_bfloat16* resid;
  const __nv_bfloat16* zin;
  __nv_bfloat16* out_z;
  __nv_bfloat16* out_h;
  float* out_f32;
  int32_t* status;
  int B, H, W, cin, cout, dil, mode, ntiles;
  int rx, pitch, slab, abuf, wbytes;
};

// One output row of a tile (this warp's 32 pixels, all NG * 8 output channels)
// from its tensor-memory accumulator: bias, GELU / residual or the GELU
// derivative, stores. `res` is the residual row, loaded before the accumulator
// was ready.
template <int NG>
__device__ __forceinline__ void conv_epilogue_row(const ConvDev& p, size_t o0, size_t gstride,
                                                  uint32_t tacc, const float* bias_s,
                                                  const uint4 (&res)[NG]) {
  uint32_t acc[NG / 2][16];
#pragma unroll
  for (int j = 0; j < NG / 2; ++j) tmem_ld16_async(tacc + 16 * j, acc[j]);
  tmem_ld_wait();
#pragma unroll
  for (int j = 0; j < NG / 2; ++j) tmem_reg_fence(acc[j]);
#pragma unroll
  for (int g = 0; g < NG; ++g) {
    float v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(acc[g / 2][(g & 1) * 8 + i]);
    // group g of the pixel: 8 consecutive values; the warp's 32 pixels are 512
    // (bf16) or 1024 (float32) contiguous bytes
    const size_t o = o0 + g * gstride;
    if (p.mode == FDS_CONV_FWD_LINEAR) {
#pragma unroll
      for (int i = 0; i < 8; ++i) v[i] += bias_s[g * 8 + i];
      float4* dst = reinterpret_cast<float4*>(p.out_f32 + o);
      dst[0] = make_float4(v[0], v[1], v[2], v[3]);
      dst[1] = make_float4(v[4], v[5], v[6], v[7]);
    } else if (p.mode == FDS_CONV_FWD_GELU) {
#pragma unroll
      for (int i = 0; i < 8; ++i) v[i] += bias_s[g * 8 + i];
      if (p.out_z) *reinterpret_cast<uint4*>(p.out_z + o) = pack8(v);
      float rr[8];
      unpack8(res[g], rr);
#pragma unroll
      for (int i = 0; i < 8; ++i) v[i] = gelu(v[i]) + rr[i];
      *reinterpret_cast<uint4*>(p.out_h + o) = pack8(v);
    } else {  // FDS_CONV_BWD_DATA
      float rr[8], z[8];
      unpack8(res[g], rr);
#pragma unroll
      for (int i = 0; i < 8; ++i) v[i] += rr[i];
      if (p.out_h) *reinterpret_cast<uint4*>(p.out_h + o) = pack8(v);
      unpack8(*reinterpret_cast<const uint4*>(p.zin + o), z);
#pragma unroll
      for (int i = 0; i < 8; ++i) v[i] *= gelu_grad(z[i]);
      *reinterpret_cast<uint4*>(p.out_z + o) = pack8(v);
    }
  }
}

// The epilogue role: warp w handles tensor-memory lane quarter w % 4 (the quarter
// it may read) of output row (w - 2) / 4 of every tile of the CTA.
// A bounded wait on an mbarrier phase that every lane of the warp takes together.
__device__ __forceinline__ bool warp_wait(uint64_t* bar, uint32_t parity) {
  const bool ok = mbar_wait(bar, parity, kWaitLimit);
  return __all_sync(0xffffffffu, ok);
}

// Warp-uniform read of the CTA's abort flag.
__device__ __forceinline__ bool aborted(volatile int* flag) {
  return __shfl_sync(0xffffffffu, *flag, 0) != 0;
}

// Tiles of this CTA: blockIdx.x, blockIdx.x + gridDim.x, ...
__device__ __forceinline__ int my_tiles(int ntiles) {
  return blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
}

// The epilogue role: warp w handles tensor-memory lane quarter w % 4 (the quarter
// it may read) of output row (w - 2) / 4 of every tile of the CTA.
template <int NG>
__device__ void conv_epilogue_role(const ConvDev& p, uint32_t tm, uint64_t* acc_full,
                                   uint64_t* acc_empty, volatile int* abort_flag,
                                   const float* bias_s, int nmine) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int q = warp & 3, r = (warp - 2) >> 2;
  const size_t plane = (size_t)p.H * p.W;
  const size_t gstride = plane * 8;
  for (int k = 0; k < nmine; ++k) {
    const int a = k & 1, u = k >> 1;
    if (aborted(abort_flag)) break;
    const Tile tl = decode_tile(blockIdx.x + k * gridDim.x, p.H, p.W, p.dil, kRows);
    const size_t pix = (size_t)(tl.y0 + r * p.dil) * p.W + tl.x0 + 32 * q + lane;
    const size_t o0 = ((size_t)tl.b * NG * plane + pix) * 8;
    uint4 res[NG];
#pragma unroll
    for (int g = 0; g < NG; ++g)
      res[g] = p.resid ? *reinterpret_cast<const uint4*>(p.resid + o0 + g * gstride)
                       : make_uint4(0u, 0u, 0u, 0u);
    if (!warp_wait(acc_full + a, (uint32_t)(u & 1))) {
      if (lane == 0) *abort_flag = 1;
      break;
    }
    tc_fence_after();
    conv_epilogue_row<NG>(p, o0, gstride,
                          tm + ((uint32_t)(32 * q) << 16) +
                              (uint32_t)(a * kRows * kAccStride + r * kAccStride),
                          bias_s, res);
    tc_fence_before();
    __syncwarp();
    if (lane == 0) mbar_arrive(acc_empty + a);
  }
}

// The MMA role (one thread issues): per tile and output row r, 9 taps x KC
// 16-channel chunks accumulate into one tensor-memory accumulator. Descriptors
// are built once; a tap or chunk only adds its byte offset / 16 to the start
// address field (addresses stay below 256 KB, so the field cannot carry).
template <int KC, int NOUT>
__device__ void conv_mma_role(const ConvDev& p, unsigned char* sm, unsigned char* abuf0,
                              uint64_t* full, uint64_t* empty, uint64_t* acc_full,
                              uint64_t* acc_empty, volatile int* abort_flag, uint32_t tm,
                              int nmine) {
  const int lane = threadIdx.x & 31;
  constexpr uint32_t idesc = umma_idesc_bf16(128, NOUT);
  const uint64_t bdesc0 = umma_desc(smem_addr(sm), NOUT * 16u, 128u);
  const uint32_t pitch = (uint32_t)p.pitch, dil = (uint32_t)p.dil, slab16 = (uint32_t)p.slab >> 4;
  int last = -1;
  for (int k = 0; k < nmine; ++k) {
    const int s = k & 1, u = k >> 1;
    if (aborted(abort_flag)) break;
    if (!warp_wait(full + s, (uint32_t)(u & 1)) ||
        (u > 0 && !warp_wait(acc_empty + s, (uint32_t)((u - 1) & 1)))) {
      if (lane == 0) *abort_flag = 1;
      break;
    }
    tc_fence_after();
    if (lane == 0) {
      const uint64_t adesc0 = umma_desc(smem_addr(abuf0 + s * p.abuf), (uint32_t)p.slab, 128u);
      const uint32_t acc0 = tm + (uint32_t)(s * kRows * kAccStride);
#pragma unroll 1
      for (int r = 0; r < kRows; ++r) {
#pragma unroll
        for (int tap = 0; tap < 9; ++tap) {
          const uint32_t arow = (uint32_t)(r + tap / 3) * pitch + (uint32_t)(tap % 3) * dil;
#pragma unroll
          for (int kc = 0; kc < KC; ++kc) {
            umma_bf16(acc0 + r * kAccStride, adesc0 + (arow + 2u * kc * slab16),
                      bdesc0 + (uint64_t)((tap * KC + kc) * NOUT * 2), idesc,
                      (tap | kc) != 0 ? 1u : 0u);
          }
        }
      }
      umma_commit(empty + s);
      umma_commit(acc_full + s);
    }
    __syncwarp();
    last = k;
  }
  if (aborted(abort_flag) && last >= 0)  // MMAs complete in order: wait for the last
    warp_wait(acc_full + (last & 1), (uint32_t)((last >> 1) & 1));
}

// Warp roles: warp 0 stages tiles with TMA, warp 1 issues the MMAs, warps 2 ..
// 2 + 4 kRows - 1 are the epilogue, warp w handling tensor-memory lane quarter
// w % 4 (the quarter a warp may read) of output row (w - 2) / 4. Hand-offs are
// mbarriers only: full[s] (copies landed) / empty[s] (the MMAs reading buffer s
// completed), acc_full[a] (accumulator a complete) / acc_empty[a] (its 16
// epilogue warps are done with it).
__global__ void __launch_bounds__(kConvThreads, 1)
    conv3x3_kernel(const __grid_constant__ CUtensorMap xmap, const ConvDev p) {
  extern __shared__ __align__(1024) unsigned char sm[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  unsigned char* abuf0 = sm + round_up(p.wbytes, 128);
  uint64_t* bars = reinterpret_cast<uint64_t*>(abuf0 + 2 * p.abuf);
  uint64_t* full = bars;
  uint64_t* empty = bars + 2;
  uint64_t* acc_full = bars + 4;
  uint64_t* acc_empty = bars + 6;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 8);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  float* bias_s = reinterpret_cast<float*>(tmem_slot + 4);  // [64]
  if ((smem_addr(sm) & 127u) != 0) {  // TMA destinations need 128-byte alignment
    if (tid == 0 && p.status) atomicOr(p.status, FDS_SURR_STATUS_ALIGN);
    return;
  }
  if (tid < 64) bias_s[tid] = (p.bias && tid < p.cout) ? p.bias[tid] : 0.0f;
  if (tid == 0) {
    for (int i = 0; i < 2; ++i) {
      mbar_init(full + i, 1);
      mbar_init(empty + i, 1);
      mbar_init(acc_full + i, 1);
      mbar_init(acc_empty + i, 4 * kRows);
    }
    *abort_flag = 0;
  }
  if (warp == 0) tmem_alloc(tmem_slot, kTmemCols);
  {
    const uint4* src = reinterpret_cast<const uint4*>(p.w);
    uint4* dst = reinterpret_cast<uint4*>(sm);
    for (int i = tid; i < p.wbytes / 16; i += blockDim.x) dst[i] = src[i];
  }
  // weights written by the generic proxy are read by the tensor core (async proxy)
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tm = *tmem_slot;
  const int grid = gridDim.x;
  const int nmine = my_tiles(p.ntiles);

  if (warp == 0) {
    // ---- producer
    const uint32_t tx_bytes = (uint32_t)((p.cin / 8) * (kRows + 2) * p.rx * 16);
    int issued[2] = {0, 0};
    for (int k = 0; k < nmine; ++k) {
      const int s = k & 1, u = k >> 1;
      if (aborted(abort_flag)) break;
      if (u > 0 && !warp_wait(empty + s, (uint32_t)((u - 1) & 1))) {
        if (lane == 0) *abort_flag = 1;
        break;
      }
      if (lane == 0) {
        mbar_arrive_expect_tx(full + s, tx_bytes);
        issue_rows(&xmap, decode_tile(blockIdx.x + k * grid, p.H, p.W, p.dil, kRows), p.dil,
                   p.cin / 8, kRows + 2, p.rx, p.slab, p.pitch * 16, 1, abuf0 + s * p.abuf,
                   full + s);
      }
      __syncwarp();
      ++issued[s];
    }
    if (aborted(abort_flag))  // let copies in flight land before the memory goes away
      for (int s = 0; s < 2; ++s)
        if (issued[s] > 0) warp_wait(full + s, (uint32_t)((issued[s] - 1) & 1));
  } else if (warp == 1) {
    // ---- MMA issuer
    switch (p.cin * 4 + p.cout / 16) {
      case 16 * 4 + 1: conv_mma_role<1, 16>(p, sm, abuf0, full, empty, acc_full, acc_empty, abort_flag, tm, nmine); break;
      case 16 * 4 + 2: conv_mma_role<1, 32>(p, sm, abuf0, full, empty, acc_full, acc_empty, abort_flag, tm, nmine); break;
      case 16 * 4 + 3: conv_mma_role<1, 48>(p, sm, abuf0, full, empty, acc_full, acc_empty, abort_flag, tm, nmine); break;
      case 32 * 4 + 1: conv_mma_role<2, 16>(p, sm, abuf0, full, empty, acc_full, acc_empty, abort_flag, tm, nmine); break;
      case 32 * 4 + 2: conv_mma_role<2, 32>(p, sm, abuf0, full, empty, acc_full, acc_empty, abort_flag, tm, nmine); break;
      case 32 * 4 + 3: conv_mma_role<2, 48>(p, sm, abuf0, full, empty, acc_full, acc_empty, abort_flag, tm, nmine); break;
      case 48 * 4 + 1: conv_mma_role<3, 16>(p, sm, abuf0, full, empty, acc_full, acc_empty, abort_flag, tm, nmine); break;
      case 48 * 4 + 2: conv_mma_role<3, 32>(p, sm, abuf0, full, empty, acc_full, acc_empty, abort_flag, tm, nmine); break;
      default: conv_mma_role<3, 48>(p, sm, abuf0, full, empty, acc_full, acc_empty, abort_flag, tm, nmine); break;
    }
  } else {
    // ---- epilogue
    switch (p.cout) {
      case 16: conv_epilogue_role<2>(p, tm, acc_full, acc_empty, abort_flag, bias_s, nmine); break;
      case 32: conv_epilogue_role<4>(p, tm, acc_full, acc_empty, abort_flag, bias_s, nmine); break;
      default: conv_epilogue_role<6>(p, tm, acc_full, acc_empty, abort_flag, bias_s, nmine); break;
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (tid == 0 && *abort_flag && p.status) atomicOr(p.status, FDS_SURR_STATUS_TIMEOUT);
  if (warp == 0) tmem_dealloc(tm, kTmemCols);
}

// ------------------------------------------------------------------ weight gradient

// Shared memory of a weight-gradient stage: the input rows as [row][group][pixel][8]
// (group stride pitch * 16 bytes, row stride xrow = cin/8 groups), so that the
// 8-channel groups of three consecutive rows (taps dy = 0, 1, 2) are N-groups at a
// constant stride of one MMA; then the gradient rows as [group][row][128][8].
struct WgradDev {
  float* partial;
  int32_t* status;
  int B, H, W, cin, cout, dil, ntiles;
  int rx, pitch, xrow, dzslab, xbytes, buf;
};

// The weight-gradient MMA role (one thread issues): per tile, output row r and
// 16-pixel window, one MMA per horizontal tap dx (M = 64 output channels, N = 3 cin
// = the three vertical taps x cin, K = 16 pixels, both operands MN-major) into the
// accumulator of that dx; descriptors are built once and advanced by offset / 16.
template <int CIN>
__device__ void wgrad_mma_role(const WgradDev& p, unsigned char* sm, uint64_t* full, uint64_t* empty,
                               volatile int* abort_flag, uint32_t tm, int nmine) {
  const int lane = threadIdx.x & 31;
  constexpr uint32_t idesc = umma_idesc_bf16(64, 3 * CIN) | kUmmaAMajorMN | kUmmaBMajorMN;
  const uint32_t pitch = (uint32_t)p.pitch, dil = (uint32_t)p.dil;
  const uint32_t row16 = (uint32_t)p.xrow >> 4;
  for (int k = 0; k < nmine; ++k) {
    const int s = k & 1, u = k >> 1;
    if (aborted(abort_flag) || !warp_wait(full + s, (uint32_t)(u & 1))) {
      if (lane == 0) *abort_flag = 1;
      break;
    }
    tc_fence_after();
    if (lane == 0) {
      const uint32_t xb = smem_addr(sm + s * p.buf);
      const uint64_t zd0 = umma_desc(xb + (uint32_t)p.xbytes, 128u, (uint32_t)p.dzslab);
      const uint64_t xd0 = umma_desc(xb, 128u, pitch * 16u);
#pragma unroll 1
      for (int r = 0; r < kWRows; ++r)
#pragma unroll 1
        for (int w16 = 0; w16 < kTilePx / 16; ++w16) {
          const uint64_t ad = zd0 + (uint64_t)(r * kTilePx + w16 * 16);
          const uint32_t acc = (k > 0 || r > 0 || w16 > 0) ? 1u : 0u;
#pragma unroll
          for (int dx = 0; dx < 3; ++dx) {
            const uint32_t off = (uint32_t)r * row16 + (uint32_t)(w16 * 16) + (uint32_t)dx * dil;
            umma_bf16(tm + (uint32_t)(dx * 3 * CIN), ad, xd0 + off, idesc, acc);
          }
        }
      umma_commit(empty + s);
    }
    __syncwarp();
  }
}

// Warp roles: warp 0 stages tiles (input rows and gradient rows) with TMA, warp 1
// issues the MMAs (every tile of the CTA accumulates into the same 9 per-tap
// accumulators), warps 2..9 sum the bias gradient of each staged tile (thread =
// pixel) and, at the end, read the accumulators out. A staging buffer is free once
// its MMAs completed (commit) and the 8 bias warps arrived.
__global__ void __launch_bounds__(kWgradThreads, 1)
    wgrad_kernel(const __grid_constant__ CUtensorMap xmap, const __grid_constant__ CUtensorMap dzmap,
                 const WgradDev p) {
  extern __shared__ __align__(1024) unsigned char sm[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + 2 * p.buf);
  uint64_t* full = bars;
  uint64_t* empty = bars + 2;
  uint64_t* done = bars + 4;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 5);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  float* dbw = reinterpret_cast<float*>(tmem_slot + 4);  // [8 warps][64] bias partials
  if ((smem_addr(sm) & 127u) != 0) {  // TMA destinations need 128-byte alignment
    if (tid == 0 && p.status) atomicOr(p.status, FDS_SURR_STATUS_ALIGN);
    return;
  }
  if (tid == 0) {
    for (int i = 0; i < 2; ++i) {
      mbar_init(full + i, 1);
      mbar_init(empty + i, 1 + kBiasWarps);
    }
    mbar_init(done, 1);
    *abort_flag = 0;
  }
  if (warp == 0) tmem_alloc(tmem_slot, kTmemCols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tm = *tmem_slot;
  const int grid = gridDim.x;
  const int nmine = my_tiles(p.ntiles);
  const int KGx = p.cin / 8, KGz = p.cout / 8;
  float db[48];
#pragma unroll
  for (int i = 0; i < 48; ++i) db[i] = 0.0f;

  if (warp == 0) {
    const uint32_t tx_bytes =
        (uint32_t)(KGx * (kWRows + 2) * p.rx * 16 + KGz * kWRows * kTilePx * 16);
    int issued[2] = {0, 0};
    for (int k = 0; k < nmine; ++k) {
      const int s = k & 1, u = k >> 1;
      if (aborted(abort_flag)) break;
      if (u > 0 && !warp_wait(empty + s, (uint32_t)((u - 1) & 1))) {
        if (lane == 0) *abort_flag = 1;
        break;
      }
      if (lane == 0) {
        const Tile tl = decode_tile(blockIdx.x + k * grid, p.H, p.W, p.dil, kWRows);
        unsigned char* base = sm + s * p.buf;
        mbar_arrive_expect_tx(full + s, tx_bytes);
        issue_rows(&xmap, tl, p.dil, KGx, kWRows + 2, p.rx, p.pitch * 16, p.xrow, 1, base,
                   full + s);
        issue_rows(&dzmap, tl, p.dil, KGz, kWRows, kTilePx, p.dzslab, kTilePx * 16, 0,
                   base + p.xbytes, full + s);
      }
      __syncwarp();
      ++issued[s];
    }
    if (aborted(abort_flag))
      for (int s = 0; s < 2; ++s)
        if (issued[s] > 0) warp_wait(full + s, (uint32_t)((issued[s] - 1) & 1));
  } else if (warp == 1) {
    switch (p.cin) {
      case 16: wgrad_mma_role<16>(p, sm, full, empty, abort_flag, tm, nmine); break;
      case 32: wgrad_mma_role<32>(p, sm, full, empty, abort_flag, tm, nmine); break;
      default: wgrad_mma_role<48>(p, sm, full, empty, abort_flag, tm, nmine); break;
    }
    // completion of every MMA of this CTA (also when there were none, or on abort)
    if (lane == 0) umma_commit(done);
    __syncwarp();
  } else {
    const int px = tid - 64;  // pixel of the tile: row px / 128, column px % 128
    for (int k = 0; k < nmine; ++k) {
      const int s = k & 1, u = k >> 1;
      if (aborted(abort_flag)) break;
      if (!warp_wait(full + s, (uint32_t)(u & 1))) {
        if (lane == 0) *abort_flag = 1;
        break;
      }
      const unsigned char* zs = sm + s * p.buf + p.xbytes + px * 16;
      for (int g = 0; g < KGz; ++g) {
        float f[8];
        unpack8(*reinterpret_cast<const uint4*>(zs + g * p.dzslab), f);
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
          for (int gg = 0; gg < 6; ++gg)
            if (gg == g) db[gg * 8 + i] += f[i];
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(empty + s);
    }
  }
  __syncthreads();
  const bool ok = !*abort_flag && warp_wait(done, 0u);
  tc_fence_after();
  if (ok && warp >= 2) {
    // D row m (output channel) sits in lane 32 (m / 16) + m % 16; tap (dy, dx) is
    // columns (3 dx + dy) cin .. + cin - 1
    const int q = warp & 3, half = (warp - 2) >> 2;
    const int m = 16 * q + lane;
    const int hc = p.cin / 2;
    const size_t row_len = (size_t)9 * p.cout * p.cin + p.cout;
    float* out = p.partial + (size_t)blockIdx.x * row_len;
    for (int tap = 0; tap < 9; ++tap)
      for (int c0 = half * hc; c0 < (half + 1) * hc; c0 += 8) {
        float v[8];
        if (nmine > 0) {
          tmem_ld8(tm + ((uint32_t)(32 * q) << 16) +
                       (uint32_t)((3 * (tap % 3) + tap / 3) * p.cin + c0),
                   v);
        } else {
#pragma unroll
          for (int i = 0; i < 8; ++i) v[i] = 0.0f;
        }
        if (lane < 16 && m < p.cout) {
          float4* dst = reinterpret_cast<float4*>(out + ((size_t)tap * p.cout + m) * p.cin + c0);
          dst[0] = make_float4(v[0], v[1], v[2], v[3]);
          dst[1] = make_float4(v[4], v[5], v[6], v[7]);
        }
      }
    // bias: warp sums in a fixed order, then the 8 warp sums in warp order
#pragma unroll
    for (int i = 0; i < 48; ++i) {
      float v = db[i];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) dbw[(warp - 2) * 64 + i] = v;
    }
  }
  __syncthreads();
  if (ok && tid < p.cout) {
    float v = 0.0f;
    for (int w = 0; w < kBiasWarps; ++w) v += dbw[w * 64 + tid];
    p.partial[(size_t)blockIdx.x * ((size_t)9 * p.cout * p.cin + p.cout) +
              (size_t)9 * p.cout * p.cin + tid] = v;
  }
  if (tid == 0 && !ok && p.status) atomicOr(p.status, FDS_SURR_STATUS_TIMEOUT);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tm, kTmemCols);
}

// ------------------------------------------------------------------ optimiser, packing

__global__ void pack_kernel(int cin, int cout, const float* __restrict__ w,
                            __nv_bfloat16* __restrict__ wfwd, __nv_bfloat16* __restrict__ wbwd) {
  const int n = 9 * cout * cin;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int ci = i % cin, co = (i / cin) % cout, tap = i / (cin * cout);
    const __nv_bfloat16 h = __float2bfloat16_rn(w[i]);
    wfwd[packed_index(tap, co, ci, cin, cout)] = h;
    if (wbwd) wbwd[packed_index(8 - tap, ci, co, cout, cin)] = h;
  }
}

struct AdamDev {
  int cin, cout, nparts;
  float lr, beta1, beta2, eps, wd, scale, corr1, corr2_sqrt;
  const float* partial;
  float *w, *b, *m, *v;
  __nv_bfloat16 *wfwd, *wbwd;
  float* grad_out;
};

__global__ void adamw_kernel(const AdamDev a) {
  const int nw = 9 * a.cout * a.cin, n = nw + a.cout;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float g = 0.0f;
    for (int r = 0; r < a.nparts; ++r) g += a.partial[(size_t)r * n + i];
    g *= a.scale;
    if (a.grad_out) a.grad_out[i] = g;
    if (a.lr == 0.0f) continue;
    float* param = i < nw ? a.w + i : a.b + (i - nw);
    float x = *param * (1.0f - a.lr * a.wd);
    const float m = a.beta1 * a.m[i] + (1.0f - a.beta1) * g;
    const float v = a.beta2 * a.v[i] + (1.0f - a.beta2) * g * g;
    a.m[i] = m;
    a.v[i] = v;
    x -= a.lr / a.corr1 * m / (sqrtf(v) / a.corr2_sqrt + a.eps);
    *param = x;
    if (i < nw) {
      const int ci = i % a.cin, co = (i / a.cin) % a.cout, tap = i / (a.cin * a.cout);
      const __nv_bfloat16 h = __float2bfloat16_rn(x);
      a.wfwd[packed_index(tap, co, ci, a.cin, a.cout)] = h;
      if (a.wbwd) a.wbwd[packed_index(8 - tap, ci, co, a.cout, a.cin)] = h;
    }
  }
}

// ------------------------------------------------------------------ data plumbing

template <typename T>
__device__ __forceinline__ const T* state_at(const FdsSurrData& d, int k, int snap_shift) {
  const size_t plane = (size_t)d.height * d.width;
  return reinterpret_cast<const T*>(d.state) +
         ((size_t)d.inst[k] * d.nsnap + d.snap[k] + snap_shift) * 3 * plane;
}

// Block-wide sum over blockDim.x = 32 * NW threads, the same order on every call.
template <int NW>
__device__ __forceinline__ float block_sum(float v, float* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  float s = 0.0f;
  if (threadIdx.x == 0)
    for (int w = 0; w < NW; ++w) s += red[w];
  __syncthreads();
  return s;
}

template <typename T>
struct Vec4;
template <>
struct Vec4<float> {
  using type = float4;
};
template <>
struct Vec4<double> {
  using type = double4;
};

// Energy norm of each sample's input state: one 1024-thread CTA per sample, four
// cells per load (the plane is a multiple of 128 cells).
template <typename T>
__global__ void __launch_bounds__(1024) scale_kernel(const FdsSurrData d) {
  __shared__ float red[32];
  using V = typename Vec4<T>::type;
  const int k = blockIdx.x;
  const size_t plane = (size_t)d.height * d.width;
  const T* st = state_at<T>(d, k, 0);
  const float z = d.zref[d.inst[k]];
  const V* p4 = reinterpret_cast<const V*>(st);
  const V* x4 = reinterpret_cast<const V*>(st + plane);
  const V* y4 = reinterpret_cast<const V*>(st + 2 * plane);
  float acc = 0.0f;
  for (size_t i = threadIdx.x; i < plane / 4; i += blockDim.x) {
    const V a = p4[i], b = x4[i], c = y4[i];
    acc += (float)a.x * (float)a.x + (float)a.y * (float)a.y + (float)a.z * (float)a.z +
           (float)a.w * (float)a.w;
    const float bx = z * (float)b.x, by = z * (float)b.y, bz = z * (float)b.z, bw = z * (float)b.w;
    const float cx = z * (float)c.x, cy = z * (float)c.y, cz = z * (float)c.z, cw = z * (float)c.w;
    acc += bx * bx + by * by + bz * bz + bw * bw + cx * cx + cy * cy + cz * cz + cw * cw;
  }
  const float s = block_sum<32>(acc, red);
  if (threadIdx.x == 0) d.scale[k] = sqrtf(s / (float)plane);
}

template <typename T>
__global__ void __launch_bounds__(256) pack_input_kernel(const FdsSurrData d) {
  const size_t plane = (size_t)d.height * d.width;
  const int k = blockIdx.y;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= plane) return;
  const int inst = d.inst[k];
  const float sc = d.scale[k];
  const float inv = sc > 0.0f ? 1.0f / sc : 0.0f;
  const float z = d.zref[inst];
  const T* st = state_at<T>(d, k, 0);
  const float* md = d.media + (size_t)inst * 2 * plane;
  const float sp = (float)st[i] * inv, svx = z * (float)st[plane + i] * inv,
              svy = z * (float)st[2 * plane + i] * inv;
  float f[8] = {md[i], md[plane + i], sp, svx, svy, d.freq[inst], 0.0f, 0.0f};
  uint4* x = reinterpret_cast<uint4*>(d.x);  // [count][2][plane] rows of 8 channels
  x[(size_t)k * 2 * plane + i] = pack8(f);
  x[((size_t)k * 2 + 1) * plane + i] = make_uint4(0u, 0u, 0u, 0u);
  reinterpret_cast<float4*>(d.s)[(size_t)k * plane + i] = make_float4(sp, svx, svy, 0.0f);
  if (d.t) {
    const T* tg = state_at<T>(d, k, 1);
    reinterpret_cast<float4*>(d.t)[(size_t)k * plane + i] =
        make_float4((float)tg[i] * inv, z * (float)tg[plane + i] * inv,
                    z * (float)tg[2 * plane + i] * inv, 0.0f);
  }
}

__global__ void __launch_bounds__(256)
    loss_kernel(const FdsSurrData d, const float* __restrict__ y, __nv_bfloat16* __restrict__ dy,
                float* __restrict__ parts, float gscale) {
  __shared__ float red[8];
  const size_t n = (size_t)d.count * d.height * d.width;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  float err = 0.0f;
  if (i < n) {
    const size_t plane = (size_t)d.height * d.width;
    const size_t k = i / plane, pix = i % plane;
    // y: float32 [count][2][plane][8]; the state channels are group 0, values 0..2
    const float4 o = reinterpret_cast<const float4*>(y)[(k * 2 * plane + pix) * 2];
    const float4 s = reinterpret_cast<const float4*>(d.s)[i];
    const float4 t = reinterpret_cast<const float4*>(d.t)[i];
    const float e0 = s.x + o.x - t.x, e1 = s.y + o.y - t.y, e2 = s.z + o.z - t.z;
    err = e0 * e0 + e1 * e1 + e2 * e2;
    float f[8] = {gscale * e0, gscale * e1, gscale * e2, 0, 0, 0, 0, 0};
    uint4* g = reinterpret_cast<uint4*>(dy);
    g[k * 2 * plane + pix] = pack8(f);
    g[(k * 2 + 1) * plane + pix] = make_uint4(0u, 0u, 0u, 0u);
  }
  const float s = block_sum<8>(err, red);
  if (threadIdx.x == 0) parts[blockIdx.x] = s;
}

template <typename T>
__global__ void __launch_bounds__(256) unpack_kernel(const FdsSurrData d, const float* __restrict__ y) {
  const size_t plane = (size_t)d.height * d.width;
  const int k = blockIdx.y;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= plane) return;
  const int inst = d.inst[k];
  const float sc = d.scale[k];
  const float z = d.zref[inst];
  const float4 o = reinterpret_cast<const float4*>(y)[((size_t)k * 2 * plane + i) * 2];
  const float4 s = reinterpret_cast<const float4*>(d.s)[(size_t)k * plane + i];
  T* st = const_cast<T*>(state_at<T>(d, k, 0));
  float pv = (s.x + o.x) * sc;
  const int xx = (int)(i % d.width), yy = (int)(i / d.width);
  if (d.edge_zero_p && (xx == 0 || yy == 0 || xx == d.width - 1 || yy == d.height - 1)) pv = 0.0f;
  st[i] = (T)pv;
  st[plane + i] = (T)((s.y + o.y) * sc / z);
  st[2 * plane + i] = (T)((s.z + o.z) * sc / z);
}

__global__ void __launch_bounds__(256)
    compare_kernel(int H, int W, const int32_t* inst, const double* a, const double* b,
                   const float* zref, double* out) {
  __shared__ double red[8];
  const int k = blockIdx.x;
  const size_t plane = (size_t)H * W;
  const int n = inst[k];
  const double z = zref[n];
  const double* pa = a + (size_t)n * 3 * plane;
  const double* pb = b + (size_t)n * 3 * plane;
  double dd = 0.0, bb = 0.0;
  for (size_t i = threadIdx.x; i < 3 * plane; i += blockDim.x) {
    const double wgt = i < plane ? 1.0 : z;
    const double e = (pa[i] - pb[i]) * wgt, v = pb[i] * wgt;
    dd += e * e;
    bb += v * v;
  }
  for (int pass = 0; pass < 2; ++pass) {
    double v = pass == 0 ? dd : bb;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0.0;
      for (int w = 0; w < 8; ++w) s += red[w];
      out[2 * k + pass] = s;
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------ host side

int sm_count() {
  static const int n = []() {
    int dev = 0, count = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        count <= 0)
      return 148;
    return count;
  }();
  return n;
}

// [B][C/8][H][W][8] bf16 activations as a 4-D tensor (8, W, H, B * C/8); boxes of
// 8 channels x bw pixels x 1 row x 1 group.
bool encode_act_map(CUtensorMap* m, const void* base, int B, int H, int W, int C, int bw) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc || !base || ((uintptr_t)base & 15) != 0 || bw > 256) return false;
  const cuuint64_t dims[4] = {8, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)B * (C / 8)};
  const cuuint64_t strides[3] = {16, (cuuint64_t)W * 16, (cuuint64_t)H * W * 16};
  const cuuint32_t box[4] = {8, (cuuint32_t)bw, 1, 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(base), dims, strides, box,
             estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
             CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool channels_ok(int c) { return c == 16 || c == 32 || c == 48; }
bool dil_ok(int d) { return d == 1 || d == 2 || d == 4 || d == 8; }
bool aligned16(const void* p) { return ((uintptr_t)p & 15) == 0; }

int32_t launch_error(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(FDS_E_LAUNCH, "%s: %s", what, cudaGetErrorString(e));
  return FDS_OK;
}

int32_t set_smem(const void* fn, int bytes) {
  const cudaError_t e =
      cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxSmem);
  if (e != cudaSuccess)
    return set_error(FDS_E_LAUNCH, "cudaFuncSetAttribute: %s", cudaGetErrorString(e));
  (void)bytes;
  return FDS_OK;
}

}  // namespace surr
}  // namespace fds

using namespace fds;
using namespace fds::surr;

extern "C" int64_t fds_conv_packed_elems(int32_t cin, int32_t cout) {
  return (int64_t)9 * cin * cout;
}

extern "C" int32_t fds_conv3x3(const FdsConvArgs* a, void* stream) {
  if (!a) return set_error(FDS_E_ARG, "null FdsConvArgs");
  if (a->batch < 1 || a->height < 1 || a->width < 1)
    return set_error(FDS_E_ARG, "bad activation shape %dx%dx%d", a->batch, a->height, a->width);
  if (!channels_ok(a->cin) || !channels_ok(a->cout))
    return set_error(FDS_E_ARG, "channels %d -> %d: each must be 16, 32 or 48", a->cin, a->cout);
  if (!dil_ok(a->dilation)) return set_error(FDS_E_ARG, "dilation %d not in {1,2,4,8}", a->dilation);
  if (a->width % kTilePx != 0 || a->height % (kRows * a->dilation) != 0)
    return set_error(FDS_E_ARG, "%dx%d image: width must be a multiple of %d, height of %d",
                     a->width, a->height, kTilePx, kRows * a->dilation);
  if (!a->x || !a->weight || !aligned16(a->x) || !aligned16(a->weight))
    return set_error(FDS_E_ARG, "x / weight missing or not 16-byte aligned");
  switch (a->mode) {
    case FDS_CONV_FWD_GELU:
      if (!a->out_h || !aligned16(a->out_h) || (a->out_z && !aligned16(a->out_z)) ||
          (a->resid && !aligned16(a->resid)))
        return set_error(FDS_E_ARG, "FWD_GELU needs a 16-byte aligned out_h");
      break;
    case FDS_CONV_FWD_LINEAR:
      if (!a->out_f32 || !aligned16(a->out_f32))
        return set_error(FDS_E_ARG, "FWD_LINEAR needs a 16-byte aligned out_f32");
      break;
    case FDS_CONV_BWD_DATA:
      if (!a->out_z || !a->zin || !aligned16(a->out_z) || !aligned16(a->zin) ||
          (a->out_h && !aligned16(a->out_h)) || (a->resid && !aligned16(a->resid)))
        return set_error(FDS_E_ARG, "BWD_DATA needs 16-byte aligned out_z and zin");
      break;
    default:
      return set_error(FDS_E_ARG, "unknown convolution mode %d", a->mode);
  }
  ConvDev p{};
  p.w = static_cast<const __nv_bfloat16*>(a->weight);
  p.bias = a->bias;
  p.resid = static_cast<const __nv_bfloat16*>(a->resid);
  p.zin = static_cast<const __nv_bfloat16*>(a->zin);
  p.out_z = static_cast<__nv_bfloat16*>(a->out_z);
  p.out_h = static_cast<__nv_bfloat16*>(a->out_h);
  p.out_f32 = a->out_f32;
  p.status = a->status;
  p.B = a->batch;
  p.H = a->height;
  p.W = a->width;
  p.cin = a->cin;
  p.cout = a->cout;
  p.dil = a->dilation;
  p.mode = a->mode;
  p.ntiles = a->batch * (a->height / (kRows * a->dilation)) * a->dilation * (a->width / kTilePx);
  p.rx = kTilePx + 2 * a->dilation;
  p.pitch = round_up(p.rx, 8);
  p.slab = (kRows + 2) * p.pitch * 16;
  p.abuf = (a->cin / 8) * p.slab;
  p.wbytes = 9 * a->cin * a->cout * 2;
  const int smem = round_up(p.wbytes, 128) + 2 * p.abuf + 96 + 64 * 4;
  if (smem > kMaxSmem)
    return set_error(FDS_E_SIZE, "convolution %d->%d dilation %d needs %d bytes of shared memory",
                     a->cin, a->cout, a->dilation, smem);
  CUtensorMap map;
  if (!encode_act_map(&map, a->x, a->batch, a->height, a->width, a->cin, p.rx))
    return set_error(FDS_E_LAUNCH, "tensor map encoding failed for the convolution input");
  int32_t rc = set_smem(reinterpret_cast<const void*>(conv3x3_kernel), smem);
  if (rc != FDS_OK) return rc;
  const int grid = p.ntiles < sm_count() ? p.ntiles : sm_count();
  conv3x3_kernel<<<grid, kConvThreads, smem > kMinSmem ? smem : kMinSmem,
                   static_cast<cudaStream_t>(stream)>>>(map, p);
  return launch_error("conv3x3_kernel");
}

extern "C" int32_t fds_conv_wgrad_max_grid(void) { return sm_count(); }

extern "C" int32_t fds_conv3x3_wgrad(const FdsWgradArgs* a, void* stream) {
  if (!a) return set_error(FDS_E_ARG, "null FdsWgradArgs");
  if (a->batch < 1 || a->height < 1 || a->width < 1)
    return set_error(FDS_E_ARG, "bad activation shape");
  if (!channels_ok(a->cin) || !channels_ok(a->cout))
    return set_error(FDS_E_ARG, "channels %d -> %d: each must be 16, 32 or 48", a->cin, a->cout);
  if (!dil_ok(a->dilation)) return set_error(FDS_E_ARG, "dilation %d not in {1,2,4,8}", a->dilation);
  if (a->width % kTilePx != 0 || a->height % (kWRows * a->dilation) != 0)
    return set_error(FDS_E_ARG, "%dx%d image: width must be a multiple of %d, height of %d",
                     a->width, a->height, kTilePx, kWRows * a->dilation);
  if (a->grid < 1 || a->grid > sm_count())
    return set_error(FDS_E_ARG, "grid %d not in [1, %d]", a->grid, sm_count());
  if (!a->x || !a->dz || !a->partial || !aligned16(a->x) || !aligned16(a->dz) ||
      !aligned16(a->partial))
    return set_error(FDS_E_ARG, "x / dz / partial missing or not 16-byte aligned");
  WgradDev p{};
  p.partial = a->partial;
  p.status = a->status;
  p.B = a->batch;
  p.H = a->height;
  p.W = a->width;
  p.cin = a->cin;
  p.cout = a->cout;
  p.dil = a->dilation;
  p.ntiles = a->batch * (a->height / (kWRows * a->dilation)) * a->dilation * (a->width / kTilePx);
  p.rx = kTilePx + 2 * a->dilation;
  p.pitch = round_up(p.rx, 8);
  p.xrow = (a->cin / 8) * p.pitch * 16;
  p.dzslab = kWRows * kTilePx * 16;
  p.xbytes = (kWRows + 2) * p.xrow;
  // the M = 64 operand spans 8 channel groups; the ones past cout are never used
  p.buf = p.xbytes + 8 * p.dzslab;
  const int smem = 2 * p.buf + 64 + kBiasWarps * 64 * 4;
  if (smem > kMaxSmem)
    return set_error(FDS_E_SIZE, "weight gradient %d->%d dilation %d needs %d bytes of shared memory",
                     a->cin, a->cout, a->dilation, smem);
  CUtensorMap xm, zm;
  if (!encode_act_map(&xm, a->x, a->batch, a->height, a->width, a->cin, p.rx) ||
      !encode_act_map(&zm, a->dz, a->batch, a->height, a->width, a->cout, kTilePx))
    return set_error(FDS_E_LAUNCH, "tensor map encoding failed for the weight gradient");
  int32_t rc = set_smem(reinterpret_cast<const void*>(wgrad_kernel), smem);
  if (rc != FDS_OK) return rc;
  wgrad_kernel<<<a->grid, kWgradThreads, smem > kMinSmem ? smem : kMinSmem,
                 static_cast<cudaStream_t>(stream)>>>(xm, zm, p);
  return launch_error("wgrad_kernel");
}

extern "C" int32_t fds_conv_pack(int32_t cin, int32_t cout, const float* w, void* wfwd, void* wbwd,
                                 void* stream) {
  if (!channels_ok(cin) || !channels_ok(cout) || !w || !wfwd)
    return set_error(FDS_E_ARG, "bad fds_conv_pack arguments");
  pack_kernel<<<64, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      cin, cout, w, static_cast<__nv_bfloat16*>(wfwd), static_cast<__nv_bfloat16*>(wbwd));
  return launch_error("pack_kernel");
}

extern "C" int32_t fds_adamw(const FdsAdamArgs* a, void* stream) {
  if (!a || !channels_ok(a->cin) || !channels_ok(a->cout) || a->nparts < 1 || !a->partial ||
      a->step < 1)
    return set_error(FDS_E_ARG, "bad FdsAdamArgs");
  if (a->lr != 0.0f && (!a->weight || !a->bias || !a->m || !a->v || !a->wfwd))
    return set_error(FDS_E_ARG, "AdamW step needs weight, bias, moments and wfwd");
  AdamDev d{};
  d.cin = a->cin;
  d.cout = a->cout;
  d.nparts = a->nparts;
  d.lr = a->lr;
  d.beta1 = a->beta1;
  d.beta2 = a->beta2;
  d.eps = a->eps;
  d.wd = a->weight_decay;
  d.scale = a->grad_scale;
  d.corr1 = (float)(1.0 - pow((double)a->beta1, (double)a->step));
  d.corr2_sqrt = (float)sqrt(1.0 - pow((double)a->beta2, (double)a->step));
  d.partial = a->partial;
  d.w = a->weight;
  d.b = a->bias;
  d.m = a->m;
  d.v = a->v;
  d.wfwd = static_cast<__nv_bfloat16*>(a->wfwd);
  d.wbwd = static_cast<__nv_bfloat16*>(a->wbwd);
  d.grad_out = a->grad_out;
  const int n = 9 * a->cout * a->cin + a->cout;
  adamw_kernel<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(d);
  return launch_error("adamw_kernel");
}

static int32_t check_data(const FdsSurrData* d, bool need_t) {
  if (!d || d->count < 1 || d->height < 1 || d->width < 1 || d->nsnap < 1 || !d->inst ||
      !d->snap || !d->state || !d->scale || !d->s || !d->zref)
    return set_error(FDS_E_ARG, "bad FdsSurrData");
  if (need_t && !d->t) return set_error(FDS_E_ARG, "FdsSurrData.t is required here");
  if (!aligned16(d->s) || (d->t && !aligned16(d->t)) || (d->x && !aligned16(d->x)))
    return set_error(FDS_E_ARG, "FdsSurrData buffers must be 16-byte aligned");
  return FDS_OK;
}

extern "C" int32_t fds_surr_pack(const FdsSurrData* d, void* stream) {
  int32_t rc = check_data(d, false);
  if (rc != FDS_OK) return rc;
  if (!d->x || !d->media || !d->freq) return set_error(FDS_E_ARG, "pack needs x, media, freq");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t plane = (size_t)d->height * d->width;
  const dim3 grid((unsigned)((plane + 255) / 256), (unsigned)d->count);
  if (d->state_f64) {
    scale_kernel<double><<<d->count, 1024, 0, s>>>(*d);
    pack_input_kernel<double><<<grid, 256, 0, s>>>(*d);
  } else {
    scale_kernel<float><<<d->count, 1024, 0, s>>>(*d);
    pack_input_kernel<float><<<grid, 256, 0, s>>>(*d);
  }
  return launch_error("pack_input_kernel");
}

extern "C" int32_t fds_surr_loss_parts(int32_t count, int32_t height, int32_t width) {
  return (int32_t)(((int64_t)count * height * width + 255) / 256);
}

extern "C" int32_t fds_surr_loss(const FdsSurrData* d, const float* y, void* dy, float* loss_parts,
                                 void* stream) {
  int32_t rc = check_data(d, true);
  if (rc != FDS_OK) return rc;
  if (!y || !dy || !loss_parts || !aligned16(y) || !aligned16(dy))
    return set_error(FDS_E_ARG, "loss needs aligned y, dy and loss_parts");
  const int nb = fds_surr_loss_parts(d->count, d->height, d->width);
  const float gscale = 2.0f / (3.0f * (float)d->count * d->height * d->width);
  loss_kernel<<<nb, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      *d, y, static_cast<__nv_bfloat16*>(dy), loss_parts, gscale);
  return launch_error("loss_kernel");
}

extern "C" int32_t fds_surr_unpack(const FdsSurrData* d, const float* y, void* stream) {
  int32_t rc = check_data(d, false);
  if (rc != FDS_OK) return rc;
  if (!y || !aligned16(y)) return set_error(FDS_E_ARG, "unpack needs an aligned y");
  const size_t plane = (size_t)d->height * d->width;
  const dim3 grid((unsigned)((plane + 255) / 256), (unsigned)d->count);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (d->state_f64)
    unpack_kernel<double><<<grid, 256, 0, s>>>(*d, y);
  else
    unpack_kernel<float><<<grid, 256, 0, s>>>(*d, y);
  return launch_error("unpack_kernel");
}

extern "C" int32_t fds_surr_compare(int32_t count, int32_t height, int32_t width,
                                    const int32_t* inst, const double* a, const double* b,
                                    const float* zref, double* out, void* stream) {
  if (count < 1 || height < 1 || width < 1 || !inst || !a || !b || !zref || !out)
    return set_error(FDS_E_ARG, "bad fds_surr_compare arguments");
  compare_kernel<<<count, 256, 0, static_cast<cudaStream_t>(stream)>>>(height, width, inst, a, b,
                                                                       zref, out);
  return launch_error("compare_kernel");
}
