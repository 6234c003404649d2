// Step loop and variant dispatch of the fused staggered-grid kernel, for one
// precision (included by one translation unit per precision).
#pragma once

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <utility>
#include <vector>

#include "fds_internal.h"
#include "batch_kernel.cuh"
#include "march_kernel.cuh"
#include "cluster_1d.cuh"
#include "warp_1d.cuh"
#include "resident_1d.cuh"
#include "stag_kernel.cuh"

namespace fds {

constexpr int kTile2dX = 64, kTile2dY = 16, kTile1dX = 1024;
constexpr int kThreads = 256;

// Tensor maps of one call, built by the first launch (which knows the box shape)
// for both ping-pong buffers of each state array.
struct StagTmaCache {
  bool tried = false;
  bool ok = false;
  const void* pbuf[2] = {nullptr, nullptr};
  const void* ubuf[2] = {nullptr, nullptr};
  const void* vbuf[2] = {nullptr, nullptr};
  const void* state[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  CUtensorMap p[2], u[2], v[2], bx, kx, by, ky;
};

template <typename TP, typename TF, typename TC>
using StagLaunch = int32_t (*)(StagArgs<TP, TF, TC>&, cudaStream_t, StagTmaCache*);

// Use TMA staging for this launch if the variant and the arrays allow it.
template <class C, typename TP, typename TF, typename TC>
void select_tma(StagArgs<TP, TF, TC>& a, StagTmaCache* tc, const void* const* state_bufs) {
  a.use_tma = 0;
  if (!tc || !C::HAS_V || C::RX > 256 || C::RY > 256) return;
  if (!tc->tried) {
    tc->tried = true;
    bool ok = true;
    for (int k = 0; k < 2; ++k) {
      tc->pbuf[k] = state_bufs[k];
      ok = ok && encode_tile_map(&tc->p[k], state_bufs[k], sizeof(TP), a.nx, a.ny, C::RX, C::RY);
      if (C::MEMORY) {
        tc->ubuf[k] = state_bufs[2 + k];
        tc->vbuf[k] = state_bufs[4 + k];
        ok = ok && encode_tile_map(&tc->u[k], state_bufs[2 + k], sizeof(TF), a.nx, a.ny, C::RX, C::RY);
        ok = ok && encode_tile_map(&tc->v[k], state_bufs[4 + k], sizeof(TF), a.nx, a.ny, C::RX, C::RY);
      }
    }
    ok = ok && encode_tile_map(&tc->bx, a.bx, sizeof(TC), a.nx, a.ny, C::RX, C::RY);
    ok = ok && encode_tile_map(&tc->kx, a.kx, sizeof(TC), a.nx, a.ny, C::RX, C::RY);
    ok = ok && encode_tile_map(&tc->by, a.by, sizeof(TC), a.nx, a.ny, C::RX, C::RY);
    ok = ok && encode_tile_map(&tc->ky, a.ky, sizeof(TC), a.nx, a.ny, C::RX, C::RY);
    tc->ok = ok;
  }
  if (!tc->ok) return;
  const int ip = (a.p_in == tc->pbuf[0]) ? 0 : (a.p_in == tc->pbuf[1] ? 1 : -1);
  if (ip < 0) return;
  a.tm[0] = tc->p[ip];
  if (C::MEMORY) {
    const int iu = (a.u_in == tc->ubuf[0]) ? 0 : (a.u_in == tc->ubuf[1] ? 1 : -1);
    const int iv = (a.v_in == tc->vbuf[0]) ? 0 : (a.v_in == tc->vbuf[1] ? 1 : -1);
    if (iu < 0 || iv < 0) return;
    a.tm[1] = tc->u[iu];
    a.tm[2] = tc->v[iv];
  }
  a.tm[3] = tc->bx;
  a.tm[4] = tc->kx;
  a.tm[5] = tc->by;
  a.tm[6] = tc->ky;
  a.use_tma = 1;
}

// Device limits, the dynamic shared-memory attribute and the resident CTAs per SM of
// one tile-kernel instantiation (KERNEL), cached per instantiation, device and staging
// layout (isotropic or not; the shared-memory size follows from it). Safe to call from
// several host threads. Returns FDS_OK or an error code.
struct LaunchShape {
  int nsm;  // SMs of the device
  int occ;  // resident CTAs per SM at this shared-memory size
};

constexpr int kMaxDevices = 64;

template <auto KERNEL>
int32_t kernel_shape(size_t smem, int threads, bool iso, LaunchShape* out) {
  struct Entry {
    int optin = -1, nsm = -1;
    size_t attr_bytes = 0;  // dynamic shared memory the attribute allows so far
    int occ[2] = {-1, -1};
  };
  static std::mutex mu;
  static Entry cache[kMaxDevices];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_error(FDS_E_LAUNCH, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices)
    return set_error(FDS_E_LAUNCH, "device %d: at most %d devices per process", dev, kMaxDevices);
  std::lock_guard<std::mutex> lock(mu);
  Entry& c = cache[dev];
  if (c.optin < 0) {
    int optin = -1, nsm = -1;
    e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess || optin < 1 || nsm < 1)
      return set_error(FDS_E_LAUNCH, "device attributes: %s", cudaGetErrorString(e));
    c.nsm = nsm;
    c.optin = optin;
  }
  if (smem > (size_t)c.optin)
    return set_error(FDS_E_SIZE, "tile needs %zu bytes of shared memory (device allows %d)", smem,
                     c.optin);
  if (smem > c.attr_bytes) {
    e = cudaFuncSetAttribute(KERNEL, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return set_error(FDS_E_LAUNCH, "smem attribute: %s", cudaGetErrorString(e));
    c.attr_bytes = smem;
  }
  int& o = c.occ[iso ? 1 : 0];
  if (o < 0) {
    int n = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, KERNEL, threads, smem);
    o = (e == cudaSuccess && n >= 1) ? n : 1;
  }
  out->nsm = c.nsm;
  out->occ = o;
  return FDS_OK;
}

// L2 prefetch distance of the one-stage TMA path: the tile 0.4 waves of resident CTAs
// ahead (measured on the 2048^2 step against 0 to 2 waves: double words +6 %, float32
// +5 %, float64 +1 %; two waves already lose)
inline int32_t prefetch_distance(const LaunchShape& ls) {
  return (int32_t)(0.4 * ls.occ * ls.nsm);
}

// Launch one step. STAGES == 1: one CTA per tile. STAGES == 2: persistent CTAs,
// as many as fit on the device at this variant's occupancy.
template <class C, typename TP, typename TF, typename TC>
int32_t launch_stag(StagArgs<TP, TF, TC>& a, cudaStream_t s, StagTmaCache* tc) {
  const bool iso = a.iso != 0 || !C::HAS_V;
  // the TMA barriers (16 bytes per stage) follow the buffers
  const size_t smem = (size_t)C::STAGES * stag_buffer_bytes<C, TP, TF, TC>(iso) + 16 * C::STAGES;
  LaunchShape ls;
  const int32_t rc = kernel_shape<stag_step_kernel<C, TP, TF, TC>>(smem, C::NT, iso, &ls);
  if (rc != FDS_OK) return rc;
  select_tma<C>(a, tc, tc ? tc->state : nullptr);
  int grid = a.ntiles;
  if (C::STAGES > 1) grid = a.ntiles < ls.occ * ls.nsm ? a.ntiles : ls.occ * ls.nsm;
  a.prefetch = (C::STAGES == 1 && a.use_tma) ? prefetch_distance(ls) : 0;
  stag_step_kernel<C, TP, TF, TC><<<grid, C::NT, smem, s>>>(a);
  return FDS_OK;
}

// Launch one or two steps (a.substeps) of the two-step kernel: one CTA per tile.
template <class C, typename TP, typename TF, typename TC>
int32_t launch_tb2(StagArgs<TP, TF, TC>& a, cudaStream_t s, StagTmaCache* tc) {
  const bool iso = a.iso != 0;
  const size_t smem = stag_buffer_bytes<C, TP, TF, TC>(iso) + 16;
  LaunchShape ls;
  const int32_t rc = kernel_shape<stag_tb2_kernel<C, TP, TF, TC>>(smem, C::NT, iso, &ls);
  if (rc != FDS_OK) return rc;
  select_tma<C>(a, tc, tc ? tc->state : nullptr);
  a.prefetch = a.use_tma ? prefetch_distance(ls) : 0;
  stag_tb2_kernel<C, TP, TF, TC><<<a.ntiles, C::NT, smem, s>>>(a);
  return FDS_OK;
}

template <class C, typename TP, typename TF, typename TC>
int32_t launch_march(StagArgs<TP, TF, TC>& a, cudaStream_t s, StagTmaCache*) {
  const int grid = (a.ntiles + C::NW - 1) / C::NW;
  march_step_kernel<C, TP, TF, TC><<<grid, C::NT, 0, s>>>(a);
  return FDS_OK;
}

// Kernel of one variant; nullptr when not built for this precision or tile.
template <typename TP, typename TF, typename TC, bool ALLOW_EXACT, bool ALLOW_ACOUSTIC>
StagLaunch<TP, TF, TC> pick_stag(int family, bool has_v, bool absorb, bool axi, bool exact,
                                 int tx, int ty, int stages) {
  constexpr int T = kThreads;
  const bool acoustic = (family == FDS_FAMILY_ACOUSTIC);
  if (exact && !ALLOW_EXACT) return nullptr;
  if (acoustic && !ALLOW_ACOUSTIC) return nullptr;
  if (!acoustic && absorb) return nullptr;
  if (stages == 3) {
    // two steps per tile: lossless 2-D (axisymmetric without losses steps as planar),
    // potential and fluxes of one type
    if constexpr (sizeof(TP) == sizeof(TF)) {
#define FDS_PICK_TB2(TX, TY, NT)                                                            \
  if (has_v && !absorb && !exact && tx == TX && ty == TY) {                                  \
    if (acoustic) {                                                                         \
      if constexpr (ALLOW_ACOUSTIC) return &launch_tb2<Tb2Cfg<TX, TY, NT, true>, TP, TF, TC>; \
    } else {                                                                                \
      return &launch_tb2<Tb2Cfg<TX, TY, NT, false>, TP, TF, TC>;                            \
    }                                                                                       \
  }
      FDS_TB2_MENU(FDS_PICK_TB2)
#undef FDS_PICK_TB2
    }
    return nullptr;
  }
  // the radius only enters the kernel through the exact pressure scaling and the
  // radial loss term; otherwise the axisymmetric step is the planar one
  if (axi && !exact && !absorb) axi = false;
  const bool dflt = stages == 1 &&
                    (has_v ? (tx == kTile2dX && ty == kTile2dY) : (tx == kTile1dX && ty == 1));
#define FDS_PICK(TX, TY, HV, MEM, ABS, AX, EX)                                              \
  if (dflt && has_v == HV && acoustic == MEM && absorb == ABS && axi == AX && exact == EX) \
    return &launch_stag<StagCfg<TX, TY, T, HV, MEM, ABS, AX, EX>, TP, TF, TC>;
#define FDS_PICK_TILE(TX, TY, NT)                                                           \
  if (has_v && !absorb && !axi && !exact && tx == TX && ty == TY) {                         \
    if (acoustic) {                                                                         \
      if constexpr (ALLOW_ACOUSTIC) {                                                       \
        if (stages == 2)                                                                    \
          return &launch_stag<StagCfg<TX, TY, NT, true, true, false, false, false, 2>, TP, TF, \
                              TC>;                                                          \
        return &launch_stag<StagCfg<TX, TY, NT, true, true, false, false, false, 1>, TP, TF, TC>; \
      }                                                                                     \
    } else {                                                                                \
      if (stages == 2)                                                                      \
        return &launch_stag<StagCfg<TX, TY, NT, true, false, false, false, false, 2>, TP, TF,  \
                            TC>;                                                            \
      return &launch_stag<StagCfg<TX, TY, NT, true, false, false, false, false, 1>, TP, TF, TC>; \
    }                                                                                       \
  }
  FDS_TILE_MENU(FDS_PICK_TILE)
#define FDS_PICK_MARCH(CX, TY, NW)                                                        \
  if (has_v && !absorb && !axi && !exact && tx == 32 * CX - 2 && ty == TY && stages == 1) { \
    if (acoustic) {                                                                       \
      if constexpr (ALLOW_ACOUSTIC) return &launch_march<MarchCfg<CX, TY, NW, true>, TP, TF, TC>; \
    } else {                                                                              \
      return &launch_march<MarchCfg<CX, TY, NW, false>, TP, TF, TC>;                      \
    }                                                                                     \
  }
  if constexpr (!std::is_same<TP, dw>::value) {  // register marching shuffles scalars
    FDS_MARCH_MENU(FDS_PICK_MARCH)
  }
#undef FDS_PICK_MARCH
  if constexpr (ALLOW_ACOUSTIC) {
    FDS_PICK(kTile1dX, 1, false, true, false, false, false)
    FDS_PICK(kTile1dX, 1, false, true, true, false, false)
    FDS_PICK(kTile2dX, kTile2dY, true, true, true, false, false)
    FDS_PICK(kTile2dX, kTile2dY, true, true, true, true, false)
    if constexpr (ALLOW_EXACT) {
      FDS_PICK(kTile1dX, 1, false, true, false, false, true)
      FDS_PICK(kTile1dX, 1, false, true, true, false, true)
      FDS_PICK(kTile2dX, kTile2dY, true, true, false, false, true)
      FDS_PICK(kTile2dX, kTile2dY, true, true, true, false, true)
      FDS_PICK(kTile2dX, kTile2dY, true, true, false, true, true)
      FDS_PICK(kTile2dX, kTile2dY, true, true, true, true, true)
    }
  }
  FDS_PICK(kTile1dX, 1, false, false, false, false, false)
  if constexpr (ALLOW_EXACT) {
    FDS_PICK(kTile1dX, 1, false, false, false, false, true)
    FDS_PICK(kTile2dX, kTile2dY, true, false, false, false, true)
    FDS_PICK(kTile2dX, kTile2dY, true, false, false, true, true)
  }
#undef FDS_PICK
#undef FDS_PICK_TILE
  return nullptr;
}

// Every step of a call in persistent wavefront launches (stages 4, stag_wave_kernel).
// Returns FDS_OK, an error code, or kWaveUnsupported when the rows cannot be staged by
// TMA (the caller then steps one launch per step). `base` carries the call's fields.
constexpr int32_t kWaveUnsupported = 1;

template <class C, typename TP, typename TF, typename TC>
int32_t run_wave(const StagArgs<TP, TF, TC>& base, const FdsStagProblem* prob, FdsStagState* st,
                 const FdsStagTables* tabs, int64_t step0, int32_t nsteps, int32_t store_flux,
                 cudaStream_t stream) {
  const bool iso = base.iso != 0;
  const size_t smem = stag_buffer_bytes<C, TP, TF, TC>(iso) + 16;
  LaunchShape ls;
  int32_t rc = kernel_shape<stag_wave_kernel<C, TP, TF, TC>>(smem, C::NT, iso, &ls);
  if (rc != FDS_OK) return rc;
  const int tiles_y = (prob->ny + C::TY - 1) / C::TY;
  if (!tabs->sync || tabs->sync_words < 1 + (int64_t)tiles_y)
    return set_error(FDS_E_ARG, "stages 4 needs FdsStagTables.sync of %d words (has %lld)",
                     1 + tiles_y, (long long)tabs->sync_words);
  StagTmaCache tma;
  tma.state[0] = st->cur[0];
  tma.state[1] = st->nxt[0];
  tma.state[2] = st->cur[1];
  tma.state[3] = st->nxt[1];
  tma.state[4] = st->cur[2];
  tma.state[5] = st->nxt[2];
  StagWaveArgs<TP, TF, TC> w{};
  auto fill = [&](void* const* in, void* const* out, StagArgs<TP, TF, TC>& a) {
    a = base;
    a.p_in = (const TP*)in[0];
    a.p_out = (TP*)out[0];
    a.u_in = (const TF*)in[1];
    a.u_out = (TF*)out[1];
    a.v_in = (const TF*)in[2];
    a.v_out = (TF*)out[2];
    a.substeps = 1;
    select_tma<C>(a, &tma, tma.state);
  };
  fill(st->cur, st->nxt, w.par[0]);
  fill(st->nxt, st->cur, w.par[1]);
  if (!w.par[0].use_tma || !w.par[1].use_tma) return kWaveUnsupported;
  const int ntiles = base.ntiles;
  const int64_t resident = (int64_t)ls.occ * ls.nsm;
  // the item counter (and each row's counter) stays below 2^31
  const int64_t per_launch = (0x7fffffffll - resident) / ntiles;
  if (per_launch < 1) return set_error(FDS_E_SIZE, "grid has too many tiles for stages 4");
  w.sync = tabs->sync;
  w.tiles_y = tiles_y;
  w.flux_all = store_flux;
  // L2 prefetch 0.4 waves of resident CTAs ahead in the queue (measured on the 2048^2
  // float64 step against 0, 1 and 2 waves: 61.8, 63.2 and 60.2 against 64.0 Gcell/s)
  w.prefetch = prefetch_distance(ls);
  // potential bounds and probes of the first step
  const FdsCompTables& t0 = tabs->comp[0];
  if (t0.bound_tile_start || t0.probe_tile_start) {
    stag_prologue_kernel<TP><<<1, 1024, 0, stream>>>((TP*)st->cur[0], t0, tabs->pool, step0,
                                                      ntiles, 0);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(FDS_E_LAUNCH, "prologue launch: %s", cudaGetErrorString(e));
  }
  for (int64_t done = 0; done < nsteps;) {
    const int32_t m = (int32_t)std::min<int64_t>(per_launch, nsteps - done);
    fill(st->cur, st->nxt, w.par[0]);
    fill(st->nxt, st->cur, w.par[1]);
    w.nsteps = m;
    w.step = step0 + done;
    w.more = done + m < nsteps ? 1 : 0;
    const int64_t items = (int64_t)m * ntiles;
    const int grid = (int)std::min<int64_t>(resident, items);
    cudaError_t e = cudaMemsetAsync(tabs->sync, 0, sizeof(uint32_t) * (1 + (size_t)tiles_y), stream);
    if (e != cudaSuccess) return set_error(FDS_E_LAUNCH, "wavefront counters: %s", cudaGetErrorString(e));
    stag_wave_kernel<C, TP, TF, TC><<<grid, C::NT, smem, stream>>>(w);
    e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(FDS_E_LAUNCH, "wavefront launch: %s", cudaGetErrorString(e));
    if (m & 1)
      for (int k = 0; k < 3; ++k) std::swap(st->cur[k], st->nxt[k]);
    done += m;
  }
  return FDS_OK;
}

template <typename TP, typename TF, typename TC>
using WaveRun = int32_t (*)(const StagArgs<TP, TF, TC>&, const FdsStagProblem*, FdsStagState*,
                            const FdsStagTables*, int64_t, int32_t, int32_t, cudaStream_t);

// Wavefront variant of a lossless 2-D non-exact field at a default tile shape.
template <typename TP, typename TF, typename TC, bool ALLOW_ACOUSTIC>
WaveRun<TP, TF, TC> pick_wave(int family, int tx, int ty) {
  const bool acoustic = family == FDS_FAMILY_ACOUSTIC;
#define FDS_PICK_WAVE(TX, TY)                                                                \
  if (tx == TX && ty == TY) {                                                                \
    if (acoustic) {                                                                          \
      if constexpr (ALLOW_ACOUSTIC)                                                          \
        return &run_wave<StagCfg<TX, TY, kThreads, true, true, false, false, false, 1>, TP, TF, TC>; \
    } else {                                                                                 \
      return &run_wave<StagCfg<TX, TY, kThreads, true, false, false, false, false, 1>, TP, TF, TC>; \
    }                                                                                        \
  }
  FDS_PICK_WAVE(64, 16)
  FDS_PICK_WAVE(64, 12)
#undef FDS_PICK_WAVE
  return nullptr;
}

// Every step of a call of a 1-D field in one CTA (stag_1d_resident_kernel): the
// first step's potential bounds and probes in the prologue, then one launch.
template <class C, typename TP, typename TF, typename TC>
int32_t run_resident(StagArgs<TP, TF, TC>& a, FdsStagState* st, const FdsStagTables* tabs,
                     int64_t step0, int32_t nsteps, cudaStream_t stream, int) {
  const int n = (int)a.n;
  // state and coefficients, the table area, and the signal pool when it fits
  size_t smem = resident_smem<TP, TF, TC>(n) + kResidentTableBytes;
  int64_t pool_cached = 0;
  if (tabs->pool && tabs->pool_len > 0 &&
      smem + (size_t)tabs->pool_len * sizeof(double) <= kResidentMaxSmem) {
    pool_cached = tabs->pool_len;
    smem += (size_t)pool_cached * sizeof(double);
  }
  LaunchShape ls;
  const int32_t rc =
      kernel_shape<stag_1d_resident_kernel<C, TP, TF, TC>>(smem, kResidentThreads, false, &ls);
  if (rc != FDS_OK) return rc;
  const FdsCompTables& t0 = tabs->comp[0];
  if (t0.bound_tile_start || t0.probe_tile_start) {
    stag_prologue_kernel<TP><<<1, 1024, 0, stream>>>((TP*)st->cur[0], t0, tabs->pool, step0,
                                                      a.ntiles, 0);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(FDS_E_LAUNCH, "prologue launch: %s", cudaGetErrorString(e));
  }
  a.p_in = (const TP*)st->cur[0];
  a.u_in = (const TF*)st->cur[1];
  a.step = step0;
  // the state ends where nsteps ping-pong swaps leave it
  const bool odd = (nsteps & 1) != 0;
  TP* p_fin = (TP*)(odd ? st->nxt[0] : st->cur[0]);
  TF* u_fin = (TF*)(odd ? st->nxt[1] : st->cur[1]);
  stag_1d_resident_kernel<C, TP, TF, TC><<<1, kResidentThreads, smem, stream>>>(
      a, nsteps, p_fin, u_fin, pool_cached);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(FDS_E_LAUNCH, "1-D launch: %s", cudaGetErrorString(e));
  if (odd)
    for (int k = 0; k < 3; ++k) std::swap(st->cur[k], st->nxt[k]);
  return FDS_OK;
}

// Whether the device schedules one cluster of `ctas` CTAs of `kernel` (beyond the
// portable size: the non-portable size is allowed first) with `threads` threads and
// `smem` bytes of dynamic shared memory.
template <typename Kernel>
bool cluster_fits(Kernel kernel, int ctas, int threads, size_t smem) {
  if (ctas <= kClusterPortableCta) return true;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)ctas;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3((unsigned)ctas, 1, 1);
  cfg.blockDim = dim3((unsigned)threads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int clusters = 0;
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
          cudaSuccess ||
      cudaOccupancyMaxActiveClusters(&clusters, kernel, &cfg) != cudaSuccess || clusters < 1) {
    (void)cudaGetLastError();
    return false;
  }
  return true;
}

// The first step's potential bounds and probes of a resident 1-D run, and the state
// pointers and step of its launch; returns FDS_OK or an error code.
template <typename TP, typename TF, typename TC>
int32_t resident_prologue(StagArgs<TP, TF, TC>& a, FdsStagState* st, const FdsStagTables* tabs,
                          int64_t step0, cudaStream_t stream) {
  const FdsCompTables& t0 = tabs->comp[0];
  if (t0.bound_tile_start || t0.probe_tile_start) {
    stag_prologue_kernel<TP><<<1, 1024, 0, stream>>>((TP*)st->cur[0], t0, tabs->pool, step0,
                                                      a.ntiles, 0);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(FDS_E_LAUNCH, "prologue launch: %s", cudaGetErrorString(e));
  }
  a.p_in = (const TP*)st->cur[0];
  a.u_in = (const TF*)st->cur[1];
  a.step = step0;
  return FDS_OK;
}

// One launch of `kernel` as a single cluster of `ctas` CTAs.
template <typename... Params, typename... Args>
cudaError_t launch_cluster(void (*kernel)(Params...), int ctas, int threads, size_t smem,
                           cudaStream_t stream, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)ctas;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3((unsigned)ctas, 1, 1);
  cfg.blockDim = dim3((unsigned)threads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// Every step of a call of a 1-D field on the warps of one cluster of up to `max_ctas`
// CTAs (stag_1d_warp_kernel, K steps per exchange block): the prologue, then one
// cluster launch; kWaveUnsupported where the field needs more warps than that.
template <class C, typename TP, typename TF, typename TC>
int32_t run_warp1d(StagArgs<TP, TF, TC>& a, FdsStagState* st, const FdsStagTables* tabs,
                   int64_t step0, int32_t nsteps, cudaStream_t stream, int max_ctas, int want_k) {
  const int n = (int)a.n;
  const int K = std::min(kWarpMaxBlockSteps,
                         std::max(1, want_k > 0 ? want_k : kWarpDefaultBlockSteps));
  const int m = warp_owned_cells(K);
  const int nw = (n + m - 1) / m;  // warps with cells
  const auto kernel = stag_1d_warp_kernel<C, TP, TF, TC>;
  int ncta = 0, nwc = 0;
  size_t smem = 0;
  int64_t pool_cached = 0;
  auto shape = [&](int ctas) {
    ncta = std::min(ctas, nw);
    nwc = (nw + ncta - 1) / ncta;
    ncta = (nw + nwc - 1) / nwc;
    smem = warp_inbox_bytes<TP, TF>(nwc, K + 1) +
           warp_slot_bytes((nwc - 1) * m + kWarpLanes) + kResidentTableBytes;
    pool_cached = 0;
    if (tabs->pool && tabs->pool_len > 0 &&
        smem + (size_t)tabs->pool_len * sizeof(double) <= kResidentMaxSmem) {
      pool_cached = tabs->pool_len;
      smem += (size_t)pool_cached * sizeof(double);
    }
    return nwc <= kWarpMaxPerCta && smem <= kResidentMaxSmem;
  };
  if (!shape(max_ctas)) return kWaveUnsupported;
  LaunchShape ls;
  int32_t rc = kernel_shape<stag_1d_warp_kernel<C, TP, TF, TC>>(smem, nwc * 32, false, &ls);
  if (rc != FDS_OK) return rc;
  if (!cluster_fits(kernel, ncta, nwc * 32, smem)) {
    if (!shape(std::min(max_ctas, kClusterPortableCta))) return kWaveUnsupported;
    rc = kernel_shape<stag_1d_warp_kernel<C, TP, TF, TC>>(smem, nwc * 32, false, &ls);
    if (rc != FDS_OK) return rc;
  }
  rc = resident_prologue(a, st, tabs, step0, stream);
  if (rc != FDS_OK) return rc;
  const bool odd = (nsteps & 1) != 0;  // the state ends where nsteps swaps leave it
  TP* p_fin = (TP*)(odd ? st->nxt[0] : st->cur[0]);
  TF* u_fin = (TF*)(odd ? st->nxt[1] : st->cur[1]);
  const cudaError_t e = launch_cluster(kernel, ncta, nwc * 32, smem, stream, a, nsteps, p_fin,
                                       u_fin, pool_cached, (int32_t)K);
  if (e != cudaSuccess) return set_error(FDS_E_LAUNCH, "1-D warp launch: %s", cudaGetErrorString(e));
  if (odd)
    for (int k = 0; k < 3; ++k) std::swap(st->cur[k], st->nxt[k]);
  return FDS_OK;
}

// Every step of a call of a 1-D field on one thread-block cluster of up to `ncta` CTAs:
// on warps with one cell per lane (stag_1d_warp_kernel) where the field fits them, else
// on shared-memory windows (stag_1d_cluster_kernel), halo cells exchanged once per block
// of K steps either way. Tuning overrides: FDS_CLUSTER_CTAS caps the cluster size,
// FDS_CLUSTER_BLOCK_STEPS sets K, FDS_1D_KERNEL=window selects the window kernel.
template <class C, typename TP, typename TF, typename TC>
int32_t run_cluster(StagArgs<TP, TF, TC>& a, FdsStagState* st, const FdsStagTables* tabs,
                    int64_t step0, int32_t nsteps, cudaStream_t stream, int ncta) {
  const int n = (int)a.n;
  const char* env_ctas = std::getenv("FDS_CLUSTER_CTAS");
  const char* env_steps = std::getenv("FDS_CLUSTER_BLOCK_STEPS");
  const char* env_kernel = std::getenv("FDS_1D_KERNEL");
  const int want_k = env_steps ? std::atoi(env_steps) : 0;
  int max_ctas = kClusterMaxCta;
  if (env_ctas && std::atoi(env_ctas) >= 2) max_ctas = std::min(max_ctas, std::atoi(env_ctas));
  ncta = std::min(ncta, max_ctas);
  if (!(env_kernel && std::strcmp(env_kernel, "window") == 0)) {
    const int32_t rw = run_warp1d<C>(a, st, tabs, step0, nsteps, stream, max_ctas, want_k);
    if (rw != kWaveUnsupported) return rw;
  }
  const auto kernel = stag_1d_cluster_kernel<C, TP, TF, TC>;
  int m = 0, K = 0;
  size_t smem = 0;
  int64_t pool_cached = 0;
  auto shape = [&](int ctas) {
    m = (n + ctas - 1) / ctas;
    K = cluster_block_steps(m, want_k);
    smem = cluster_inbox_bytes<TP, TF>(K + 1) + cluster_window_bytes<TP, TF, TC>(m + 2 * (K + 1)) +
           kResidentTableBytes;
    pool_cached = 0;
    if (tabs->pool && tabs->pool_len > 0 &&
        smem + (size_t)tabs->pool_len * sizeof(double) <= kResidentMaxSmem) {
      pool_cached = tabs->pool_len;
      smem += (size_t)pool_cached * sizeof(double);
    }
    return (n + m - 1) / m;  // every CTA owns at least one cell
  };
  ncta = shape(ncta);
  LaunchShape ls;
  int32_t rc = kernel_shape<stag_1d_cluster_kernel<C, TP, TF, TC>>(smem, kClusterThreads, false, &ls);
  if (rc != FDS_OK) return rc;
  if (!cluster_fits(kernel, ncta, kClusterThreads, smem)) {
    ncta = shape(kClusterPortableCta);
    rc = kernel_shape<stag_1d_cluster_kernel<C, TP, TF, TC>>(smem, kClusterThreads, false, &ls);
    if (rc != FDS_OK) return rc;
  }
  rc = resident_prologue(a, st, tabs, step0, stream);
  if (rc != FDS_OK) return rc;
  const bool odd = (nsteps & 1) != 0;
  TP* p_fin = (TP*)(odd ? st->nxt[0] : st->cur[0]);
  TF* u_fin = (TF*)(odd ? st->nxt[1] : st->cur[1]);
  const cudaError_t e = launch_cluster(kernel, ncta, kClusterThreads, smem, stream, a, nsteps,
                                       p_fin, u_fin, pool_cached, (int32_t)m, (int32_t)K);
  if (e != cudaSuccess) return set_error(FDS_E_LAUNCH, "1-D cluster launch: %s", cudaGetErrorString(e));
  if (odd)
    for (int k = 0; k < 3; ++k) std::swap(st->cur[k], st->nxt[k]);
  return FDS_OK;
}

// Cells per CTA below which a 1-D field stays in one CTA (a cluster of CTAs of at
// least this many cells each otherwise, up to kClusterMaxCta)
constexpr int kClusterMinCellsPerCta = 64;
constexpr int kClusterMinCells = 256;

// A 1-D field of n cells: in one cluster (ncta > 1), in one CTA (ncta == 1), or not
// resident at all (0, one launch per step).
template <typename TP, typename TF, typename TC>
int resident_ctas(int64_t n) {
  // (up to the cells that the portable cluster size holds: run_cluster falls back to
  // it where the device refuses a larger cluster)
  if (n >= kClusterMinCells && n <= (int64_t)kClusterPortableCta * kClusterMaxCellsPerCta) {
    const int ncta = (int)std::min<int64_t>(kClusterMaxCta,
                                            (n + kClusterMinCellsPerCta - 1) / kClusterMinCellsPerCta);
    const int m = (int)((n + kClusterPortableCta - 1) / kClusterPortableCta);  // the largest
    const int g = cluster_block_steps(m, kClusterWindow) + 1;  // the widest window edge
    if (cluster_inbox_bytes<TP, TF>(g) + cluster_window_bytes<TP, TF, TC>(m + 2 * g) +
            kResidentTableBytes <=
        kResidentMaxSmem)
      return ncta;
  }
  if (n <= kResidentMaxCells && resident_smem<TP, TF, TC>((int)n) + kResidentTableBytes <= kResidentMaxSmem)
    return 1;
  return 0;
}

template <typename TP, typename TF, typename TC>
using ResidentRun = int32_t (*)(StagArgs<TP, TF, TC>&, FdsStagState*, const FdsStagTables*,
                                int64_t, int32_t, cudaStream_t, int);

template <typename TP, typename TF, typename TC, bool ALLOW_EXACT, bool ALLOW_ACOUSTIC>
ResidentRun<TP, TF, TC> pick_resident(int family, bool absorb, bool exact, bool cluster) {
  if (exact && !ALLOW_EXACT) return nullptr;
  const bool acoustic = family == FDS_FAMILY_ACOUSTIC;
#define FDS_PICK_RES(MEM, ABS, EX)                                                          \
  if (acoustic == MEM && absorb == ABS && exact == EX)                                      \
    return cluster ? &run_cluster<StagCfg<kTile1dX, 1, kThreads, false, MEM, ABS, false, EX>, TP, TF, TC> \
                   : &run_resident<StagCfg<kTile1dX, 1, kThreads, false, MEM, ABS, false, EX>, TP, TF, TC>;
  if constexpr (ALLOW_ACOUSTIC) {
    FDS_PICK_RES(true, false, false)
    FDS_PICK_RES(true, true, false)
    if constexpr (ALLOW_EXACT) {
      FDS_PICK_RES(true, false, true)
      FDS_PICK_RES(true, true, true)
    }
  }
  FDS_PICK_RES(false, false, false)
  if constexpr (ALLOW_EXACT) FDS_PICK_RES(false, false, true)
#undef FDS_PICK_RES
  return nullptr;
}

template <typename TP, typename TF, typename TC, bool ALLOW_EXACT, bool ALLOW_ACOUSTIC>
int32_t run_stag_typed(const FdsStagProblem* prob, FdsStagState* st, const FdsStagTables* tabs,
                       int64_t step0, int32_t nsteps, int32_t store_flux, cudaStream_t stream) {
  const bool has_v = (prob->flags & FDS_FLAG_HAS_V) != 0;
  const bool absorb = (prob->flags & FDS_FLAG_ABSORB) != 0;
  const bool axi = (prob->flags & FDS_FLAG_AXI) != 0;
  const bool exact = (prob->flags & FDS_FLAG_EXACT) != 0;
  const bool flow = (prob->flags & FDS_FLAG_FLOW) != 0;
  // stages: 0 (automatic) and 1 = one CTA per tile; 2 = the persistent two-stage
  // pipeline (built for the tile menu; measured slower on GB300 for one field);
  // 3 = two steps per tile and launch (stag_tb2_kernel; the host picks it)
  StagLaunch<TP, TF, TC> fn = nullptr;
  const bool two_step = prob->stages == 3;
  if (two_step) {
    if (flow) return set_error(FDS_E_ARG, "two steps per tile do not cover a moving medium");
    fn = pick_stag<TP, TF, TC, ALLOW_EXACT, ALLOW_ACOUSTIC>(prob->family, has_v, absorb, axi,
                                                            exact, prob->tile_x, prob->tile_y, 3);
  } else if (prob->stages == 2)
    fn = pick_stag<TP, TF, TC, ALLOW_EXACT, ALLOW_ACOUSTIC>(prob->family, has_v, absorb, axi,
                                                            exact, prob->tile_x, prob->tile_y, 2);
  // a two-step request never falls back: its tables are built for slot layout 2
  if (!fn && prob->stages != 2 && !two_step)
    fn = pick_stag<TP, TF, TC, ALLOW_EXACT, ALLOW_ACOUSTIC>(prob->family, has_v, absorb, axi,
                                                            exact, prob->tile_x, prob->tile_y, 1);
  if (!fn)
    return set_error(FDS_E_NOKERNEL,
                     "no kernel built for family=%d precision=%d flags=%u tile=%dx%d stages=%d",
                     prob->family, prob->precision, prob->flags, prob->tile_x, prob->tile_y,
                     prob->stages);
  const int tiles_x = (prob->nx + prob->tile_x - 1) / prob->tile_x;
  const int tiles_y = (prob->ny + prob->tile_y - 1) / prob->tile_y;
  const int64_t ntiles64 = (int64_t)tiles_x * tiles_y;
  if (ntiles64 > 0x7fffffff) return set_error(FDS_E_SIZE, "grid has too many tiles");
  const int ntiles = (int)ntiles64;

  StagArgs<TP, TF, TC> a{};
  a.nx = prob->nx;
  a.ny = prob->ny;
  a.n = (int64_t)prob->nx * prob->ny;
  a.tiles_x = tiles_x;
  tile_divider(tiles_x, &a.tx_mul, &a.tx_shift);
  a.ntiles = ntiles;
  const FdsCoefs& c = prob->coefs;
  a.bx = (const TC*)c.bx;
  a.by = (const TC*)(c.by ? c.by : c.bx);
  a.kx = (const TC*)c.kx;
  a.ky = (const TC*)(c.ky ? c.ky : c.kx);
  a.aym = (const TC*)c.aym;
  a.axm = (const TC*)c.axm;
  a.ad = (const TC*)c.ad;
  a.axp = (const TC*)c.axp;
  a.ayp = (const TC*)c.ayp;
  a.ex = (const TC*)c.ex;
  a.rx = (const TC*)c.rx;
  a.iso = (a.by == a.bx && a.ky == a.kx) ? 1 : 0;
  a.offset = prob->offset;
  for (int k = 0; k < 3; ++k) a.tab[k] = tabs->comp[k];
  a.pool = tabs->pool;
  a.status = tabs->status;
  a.step0 = step0;
  StagTmaCache tma;
  tma.state[0] = st->cur[0];
  tma.state[1] = st->nxt[0];
  tma.state[2] = st->cur[1];
  tma.state[3] = st->nxt[1];
  tma.state[4] = st->cur[2];
  tma.state[5] = st->nxt[2];

  // a 1-D field that fits shared memory: every step in one launch, on a cluster of
  // CTAs from 256 cells on, else on one CTA (stages 0 or 4, calls of two steps or more;
  // stages 1 keeps one launch per step, and a single step is a tile-kernel launch)
  if (!has_v && !flow && (prob->stages == 0 || prob->stages == 4) && nsteps > 1) {
    const int ncta = resident_ctas<TP, TF, TC>(a.n);
    ResidentRun<TP, TF, TC> rr =
        ncta > 0 ? pick_resident<TP, TF, TC, ALLOW_EXACT, ALLOW_ACOUSTIC>(prob->family, absorb,
                                                                           exact, ncta > 1)
                 : nullptr;
    if (rr) return rr(a, st, tabs, step0, nsteps, stream, ncta);
  }
  if (prob->stages == 4 && has_v && !absorb && !exact && !flow) {
    WaveRun<TP, TF, TC> wr =
        pick_wave<TP, TF, TC, ALLOW_ACOUSTIC>(prob->family, prob->tile_x, prob->tile_y);
    if (wr) {
      const int32_t rw = wr(a, prob, st, tabs, step0, nsteps, store_flux, stream);
      if (rw != kWaveUnsupported) return rw;
    }
  }

  // potential bounds and probes of the first step
  const FdsCompTables& t0 = tabs->comp[0];
  if (nsteps > 0 && (t0.bound_tile_start || t0.probe_tile_start)) {
    stag_prologue_kernel<TP><<<1, 1024, 0, stream>>>((TP*)st->cur[0], t0, tabs->pool, step0,
                                                      ntiles, 0);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(FDS_E_LAUNCH, "prologue launch: %s", cudaGetErrorString(e));
  }
  // a moving medium with a host copy of its shift periods: steps on which no row is
  // due need neither the shift launch nor the prologue after it (the periods that
  // occur, deduplicated; numpy's step % f == 0, f == 0 always due)
  std::vector<int64_t> periods;
  if (flow && prob->flow_period_host) {
    periods.assign(prob->flow_period_host, prob->flow_period_host + prob->ny);
    std::sort(periods.begin(), periods.end());
    periods.erase(std::unique(periods.begin(), periods.end()), periods.end());
  }
  auto shift_due = [&](int64_t step) {
    if (!flow) return false;
    if (!prob->flow_period_host) return true;
    for (const int64_t f : periods)
      if (f == 0 || step % f == 0) return true;
    return false;
  };
  for (int32_t s = 0; s < nsteps;) {
    // the two-step kernel advances two steps per launch (one for an odd last step)
    const int take = (two_step && s + 1 < nsteps) ? 2 : 1;
    a.substeps = take;
    a.p_in = (const TP*)st->cur[0];
    a.p_out = (TP*)st->nxt[0];
    a.u_in = (const TF*)st->cur[1];
    a.u_out = (TF*)st->nxt[1];
    a.v_in = (const TF*)st->cur[2];
    a.v_out = (TF*)st->nxt[2];
    a.step = step0 + s;
    // a moving medium shifts rows between the pressure update and the next step's
    // pressure bounds / probes, which then run in the prologue kernel instead
    const bool due = shift_due(step0 + s);
    a.apply_next = (s + take < nsteps && !due) ? 1 : 0;
    a.store_flux = (store_flux || s + take == nsteps) ? 1 : 0;
    const int32_t rc = fn(a, stream, &tma);
    if (rc != FDS_OK) return rc;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(FDS_E_LAUNCH, "step launch: %s", cudaGetErrorString(e));
    for (int k = 0; k < 3; ++k) std::swap(st->cur[k], st->nxt[k]);
    if (due) {
      const int32_t rf = launch_flow_shift(prob, st->cur, step0 + s, stream);
      if (rf != FDS_OK) return rf;
      if (s + 1 < nsteps && (t0.bound_tile_start || t0.probe_tile_start)) {
        stag_prologue_kernel<TP><<<1, 1024, 0, stream>>>((TP*)st->cur[0], t0, tabs->pool,
                                                          step0 + s + 1, ntiles, s + 1);
        e = cudaGetLastError();
        if (e != cudaSuccess)
          return set_error(FDS_E_LAUNCH, "prologue launch: %s", cudaGetErrorString(e));
      }
    }
    s += take;
  }
  return FDS_OK;
}


// ------------------------------------------------------------------ batched path

inline size_t batch_desc_bytes(size_t desc_size, int32_t count) {
  return (2 * (size_t)count * desc_size + 255) / 256 * 256;
}

// Build the descriptors and work list of one batched call for kernel variant C,
// upload them into the caller's workspace and run the steps.
template <class C, typename TP, typename TF, typename TC>
int32_t batch_run_variant(const FdsStagProblem* probs, FdsStagState* states,
                          const FdsStagTables* tables, int32_t count, void* workspace,
                          size_t workspace_bytes, int64_t step0, int32_t nsteps,
                          int32_t store_flux, uint32_t mode, cudaStream_t stream) {
  using Args = StagArgs<TP, TF, TC>;
  const size_t dbytes = batch_desc_bytes(sizeof(Args), count);
  int64_t nwork = 0;
  for (int i = 0; i < count; ++i) {
    const int tx = (probs[i].nx + C::TX - 1) / C::TX, ty = (probs[i].ny + C::TY - 1) / C::TY;
    nwork += (int64_t)tx * ty;
  }
  if (nwork > 0x7fffffff) return set_error(FDS_E_SIZE, "too many tiles in the batch");
  if (dbytes + (size_t)nwork * sizeof(int2) > workspace_bytes)
    return set_error(FDS_E_SIZE, "workspace holds %zu bytes, batch needs %zu", workspace_bytes,
                     dbytes + (size_t)nwork * sizeof(int2));
  Args* d_desc = (Args*)workspace;
  int2* d_work = (int2*)((char*)workspace + dbytes);
  cudaError_t e = cudaSuccess;
  if (mode & FDS_BATCH_UPLOAD) {
  std::vector<Args> desc(2 * (size_t)count);
  std::vector<int2> work;
  work.reserve((size_t)nwork);
  for (int i = 0; i < count; ++i) {
    const FdsStagProblem& pr = probs[i];
    const FdsCoefs& c = pr.coefs;
    const FdsStagState& st = states[i];
    Args base{};
    base.nx = pr.nx;
    base.ny = pr.ny;
    base.n = (int64_t)pr.nx * pr.ny;
    base.tiles_x = (pr.nx + C::TX - 1) / C::TX;
    tile_divider(base.tiles_x, &base.tx_mul, &base.tx_shift);
    base.ntiles = base.tiles_x * ((pr.ny + C::TY - 1) / C::TY);
    base.bx = (const TC*)c.bx;
    base.by = (const TC*)(c.by ? c.by : c.bx);
    base.kx = (const TC*)c.kx;
    base.ky = (const TC*)(c.ky ? c.ky : c.kx);
    base.rx = (const TC*)c.rx;
    base.iso = (base.by == base.bx && base.ky == base.kx) ? 1 : 0;
    base.offset = pr.offset;
    for (int k = 0; k < 3; ++k) base.tab[k] = tables[i].comp[k];
    base.pool = tables[i].pool;
    base.status = tables[i].status;
    bool tma = encode_tile_map(&base.tm[3], base.bx, sizeof(TC), pr.nx, pr.ny, C::RX, C::RY) &&
               encode_tile_map(&base.tm[4], base.kx, sizeof(TC), pr.nx, pr.ny, C::RX, C::RY) &&
               encode_tile_map(&base.tm[5], base.by, sizeof(TC), pr.nx, pr.ny, C::RX, C::RY) &&
               encode_tile_map(&base.tm[6], base.ky, sizeof(TC), pr.nx, pr.ny, C::RX, C::RY);
    for (int par = 0; par < 2; ++par) {
      Args d = base;
      void* const* in = par ? st.nxt : st.cur;
      void* const* out = par ? st.cur : st.nxt;
      d.p_in = (const TP*)in[0];
      d.p_out = (TP*)out[0];
      d.u_in = (const TF*)in[1];
      d.u_out = (TF*)out[1];
      d.v_in = (const TF*)in[2];
      d.v_out = (TF*)out[2];
      bool t = tma && encode_tile_map(&d.tm[0], in[0], sizeof(TP), pr.nx, pr.ny, C::RX, C::RY);
      if (C::MEMORY)
        t = t && encode_tile_map(&d.tm[1], in[1], sizeof(TF), pr.nx, pr.ny, C::RX, C::RY) &&
            encode_tile_map(&d.tm[2], in[2], sizeof(TF), pr.nx, pr.ny, C::RX, C::RY);
      d.use_tma = t ? 1 : 0;
      desc[2 * (size_t)i + par] = d;
    }
    for (int t = 0; t < base.ntiles; ++t) work.push_back(make_int2(i, t));
  }
  e = cudaMemcpyAsync(d_desc, desc.data(), desc.size() * sizeof(Args), cudaMemcpyHostToDevice,
                      stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_work, work.data(), work.size() * sizeof(int2), cudaMemcpyHostToDevice,
                        stream);
  if (e != cudaSuccess) return set_error(FDS_E_LAUNCH, "descriptor upload: %s", cudaGetErrorString(e));
  }
  if (!(mode & FDS_BATCH_LAUNCH)) return FDS_OK;

  // launch configuration: staging sized for the isotropic layout when every
  // instance is isotropic (by == bx and ky == kx, as the descriptors record it)
  bool all_iso = true;
  for (int i = 0; i < count; ++i) {
    const FdsCoefs& c = probs[i].coefs;
    const void* by = c.by ? c.by : c.bx;
    const void* ky = c.ky ? c.ky : c.kx;
    all_iso = all_iso && by == c.bx && ky == c.kx;
  }
  const size_t smem = batch_smem_bytes<C, TP, TF, TC>(all_iso);
  LaunchShape ls;
  const int32_t rs = kernel_shape<stag_batch_kernel<C, TP, TF, TC>>(smem, C::NT, all_iso, &ls);
  if (rs != FDS_OK) return rs;
  int grid = (int)nwork;
  if (C::STAGES > 1) grid = (int)std::min<int64_t>(nwork, (int64_t)ls.occ * ls.nsm);
  // one-stage: prefetch the work item 0.4 waves of resident CTAs ahead (as the
  // single-field kernel)
  const int prefetch = C::STAGES == 1 ? prefetch_distance(ls) : 0;
  if (nsteps > 0) {
    stag_batch_prologue_kernel<TP, TF, TC><<<count, 256, 0, stream>>>(d_desc, count, step0);
    e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(FDS_E_LAUNCH, "batch prologue: %s", cudaGetErrorString(e));
  }
  // one step per launch, or for a two-step configuration n2 launches of two steps
  // then n1 of one, with n2 + n1 even whenever nsteps >= 2 (a captured run then ends
  // with the ping-pong buffers where it started); the parity follows the launches
  int32_t n2 = C::TWO_STEP ? nsteps / 2 : 0;
  int32_t n1 = nsteps - 2 * n2;
  if (((n2 + n1) & 1) && n2 > 0) {
    --n2;
    n1 += 2;
  }
  int32_t launches = 0;
  for (int32_t s = 0; s < nsteps; ++launches) {
    const int take = launches < n2 ? 2 : 1;
    const StepInfo si{step0 + s, step0, (s + take < nsteps) ? 1 : 0,
                      (store_flux || s + take == nsteps) ? 1 : 0, take};
    stag_batch_kernel<C, TP, TF, TC><<<grid, C::NT, smem, stream>>>(d_desc, d_work, (int)nwork, si,
                                                                    launches & 1, prefetch,
                                                                    all_iso ? 1 : 0);
    e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(FDS_E_LAUNCH, "batch step: %s", cudaGetErrorString(e));
    s += take;
  }
  if (launches & 1)
    for (int i = 0; i < count; ++i)
      for (int k = 0; k < 3; ++k) std::swap(states[i].cur[k], states[i].nxt[k]);
  return FDS_OK;
}

template <typename TP, typename TF, typename TC, bool ALLOW_ACOUSTIC>
int32_t run_batch_typed(const FdsStagProblem* probs, FdsStagState* states,
                        const FdsStagTables* tables, int32_t count, void* workspace,
                        size_t workspace_bytes, int64_t step0, int32_t nsteps, int32_t store_flux,
                        uint32_t mode, cudaStream_t stream) {
  const FdsStagProblem& p0 = probs[0];
  const bool acoustic = p0.family == FDS_FAMILY_ACOUSTIC;
  const int stages = p0.stages == 2 ? 2 : 1;
  if (p0.stages == 3) {
    // two steps per tile: potential and fluxes of one type
    if constexpr (sizeof(TP) == sizeof(TF)) {
#define FDS_BATCH_TB2(TX, TY, NT)                                                                \
  if (p0.tile_x == TX && p0.tile_y == TY) {                                                      \
    if (acoustic) {                                                                              \
      if constexpr (ALLOW_ACOUSTIC)                                                              \
        return batch_run_variant<Tb2Cfg<TX, TY, NT, true>, TP, TF, TC>(                          \
            probs, states, tables, count, workspace, workspace_bytes, step0, nsteps, store_flux, \
            mode, stream);                                                                       \
    } else {                                                                                     \
      return batch_run_variant<Tb2Cfg<TX, TY, NT, false>, TP, TF, TC>(                           \
          probs, states, tables, count, workspace, workspace_bytes, step0, nsteps, store_flux,   \
          mode, stream);                                                                         \
    }                                                                                            \
  }
      FDS_TB2_MENU(FDS_BATCH_TB2)
#undef FDS_BATCH_TB2
    }
    return set_error(FDS_E_NOKERNEL, "no two-step batched kernel for family=%d tile=%dx%d",
                     p0.family, p0.tile_x, p0.tile_y);
  }
#define FDS_BATCH_TILE(TX, TY, NT)                                                              \
  if (p0.tile_x == TX && p0.tile_y == TY) {                                                     \
    if (acoustic) {                                                                             \
      if constexpr (ALLOW_ACOUSTIC) {                                                           \
        if (stages == 2)                                                                        \
          return batch_run_variant<StagCfg<TX, TY, NT, true, true, false, false, false, 2>, TP, \
                                   TF, TC>(probs, states, tables, count, workspace,             \
                                           workspace_bytes, step0, nsteps, store_flux, mode,     \
                                           stream);                                              \
        return batch_run_variant<StagCfg<TX, TY, NT, true, true, false, false, false, 1>, TP,   \
                                 TF, TC>(probs, states, tables, count, workspace,               \
                                         workspace_bytes, step0, nsteps, store_flux, mode,       \
                                         stream);                                                \
      }                                                                                         \
    } else {                                                                                    \
      if (stages == 2)                                                                          \
        return batch_run_variant<StagCfg<TX, TY, NT, true, false, false, false, false, 2>, TP,  \
                                 TF, TC>(probs, states, tables, count, workspace,               \
                                         workspace_bytes, step0, nsteps, store_flux, mode,       \
                                         stream);                                                \
      return batch_run_variant<StagCfg<TX, TY, NT, true, false, false, false, false, 1>, TP,    \
                               TF, TC>(probs, states, tables, count, workspace,                 \
                                       workspace_bytes, step0, nsteps, store_flux, mode,         \
                                       stream);                                                  \
    }                                                                                           \
  }
  FDS_TILE_MENU(FDS_BATCH_TILE)
#undef FDS_BATCH_TILE
  return set_error(FDS_E_NOKERNEL, "no batched kernel for family=%d tile=%dx%d", p0.family,
                   p0.tile_x, p0.tile_y);
}
}  // namespace fds
