// Step loop and variant dispatch of the fused staggered-grid kernel, for one
// precision (included by one translation unit per precision).
#pragma once

#include <cstdio>
#include <utility>

#include "fds_internal.h"
#include "march_kernel.cuh"
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

// Launch one step. STAGES == 1: one CTA per tile. STAGES == 2: persistent CTAs,
// as many as fit on the device at this variant's occupancy.
template <class C, typename TP, typename TF, typename TC>
int32_t launch_stag(StagArgs<TP, TF, TC>& a, cudaStream_t s, StagTmaCache* tc) {
  const bool iso = a.iso != 0 || !C::HAS_V;
  // the TMA barriers (8 bytes per stage) follow the buffers
  const size_t smem = (size_t)C::STAGES * stag_buffer_bytes<C, TP, TF, TC>(iso) + 16 * C::STAGES;
  static int optin = -1, nsm = -1;
  static size_t attr_bytes = 0;
  static int occ[2] = {-1, -1};
  if (optin < 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  }
  if (smem > (size_t)optin)
    return set_error(FDS_E_SIZE, "tile %dx%d with %d stages needs %zu bytes of shared memory "
                     "(device allows %d)", C::TX, C::TY, C::STAGES, smem, optin);
  if (smem > attr_bytes) {
    cudaError_t e = cudaFuncSetAttribute(stag_step_kernel<C, TP, TF, TC>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return set_error(FDS_E_LAUNCH, "smem attribute: %s", cudaGetErrorString(e));
    attr_bytes = smem;
  }
  select_tma<C>(a, tc, tc ? tc->state : nullptr);
  int grid = a.ntiles;
  if (C::STAGES > 1) {
    int& o = occ[iso ? 1 : 0];
    if (o < 0) {
      cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &o, stag_step_kernel<C, TP, TF, TC>, C::NT, smem);
      if (e != cudaSuccess || o < 1) o = 1;
    }
    grid = a.ntiles < o * nsm ? a.ntiles : o * nsm;
  }
  stag_step_kernel<C, TP, TF, TC><<<grid, C::NT, smem, s>>>(a);
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
  FDS_MARCH_MENU(FDS_PICK_MARCH)
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

template <typename TP, typename TF, typename TC, bool ALLOW_EXACT, bool ALLOW_ACOUSTIC>
int32_t run_stag_typed(const FdsStagProblem* prob, FdsStagState* st, const FdsStagTables* tabs,
                       int64_t step0, int32_t nsteps, int32_t store_flux, cudaStream_t stream) {
  const bool has_v = (prob->flags & FDS_FLAG_HAS_V) != 0;
  const bool absorb = (prob->flags & FDS_FLAG_ABSORB) != 0;
  const bool axi = (prob->flags & FDS_FLAG_AXI) != 0;
  const bool exact = (prob->flags & FDS_FLAG_EXACT) != 0;
  // stages: 0 = two-stage persistent pipeline where it is built, else one stage
  StagLaunch<TP, TF, TC> fn = nullptr;
  if (prob->stages == 0 || prob->stages == 2)
    fn = pick_stag<TP, TF, TC, ALLOW_EXACT, ALLOW_ACOUSTIC>(prob->family, has_v, absorb, axi,
                                                            exact, prob->tile_x, prob->tile_y, 2);
  if (!fn && prob->stages != 2)
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

  // potential bounds and probes of the first step
  const FdsCompTables& t0 = tabs->comp[0];
  if (nsteps > 0 && (t0.bound_tile_start || t0.probe_tile_start)) {
    stag_prologue_kernel<TP><<<1, 1024, 0, stream>>>((TP*)st->cur[0], t0, tabs->pool, step0,
                                                      ntiles);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(FDS_E_LAUNCH, "prologue launch: %s", cudaGetErrorString(e));
  }
  for (int32_t s = 0; s < nsteps; ++s) {
    a.p_in = (const TP*)st->cur[0];
    a.p_out = (TP*)st->nxt[0];
    a.u_in = (const TF*)st->cur[1];
    a.u_out = (TF*)st->nxt[1];
    a.v_in = (const TF*)st->cur[2];
    a.v_out = (TF*)st->nxt[2];
    a.step = step0 + s;
    a.apply_next = (s + 1 < nsteps) ? 1 : 0;
    a.store_flux = (store_flux || s + 1 == nsteps) ? 1 : 0;
    const int32_t rc = fn(a, stream, &tma);
    if (rc != FDS_OK) return rc;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(FDS_E_LAUNCH, "step launch: %s", cudaGetErrorString(e));
    for (int k = 0; k < 3; ++k) std::swap(st->cur[k], st->nxt[k]);
  }
  return FDS_OK;
}

}  // namespace fds
