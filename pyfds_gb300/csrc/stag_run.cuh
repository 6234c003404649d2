// Step loop and variant dispatch of the fused staggered-grid kernel, for one
// precision (included by one translation unit per precision).
#pragma once

#include <cstdio>
#include <utility>

#include "fds_internal.h"
#include "stag_kernel.cuh"

namespace fds {

constexpr int kTile2dX = 64, kTile2dY = 16, kTile1dX = 1024;
constexpr int kThreads = 256;

template <typename TP, typename TF, typename TC>
using StagLaunch = void (*)(const StagArgs<TP, TF, TC>&, int, cudaStream_t);

template <class C, typename TP, typename TF, typename TC>
void launch_stag(const StagArgs<TP, TF, TC>& a, int ntiles, cudaStream_t s) {
  const size_t smem = stag_smem_bytes<C, TP, TF, TC>(a.iso != 0);
  static bool attr_set = false;  // opt in once per kernel variant (largest size)
  if (!attr_set) {
    cudaFuncSetAttribute(stag_step_kernel<C, TP, TF, TC>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)stag_smem_bytes<C, TP, TF, TC>(false));
    attr_set = true;
  }
  stag_step_kernel<C, TP, TF, TC><<<ntiles, C::NT, smem, s>>>(a);
}

// Kernel of one variant; nullptr when not built for this precision or tile.
template <typename TP, typename TF, typename TC, bool ALLOW_EXACT, bool ALLOW_ACOUSTIC>
StagLaunch<TP, TF, TC> pick_stag(int family, bool has_v, bool absorb, bool axi, bool exact,
                                 int tx, int ty) {
  constexpr int T = kThreads;
  const bool acoustic = (family == FDS_FAMILY_ACOUSTIC);
  if (exact && !ALLOW_EXACT) return nullptr;
  if (acoustic && !ALLOW_ACOUSTIC) return nullptr;
  if (!acoustic && absorb) return nullptr;
  // the radius only enters the kernel through the exact pressure scaling and the
  // radial loss term; otherwise the axisymmetric step is the planar one
  if (axi && !exact && !absorb) axi = false;
  const bool dflt = has_v ? (tx == kTile2dX && ty == kTile2dY) : (tx == kTile1dX && ty == 1);
#define FDS_PICK(TX, TY, HV, MEM, ABS, AX, EX)                                              \
  if (dflt && has_v == HV && acoustic == MEM && absorb == ABS && axi == AX && exact == EX) \
    return &launch_stag<StagCfg<TX, TY, T, HV, MEM, ABS, AX, EX>, TP, TF, TC>;
#define FDS_PICK_TILE(TX, TY, NT)                                                            \
  if (has_v && !absorb && !axi && !exact && tx == TX && ty == TY) {                          \
    if (acoustic) {                                                                          \
      if constexpr (ALLOW_ACOUSTIC)                                                          \
        return &launch_stag<StagCfg<TX, TY, NT, true, true, false, false, false>, TP, TF, TC>; \
    } else {                                                                                 \
      return &launch_stag<StagCfg<TX, TY, NT, true, false, false, false, false>, TP, TF, TC>;  \
    }                                                                                        \
  }
  FDS_TILE_MENU(FDS_PICK_TILE)
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
  StagLaunch<TP, TF, TC> fn =
      pick_stag<TP, TF, TC, ALLOW_EXACT, ALLOW_ACOUSTIC>(prob->family, has_v, absorb, axi, exact,
                                                         prob->tile_x, prob->tile_y);
  if (!fn)
    return set_error(FDS_E_NOKERNEL,
                     "no kernel built for family=%d precision=%d flags=%u tile=%dx%d",
                     prob->family, prob->precision, prob->flags, prob->tile_x, prob->tile_y);
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
  a.step0 = step0;

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
    fn(a, ntiles, stream);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(FDS_E_LAUNCH, "step launch: %s", cudaGetErrorString(e));
    for (int k = 0; k < 3; ++k) std::swap(st->cur[k], st->nxt[k]);
  }
  return FDS_OK;
}

}  // namespace fds
