// C ABI entry points of libfdsgpu.so (declared in include/fds_capi.h).
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>

#include "fds_capi.h"
#include "fds_internal.h"
#include "stag_kernel.cuh"

namespace fds {

static thread_local std::string g_last_error;

int32_t set_error(int32_t code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

static int32_t tile_shape(int32_t precision, uint32_t flags, int32_t* tx, int32_t* ty) {
  if (flags & FDS_FLAG_HAS_V) {
    *tx = 64;
    *ty = 16;
    // double words: 64 x 12 stages 43 KB per CTA instead of 55 KB, which fits a
    // fifth CTA per SM (lossless variants; measured 8 % faster on the 2048^2 step)
    if (precision == FDS_PREC_DW && !(flags & (FDS_FLAG_ABSORB | FDS_FLAG_EXACT))) *ty = 12;
  } else {
    *tx = 1024;
    *ty = 1;
  }
  return FDS_OK;
}

}  // namespace fds

extern "C" {

int32_t fds_abi_version(void) { return FDS_ABI_VERSION; }

int32_t fds_last_error(char* buf, size_t len) {
  const std::string& m = fds::g_last_error;
  if (buf && len > 0) {
    size_t k = m.size() < len - 1 ? m.size() : len - 1;
    memcpy(buf, m.data(), k);
    buf[k] = '\0';
  }
  return (int32_t)m.size();
}

int32_t fds_stag_tile_shape(int32_t family, int32_t precision, uint32_t flags, int32_t nx,
                            int32_t ny, int32_t* tile_x, int32_t* tile_y) {
  (void)family;
  (void)nx;
  (void)ny;
  if (!tile_x || !tile_y) return fds::set_error(FDS_E_ARG, "null output pointer");
  return fds::tile_shape(precision, flags, tile_x, tile_y);
}

int32_t fds_stag_tile_menu(int32_t* tile_x, int32_t* tile_y, int32_t* layout, int32_t capacity) {
  int32_t k = 0;
#define FDS_MENU_ENTRY(TX, TY, NT)                    \
  if (tile_x && tile_y && layout && k < capacity) {   \
    tile_x[k] = TX;                                   \
    tile_y[k] = TY;                                   \
    layout[k] = 0;                                    \
  }                                                   \
  ++k;
#define FDS_MARCH_ENTRY(CX, TY, NW)                   \
  if (tile_x && tile_y && layout && k < capacity) {   \
    tile_x[k] = 32 * CX - 2;                          \
    tile_y[k] = TY;                                   \
    layout[k] = 1;                                    \
  }                                                   \
  ++k;
  FDS_TILE_MENU(FDS_MENU_ENTRY)
  FDS_MARCH_MENU(FDS_MARCH_ENTRY)
#undef FDS_MENU_ENTRY
#undef FDS_MARCH_ENTRY
  return k;
}

int32_t fds_stag_run(const FdsStagProblem* prob, FdsStagState* state,
                     const FdsStagTables* tables, int64_t step0, int32_t nsteps,
                     int32_t store_flux, void* stream) {
  using namespace fds;
  if (!prob || !state || !tables) return set_error(FDS_E_ARG, "null argument");
  if (prob->nx < 1 || prob->ny < 1) return set_error(FDS_E_ARG, "bad grid %d x %d", prob->nx, prob->ny);
  if (prob->stages < 0 || prob->stages > 4) return set_error(FDS_E_ARG, "bad stages %d", prob->stages);
  if (nsteps < 0 || step0 < 0) return set_error(FDS_E_ARG, "bad step range");
  const bool has_v = (prob->flags & FDS_FLAG_HAS_V) != 0;
  if (!has_v && prob->ny != 1) return set_error(FDS_E_ARG, "1-D field needs ny == 1");
  if (prob->tile_x < 1 || prob->tile_y < 1 || (!has_v && prob->tile_y != 1))
    return set_error(FDS_E_ARG, "bad tile shape %dx%d", prob->tile_x, prob->tile_y);
  const FdsCoefs& c = prob->coefs;
  if (!c.bx || !c.kx) return set_error(FDS_E_ARG, "missing coefficient arrays");
  if ((prob->flags & FDS_FLAG_ABSORB) && (!c.axm || !c.ad || !c.axp || (has_v && (!c.aym || !c.ayp))))
    return set_error(FDS_E_ARG, "absorption requested without its diagonals");
  if ((prob->flags & FDS_FLAG_AXI) && !c.rx) return set_error(FDS_E_ARG, "axisymmetric field without radii");
  if ((prob->flags & FDS_FLAG_AXI) && (prob->flags & FDS_FLAG_ABSORB) && !c.ex)
    return set_error(FDS_E_ARG, "axisymmetric absorption without its radial loss factor");
  if ((prob->flags & FDS_FLAG_FLOW) &&
      (prob->family != FDS_FAMILY_ACOUSTIC || !has_v || (prob->flags & FDS_FLAG_AXI) ||
       !prob->flow_period || prob->precision == FDS_PREC_F32_T64))
    return set_error(FDS_E_ARG, "flow needs a 2-D Cartesian float64/float32/double-word "
                                "acoustic field and its flow_period array");
  const int ncomp = has_v ? 3 : 2;
  for (int k = 0; k < ncomp; ++k)
    if (!state->cur[k] || !state->nxt[k]) return set_error(FDS_E_ARG, "missing state buffer %d", k);
  if (prob->family == FDS_FAMILY_ACOUSTIC && !store_flux)
    return set_error(FDS_E_ARG, "acoustic fluxes carry state: store_flux must be set");
  for (int k = 0; k < 3; ++k) {
    const FdsCompTables& t = tables->comp[k];
    if (t.probe_tile_start && (!t.out || t.out_rows < nsteps))
      return set_error(FDS_E_ARG, "output buffer of component %d holds %d rows, need %d", k,
                       t.out_rows, nsteps);
  }
  if (nsteps == 0) return FDS_OK;
  cudaStream_t s = (cudaStream_t)stream;
  switch (prob->precision) {
    case FDS_PREC_F64:
      return run_stag_f64(prob, state, tables, step0, nsteps, store_flux, s);
    case FDS_PREC_F32:
      if (prob->flags & FDS_FLAG_EXACT) return set_error(FDS_E_ARG, "exact mode is float64 only");
      return run_stag_f32(prob, state, tables, step0, nsteps, store_flux, s);
    case FDS_PREC_F32_T64:
      if (prob->flags & FDS_FLAG_EXACT) return set_error(FDS_E_ARG, "exact mode is float64 only");
      return run_stag_f32t64(prob, state, tables, step0, nsteps, store_flux, s);
    case FDS_PREC_DW:
      if (prob->flags & FDS_FLAG_EXACT) return set_error(FDS_E_ARG, "exact mode is float64 only");
      return run_stag_dw(prob, state, tables, step0, nsteps, store_flux, s);
    default:
      return set_error(FDS_E_ARG, "unknown precision %d", prob->precision);
  }
}

int64_t fds_stag_sync_words(const FdsStagProblem* prob) {
  if (!prob) return fds::set_error(FDS_E_ARG, "null argument");
  if (prob->nx < 1 || prob->ny < 1 || prob->tile_y < 1)
    return fds::set_error(FDS_E_ARG, "bad grid %d x %d or tile height %d", prob->nx, prob->ny,
                          prob->tile_y);
  return 1 + ((int64_t)prob->ny + prob->tile_y - 1) / prob->tile_y;
}

size_t fds_stag_batch_workspace_bytes(int32_t count, int64_t total_tiles) {
  if (count < 0 || total_tiles < 0) return 0;
  const size_t d = (2 * (size_t)count * sizeof(fds::StagArgs<double, double, double>) + 255) / 256 * 256;
  return d + (size_t)total_tiles * 8;
}

int32_t fds_stag_batch_run(const FdsStagProblem* probs, FdsStagState* states,
                           const FdsStagTables* tables, int32_t count, void* workspace,
                           size_t workspace_bytes, int64_t step0, int32_t nsteps,
                           int32_t store_flux, uint32_t mode, void* stream) {
  using namespace fds;
  if ((mode & (FDS_BATCH_UPLOAD | FDS_BATCH_LAUNCH)) == 0 || (mode & ~3u) != 0)
    return set_error(FDS_E_ARG, "mode must combine FDS_BATCH_UPLOAD and FDS_BATCH_LAUNCH");
  if (!probs || !states || !tables || count < 1 || !workspace)
    return set_error(FDS_E_ARG, "null argument or empty batch");
  if (((uintptr_t)workspace & 255) != 0) return set_error(FDS_E_ARG, "workspace must be 256-byte aligned");
  if (nsteps < 0 || step0 < 0) return set_error(FDS_E_ARG, "bad step range");
  const FdsStagProblem& p0 = probs[0];
  if (p0.family == FDS_FAMILY_ACOUSTIC && !store_flux)
    return set_error(FDS_E_ARG, "acoustic fluxes carry state: store_flux must be set");
  for (int i = 0; i < count; ++i) {
    const FdsStagProblem& p = probs[i];
    if (p.family != p0.family || p.precision != p0.precision || p.flags != p0.flags ||
        p.tile_x != p0.tile_x || p.tile_y != p0.tile_y || p.stages != p0.stages)
      return set_error(FDS_E_ARG, "instance %d differs from instance 0 in variant or tile", i);
    if (p.nx < 1 || p.ny < 1) return set_error(FDS_E_ARG, "instance %d: bad grid", i);
    if (p.stages < 0 || p.stages > 3) return set_error(FDS_E_ARG, "instance %d: bad stages", i);
    if (!(p.flags & FDS_FLAG_HAS_V) || (p.flags & (FDS_FLAG_ABSORB | FDS_FLAG_EXACT | FDS_FLAG_FLOW)))
      return set_error(FDS_E_NOKERNEL, "batched runs cover lossless 2-D non-exact fields");
    if (!p.coefs.bx || !p.coefs.kx) return set_error(FDS_E_ARG, "instance %d: missing coefficients", i);
    for (int k = 0; k < 3; ++k)
      if (!states[i].cur[k] || !states[i].nxt[k])
        return set_error(FDS_E_ARG, "instance %d: missing state buffer %d", i, k);
    for (int k = 0; k < 3; ++k) {
      const FdsCompTables& t = tables[i].comp[k];
      if (t.probe_tile_start && (!t.out || t.out_rows < nsteps))
        return set_error(FDS_E_ARG, "instance %d: output buffer of component %d too small", i, k);
    }
  }
  if (nsteps == 0) return FDS_OK;
  cudaStream_t s = (cudaStream_t)stream;
  switch (p0.precision) {
    case FDS_PREC_F64:
      return run_batch_f64(probs, states, tables, count, workspace, workspace_bytes, step0, nsteps,
                           store_flux, mode, s);
    case FDS_PREC_F32:
      return run_batch_f32(probs, states, tables, count, workspace, workspace_bytes, step0, nsteps,
                           store_flux, mode, s);
    case FDS_PREC_F32_T64:
      return run_batch_f32t64(probs, states, tables, count, workspace, workspace_bytes, step0,
                              nsteps, store_flux, mode, s);
    case FDS_PREC_DW:
      return run_batch_dw(probs, states, tables, count, workspace, workspace_bytes, step0, nsteps,
                          store_flux, mode, s);
    default:
      return set_error(FDS_E_ARG, "unknown precision %d", p0.precision);
  }
}

}  // extern "C"
