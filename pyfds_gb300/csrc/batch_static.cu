// Allocation-free batched run: fds_stag_batch_run with its workspace in a
// fixed-size array compiled into this library instead of memory the caller
// allocates.
//
// Who needs it: callers that cannot (or must not) allocate device memory, for
// example a C or Fortran host code that links libfdsgpu.so directly and has no
// device allocator of its own, or a caller in a section where a cudaMalloc would
// be an error or a stall it cannot afford (a real-time loop, a region where the
// device heap is owned by someone else).
//
// The array below lives in every GPU that loads this library, for the lifetime of
// the process (FDS_BATCH_STATIC_MAX_BYTES of device memory). Host code cannot use
// the array's name as a device address, so the first call on each device (with
// that device current) resolves its address with cudaGetSymbolAddress; that first
// call should therefore come before any stream capture. All calls share the one
// array and it keeps the last call's contents; nothing in it has to start at zero
// (every call rewrites the descriptors and work list it reads). Two calls whose
// work overlaps on the GPU (different streams, or different host threads) race on
// the array and must be serialised by the caller.
#include <mutex>

#include "fds_capi.h"
#include "fds_internal.h"

static __device__ __align__(256) unsigned char g_batch_scratch[FDS_BATCH_STATIC_MAX_BYTES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
void* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device (set up once).
int32_t scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fds::set_error(FDS_E_LAUNCH, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fds::set_error(FDS_E_ARG, "device %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_batch_scratch);
    if (e != cudaSuccess || !p)
      return fds::set_error(FDS_E_LAUNCH, "cudaGetSymbolAddress(scratch): %s",
                            cudaGetErrorString(e));
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return FDS_OK;
}

}  // namespace

extern "C" int32_t fds_stag_batch_run_static(const FdsStagProblem* probs, FdsStagState* states,
                                             const FdsStagTables* tables, int32_t count,
                                             int64_t step0, int32_t nsteps, int32_t store_flux,
                                             void* stream) {
  if (!probs || count < 1) return fds::set_error(FDS_E_ARG, "null argument or empty batch");
  if (probs[0].tile_x < 1 || probs[0].tile_y < 1)
    return fds::set_error(FDS_E_ARG, "bad tile shape %dx%d", probs[0].tile_x, probs[0].tile_y);
  int64_t tiles = 0;
  for (int i = 0; i < count; ++i)
    tiles += (int64_t)((probs[i].nx + probs[0].tile_x - 1) / probs[0].tile_x) *
             ((probs[i].ny + probs[0].tile_y - 1) / probs[0].tile_y);
  const size_t need = fds_stag_batch_workspace_bytes(count, tiles);
  if (need > (size_t)FDS_BATCH_STATIC_MAX_BYTES)
    return fds::set_error(FDS_E_SIZE,
                          "batch of %d fields / %lld tiles needs %zu bytes of scratch; the "
                          "built-in scratch holds %zu (use fds_stag_batch_run with a workspace)",
                          count, (long long)tiles, need, (size_t)FDS_BATCH_STATIC_MAX_BYTES);
  void* ws = nullptr;
  const int32_t rc = scratch_address(&ws);
  if (rc != FDS_OK) return rc;
  return fds_stag_batch_run(probs, states, tables, count, ws, FDS_BATCH_STATIC_MAX_BYTES, step0,
                            nsteps, store_flux, FDS_BATCH_UPLOAD | FDS_BATCH_LAUNCH, stream);
}
