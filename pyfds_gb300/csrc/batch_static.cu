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
// the array's name as a device address, so every call resolves the address on the
// current device with cudaGetSymbolAddress (a lookup, no allocation). Resolving
// it per call instead of caching it keeps the address right after a device reset
// or a new primary context, which reloads this module at another address. The
// first call on a device also loads the module, so make it before any stream
// capture. A call made while its stream is capturing is rejected (FDS_E_ARG): the
// call uploads its descriptors from host memory that is freed when it returns,
// which a captured copy would read again at every replay. All calls share the one
// array and it keeps the last call's contents; nothing in it has to start at
// zero (every call rewrites the descriptors and work list it reads). Two calls
// whose work overlaps on the GPU (different streams, or different host threads)
// race on the array and must be serialised by the caller.
#include "fds_capi.h"
#include "fds_internal.h"

static __device__ __align__(256) unsigned char g_batch_scratch[FDS_BATCH_STATIC_MAX_BYTES];

namespace {

// Device address of the scratch array in the current device's context.
int32_t scratch_address(void** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_batch_scratch);
  if (e != cudaSuccess || !p)
    return fds::set_error(FDS_E_LAUNCH, "cudaGetSymbolAddress(scratch): %s",
                          cudaGetErrorString(e));
  *out = p;
  return FDS_OK;
}

// FDS_OK unless `stream` is being captured into a graph (or its capture state
// cannot be read, as for the legacy stream while another stream captures).
int32_t require_not_capturing(cudaStream_t stream) {
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  const cudaError_t e = cudaStreamIsCapturing(stream, &st);
  if (e == cudaErrorStreamCaptureImplicit || e == cudaErrorStreamCaptureUnsupported) {
    (void)cudaGetLastError();
    return fds::set_error(FDS_E_ARG, "stream capture state: %s (this entry point cannot be "
                          "called during a stream capture)", cudaGetErrorString(e));
  }
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    return fds::set_error(FDS_E_LAUNCH, "cudaStreamIsCapturing: %s", cudaGetErrorString(e));
  }
  if (st != cudaStreamCaptureStatusNone)
    return fds::set_error(FDS_E_ARG, "fds_stag_batch_run_static cannot be called while its "
                          "stream is capturing (it uploads descriptors from host memory)");
  return FDS_OK;
}

}  // namespace

extern "C" int32_t fds_stag_batch_run_static(const FdsStagProblem* probs, FdsStagState* states,
                                             const FdsStagTables* tables, int32_t count,
                                             int64_t step0, int32_t nsteps, int32_t store_flux,
                                             void* stream) {
  if (!probs || count < 1) return fds::set_error(FDS_E_ARG, "null argument or empty batch");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int32_t rc = require_not_capturing(s);
  if (rc != FDS_OK) return rc;
  void* ws = nullptr;
  rc = scratch_address(&ws);
  if (rc != FDS_OK) return rc;
  // the size check is the workspace entry point's own (same tile shapes)
  rc = fds_stag_batch_run(probs, states, tables, count, ws, FDS_BATCH_STATIC_MAX_BYTES, step0,
                          nsteps, store_flux, FDS_BATCH_UPLOAD | FDS_BATCH_LAUNCH, stream);
  if (rc == FDS_E_SIZE) {
    char msg[384];
    fds_last_error(msg, sizeof(msg));
    return fds::set_error(FDS_E_SIZE,
                          "%s; the built-in scratch holds %zu bytes (use fds_stag_batch_run "
                          "with a workspace)", msg, (size_t)FDS_BATCH_STATIC_MAX_BYTES);
  }
  return rc;
}
