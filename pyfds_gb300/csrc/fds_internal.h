// Internal helpers shared by the translation units of libfdsgpu.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "fds_capi.h"

// Tile shapes built for the lossless 2-D variants: the search space of the
// host-side autotuner. Every other variant uses the default 64 x 16 (2-D) or
// 1024 x 1 (1-D) shared-memory tile.
//   FDS_TILE_MENU:  shared-memory tiles (cells x, cells y, threads); slot layout 0
//   FDS_MARCH_MENU: register-marching warps (cells per lane CX, rows TY, warps per
//                   CTA); the tile is (32*CX - 2) x TY cells; slot layout 1
#define FDS_TILE_MENU(X)                                                                   \
  X(64, 16, 256) X(32, 32, 256) X(128, 8, 256) X(64, 32, 512) X(128, 16, 512) X(64, 12, 256) \
  X(64, 8, 256)
// two steps per tile (stages = 3): shared-memory tiles of slot layout 2
#define FDS_TB2_MENU(X) X(64, 16, 256) X(64, 12, 256) X(64, 8, 256) X(32, 32, 256)
#define FDS_MARCH_MENU(X) X(2, 16, 4) X(2, 8, 4) X(2, 32, 4) X(1, 16, 4) X(1, 32, 4)

namespace fds {

// Records a printf-style message as the calling thread's last error; returns code.
int32_t set_error(int32_t code, const char* fmt, ...);

int32_t run_stag_f64(const FdsStagProblem*, FdsStagState*, const FdsStagTables*, int64_t,
                     int32_t, int32_t, cudaStream_t);
int32_t run_stag_f32(const FdsStagProblem*, FdsStagState*, const FdsStagTables*, int64_t,
                     int32_t, int32_t, cudaStream_t);
int32_t run_stag_f32t64(const FdsStagProblem*, FdsStagState*, const FdsStagTables*, int64_t,
                        int32_t, int32_t, cudaStream_t);
int32_t run_stag_dw(const FdsStagProblem*, FdsStagState*, const FdsStagTables*, int64_t, int32_t,
                    int32_t, cudaStream_t);

int32_t run_batch_f64(const FdsStagProblem*, FdsStagState*, const FdsStagTables*, int32_t, void*,
                      size_t, int64_t, int32_t, int32_t, uint32_t, cudaStream_t);
int32_t run_batch_f32(const FdsStagProblem*, FdsStagState*, const FdsStagTables*, int32_t, void*,
                      size_t, int64_t, int32_t, int32_t, uint32_t, cudaStream_t);
int32_t run_batch_dw(const FdsStagProblem*, FdsStagState*, const FdsStagTables*, int32_t, void*,
                     size_t, int64_t, int32_t, int32_t, uint32_t, cudaStream_t);
int32_t run_batch_f32t64(const FdsStagProblem*, FdsStagState*, const FdsStagTables*, int32_t,
                         void*, size_t, int64_t, int32_t, int32_t, uint32_t, cudaStream_t);
size_t batch_workspace_bytes(int32_t count, int64_t total_tiles);

// The moving-medium row shift of one step on the current state (flow.cu).
int32_t launch_flow_shift(const FdsStagProblem* prob, void* const* cur, int64_t step,
                          cudaStream_t stream);

}  // namespace fds
