// Internal helpers shared by the translation units of libfdsgpu.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "fds_capi.h"

namespace fds {

// Records a printf-style message as the calling thread's last error; returns code.
int32_t set_error(int32_t code, const char* fmt, ...);

int32_t run_stag_f64(const FdsStagProblem*, FdsStagState*, const FdsStagTables*, int64_t,
                     int32_t, int32_t, cudaStream_t);
int32_t run_stag_f32(const FdsStagProblem*, FdsStagState*, const FdsStagTables*, int64_t,
                     int32_t, int32_t, cudaStream_t);
int32_t run_stag_f32t64(const FdsStagProblem*, FdsStagState*, const FdsStagTables*, int64_t,
                        int32_t, int32_t, cudaStream_t);

}  // namespace fds
