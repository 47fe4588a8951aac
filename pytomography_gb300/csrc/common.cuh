// Shared helpers for the gbtomo CUDA library: status handling, thread-local last
// error, launch checks.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>
#include <string>

#include "gbtomo.h"

namespace gb {

// Thread-local message of the last failed call (read back through gb_last_error()).
void set_error(const char *fmt, ...);
void clear_error();

#define GB_CHECK_ARG(cond, ...)            \
    do {                                   \
        if (!(cond)) {                     \
            ::gb::set_error(__VA_ARGS__);  \
            return GB_ERR_ARG;             \
        }                                  \
    } while (0)

#define GB_CUDA(call)                                                                   \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) {                                                        \
            ::gb::set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_),     \
                            __FILE__, __LINE__);                                        \
            return e_ == cudaErrorMemoryAllocation ? GB_ERR_OOM : GB_ERR_CUDA;          \
        }                                                                               \
    } while (0)

#define GB_LAUNCH_CHECK()                                                               \
    do {                                                                                \
        cudaError_t e_ = cudaGetLastError();                                            \
        if (e_ != cudaSuccess) {                                                        \
            ::gb::set_error("kernel launch failed: %s (%s:%d)", cudaGetErrorString(e_), \
                            __FILE__, __LINE__);                                        \
            return GB_ERR_CUDA;                                                         \
        }                                                                               \
    } while (0)

inline cudaStream_t as_stream(gb_stream_t s) { return reinterpret_cast<cudaStream_t>(s); }

int device_sm_count();

}  // namespace gb
