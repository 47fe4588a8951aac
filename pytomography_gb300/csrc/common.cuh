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

// Host-side fault injection (tests of the error paths without a GPU fault).  A site armed
// with a countdown n makes its n-th check from then on report a failure, once; sites are
// armed by gb_inject_fault() or, at the first check, by the environment variable
// GBTOMO_INJECT ("alloc:1", "launch:2,arg:1", ...).
enum FaultSite { FAULT_ALLOC = 0, FAULT_LAUNCH = 1, FAULT_ARG = 2, FAULT_SITES = 3 };
bool fault_injected(FaultSite site);

// Device memory of plans, batches and their scratch, with the allocation fault site in
// front of it.  Blocks come from a library-owned stream-ordered pool per device
// (cudaMemPool) that keeps up to kPoolKeepBytes of freed memory reserved, so a plan
// created after another was destroyed reuses its memory without new driver mappings.
// dev_alloc returns memory usable from any stream; dev_free waits for the device first
// (as cudaFree does), so no kernel in flight can see a block handed out again.
constexpr unsigned long long kPoolKeepBytes = 16ull << 30;
cudaError_t dev_alloc(void **p, size_t bytes);
void dev_free(void *p);
// Returns the current device pool's reserved, unused blocks to the driver (after a device
// synchronize).
cudaError_t release_pool_memory();
template <typename T>
inline cudaError_t dev_alloc(T **p, size_t bytes) {
    return dev_alloc(reinterpret_cast<void **>(p), bytes);
}

// Entry-point checks of the launch and argument fault sites: set the error message and
// return the status the real failure would return.
#define GB_INJECT_LAUNCH()                                                  \
    do {                                                                    \
        if (::gb::fault_injected(::gb::FAULT_LAUNCH)) {                     \
            ::gb::set_error("kernel launch failed: injected launch failure"); \
            return GB_ERR_CUDA;                                             \
        }                                                                   \
    } while (0)
#define GB_INJECT_ARG()                                             \
    do {                                                            \
        if (::gb::fault_injected(::gb::FAULT_ARG)) {                \
            ::gb::set_error("invalid argument: injected bad argument"); \
            return GB_ERR_ARG;                                      \
        }                                                           \
    } while (0)

int device_sm_count();

}  // namespace gb
