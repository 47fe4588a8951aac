// Forward projection that allocates nothing: its cross-chunk partial sums live in a
// fixed file-scope device array instead of the plan's scratch buffer.
//
// Who needs it: callers that must not allocate device memory while they run — code on a
// stream whose memory pool forbids further cudaMalloc, host processes whose device memory
// is owned by another framework's allocator, or long-running services that budget every
// allocation up front.  They
// create their plan once at set-up; afterwards this entry point touches only the plan's
// read-only tables, the caller's input and output, and the static array below.
//
// Limits and behaviour:
//   * the array holds GB_FWD_STATIC_FLOATS floats (16 MiB); every GPU that loads the
//     library keeps it until the process exits;
//   * the plan's work items times nx * nz partial sums must fit (at least one item per
//     angle); larger requests are rejected with GB_ERR_SHAPE;
//   * every call shares the array and the kernels overwrite every partial they later
//     read (nothing needs to start at zero), so calls that overlap on the GPU (other
//     streams, other threads) race: order them on one stream;
//   * the first call on a device looks the array's device address up with
//     cudaGetSymbolAddress (with that device current) and caches it; make that first
//     call before any stream capture.
#include <algorithm>
#include <mutex>

#include "common.cuh"
#include "spect_launch.h"

#define GB_FWD_STATIC_FLOATS (4u * 1024u * 1024u)

namespace gb {

static __device__ __align__(256) float g_fwd_static_scratch[GB_FWD_STATIC_FLOATS];

static std::mutex g_static_mu;
static float *g_static_ptr[64] = {nullptr};

// Device address of the static array on the current device (looked up once per device).
static gb_status static_scratch(float **out) {
    int dev = 0;
    GB_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) {
        set_error("device ordinal %d out of range", dev);
        return GB_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (!g_static_ptr[dev]) {
        void *p = nullptr;
        GB_CUDA(cudaGetSymbolAddress(&p, g_fwd_static_scratch));
        g_static_ptr[dev] = static_cast<float *>(p);
    }
    *out = g_static_ptr[dev];
    return GB_OK;
}

}  // namespace gb

using namespace gb;

extern "C" gb_status gb_spect_forward_static(gb_spect_plan *plan, const float *object,
                                             float *proj, int32_t subset, gb_stream_t stream) {
    clear_error();
    GB_CHECK_ARG(plan && object && proj, "null argument");
    FwdArgs a;
    if (!plan_forward_args(plan, subset, &a)) {
        set_error("subset %d out of range", subset);
        return GB_ERR_STATE;
    }
    const size_t need = (size_t)a.n_items * a.g.N * a.g.nz;
    if (need > GB_FWD_STATIC_FLOATS) {
        set_error("forward of %d angles (%d work items) x %d x %d needs %zu floats of scratch; "
                  "the static array holds %u",
                  a.n_sel, a.n_items, a.g.N, a.g.nz, need, (unsigned)GB_FWD_STATIC_FLOATS);
        return GB_ERR_SHAPE;
    }
    float *scratch = nullptr;
    gb_status s = static_scratch(&scratch);
    if (s != GB_OK) return s;
    cudaStream_t st = as_stream(stream);
    GB_CUDA(launch_fwd(a.g, object, a.alist, a.items, a.n_items, a.Zt, a.tpb, a.variant, scratch,
                       st));
    GB_CUDA(launch_reduce(a.n_sel, a.ioff, a.g.N * a.g.nz, scratch, proj, 0, nullptr, nullptr,
                          a.alist, nullptr, st));
    return GB_OK;
}
