// Host-side launchers of the SPECT kernels (implemented in spect_fwd.cu / spect_bwd.cu).
#pragma once
#include <cuda_runtime.h>

#include "gbtomo.h"
#include "spect_kernels.cuh"

// PSF tap-count buckets compiled into the library: a plan's taps are zero-padded
// (centred) to the smallest bucket that holds its widest kernel.
#define GB_FOR_EACH_K(X) X(7) X(11) X(15) X(21) X(25) X(29) X(37) X(45)
// the buckets the second forward variant (k_fwd_psf2) is compiled for
#define GB_FOR_EACH_K2(X) X(7) X(11) X(15) X(21) X(25) X(29)

namespace gb {

inline int psf_bucket(int k) {
    const int b[] = {7, 11, 15, 21, 25, 29, 37, 45};
    for (int v : b)
        if (k <= v) return v;
    return -1;
}

// Forward PSF kernel: rows per TMA box of its attenuation copy, and the length of its
// sample rows in shared memory for a z slab of zw (rounded to the output block) with
// half-halo hp: a multiple of 32 floats, so every row starts 128-byte aligned.
constexpr int kBoxRows = 8;
__host__ __device__ constexpr int fwd_s_cols(int zw, int hp) { return (zw + 2 * hp + 31) & ~31; }

// tpb: threads per forward CTA, 512 or 768 (one CTA per SM)
size_t fwd_psf_smem_bytes(int K, int N, int Zt, int tpb);
size_t b1_psf_smem_bytes(int K, int N, int Zt);
// Raise the dynamic shared-memory limit of the PSF kernels (done once at plan creation,
// outside any stream capture).
cudaError_t setup_fwd(int K, size_t smem, int tpb);
cudaError_t setup_b1(int K, size_t smem);

// Work items (int4: slot, first plane, end plane, unused) split each angle's planes
// into ranges of about equal work; partial sums are indexed by item.
// variant 1: k_fwd_psf (tpb 512 or 768); variant 2: k_fwd_psf2 (cp.async ring, z blur first;
// attenuation before a 2-D PSF, N <= 128, nz <= 128, nz % 4 == 0, at most 29 taps)
cudaError_t launch_fwd(const SpectDev &g, const float *f, const int *alist, const int4 *items,
                       int n_items, int Zt, int tpb, int variant, float *partials,
                       cudaStream_t st);
bool fwd2_eligible(const SpectDev &g, size_t smem_cap);
cudaError_t setup_fwd2(int K);
// ioff[slot] .. ioff[slot+1]: the items of a slot
cudaError_t launch_reduce(int n_slots, const int *ioff, int NZ, const float *partials, float *out,
                          int ratio, const float *gproj, const float *sadd, const int *alist,
                          float *pred, cudaStream_t st);
cudaError_t launch_b1(const SpectDev &g, const float *proj, const int *alist, int n_slots,
                      const int4 *items, int n_items, int Zt, float *W, cudaStream_t st);
cudaError_t launch_b2_gather(const SpectDev &g, const float *W, const int *alist, int n_slots,
                             float *out, int mode, const UpdateArgs &u, cudaStream_t st);
cudaError_t launch_b2_scatter(const SpectDev &g, const float *W, const int *alist, int n_slots,
                              float *out, cudaStream_t st);
cudaError_t launch_atten(const SpectDev &g, const float *mu, float dx, int n_angles, float *A,
                         cudaStream_t st);
cudaError_t launch_rdp(const float *f, float *grad, int nx, int ny, int nz, const UpdateArgs &u,
                       float beta_scale, cudaStream_t st);
cudaError_t launch_rdp_hvp(const float *f, const float *x, float *out, int nx, int ny, int nz,
                           const UpdateArgs &u, float beta_scale, cudaStream_t st);

// ------------------------------------------------------------------ batches
// Persistent / flat launches over several "entries" (a reconstruction, or one object of a
// batch on a shared plan) at once.  Each entry carries its plan's device description and
// its own buffers; the structures travel as kernel parameters (__grid_constant__), so a
// launch reads no descriptor from global memory and can be recorded in a CUDA graph.
constexpr int kMaxBatch = 32;

struct FwdBatch {
    CUtensorMap tm[kMaxBatch];  // attenuation boxes of each entry (64-byte aligned)
    SpectDev g[kMaxBatch];
    const float *f[kMaxBatch];      // object of each entry
    const int *alist[kMaxBatch];    // angle list of the launch's subset, per entry
    const int4 *items;              // (slot, first plane, end plane, entry), largest first
    int n_items;
    int *counter;                   // work-queue position, zeroed before the launch
    float *partials;                // [n_items][nz_max]
    int nz_max;
};

struct ReduceBatch {
    float *out[kMaxBatch];          // [n_sel][N][nz] of each entry
    const float *gproj[kMaxBatch];  // measured projections [n_angles][N][nz] (ratio mode)
    const float *sadd[kMaxBatch];   // additive term, same layout, or null
    const int *alist[kMaxBatch];
    int NZ[kMaxBatch];              // N * nz of each entry
    const int2 *rows;               // (entry, slot) of every output row
    const int *row_off;             // [n_rows + 1] offsets into row_items
    const int *row_items;           // work items of each row in plane order
    const float *partials;
    int nz_max;
    int ratio;                      // 1: out = g / (sum + s + delta)
};

struct B1Batch {
    SpectDev g[kMaxBatch];          // wrange: the entry's own row ranges
    const float *proj[kMaxBatch];   // projection rows of the group's slots
    const int *alist[kMaxBatch];    // the group's angles
    float *W[kMaxBatch];            // [slots][Lp][nya][nz]
    const int4 *items;              // (slot in group, first plane, end plane, entry)
    int n_items;
    int *counter;
};

struct B2Batch {
    SpectDev g[kMaxBatch];
    const float *W[kMaxBatch];
    const int *alist[kMaxBatch];    // the group's angles
    int n_slots[kMaxBatch];
    float *out[kMaxBatch];          // target (write / add / scatter) or OSEM object
    const float *nbp[kMaxBatch];    // OSEM: H_m^T 1
    const float *acc[kMaxBatch];    // OSEM: back projection of earlier groups, or null
    int block_off[kMaxBatch + 1];   // first block of each entry (total for unused entries)
    int mode[kMaxBatch];            // gather: B2_WRITE, B2_ADD or B2_OSEM per entry
};

#define GB_DECL_FWD_BATCH(KK)                                                               \
    cudaError_t setup_fwd_psf_batch_##KK();                                                 \
    cudaError_t launch_fwd_psf_batch_##KK(const FwdBatch &p, int grid, cudaStream_t st);
GB_FOR_EACH_K(GB_DECL_FWD_BATCH)
#undef GB_DECL_FWD_BATCH
// Tensor map of a plan's attenuation table for the forward kernel's box copies (a zeroed map
// when the kernel makes none); s_cols is the kernel's S row length.
cudaError_t make_att_tmap(const SpectDev &g, int s_cols, CUtensorMap *out);
cudaError_t setup_b1_batch(int K);
cudaError_t launch_b1_batch(int K, const B1Batch &p, int grid, cudaStream_t st);
cudaError_t launch_reduce_batch(const ReduceBatch &p, int n_rows, cudaStream_t st);
cudaError_t launch_b2_gather_batch(const B2Batch &p, int n_blocks, cudaStream_t st);
cudaError_t launch_b2_scatter_batch(const B2Batch &p, int n_blocks, cudaStream_t st);
// blocks of 256 threads of one entry in the batched gather / scatter kernels
int b2_gather_blocks(const SpectDev &g);
int b2_scatter_blocks(const SpectDev &g, int n_slots);

// Launch geometry of one forward projection of a plan (for entry points defined outside
// spect_plan.cu): false when the subset is out of range.
struct FwdArgs {
    SpectDev g;
    const int *alist;
    int n_sel;
    const int4 *items;
    int n_items;
    const int *ioff;
    int Zt;
    int tpb;
    int variant;
};
bool plan_forward_args(const gb_spect_plan *p, int subset, FwdArgs *a);

}  // namespace gb
