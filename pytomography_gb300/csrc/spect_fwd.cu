// Fused SPECT forward projector (rotate -> attenuate -> depth-dependent PSF -> ray sum)
// and the cross-chunk reduction with its likelihood-ratio epilogue: the projector without
// PSF, the reduction and the launchers (the PSF kernel is in spect_fwd_psf.cuh).
//
// Reference: SPECTSystemMatrix.forward (projectors/SPECT/spect_system_matrix.py:120-157)
// with SPECTAttenuationTransform.forward (transforms/SPECT/attenuation.py:72-92); the
// ratio epilogue is PoissonLogLikelihood.compute_gradient's g / (H f + s + delta)
// (likelihoods/poisson_log_likelihood.py:33-36).
#include <cudaTypedefs.h>

#include <cstring>

#include "spect_fwd_v2.cuh"
#include "spect_kernels.cuh"
#include "spect_launch.h"

namespace gb {

// per-bucket PSF forward entry points (spect_fwd_k*.cu)
#define GB_DECL_FWD(KK)                                                                      \
    cudaError_t launch_fwd_psf_##KK(const SpectDev &g, const float *f, const int *alist,     \
                                    const int4 *items, int n_items, int Zt, int tpb,         \
                                    float *partials, cudaStream_t st);                      \
    cudaError_t setup_fwd_##KK(size_t smem, int tpb);
GB_FOR_EACH_K(GB_DECL_FWD)
#undef GB_DECL_FWD
#define GB_DECL_FWD2(KK)                                                                     \
    cudaError_t setup_fwd2_##KK();                                                           \
    cudaError_t launch_fwd2_##KK(const SpectDev &g, const float *f, const int *alist,        \
                                 const int4 *items, int n_items, float *partials,            \
                                 cudaStream_t st);
GB_FOR_EACH_K2(GB_DECL_FWD2)
#undef GB_DECL_FWD2

// ------------------------------------------------------------- without PSF
// One thread per output (y, z) of an item's planes, or per (y, z quad) with nz % 4 == 0;
// A read on the fly.  The samples of PU planes are gathered before they are added, in
// plane order, so those loads are in flight together.
template <bool VEC>
__global__ void __launch_bounds__(256)
    k_fwd_nopsf(SpectDev g, const float *__restrict__ f, const int *__restrict__ alist,
                const int4 *__restrict__ items, float *__restrict__ partials) {
    constexpr int V = VEC ? 4 : 1, PU = VEC ? 4 : 8;
    const int4 item = items[blockIdx.x];
    const int ga = alist[item.x];
    const int N = g.N, nz = g.nz, nzv = nz / V;
    const int i = blockIdx.y * blockDim.x + threadIdx.x;
    if (i >= N * nzv) return;
    const int y = i / nzv, z = (i % nzv) * V;
    float th[6];
#pragma unroll
    for (int k = 0; k < 6; k++) th[k] = g.theta_fwd[6 * ga + k];
    const float *A = g.att ? g.A + (size_t)ga * g.Lp * g.nya * nz : nullptr;
    const int yp = g.pad + y;
    const float lc = g.lin[yp];
    float acc[V];
#pragma unroll
    for (int w = 0; w < V; w++) acc[w] = 0.f;
    for (int x0 = item.y; x0 < item.z; x0 += PU) {
        float v[PU][V];
#pragma unroll
        for (int u = 0; u < PU; u++) {
            const int xp = min(x0 + u, item.z - 1);
            float ix, iy;
            rot_coords(th, g.lin[xp], lc, g.half, ix, iy);
            const Bilin b = bilin(ix, iy);
            const size_t ao = ((size_t)xp * g.nya + (yp - g.ya_lo)) * nz + z;
            if constexpr (VEC) {
                float4 s4;
                sample4(f, N, N, nz, g.pad, g.pad, b, z, s4);
                if (A) s4 = mul4(s4, __ldg(reinterpret_cast<const float4 *>(A + ao)));
                v[u][0] = s4.x;
                v[u][1] = s4.y;
                v[u][2] = s4.z;
                v[u][3] = s4.w;
            } else {
                float s1 = sample(f, N, N, nz, g.pad, g.pad, b, z);
                if (A) s1 = __fmul_rn(s1, __ldg(A + ao));
                v[u][0] = s1;
            }
        }
#pragma unroll
        for (int u = 0; u < PU; u++) {
            if (x0 + u >= item.z) break;
#pragma unroll
            for (int w = 0; w < V; w++) acc[w] += v[u][w];
        }
    }
    float *out = partials + (size_t)blockIdx.x * N * nz + (size_t)y * nz + z;
    if constexpr (VEC)
        *reinterpret_cast<float4 *>(out) = make_float4(acc[0], acc[1], acc[2], acc[3]);
    else
        out[0] = acc[0];
}

// --------------------------------------------------------------- reduction
// out[slot][i] = sum of the partials of the slot's items, in item order.  With
// `ratio`, out = g[ga][i] / (sum + s[ga][i] + delta) and pred (optional) = sum + s.
__global__ void k_reduce(const int *__restrict__ ioff, int NZ, const float *__restrict__ partials,
                         float *__restrict__ out, int ratio, const float *__restrict__ gproj,
                         const float *__restrict__ sadd, const int *__restrict__ alist,
                         float *__restrict__ pred) {
    const int slot = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= NZ) return;
    const int c0 = ioff[slot], c1 = ioff[slot + 1];
    float v = 0.f;
    int c = c0;
    for (; c + 4 <= c1; c += 4) {  // four partials' loads in flight, added in item order
        const float p0 = partials[(size_t)c * NZ + i], p1 = partials[(size_t)(c + 1) * NZ + i];
        const float p2 = partials[(size_t)(c + 2) * NZ + i], p3 = partials[(size_t)(c + 3) * NZ + i];
        v = (((v + p0) + p1) + p2) + p3;
    }
    for (; c < c1; c++) v += partials[(size_t)c * NZ + i];
    size_t o = (size_t)slot * NZ + i;
    if (!ratio) {
        out[o] = v;
        return;
    }
    const int ga = alist[slot];
    size_t gi = (size_t)ga * NZ + i;
    float pr = sadd ? v + sadd[gi] : v;
    if (pred) pred[o] = pr;
    out[o] = gproj[gi] / (pr + kDelta);
}

// Batched reduction: one row (entry, slot) per grid row; the items of the row are added
// in plane order (the order of row_items), so results do not depend on the work queue.
__global__ void k_reduce_batch(const __grid_constant__ ReduceBatch p) {
    const int2 row = p.rows[blockIdx.y];
    const int e = row.x, slot = row.y;
    const int NZ = p.NZ[e];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= NZ) return;
    float v = 0.f;
    for (int c = p.row_off[blockIdx.y]; c < p.row_off[blockIdx.y + 1]; c++)
        v += p.partials[(size_t)p.row_items[c] * p.nz_max + i];
    const size_t o = (size_t)slot * NZ + i;
    if (!p.ratio) {
        p.out[e][o] = v;
        return;
    }
    const size_t gi = (size_t)p.alist[e][slot] * NZ + i;
    const float pr = p.sadd[e] ? v + p.sadd[e][gi] : v;
    p.out[e][o] = p.gproj[e][gi] / (pr + kDelta);
}

cudaError_t launch_reduce_batch(const ReduceBatch &p, int n_rows, cudaStream_t st) {
    if (n_rows <= 0) return cudaSuccess;
    dim3 grid((p.nz_max + 255) / 256, n_rows);
    k_reduce_batch<<<grid, 256, 0, st>>>(p);
    return cudaGetLastError();
}

// ------------------------------------------------------------- launchers
static bool fwd_fixed_host(int K, int N, int Zt, int tpb) {
    int OB = (K <= 31) ? 8 : 4;
    (void)tpb;
    return (N + OB - 1) / OB * OB <= 128 && (Zt + OB - 1) / OB * OB <= 128;
}

size_t fwd_psf_smem_bytes(int K, int N, int Zt, int tpb) {
    int H = K / 2, HP = (H + 3) / 4 * 4, OB = (K <= 31) ? 8 : 4;
    int N8 = (N + OB - 1) / OB * OB;
    int Z8 = (Zt + OB - 1) / OB * OB;
    const bool fx = fwd_fixed_host(K, N, Zt, tpb);
    const int ZW = 128;
    // Tt row stride: even (float2 row pairs) with 512 threads, odd with 768
    const int ts_pad = tpb <= 512 ? 2 : 1;
    size_t SC = fwd_s_cols(fx ? ZW : Z8, HP), TS = fx ? 128 + ts_pad : N8 + ts_pad;
    return sizeof(float) * ((size_t)(N8 + 2 * H) * SC + (size_t)(Z8 + 2 * HP) * TS +
                            ((4 * K + 1) & ~1)) +
           sizeof(unsigned long long);
}

// cuTensorMapEncodeTiled from the driver, looked up once through the runtime.
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

cudaError_t make_att_tmap(const SpectDev &g, int s_cols, CUtensorMap *out) {
    std::memset(out, 0, sizeof(*out));
    // the kernel copies boxes only for an attenuation-first table with z quads
    if (!g.att || !g.att_first || !g.A || g.nz % 4 != 0 || s_cols > 256) return cudaSuccess;
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) return cudaErrorNotSupported;
    const cuuint64_t dims[2] = {(cuuint64_t)g.nz, (cuuint64_t)g.n_angles * g.Lp * g.nya};
    const cuuint64_t strides[1] = {(cuuint64_t)g.nz * sizeof(float)};
    const cuuint32_t box[2] = {(cuuint32_t)s_cols, (cuuint32_t)kBoxRows};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(out, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(g.A), dims,
                     strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

cudaError_t setup_fwd(int K, size_t smem, int tpb) {
    (void)tensor_map_encoder();  // driver lookup outside any stream capture
    switch (K) {
#define GB_SETUP_CASE(KK) \
    case KK:              \
        return setup_fwd_##KK(smem, tpb);
        GB_FOR_EACH_K(GB_SETUP_CASE)
#undef GB_SETUP_CASE
        default:
            return cudaErrorInvalidValue;
    }
}

bool fwd2_eligible(const SpectDev &g, size_t smem_cap) {
    return g.psf && g.psf2d && g.att && g.att_first && g.A && g.K <= kFwd2MaxK &&
           g.N <= 128 && g.nz <= 128 && g.nz % 4 == 0 &&
           fwd2_smem_floats(g.K, g.N, g.nz) * sizeof(float) <= smem_cap;
}

cudaError_t setup_fwd2(int K) {
    switch (K) {
#define GB_SETUP2_CASE(KK) \
    case KK:               \
        return setup_fwd2_##KK();
        GB_FOR_EACH_K2(GB_SETUP2_CASE)
#undef GB_SETUP2_CASE
        default:
            return cudaErrorNotSupported;
    }
}

cudaError_t launch_fwd(const SpectDev &g, const float *f, const int *alist, const int4 *items,
                       int n_items, int Zt, int tpb, int variant, float *partials,
                       cudaStream_t st) {
    if (variant == 2 && g.psf) {
        switch (g.K) {
#define GB_FWD2_CASE(KK) \
    case KK:             \
        return launch_fwd2_##KK(g, f, alist, items, n_items, partials, st);
            GB_FOR_EACH_K2(GB_FWD2_CASE)
#undef GB_FWD2_CASE
            default:
                return cudaErrorNotSupported;
        }
    }
    if (!g.psf) {
        if (g.nz % 4 == 0) {
            dim3 grid(n_items, (g.N * (g.nz / 4) + 255) / 256);
            k_fwd_nopsf<true><<<grid, 256, 0, st>>>(g, f, alist, items, partials);
        } else {
            dim3 grid(n_items, (g.N * g.nz + 255) / 256);
            k_fwd_nopsf<false><<<grid, 256, 0, st>>>(g, f, alist, items, partials);
        }
        return cudaGetLastError();
    }
    switch (g.K) {
#define GB_FWD_CASE(KK) \
    case KK:            \
        return launch_fwd_psf_##KK(g, f, alist, items, n_items, Zt, tpb, partials, st);
        GB_FOR_EACH_K(GB_FWD_CASE)
#undef GB_FWD_CASE
        default:
            return cudaErrorInvalidValue;
    }
}


cudaError_t launch_reduce(int n_slots, const int *ioff, int NZ, const float *partials, float *out,
                          int ratio, const float *gproj, const float *sadd, const int *alist,
                          float *pred, cudaStream_t st) {
    dim3 grid((NZ + 255) / 256, n_slots);
    k_reduce<<<grid, 256, 0, st>>>(ioff, NZ, partials, out, ratio, gproj, sadd, alist, pred);
    return cudaGetLastError();
}

}  // namespace gb
