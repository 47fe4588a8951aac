// Fused SPECT forward projector (rotate -> attenuate -> depth-dependent PSF -> ray sum)
// and the cross-chunk reduction with its likelihood-ratio epilogue.
//
// Reference: SPECTSystemMatrix.forward (projectors/SPECT/spect_system_matrix.py:120-157)
// with SPECTAttenuationTransform.forward (transforms/SPECT/attenuation.py:72-92) and
// SPECTPSFTransform.forward -> Seperable1DBlurNet.forward (transforms/SPECT/psf.py:27-41,
// 199-214); the ratio epilogue is PoissonLogLikelihood.compute_gradient's
// g / (H f + s + delta) (likelihoods/poisson_log_likelihood.py:33-36).
//
// Work decomposition: one CTA per (angle, chunk of x planes, z slab).  The CTA sweeps
// its planes; per plane it samples the rotated object (times A) into shared memory,
// blurs along y into a transposed buffer, blurs along z and accumulates the ray sum
// in registers.  Partial sums of the chunks go to a scratch buffer and are reduced
// in a fixed order by k_reduce (deterministic results).
#include "spect_kernels.cuh"
#include "spect_launch.h"

namespace gb {

// Does the sample segment of plane xp (rows y in [ya, yb]) touch the object square
// [pad-1, pad+N] x [pad-1, pad+N] in padded coordinates?  Liang-Barsky clip.
__device__ __forceinline__ bool plane_hits(const SpectDev &g, const float *th, int xp, int ya,
                                           int yb) {
    float ixa, iya, ixb, iyb;
    rot_coords(th, g.lin[xp], g.lin[ya], g.half, ixa, iya);
    rot_coords(th, g.lin[xp], g.lin[yb], g.half, ixb, iyb);
    float lo = (float)g.pad - 1.5f, hi = (float)(g.pad + g.N) + 0.5f;
    float t0 = 0.f, t1 = 1.f;
    float p[2] = {ixa, iya}, d[2] = {ixb - ixa, iyb - iya};
#pragma unroll
    for (int k = 0; k < 2; k++) {
        if (fabsf(d[k]) < 1e-12f) {
            if (p[k] < lo || p[k] > hi) return false;
        } else {
            float ta = (lo - p[k]) / d[k], tb = (hi - p[k]) / d[k];
            if (ta > tb) { float t = ta; ta = tb; tb = t; }
            t0 = fmaxf(t0, ta);
            t1 = fminf(t1, tb);
        }
    }
    return t0 <= t1;
}

// ---------------------------------------------------------------- with PSF
// Shared-memory layout (per CTA):
//   S  [SR][SC]: rotated, attenuated samples; row r <-> padded y = pad - H + r,
//                column c <-> z = z0 - HP + c  (HP = H rounded up to 4: 16-byte aligned
//                z quads)
//   Tt [TR][TS]: y-blurred plane, transposed; row c <-> z = z0 - HP + c, column = output y
//   taps [2][2][K]: double-buffered y / z taps of the current plane
template <int K, bool VEC>
__global__ void __launch_bounds__(512, 1)
    k_fwd_psf(SpectDev g, const float *__restrict__ f, const int *__restrict__ alist,
              int n_chunks, int Zt, float *__restrict__ partials) {
    constexpr int H = K / 2;
    constexpr int HP = (H + 3) / 4 * 4;
    constexpr int OB = (K <= 31) ? 8 : 4;  // outputs per task
    constexpr int NACC = 32 / OB;          // phase-3 tasks per thread
    const int slot = blockIdx.y, chunk = blockIdx.x;
    const int ga = alist[slot];
    const int N = g.N, nz = g.nz;
    const int z0 = blockIdx.z * Zt;
    const int Zc = min(Zt, nz - z0);
    const int N8 = (N + OB - 1) / OB * OB;
    const int Z8 = (Zc + OB - 1) / OB * OB;
    const int SC = Z8 + 2 * HP, SR = N8 + 2 * H;
    const int TS = N8 + 1, TR = Z8 + 2 * HP;
    extern __shared__ __align__(16) float sm[];
    float *S = sm;
    float *Tt = S + SR * SC;
    float *tp = Tt + TR * TS;
    for (int i = threadIdx.x; i < SR * SC + TR * TS; i += blockDim.x) sm[i] = 0.f;

    float th[6];
#pragma unroll
    for (int k = 0; k < 6; k++) th[k] = g.theta_fwd[6 * ga + k];
    const int grp = g.group[ga];
    const float *A = g.att ? g.A + (size_t)ga * g.Lp * g.nya * nz : nullptr;
    const int x0 = chunk * g.Lp / n_chunks, x1 = (chunk + 1) * g.Lp / n_chunks;
    const int zv_lo = max(0, z0 - H), zv_hi = min(nz, z0 + Zc + H);  // z needed by the blur
    const int cz_lo = zv_lo - z0 + HP, cz_hi = zv_hi - z0 + HP;
    const int ncol = cz_hi - cz_lo;
    const int ylo = max(0, g.pad - H), yhi = min(g.Lp, g.pad + N + H);  // sampled rows
    const int n3 = N8 * (Z8 / OB);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
    // z quads covering [zv_lo, zv_hi) (vector path)
    const int zq_lo = zv_lo & ~3, zq_hi = (zv_hi + 3) & ~3;
    const int nq = (zq_hi - zq_lo) >> 2;
    float acc[NACC][OB];
#pragma unroll
    for (int k = 0; k < NACC; k++)
#pragma unroll
        for (int j = 0; j < OB; j++) acc[k][j] = 0.f;
    __syncthreads();

    int parity = 0;
    for (int xp = x0; xp < x1; ++xp) {
        if (!plane_hits(g, th, xp, ylo, yhi - 1)) continue;
        const float lr = g.lin[xp];
        float *tap = tp + parity * 2 * K;
        if (threadIdx.x < K) {
            tap[threadIdx.x] = g.taps_r[((size_t)grp * g.Lp + xp) * g.K + threadIdx.x];
            tap[K + threadIdx.x] =
                g.psf2d ? g.taps_z[((size_t)grp * g.Lp + xp) * g.K + threadIdx.x] : 0.f;
        }
        // phase 1: rotated samples (times A when attenuation precedes the PSF)
        const float *Ap = A ? A + (size_t)xp * g.nya * nz : nullptr;
        const bool amul = Ap && g.att_first;
        if (VEC) {
            // one row per warp, two rows in flight, z quads across lanes
            for (int y = ylo + warp; y < yhi; y += 2 * nwarp) {
                const int y2 = y + nwarp;
                const bool two = y2 < yhi;
                float ix, iy, ix2, iy2;
                rot_coords(th, lr, g.lin[y], g.half, ix, iy);
                rot_coords(th, lr, g.lin[two ? y2 : y], g.half, ix2, iy2);
                const Bilin b1 = bilin(ix, iy), b2 = bilin(ix2, iy2);
                float *S1 = S + (y - (g.pad - H)) * SC;
                float *S2 = S + (y2 - (g.pad - H)) * SC;
                for (int q = lane; q < nq; q += 32) {
                    const int z = zq_lo + 4 * q;
                    float4 v1, v2;
                    bool h1 = sample4(f, N, N, nz, g.pad, g.pad, b1, z, v1);
                    bool h2 = two && sample4(f, N, N, nz, g.pad, g.pad, b2, z, v2);
                    if (amul && h1)
                        v1 = mul4(v1, __ldg(reinterpret_cast<const float4 *>(
                                          Ap + (size_t)(y - g.ya_lo) * nz + z)));
                    if (amul && h2)
                        v2 = mul4(v2, __ldg(reinterpret_cast<const float4 *>(
                                          Ap + (size_t)(y2 - g.ya_lo) * nz + z)));
                    *reinterpret_cast<float4 *>(S1 + (z - z0 + HP)) = v1;
                    if (two) *reinterpret_cast<float4 *>(S2 + (z - z0 + HP)) = h2 ? v2 : make_float4(0.f, 0.f, 0.f, 0.f);
                }
            }
        } else {
            for (int i = threadIdx.x; i < (yhi - ylo) * ncol; i += blockDim.x) {
                int y = ylo + i / ncol, c = cz_lo + i % ncol;
                int z = z0 - HP + c;
                float ix, iy;
                rot_coords(th, lr, g.lin[y], g.half, ix, iy);
                Bilin b = bilin(ix, iy);
                float v = sample(f, N, N, nz, g.pad, g.pad, b, z);
                if (amul && v != 0.f) v = __fmul_rn(v, Ap[(size_t)(y - g.ya_lo) * nz + z]);
                S[(y - (g.pad - H)) * SC + c] = v;
            }
        }
        __syncthreads();
        // phase 2: blur along y, write transposed
        {
            float w[K];
#pragma unroll
            for (int t = 0; t < K; t++) w[t] = tap[t];
            for (int task = threadIdx.x; task < ncol * (N8 / OB); task += blockDim.x) {
                int c = cz_lo + task % ncol, yb = task / ncol;
                float win[OB + K - 1];
#pragma unroll
                for (int i = 0; i < OB + K - 1; i++) win[i] = S[(yb * OB + i) * SC + c];
#pragma unroll
                for (int j = 0; j < OB; j++) {
                    float o = 0.f;
#pragma unroll
                    for (int t = 0; t < K; t++) o = fmaf(w[t], win[j + t], o);
                    Tt[c * TS + yb * OB + j] = o;
                }
            }
        }
        __syncthreads();
        // phase 3: blur along z (2D PSF), optional attenuation after the PSF, accumulate
        {
            float w[K];
#pragma unroll
            for (int t = 0; t < K; t++) w[t] = tap[K + t];
#pragma unroll
            for (int k = 0; k < NACC; k++) {
                int task = threadIdx.x + k * blockDim.x;
                if (task < n3) {
                    int y = task % N8, zb = task / N8;
                    float o[OB];
                    if (g.psf2d) {
                        float win[OB + K - 1];
#pragma unroll
                        for (int i = 0; i < OB + K - 1; i++)
                            win[i] = Tt[(zb * OB + i + HP - H) * TS + y];
#pragma unroll
                        for (int j = 0; j < OB; j++) {
                            float s = 0.f;
#pragma unroll
                            for (int t = 0; t < K; t++) s = fmaf(w[t], win[j + t], s);
                            o[j] = s;
                        }
                    } else {
#pragma unroll
                        for (int j = 0; j < OB; j++) o[j] = Tt[(zb * OB + j + HP) * TS + y];
                    }
                    if (Ap && !g.att_first && y < N) {
#pragma unroll
                        for (int j = 0; j < OB; j++) {
                            int z = z0 + zb * OB + j;
                            if (z < nz)
                                o[j] = __fmul_rn(
                                    o[j], Ap[(size_t)(g.pad + y - g.ya_lo) * nz + z]);
                        }
                    }
#pragma unroll
                    for (int j = 0; j < OB; j++) acc[k][j] += o[j];
                }
            }
        }
        parity ^= 1;
    }
    // partial ray sums of this chunk
    float *out = partials + ((size_t)slot * n_chunks + chunk) * N * nz;
#pragma unroll
    for (int k = 0; k < NACC; k++) {
        int task = threadIdx.x + k * blockDim.x;
        if (task < n3) {
            int y = task % N8, zb = task / N8;
            if (y < N) {
#pragma unroll
                for (int j = 0; j < OB; j++) {
                    int z = z0 + zb * OB + j;
                    if (z - z0 < Zc) out[(size_t)y * nz + z] = acc[k][j];
                }
            }
        }
    }
}

// ------------------------------------------------------------- without PSF
// One thread per output (y, z) of a chunk of planes; A read on the fly.
__global__ void __launch_bounds__(256)
    k_fwd_nopsf(SpectDev g, const float *__restrict__ f, const int *__restrict__ alist,
                int n_chunks, float *__restrict__ partials) {
    const int slot = blockIdx.y, chunk = blockIdx.x;
    const int ga = alist[slot];
    const int N = g.N, nz = g.nz;
    const int i = blockIdx.z * blockDim.x + threadIdx.x;
    if (i >= N * nz) return;
    const int y = i / nz, z = i % nz;
    float th[6];
#pragma unroll
    for (int k = 0; k < 6; k++) th[k] = g.theta_fwd[6 * ga + k];
    const float *A = g.att ? g.A + (size_t)ga * g.Lp * g.nya * nz : nullptr;
    const int yp = g.pad + y;
    const float lc = g.lin[yp];
    const int x0 = chunk * g.Lp / n_chunks, x1 = (chunk + 1) * g.Lp / n_chunks;
    float acc = 0.f;
    for (int xp = x0; xp < x1; ++xp) {
        float ix, iy;
        rot_coords(th, g.lin[xp], lc, g.half, ix, iy);
        Bilin b = bilin(ix, iy);
        float v = sample(f, N, N, nz, g.pad, g.pad, b, z);
        if (A) v = __fmul_rn(v, __ldg(A + ((size_t)xp * g.nya + (yp - g.ya_lo)) * nz + z));
        acc += v;
    }
    partials[((size_t)slot * n_chunks + chunk) * N * nz + i] = acc;
}

// --------------------------------------------------------------- reduction
// out[slot][i] = sum_c partials[slot][c][i] in chunk order.  With `ratio`,
// out = g[ga][i] / (sum + s[ga][i] + delta) and pred (optional) = sum + s.
__global__ void k_reduce(int n_chunks, int NZ, const float *__restrict__ partials,
                         float *__restrict__ out, int ratio, const float *__restrict__ gproj,
                         const float *__restrict__ sadd, const int *__restrict__ alist,
                         float *__restrict__ pred) {
    const int slot = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= NZ) return;
    const float *p = partials + (size_t)slot * n_chunks * NZ + i;
    float v = 0.f;
    for (int c = 0; c < n_chunks; c++) v += p[(size_t)c * NZ];
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

// ------------------------------------------------------------- launchers
size_t fwd_psf_smem_bytes(int K, int N, int Zt) {
    int H = K / 2, HP = (H + 3) / 4 * 4, OB = (K <= 31) ? 8 : 4;
    int N8 = (N + OB - 1) / OB * OB;
    int Z8 = (Zt + OB - 1) / OB * OB;
    return sizeof(float) *
           ((size_t)(N8 + 2 * H) * (Z8 + 2 * HP) + (size_t)(Z8 + 2 * HP) * (N8 + 1) + 4 * K);
}

template <int K>
static cudaError_t launch_fwd_psf_k(const SpectDev &g, const float *f, const int *alist,
                                    int n_slots, int n_chunks, int Zt, float *partials,
                                    cudaStream_t st) {
    size_t smem = fwd_psf_smem_bytes(K, g.N, Zt);
    dim3 grid(n_chunks, n_slots, (g.nz + Zt - 1) / Zt);
    if (g.nz % 4 == 0)
        k_fwd_psf<K, true><<<grid, 512, smem, st>>>(g, f, alist, n_chunks, Zt, partials);
    else
        k_fwd_psf<K, false><<<grid, 512, smem, st>>>(g, f, alist, n_chunks, Zt, partials);
    return cudaGetLastError();
}

template <int K>
static cudaError_t setup_fwd_k(size_t smem) {
    cudaError_t e = cudaFuncSetAttribute(k_fwd_psf<K, true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_fwd_psf<K, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem);
}

cudaError_t setup_fwd(int K, size_t smem) {
    switch (K) {
#define GB_SETUP_CASE(KK) \
    case KK:              \
        return setup_fwd_k<KK>(smem);
        GB_FOR_EACH_K(GB_SETUP_CASE)
#undef GB_SETUP_CASE
        default:
            return cudaErrorInvalidValue;
    }
}

cudaError_t launch_fwd(const SpectDev &g, const float *f, const int *alist, int n_slots,
                       int n_chunks, int Zt, float *partials, cudaStream_t st) {
    if (!g.psf) {
        dim3 grid(n_chunks, n_slots, (g.N * g.nz + 255) / 256);
        k_fwd_nopsf<<<grid, 256, 0, st>>>(g, f, alist, n_chunks, partials);
        return cudaGetLastError();
    }
    switch (g.K) {
#define GB_FWD_CASE(KK) \
    case KK:            \
        return launch_fwd_psf_k<KK>(g, f, alist, n_slots, n_chunks, Zt, partials, st);
        GB_FOR_EACH_K(GB_FWD_CASE)
#undef GB_FWD_CASE
        default:
            return cudaErrorInvalidValue;
    }
}

cudaError_t launch_reduce(int n_slots, int n_chunks, int NZ, const float *partials, float *out,
                          int ratio, const float *gproj, const float *sadd, const int *alist,
                          float *pred, cudaStream_t st) {
    dim3 grid((NZ + 255) / 256, n_slots);
    k_reduce<<<grid, 256, 0, st>>>(n_chunks, NZ, partials, out, ratio, gproj, sadd, alist, pred);
    return cudaGetLastError();
}

}  // namespace gb
