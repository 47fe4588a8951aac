// Fused SPECT forward projector, second variant: attenuation before a 2-D PSF, one z slab
// (N <= 128, nz <= 128, nz % 4 == 0), 512 threads.  Same operator as k_fwd_psf (rotate ->
// attenuate -> depth-dependent separable PSF -> ray sum, projectors/SPECT/
// spect_system_matrix.py:145-154 with transforms/SPECT/attenuation.py:72-92 and
// transforms/SPECT/psf.py:27-41); the two 1-D blurs of a plane are applied z first, then
// y (separable, so the same operator up to float rounding).
//
// Per plane x of the work item:
//   phase A  every warp takes the plane's sampled rows y = ra + warp, ra + warp + 16, ...
//            For each row the four bilinear corner rows of the object and the plane's
//            attenuation row are copied global -> shared by cp.async (16 bytes per lane
//            and row, zero-filled outside the object) into a ring of kRing slots per warp,
//            issued kRing rows ahead of use (across plane boundaries), so the L2 / DRAM
//            latency of the gather is hidden behind the arithmetic of earlier rows.  The
//            lane that copied a z quad combines it (bilinear weights, times A), the row is
//            blurred along z from a per-warp row buffer, and written to Sz[y][z].
//   phase B  after a CTA barrier every warp blurs Sz along y for its RPW output rows and
//            adds the result to the ray sums held in registers (packed f32x2 FMAs over
//            z pairs).
// Shared memory: Sz [N + 2H][nz], ring [16][kRing][5][nz], row buffers [16][nz + 2 HP],
// taps [2][2][K].  No transposition buffer and no mbarrier: cp.async.wait_group waits on
// the thread's own copies, which always complete.
#pragma once
#include "spect_blur.cuh"
#include "spect_kernels.cuh"
#include "spect_launch.h"

namespace gb {

constexpr int kRing = 3;       // rows in flight per warp
constexpr int kFwd2MaxK = 29;  // tap buckets the variant is compiled for

__device__ __forceinline__ void cp_async16(void *dst, const void *src, bool valid) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)), "l"(src),
                 "r"(valid ? 16 : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
    asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int NPEND>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(NPEND) : "memory");
}

__host__ __device__ constexpr int fwd2_halo(int K) { return (K / 2 + 3) / 4 * 4; }

// shared-memory floats of the variant for N rows and nz z values
__host__ __device__ inline size_t fwd2_smem_floats(int K, int N, int nz) {
    const int H = K / 2, HP = fwd2_halo(K);
    return (size_t)(N + 2 * H) * nz + (size_t)16 * kRing * 5 * nz + (size_t)16 * (nz + 2 * HP) +
           4 * K;
}

// Per-warp cursor over the (plane, row) stream of a work item: the warp's rows of every
// plane with samples, in plane order.
struct RowCursor {
    int xp, y, rb;  // current plane, row, last sampled row of the plane; xp == x1: done
};

template <int K, int RPW>
__global__ void __launch_bounds__(512, 1)
    k_fwd_psf2(SpectDev g, const float *__restrict__ f, const int *__restrict__ alist,
               const int4 *__restrict__ items, float *__restrict__ partials) {
    constexpr int H = K / 2, HP = fwd2_halo(K);
    const int4 item = items[blockIdx.x];  // (slot, first plane, end plane)
    const int ga = alist[item.x];
    const int x0 = item.y, x1 = item.z;
    const int N = g.N, nz = g.nz, nq = nz >> 2;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool qok = lane < nq;
    const int z = 4 * lane;
    const int SR = N + 2 * H, RBW = nz + 2 * HP;
    extern __shared__ __align__(16) float sm[];
    float *Sz = sm;                                    // [SR][nz], row i <-> y = pad - H + i
    float *ring = Sz + (size_t)SR * nz;                // [16][kRing][5][nz]
    float *rowb = ring + (size_t)16 * kRing * 5 * nz;  // [16][RBW]
    float *tp = rowb + 16 * RBW;                       // [2][2][K]
    for (int i = threadIdx.x; i < SR * nz + 16 * RBW; i += 512)
        (i < SR * nz ? Sz[i] : rowb[i - SR * nz]) = 0.f;
    float th[6];
#pragma unroll
    for (int k = 0; k < 6; k++) th[k] = g.theta_fwd[6 * ga + k];
    const int grp = g.group[ga];
    const float *A = g.A + (size_t)ga * g.Lp * g.nya * nz;
    const int ylo = max(0, g.pad - H), yhi = min(g.Lp, g.pad + N + H);
    float *myring = ring + (size_t)warp * kRing * 5 * nz;
    float *myrow = rowb + warp * RBW;
    float4 acc[RPW];
#pragma unroll
    for (int j = 0; j < RPW; j++) acc[j] = make_float4(0.f, 0.f, 0.f, 0.f);

    // the next plane with samples from xp on, rows [ra, rb]
    auto next_plane = [&](int xp, int &ra, int &rb) {
        for (; xp < x1; ++xp)
            if (plane_rows(g, th, xp, ylo, yhi, 0.5f, ra, rb)) return xp;
        return x1;
    };
    // move a cursor to the warp's first row from plane xp on
    auto cursor_first = [&](int xp, RowCursor &c) {
        for (;;) {
            int ra = 0, rb = -1;
            xp = next_plane(xp, ra, rb);
            c.xp = xp;
            if (xp >= x1) return;
            c.y = ra + warp;
            c.rb = rb;
            if (c.y <= rb) return;
            ++xp;  // this warp has no row in the plane
        }
    };
    auto cursor_next = [&](RowCursor &c) {
        c.y += 16;
        if (c.y > c.rb) cursor_first(c.xp + 1, c);
    };
    // issue the copies of the cursor's row into ring slot s (an empty group when done)
    auto issue = [&](const RowCursor &c, int s) {
        if (c.xp < x1 && qok) {
            float ix, iy;
            rot_coords(th, g.lin[c.xp], g.lin[c.y], g.half, ix, iy);
            const int r0 = (int)floorf(iy) - g.pad, c0 = (int)floorf(ix) - g.pad;
            float *dst = myring + (size_t)s * 5 * nz + z;
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int rr = r0 + (q >> 1), cc = c0 + (q & 1);
                const bool in = (unsigned)rr < (unsigned)N && (unsigned)cc < (unsigned)N;
                cp_async16(dst + q * nz, in ? f + ((size_t)rr * N + cc) * nz + z : f, in);
            }
            cp_async16(dst + 4 * nz, A + ((size_t)c.xp * g.nya + (c.y - g.ya_lo)) * nz + z,
                       true);
        }
        cp_async_commit();
    };

    RowCursor ic;  // issue cursor, kRing rows ahead of consumption
    cursor_first(x0, ic);
    int n_issued = 0;
    for (int k = 0; k < kRing; k++) {
        issue(ic, n_issued % kRing);
        ++n_issued;
        if (ic.xp < x1) cursor_next(ic);
    }
    int n_used = 0;
    int pra = 0, prb = -1;  // rows written in Sz by the previous plane
    int parity = 0;
    int ra = 0, rb = -1;
    int xp = next_plane(x0, ra, rb);
    while (xp < x1) {
        float *tap = tp + parity * 2 * K;
        if (threadIdx.x < K) {
            tap[threadIdx.x] = g.taps_r[((size_t)grp * g.Lp + xp) * g.K + threadIdx.x];
            tap[K + threadIdx.x] = g.taps_z[((size_t)grp * g.Lp + xp) * g.K + threadIdx.x];
        }
        __syncthreads();  // taps visible; every warp is done with the previous plane's Sz
        // clear the previous plane's rows this plane does not write
        for (int y = pra + warp; y <= prb; y += 16) {
            if (y >= ra && y <= rb) continue;
            if (qok)
                *reinterpret_cast<float4 *>(Sz + (size_t)(y - (g.pad - H)) * nz + z) =
                    make_float4(0.f, 0.f, 0.f, 0.f);
        }
        const int tier = g.tier ? g.tier[grp * g.Lp + xp] : kTiers - 1;
        // ---- phase A: the warp's rows of this plane
        const float lr = g.lin[xp];
        tier_dispatch<K>(tier, [&](auto kk) {
            constexpr int KK = decltype(kk)::value, OFF = (K - KK) / 2;
            float wz[KK];
            load_taps<K, KK>(tap + K, wz);
            for (int y = ra + warp; y <= rb; y += 16) {
                cp_async_wait<kRing - 1>();  // the oldest row (this one) has landed
                const int s = n_used % kRing;
                ++n_used;
                float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                if (qok) {
                    float ix, iy;
                    rot_coords(th, lr, g.lin[y], g.half, ix, iy);
                    const Bilin b = bilin(ix, iy);
                    const float *src = myring + (size_t)s * 5 * nz + z;
                    const float4 vnw = *reinterpret_cast<const float4 *>(src);
                    const float4 vne = *reinterpret_cast<const float4 *>(src + nz);
                    const float4 vsw = *reinterpret_cast<const float4 *>(src + 2 * nz);
                    const float4 vse = *reinterpret_cast<const float4 *>(src + 3 * nz);
                    const float4 a = *reinterpret_cast<const float4 *>(src + 4 * nz);
                    v.x = bilin_combine(b, vnw.x, vne.x, vsw.x, vse.x);
                    v.y = bilin_combine(b, vnw.y, vne.y, vsw.y, vse.y);
                    v.z = bilin_combine(b, vnw.z, vne.z, vsw.z, vse.z);
                    v.w = bilin_combine(b, vnw.w, vne.w, vsw.w, vse.w);
                    v = mul4(v, a);
                }
                // the slot is free again (each lane reads only its own copies): refill it
                issue(ic, s);
                ++n_issued;
                if (ic.xp < x1) cursor_next(ic);
                __syncwarp();  // the previous row's readers of the row buffer are done
                if (qok) *reinterpret_cast<float4 *>(myrow + HP + z) = v;
                __syncwarp();
                if (qok) {
                    // window z - HP .. z + 3 + HP of the row (zeros beyond [0, nz))
                    float win[4 + 2 * HP];
#pragma unroll
                    for (int i = 0; i < 1 + 2 * HP / 4; i++) {
                        const float4 t4 = *reinterpret_cast<const float4 *>(myrow + z + 4 * i);
                        win[4 * i] = t4.x;
                        win[4 * i + 1] = t4.y;
                        win[4 * i + 2] = t4.z;
                        win[4 * i + 3] = t4.w;
                    }
                    float o[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
                    for (int t = 0; t < KK; t++)
#pragma unroll
                        for (int j = 0; j < 4; j++)
                            o[j] = fmaf(wz[t], win[HP - H + OFF + t + j], o[j]);
                    *reinterpret_cast<float4 *>(Sz + (size_t)(y - (g.pad - H)) * nz + z) =
                        make_float4(o[0], o[1], o[2], o[3]);
                }
            }
        });
        __syncthreads();  // Sz complete for this plane
        // ---- phase B: y blur of the warp's output rows into the ray sums
        const int o_lo = max(0, ra - H - g.pad), o_hi = min(N, rb + H - g.pad + 1);
        const int w0 = RPW * warp;
        if (qok && w0 < o_hi && w0 + RPW > o_lo) {
            tier_dispatch<K>(tier, [&](auto kk) {
                constexpr int KK = decltype(kk)::value, OFF = (K - KK) / 2;
                float wy[KK];
                load_taps<K, KK>(tap, wy);
                // Sz row w0 + OFF + t feeds output w0 + j with tap t - j
#pragma unroll
                for (int t = 0; t < RPW + KK - 1; t++) {
                    const int i = w0 + OFF + t;
                    const float4 r4 = *reinterpret_cast<const float4 *>(Sz + (size_t)i * nz + z);
                    const float2 lo = make_float2(r4.x, r4.y), hi = make_float2(r4.z, r4.w);
#pragma unroll
                    for (int j = 0; j < RPW; j++) {
                        const int tt = t - j;
                        if (tt < 0 || tt >= KK) continue;
                        const float2 w2 = make_float2(wy[tt], wy[tt]);
                        float2 a01 = make_float2(acc[j].x, acc[j].y);
                        float2 a23 = make_float2(acc[j].z, acc[j].w);
                        a01 = __ffma2_rn(w2, lo, a01);
                        a23 = __ffma2_rn(w2, hi, a23);
                        acc[j] = make_float4(a01.x, a01.y, a23.x, a23.y);
                    }
                }
            });
        }
        pra = ra;
        prb = rb;
        parity ^= 1;
        xp = next_plane(xp + 1, ra, rb);
    }
    cp_async_wait<0>();  // nothing of this CTA stays in flight
    float *out = partials + (size_t)blockIdx.x * N * nz;
    if (qok) {
#pragma unroll
        for (int j = 0; j < RPW; j++) {
            const int y = RPW * warp + j;
            if (y < N) *reinterpret_cast<float4 *>(out + (size_t)y * nz + z) = acc[j];
        }
    }
}

template <int K>
inline cudaError_t setup_fwd2_t() {
    const int smem = (int)(fwd2_smem_floats(K, 128, 128) * sizeof(float));
    cudaError_t e = cudaFuncSetAttribute(k_fwd_psf2<K, 8>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_fwd_psf2<K, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                smem);
}

template <int K>
inline cudaError_t launch_fwd2_t(const SpectDev &g, const float *f, const int *alist,
                                 const int4 *items, int n_items, float *partials,
                                 cudaStream_t st) {
    const size_t smem = fwd2_smem_floats(K, g.N, g.nz) * sizeof(float);
    if (g.N <= 64)
        k_fwd_psf2<K, 4><<<n_items, 512, smem, st>>>(g, f, alist, items, partials);
    else
        k_fwd_psf2<K, 8><<<n_items, 512, smem, st>>>(g, f, alist, items, partials);
    return cudaGetLastError();
}

}  // namespace gb
