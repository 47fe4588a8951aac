// Fused SPECT forward projector with PSF (rotate -> attenuate -> depth-dependent PSF -> ray
// sum): the kernel template, instantiated per PSF tap bucket in spect_fwd_k*.cu.
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
#pragma once
#include "spect_blur.cuh"
#include "spect_kernels.cuh"
#include "spect_fwd_v2.cuh"
#include "spect_launch.h"

namespace gb {

#ifdef GB_PHASE_TIMING
// Per-warp cycle counts of the forward kernel's phases (diagnostic builds only, written to
// g.phase[(CTA * warps + warp) * 16 + k] when set): [0] waits for the attenuation copy,
// [1] phase 1 work, [2] wait at the barrier after phase 1, [3] phase 2 work, [4] wait at
// the barrier after phase 2, [5] phase 3 work (with the next plane's copy issue),
// [6] planes processed, [7] total, [8] rows sampled, [9] output rows x taps, [10] planes
// of the work item.
#define GB_T(k, v)                                              \
    do {                                                        \
        if ((threadIdx.x & 31) == 0) tacc[k] += (v);            \
    } while (0)
#define GB_NOW() clock64()
#else
#define GB_T(k, v) \
    do {           \
        (void)(v); \
    } while (0)
#define GB_NOW() 0LL
#endif

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
//                z quads; SC a multiple of 32: 128-byte aligned rows).  Before phase 1 of
//                a plane, the attenuation rows of that plane are copied into S by 2-D TMA
//                boxes of kBoxRows full S rows (`tmA`: A viewed as [n_angles*Lp*nya][nz],
//                z outside [0, nz) reads as zero; one 1-D bulk copy per row instead when a
//                row is wider than a box, SC > 256) and multiplied in place.
//   Tt [TR][TS]: y-blurred plane, transposed; row c <-> z = z0 - HP + c, column = output y
//                (TS even with 512 threads: float2 row pairs)
//   taps [2][2][K]: double-buffered y / z taps of the current plane
//   one mbarrier for the TMA copies
// Per plane only the rows the rotated object square can reach are sampled / blurred.
// FIXED: the tile fits 128 output rows and a z slab of at most ZW = 128, so the
// shared-memory row strides are compile-time constants (immediate-offset loads in the
// blur loops).
// TPB: 512 threads (16 warps), or 768 threads (24 warps: more rows of the gather in flight
// per SM; the taps are read from shared memory to fit the smaller register budget).  One
// CTA per SM either way.
// One work item: planes [x0_, x1_) of angle ga for the z slab starting at z0; the item's
// partial ray sums go to out ([N][nz]).  Called once per CTA by k_fwd_psf and once per
// dequeued item by the persistent batch kernel.  Returns true when this thread's bounded
// wait gave up (the plan's error word is then set).
template <int K, bool VEC, bool FIXED, int TPB>
__device__ __forceinline__ bool fwd_psf_item(const SpectDev &g, const float *__restrict__ f,
                                             const int ga, const int x0_, const int x1_,
                                             const int z0, const int Zt, float *__restrict__ out,
                                             const CUtensorMap *tmA, unsigned long long *bar) {
    constexpr int H = K / 2;
    constexpr int ZW = 128;
    constexpr bool TAPS_SMEM = TPB > 512;
    constexpr int HP = (H + 3) / 4 * 4;
    constexpr int OB = (K <= 31) ? 8 : 4;  // outputs per task
    // phase-3 tasks per thread.  512 threads: a task owns a pair of output rows (y, y + 1)
    // and blurs both with packed f32x2 FMAs, 2 (OB = 8) or 4 tasks; 768 threads: one row
    // per task, 3 or 6 tasks
    constexpr bool PAIR = !TAPS_SMEM;
    constexpr int NT = PAIR ? 16 / OB : (OB == 8 ? 3 : 6);
    using Acc = std::conditional_t<PAIR, float2, float>;
    const int N = g.N, nz = g.nz;
    const int Zc = min(Zt, nz - z0);
    const int N8 = (N + OB - 1) / OB * OB;
    const int Z8 = (Zc + OB - 1) / OB * OB;
    // Tt row stride: odd for scalar access (conflict-free columns), even for float2 pairs
    constexpr int SC_FIX = fwd_s_cols(ZW, HP), TS_FIX = PAIR ? 130 : 129;
    const int SC = FIXED ? SC_FIX : fwd_s_cols((Zt + OB - 1) / OB * OB, HP), SR = N8 + 2 * H;
    const int TS = FIXED ? TS_FIX : N8 + (PAIR ? 2 : 1), TR = Z8 + 2 * HP;
    extern __shared__ __align__(128) float sm[];
    float *S = sm;
    float *Tt = S + SR * SC;
    float *tp = Tt + TR * TS;
    for (int i = threadIdx.x; i < SR * SC + TR * TS; i += TPB) sm[i] = 0.f;

    float th[6];
#pragma unroll
    for (int k = 0; k < 6; k++) th[k] = g.theta_fwd[6 * ga + k];
    const int grp = g.group[ga];
    const float *A = g.att ? g.A + (size_t)ga * g.Lp * g.nya * nz : nullptr;
    const bool amul = A && g.att_first;
    const bool use_tma = VEC && amul;
    const bool tma_box = SC <= 256;  // 2-D boxes (else one 1-D copy per row)
    const int x0 = x0_, x1 = x1_;
    const int zv_lo = max(0, z0 - H), zv_hi = min(nz, z0 + Zc + H);  // z needed by the blur
    const int cz_lo = zv_lo - z0 + HP, cz_hi = zv_hi - z0 + HP;
    const int ncol = cz_hi - cz_lo;
    const int ylo = max(0, g.pad - H), yhi = min(g.Lp, g.pad + N + H);  // sampled rows
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int nwarp = TPB / 32;
    const int zq_lo = zv_lo & ~3, zq_hi = (zv_hi + 3) & ~3;  // z quads (vector path)
    const int nq = (zq_hi - zq_lo) >> 2;
    const unsigned row_bytes = (unsigned)(zq_hi - zq_lo) * 4u;
    const int qcol0 = zq_lo - z0 + HP;  // S column of the first quad
    if (threadIdx.x == 0 && use_tma) mbar_init(bar, 1);
    Acc acc[NT][OB];
    int ty[NT], tz[NT];  // phase-3 task (output row or first row of a pair, z block)
    // each warp owns whole z blocks and, for them, every 32-row chunk: restricting a
    // plane's rows removes the same share of work from every warp
    // (falls back to a linear task order when the rows need more chunks than tasks)
    if constexpr (TPB > 512) {
        // linear warp-task order: task t = warp + nwarp k -> (32-row chunk t % n_yc, z block
        // t / n_yc); the plan caps the slab so that every task has a thread
        const int n_yc = (N8 + 31) >> 5, n_task = n_yc * (Z8 / OB);
#pragma unroll
        for (int k = 0; k < NT; k++) {
            const int t = warp + nwarp * k;
            ty[k] = 32 * (t % n_yc) + lane;
            tz[k] = t / n_yc;
            if (t >= n_task || ty[k] >= N8) tz[k] = 1 << 20;  // no task
#pragma unroll
            for (int j = 0; j < OB; j++) acc[k][j] = Acc{};
        }
    } else {
        // row pairs: lanes take consecutive pairs of a 64-row chunk
        const int n_yc = (N8 + 63) >> 6;
        const bool balanced = n_yc <= NT;
#pragma unroll
        for (int k = 0; k < NT; k++) {
            if (balanced) {
                ty[k] = 64 * (k % n_yc) + 2 * lane;
                tz[k] = warp + nwarp * (k / n_yc);
                if (ty[k] >= N8 || k / n_yc >= NT / n_yc) tz[k] = 1 << 20;  // no task
            } else {
                const int np = N8 >> 1;  // row pairs per z block
                const int task = threadIdx.x + k * TPB;
                ty[k] = 2 * (task % np);
                tz[k] = task / np;
            }
#pragma unroll
            for (int j = 0; j < OB; j++) acc[k][j] = Acc{};
        }
    }
    __syncthreads();

    bool failed = false;  // this thread's bounded wait gave up
    unsigned failed_phase = 0;
    // next plane with any sample on the object, from xp on; rows in [ra, rb]
    auto next_plane = [&](int xp, int &ra, int &rb) {
        for (; xp < x1; ++xp)
            if (plane_rows(g, th, xp, ylo, yhi, 0.5f, ra, rb)) return xp;
        return x1;
    };
    // copy the attenuation rows [ra, rb] of plane xp into S (warp 0).  Boxes start at ra,
    // ra + kBoxRows, ...; the last one ends at rb, or starts at ylo when the range is
    // shorter than a box, so the rows written are [fa, fb] (rows outside [ra, rb] are
    // cleared in phase 1).
    auto issue_tma = [&](int xp, int ra, int rb, int &fa, int &fb) {
        const int nbox = (rb - ra + kBoxRows) / kBoxRows;
        const int last = max(ylo, rb - (kBoxRows - 1));
        fa = ra;
        fb = rb;
        if (tma_box) {
            fa = min(ra, last);
            fb = max(rb, last + kBoxRows - 1);
        }
        if (warp != 0 || __any_sync(0xffffffffu, failed)) return;
        if (lane == 0) {
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(bar, tma_box ? (unsigned)(nbox * kBoxRows * SC) * 4u
                                               : row_bytes * (unsigned)(rb - ra + 1));
        }
        __syncwarp();
        if (tma_box) {
            const int row0 = (ga * g.Lp + xp) * g.nya - g.ya_lo;  // tensor row of y = 0
            for (int k = lane; k < nbox; k += 32) {
                const int ys = min(ra + k * kBoxRows, last);
                tma_load_2d(S + (ys - (g.pad - H)) * SC, tmA, z0 - HP, row0 + ys, bar);
            }
        } else {
            const float *src = A + ((size_t)xp * g.nya + (ra - g.ya_lo)) * nz + zq_lo;
            for (int y = ra + lane; y <= rb; y += 32)
                tma_load_1d(S + (y - (g.pad - H)) * SC + qcol0, src + (size_t)(y - ra) * nz,
                            row_bytes, bar);
        }
    };

    int ra = 0, rb = -1, pra = 0, prb = -1;  // current and previous sampled rows
    int fa = 0, fb = -1;                      // rows the attenuation copy wrote
    int xp = next_plane(x0, ra, rb);
    // (the test hook dbg_skip_first_copy leaves the first copy unissued: the bounded wait
    // below then gives up, flags the plan and the kernel returns without output)
    if (use_tma && xp < x1 && !g.dbg_skip_first_copy) issue_tma(xp, ra, rb, fa, fb);
    int parity = 0;
    unsigned phase = 0;
#ifdef GB_PHASE_TIMING
    unsigned long long tacc[16] = {};
    const long long t_start = clock64();
    tacc[10] = x1 - x0;
#endif
    long long t0 = GB_NOW();
    while (xp < x1) {
        t0 = GB_NOW();
        const float lr = g.lin[xp];
        float *tap = tp + parity * 2 * K;
        if (threadIdx.x < K) {
            tap[threadIdx.x] = g.taps_r[((size_t)grp * g.Lp + xp) * g.K + threadIdx.x];
            tap[K + threadIdx.x] =
                g.psf2d ? g.taps_z[((size_t)grp * g.Lp + xp) * g.K + threadIdx.x] : 0.f;
        }
        if (use_tma) {
            // A thread whose bounded wait gives up flags the plan and stops waiting (its
            // results are invalid); every thread still reaches every barrier.
            if (!failed && !mbar_wait_bounded(bar, phase, g.wait_polls)) {
                failed = true;
                failed_phase = phase;
                if (g.err) atomicExch(g.err, GB_ERR_WAIT_TIMEOUT);
            }
            phase ^= 1u;
        }
        {
            long long t1 = GB_NOW();
            GB_T(0, t1 - t0);
            t0 = t1;
        }
        // phase 1: rotated samples of rows [ra, rb] (times A when attenuation precedes
        // the PSF); stale rows of the previous plane are cleared
        const float *Ap = A ? A + (size_t)xp * g.nya * nz : nullptr;
        if (VEC) {
            // clear the sampled quads of rows outside [ra, rb]: the previous plane's rows
            // and the rows the box copy wrote beyond the range
            for (int y = pra + warp; y <= prb; y += nwarp) {
                if (y >= ra && y <= rb) continue;
                float *Sr = S + (y - (g.pad - H)) * SC + qcol0;
                for (int q = lane; q < nq; q += 32)
                    *reinterpret_cast<float4 *>(Sr + 4 * q) = make_float4(0.f, 0.f, 0.f, 0.f);
            }
            for (int y = fa + warp; y <= fb; y += nwarp) {
                if (y >= ra && y <= rb) continue;
                float *Sr = S + (y - (g.pad - H)) * SC + qcol0;
                for (int q = lane; q < nq; q += 32)
                    *reinterpret_cast<float4 *>(Sr + 4 * q) = make_float4(0.f, 0.f, 0.f, 0.f);
            }
            // RB = 2 consecutive rows per warp and batch: neighbouring rows share about half
            // of their bilinear taps, which then hit in L1.  (Four rows per batch keep more
            // loads in flight but leave too few registers for the blur passes: slower.)
            constexpr int RB = 2;
            for (int y0 = ra + RB * warp; y0 <= rb; y0 += RB * nwarp) {
                int ys[RB];
                bool okr[RB];
                Bilin b[RB];
#pragma unroll
                for (int u = 0; u < RB; u++) {
                    ys[u] = y0 + u;
                    okr[u] = ys[u] <= rb;
                    float ix, iy;
                    rot_coords(th, lr, g.lin[okr[u] ? ys[u] : y0], g.half, ix, iy);
                    b[u] = bilin(ix, iy);
                }
                for (int q = lane; q < nq; q += 32) {
                    const int z = zq_lo + 4 * q;
                    float4 v[RB];
                    bool h[RB];
#pragma unroll
                    for (int u = 0; u < RB; u++)
                        h[u] = okr[u] && sample4(f, N, N, nz, g.pad, g.pad, b[u], z, v[u]);
#pragma unroll
                    for (int u = 0; u < RB; u++) {
                        if (!okr[u]) continue;
                        float4 *dst = reinterpret_cast<float4 *>(
                            S + (ys[u] - (g.pad - H)) * SC + qcol0 + 4 * q);
                        float4 o = v[u];
                        if (amul) {
                            float4 a = use_tma ? *dst
                                               : (h[u] ? __ldg(reinterpret_cast<const float4 *>(
                                                             Ap + (size_t)(ys[u] - g.ya_lo) * nz + z))
                                                       : make_float4(0.f, 0.f, 0.f, 0.f));
                            o = mul4(o, a);
                        }
                        *dst = h[u] ? o : make_float4(0.f, 0.f, 0.f, 0.f);
                    }
                }
            }
        } else {
            for (int i = threadIdx.x; i < (yhi - ylo) * ncol; i += TPB) {
                int y = ylo + i / ncol, c = cz_lo + i % ncol;
                int z = z0 - HP + c;
                float v = 0.f;
                if (y >= ra && y <= rb) {
                    float ix, iy;
                    rot_coords(th, lr, g.lin[y], g.half, ix, iy);
                    Bilin bb = bilin(ix, iy);
                    v = sample(f, N, N, nz, g.pad, g.pad, bb, z);
                    if (amul && v != 0.f) v = __fmul_rn(v, Ap[(size_t)(y - g.ya_lo) * nz + z]);
                }
                S[(y - (g.pad - H)) * SC + c] = v;
            }
        }
        {
            long long t1 = GB_NOW();
            GB_T(1, t1 - t0);
            t0 = t1;
        }
        __syncthreads();
        {
            long long t1 = GB_NOW();
            GB_T(2, t1 - t0);
            t0 = t1;
        }
        // output rows (local y in [0, N)) that the blurred plane can reach
        const int o_lo = max(0, ra - H - g.pad), o_hi = min(N, rb + H - g.pad + 1);
        const int b_lo = o_lo / OB, b_hi = (o_hi + OB - 1) / OB;
        // phase 2: blur along y, write transposed (tap tier of the plane; taps read from
        // shared memory, which leaves the registers to the packed windows)
        int tier = kTiers - 1;
        if constexpr (FIXED) tier = g.tier ? g.tier[grp * g.Lp + xp] : kTiers - 1;
        tier_dispatch<K>(tier, [&](auto kk) {
            constexpr int KK = decltype(kk)::value;
            if constexpr (TAPS_SMEM)
                blur_first_st<K, KK, OB>(S, Tt, tap, SC, TS, cz_lo, cz_hi, b_lo, b_hi, warp, lane,
                                         nwarp);
            else
                blur_first2_st<K, KK, OB>(S, Tt, tap, SC, TS, cz_lo, cz_hi, b_lo, b_hi, warp,
                                          lane, nwarp);
        });
        GB_T(8, rb - ra + 1);
        GB_T(9, (b_hi - b_lo) * OB * tier_taps(K, tier));
        {
            long long t1 = GB_NOW();
            GB_T(3, t1 - t0);
            t0 = t1;
        }
        __syncthreads();
        {
            long long t1 = GB_NOW();
            GB_T(4, t1 - t0);
            t0 = t1;
        }
        // S is free until the next phase 1: start the next plane's attenuation copy
        pra = ra;
        prb = rb;
        int nra = 0, nrb = -1, nfa = 0, nfb = -1;
        const int nxp = next_plane(xp + 1, nra, nrb);
        if (use_tma && nxp < x1) issue_tma(nxp, nra, nrb, nfa, nfb);
        // phase 3: blur along z (2D PSF), optional attenuation after the PSF, accumulate
        {
            const int y_lo = b_lo * OB, y_hi = b_hi * OB;
            // attenuation after the PSF multiplies the blurred plane before accumulation;
            // otherwise the z blur accumulates straight into the ray sums
            const bool post_att = Ap && !g.att_first;
            tier_dispatch<K>(tier, [&](auto kk) {
                constexpr int KK = decltype(kk)::value;
                if constexpr (PAIR) {
                    float w[KK];
                    load_taps<K, KK>(tap + K, w);
#pragma unroll
                    for (int k = 0; k < NT; k++) {
                        const int y = ty[k], zb = tz[k];  // rows y, y + 1 (y_lo, y_hi even)
                        if (zb * OB < Z8 && y >= y_lo && y < y_hi) {
                            if (g.psf2d && !post_att) {
                                blur_second2<K, KK, OB, true>(Tt, w, TS, zb * OB + HP - H, y,
                                                              acc[k]);
                                continue;
                            }
                            float2 o[OB];
                            if (g.psf2d) {
                                blur_second2<K, KK, OB, false>(Tt, w, TS, zb * OB + HP - H, y, o);
                            } else {
#pragma unroll
                                for (int j = 0; j < OB; j++)
                                    o[j] = *reinterpret_cast<const float2 *>(
                                        Tt + (zb * OB + j + HP) * TS + y);
                            }
                            if (post_att) {
#pragma unroll
                                for (int j = 0; j < OB; j++) {
                                    const int z = z0 + zb * OB + j;
                                    if (z >= nz) continue;
                                    const float *Az = Ap + (size_t)(g.pad + y - g.ya_lo) * nz + z;
                                    if (y < N) o[j].x = __fmul_rn(o[j].x, Az[0]);
                                    if (y + 1 < N) o[j].y = __fmul_rn(o[j].y, Az[nz]);
                                }
                            }
#pragma unroll
                            for (int j = 0; j < OB; j++) {
                                acc[k][j].x += o[j].x;
                                acc[k][j].y += o[j].y;
                            }
                        }
                    }
                } else {  // 768 threads: one output row per task, taps from shared memory
#pragma unroll
                    for (int k = 0; k < NT; k++) {
                        const int y = ty[k], zb = tz[k];
                        if (zb * OB < Z8 && y >= y_lo && y < y_hi) {
                            if (g.psf2d && !post_att) {
                                blur_second_st<K, KK, OB, true>(Tt, tap + K, TS, zb * OB + HP - H,
                                                                y, acc[k]);
                                continue;
                            }
                            float o[OB];
                            if (g.psf2d) {
                                blur_second_st<K, KK, OB, false>(Tt, tap + K, TS, zb * OB + HP - H,
                                                                 y, o);
                            } else {
#pragma unroll
                                for (int j = 0; j < OB; j++) o[j] = Tt[(zb * OB + j + HP) * TS + y];
                            }
                            if (post_att && y < N) {
#pragma unroll
                                for (int j = 0; j < OB; j++) {
                                    const int z = z0 + zb * OB + j;
                                    if (z < nz)
                                        o[j] = __fmul_rn(o[j],
                                                         Ap[(size_t)(g.pad + y - g.ya_lo) * nz + z]);
                                }
                            }
#pragma unroll
                            for (int j = 0; j < OB; j++) acc[k][j] += o[j];
                        }
                    }
                }
            });
        }
        {
            long long t1 = GB_NOW();
            GB_T(5, t1 - t0);
            GB_T(6, 1);
        }
        parity ^= 1;
        xp = nxp;
        ra = nra;
        rb = nrb;
        fa = nfa;
        fb = nfb;
    }
    if (failed) mbar_wait_bounded(bar, failed_phase, g.wait_polls);
#ifdef GB_PHASE_TIMING
    const int trow = (blockIdx.x * gridDim.y + blockIdx.y) * nwarp + warp;
    if (g.phase && lane == 0 && trow < 4096) {
        tacc[7] = clock64() - t_start;
        for (int k = 0; k < 16; k++) g.phase[trow * 16 + k] = tacc[k];
    }
#endif
    // partial ray sums of this item
#pragma unroll
    for (int k = 0; k < NT; k++) {
        const int y = ty[k], zb = tz[k];
        if (zb * OB < Z8 && y < N) {
#pragma unroll
            for (int j = 0; j < OB; j++) {
                int z = z0 + zb * OB + j;
                if (z - z0 >= Zc) continue;
                if constexpr (PAIR) {
                    out[(size_t)y * nz + z] = acc[k][j].x;
                    if (y + 1 < N) out[(size_t)(y + 1) * nz + z] = acc[k][j].y;
                } else {
                    out[(size_t)y * nz + z] = acc[k][j];
                }
            }
        }
    }
    return failed;
}

// One CTA per (work item, z slab) of one plan.
template <int K, bool VEC, bool FIXED, int TPB>
__global__ void __launch_bounds__(TPB, 1)
    k_fwd_psf(SpectDev g, const float *__restrict__ f, const int *__restrict__ alist,
              const int4 *__restrict__ items, int Zt, float *__restrict__ partials,
              const __grid_constant__ CUtensorMap tmA) {
    __shared__ unsigned long long bar;  // completion of the attenuation copies
    const int4 item = items[blockIdx.x];  // (slot, first plane, end plane)
    fwd_psf_item<K, VEC, FIXED, TPB>(g, f, alist[item.x], item.y, item.z, blockIdx.y * Zt, Zt,
                                     partials + (size_t)blockIdx.x * g.N * g.nz, &tmA, &bar);
}

// Persistent batch form: one CTA per SM dequeues work items of several reconstructions
// (or of several objects on one plan) from one list ordered by estimated cost, largest
// first.  Every entry uses 512 threads, 16-byte z quads and the fixed 128 x 128 tile
// (N <= 128, nz <= 128, one z slab).  The mbarrier is invalidated between items, when
// none of its copies is in flight.
template <int K>
__global__ void __launch_bounds__(512, 1) k_fwd_psf_batch(const __grid_constant__ FwdBatch p) {
    __shared__ unsigned long long bar;
    __shared__ int s_item, s_failed;
    if (threadIdx.x == 0) s_failed = 0;
    bool used = false;
    for (;;) {
        __syncthreads();  // the previous item is finished by every thread
        if (s_failed) return;  // a bounded wait gave up: stop dequeuing (error word is set)
        if (threadIdx.x == 0) {
            if (used) mbar_inval(&bar);
            s_item = atomicAdd(p.counter, 1);
        }
        __syncthreads();
        const int it = s_item;
        if (it >= p.n_items) return;
        const int4 item = p.items[it];  // (slot, first plane, end plane, entry)
        const int e = item.w;
        const SpectDev &g = p.g[e];
        if (fwd_psf_item<K, true, true, 512>(g, p.f[e], p.alist[e][item.x], item.y, item.z, 0,
                                             g.nz, p.partials + (size_t)it * p.nz_max, &p.tm[e],
                                             &bar))
            s_failed = 1;
        used = g.att && g.att_first;
    }
}

// ------------------------------------------------------------- launchers
inline bool fwd_fixed(int K, int N, int Zt, int tpb) {
    int OB = (K <= 31) ? 8 : 4;
    (void)tpb;
    return (N + OB - 1) / OB * OB <= 128 && (Zt + OB - 1) / OB * OB <= 128;
}

// Tensor map of the attenuation table for the kernel's box copies (spect_fwd.cu); s_cols
// is the kernel's S row length.  A zeroed map when the kernel makes no box copies.
cudaError_t make_att_tmap(const SpectDev &g, int s_cols, CUtensorMap *out);

template <int K, int TPB>
inline cudaError_t launch_fwd_psf_t(const SpectDev &g, const float *f, const int *alist,
                                    const int4 *items, int n_items, int Zt, float *partials,
                                    cudaStream_t st) {
    size_t smem = fwd_psf_smem_bytes(K, g.N, Zt, TPB);
    dim3 grid(n_items, (g.nz + Zt - 1) / Zt);
    const bool fx = fwd_fixed(K, g.N, Zt, TPB);
    constexpr int HP = (K / 2 + 3) / 4 * 4, OB = (K <= 31) ? 8 : 4;
    alignas(64) CUtensorMap tm;
    cudaError_t e = make_att_tmap(
        g, fx ? fwd_s_cols(128, HP) : fwd_s_cols((Zt + OB - 1) / OB * OB, HP), &tm);
    if (e != cudaSuccess) return e;
    if (g.nz % 4 == 0) {
        if (fx)
            k_fwd_psf<K, true, true, TPB><<<grid, TPB, smem, st>>>(g, f, alist, items, Zt, partials, tm);
        else
            k_fwd_psf<K, true, false, TPB><<<grid, TPB, smem, st>>>(g, f, alist, items, Zt, partials, tm);
    } else {
        if (fx)
            k_fwd_psf<K, false, true, TPB><<<grid, TPB, smem, st>>>(g, f, alist, items, Zt, partials, tm);
        else
            k_fwd_psf<K, false, false, TPB><<<grid, TPB, smem, st>>>(g, f, alist, items, Zt,
                                                                    partials, tm);
    }
    return cudaGetLastError();
}

template <int K, int TPB>
inline cudaError_t setup_fwd_t(size_t smem) {
    const void *fns[4] = {(const void *)k_fwd_psf<K, true, true, TPB>,
                          (const void *)k_fwd_psf<K, true, false, TPB>,
                          (const void *)k_fwd_psf<K, false, true, TPB>,
                          (const void *)k_fwd_psf<K, false, false, TPB>};
    for (const void *fn : fns) {
        cudaError_t e =
            cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// Entry points of one tap bucket KK (one per spect_fwd_k*.cu translation unit, so the
// buckets compile in parallel).
#define GB_FWD_PSF_INSTANCE(KK)                                                              \
    cudaError_t setup_fwd_psf_batch_##KK() {                                                 \
        return cudaFuncSetAttribute(k_fwd_psf_batch<KK>,                                     \
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,             \
                                    (int)fwd_psf_smem_bytes(KK, 128, 128, 512));             \
    }                                                                                        \
    cudaError_t launch_fwd_psf_batch_##KK(const FwdBatch &p, int grid, cudaStream_t st) {    \
        k_fwd_psf_batch<KK><<<grid, 512, fwd_psf_smem_bytes(KK, 128, 128, 512), st>>>(p);    \
        return cudaGetLastError();                                                          \
    }                                                                                        \
    cudaError_t launch_fwd_psf_##KK(const SpectDev &g, const float *f, const int *alist,     \
                                    const int4 *items, int n_items, int Zt, int tpb,         \
                                    float *partials, cudaStream_t st) {                     \
        return tpb <= 512                                                                    \
                   ? launch_fwd_psf_t<KK, 512>(g, f, alist, items, n_items, Zt, partials, st) \
                   : launch_fwd_psf_t<KK, 768>(g, f, alist, items, n_items, Zt, partials, st); \
    }                                                                                        \
    cudaError_t setup_fwd_##KK(size_t smem, int tpb) {                                       \
        return tpb <= 512 ? setup_fwd_t<KK, 512>(smem) : setup_fwd_t<KK, 768>(smem);         \
    }

// Entry points of the second forward variant for one tap bucket (spect_fwd_k*.cu, the
// buckets of GB_FOR_EACH_K2).
#define GB_FWD2_INSTANCE(KK)                                                                 \
    cudaError_t setup_fwd2_##KK() { return setup_fwd2_t<KK>(); }                             \
    cudaError_t launch_fwd2_##KK(const SpectDev &g, const float *f, const int *alist,        \
                                 const int4 *items, int n_items, float *partials,            \
                                 cudaStream_t st) {                                          \
        return launch_fwd2_t<KK>(g, f, alist, items, n_items, partials, st);                 \
    }

}  // namespace gb
