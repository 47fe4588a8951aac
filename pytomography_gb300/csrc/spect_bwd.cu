// SPECT back-projectors, attenuation precompute, OSEM/BSREM update epilogues and the
// relative-difference prior.
//
// Reference back-projector: SPECTSystemMatrix.backward
// (projectors/SPECT/spect_system_matrix.py:159-201): the projection row is broadcast
// along x inside the back-projection box (utils/spatial.py:75-79), the obj2obj
// transforms are applied in reverse order (PSF: psf.py:216-231, attenuation:
// attenuation.py:94-115), and the result is rotated back by +(270 - beta) with bilinear
// interpolation (transforms/shared/spatial.py:21-36) and summed.
//
// Two kernels per angle group:
//   k_b1_psf / k_b1_nopsf : rotated frame, W[xp][y][z] = A (.) PSF_xp(P) (or PSF(A (.) P))
//   k_b2_gather           : object frame, bilinear gather of W at the back-rotation
//                           (reference operator), fused OSEM / BSREM update epilogue
//   k_b2_scatter          : exact transpose of the forward's gather (adjoint operator)
#include "spect_blur.cuh"
#include "spect_kernels.cuh"
#include "spect_launch.h"

namespace gb {

static bool b1_fixed(int K, int N, int Zt);

#ifdef GB_PHASE_TIMING
// Per-warp cycle counts of k_b1_psf (diagnostic builds only), row CTA * warps + warp:
// [1] phase 1 work (S load), [2] wait at the barrier after it, [3] y blur work, [4] wait
// at the barrier after it, [5] z blur + W store work, [6] planes, [7] total, [8] rows,
// [9] rows x taps, [10] planes of the work item.
__device__ unsigned long long g_b1_phase_cycles[4096 * 16];
#define GB_B1T(k, v)                                  \
    do {                                              \
        if ((threadIdx.x & 31) == 0) tacc[k] += (v);  \
    } while (0)
#define GB_B1NOW() clock64()
#else
#define GB_B1T(k, v) \
    do {             \
        (void)(v);   \
    } while (0)
#define GB_B1NOW() 0LL
#endif

// ------------------------------------------------------------- attenuation
// A[a][xp][y][z] = exp(-(sum_{k>=xp} mu_rot[k]*dx - mu_rot[xp]*dx/2)) for the stored
// rows y in [ya_lo, ya_hi); mu_rot uses the forward rotation of angle a.
// (get_prob_of_detection_matrix, attenuation.py:11-21; rev_cumsum, utils/misc.py:8-19)
// The samples of PU planes are gathered before their running sums (same order of
// additions as one plane at a time), so PU planes' loads are in flight together.
template <bool VEC>
__global__ void __launch_bounds__(256)
    k_atten(SpectDev g, const float *__restrict__ mu, float dx, float *__restrict__ A) {
    constexpr int W = VEC ? 4 : 1;       // z values per thread
    constexpr int PU = VEC ? 4 : 8;      // planes sampled per step
    const int a = blockIdx.y;
    const int nzw = g.nz / W;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.nya * nzw) return;
    const int r = i / nzw, z = (i % nzw) * W;
    const int y = g.ya_lo + r;
    float th[6];
#pragma unroll
    for (int k = 0; k < 6; k++) th[k] = g.theta_fwd[6 * a + k];
    const float lc = g.lin[y];
    float *out = A + (size_t)a * g.Lp * g.nya * g.nz + (size_t)r * g.nz + z;
    const size_t plane = (size_t)g.nya * g.nz;
    float run[W];
#pragma unroll
    for (int w = 0; w < W; w++) run[w] = 0.f;
    for (int x0 = g.Lp - 1; x0 >= 0; x0 -= PU) {
        float v[PU][W];
#pragma unroll
        for (int u = 0; u < PU; u++) {
            const int xp = max(x0 - u, 0);
            float ix, iy;
            rot_coords(th, g.lin[xp], lc, g.half, ix, iy);
            const Bilin b = bilin(ix, iy);
            if constexpr (VEC) {
                float4 s4;
                sample4(mu, g.N, g.N, g.nz, g.pad, g.pad, b, z, s4);
                v[u][0] = __fmul_rn(s4.x, dx);
                v[u][1] = __fmul_rn(s4.y, dx);
                v[u][2] = __fmul_rn(s4.z, dx);
                v[u][3] = __fmul_rn(s4.w, dx);
            } else {
                v[u][0] = __fmul_rn(sample(mu, g.N, g.N, g.nz, g.pad, g.pad, b, z), dx);
            }
        }
#pragma unroll
        for (int u = 0; u < PU; u++) {
            const int xp = x0 - u;
            if (xp < 0) break;
            float e[W];
#pragma unroll
            for (int w = 0; w < W; w++) {
                run[w] = __fadd_rn(run[w], v[u][w]);
                e[w] = expf(-__fsub_rn(run[w], __fmul_rn(v[u][w], 0.5f)));
            }
            if constexpr (VEC)
                *reinterpret_cast<float4 *>(out + (size_t)xp * plane) =
                    make_float4(e[0], e[1], e[2], e[3]);
            else
                out[(size_t)xp * plane] = e[0];
        }
    }
}

cudaError_t launch_atten(const SpectDev &g, const float *mu, float dx, int n_angles, float *A,
                         cudaStream_t st) {
    if (g.nz % 4 == 0) {
        dim3 grid((g.nya * (g.nz / 4) + 255) / 256, n_angles);
        k_atten<true><<<grid, 256, 0, st>>>(g, mu, dx, A);
    } else {
        dim3 grid((g.nya * g.nz + 255) / 256, n_angles);
        k_atten<false><<<grid, 256, 0, st>>>(g, mu, dx, A);
    }
    return cudaGetLastError();
}

// OP consecutive floats (OP = 2 or 4, aligned to 4 * OP bytes) as one vector access
template <int OP>
__device__ __forceinline__ void ldg_vec(const float *p, float (&v)[OP]) {
    if constexpr (OP == 4) {
        const float4 t = __ldg(reinterpret_cast<const float4 *>(p));
        v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
    } else {
        static_assert(OP == 2, "vector of 2 or 4");
        const float2 t = __ldg(reinterpret_cast<const float2 *>(p));
        v[0] = t.x; v[1] = t.y;
    }
}
template <int OP>
__device__ __forceinline__ void st_vec(float *p, const float (&v)[OP]) {
    if constexpr (OP == 4) {
        *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
    } else {
        static_assert(OP == 2, "vector of 2 or 4");
        *reinterpret_cast<float2 *>(p) = make_float2(v[0], v[1]);
    }
}

// ---------------------------------------------------------------- B1 (PSF)
// Grid (chunk of planes, angle slot, z slab).  Output rows o <-> padded y = pad-H+o,
// o in [0, N+2H); input S rows i <-> padded y = pad-2H+i (projection rows at i in
// [2H, 2H+N), zero elsewhere).
// FIXED: N <= 128 and a z slab <= 128 wide: compile-time shared-memory strides.
// One work item: planes [x0_, x1_) of angle ga (projection rows P, [N][nz]) for the z slab
// at z0; writes the item's planes of the slot's W stack Ws ([Lp][nya][nz]) and row ranges
// wr ([Lp]).  Called once per CTA by k_b1_psf and per dequeued item by the batch kernel.
template <int K, bool VEC, bool FIXED>
__device__ __forceinline__ void b1_psf_item(const SpectDev &g, const float *__restrict__ P,
                                            const int ga, int2 *__restrict__ wr, const int x0_,
                                            const int x1_, const int z0, const int Zt,
                                            float *__restrict__ Ws) {
    constexpr int H = K / 2;
    constexpr int OB = (K <= 31) ? 8 : 4;
    const int N = g.N, nz = g.nz;
    const int Zc = min(Zt, nz - z0);
    const int NO = N + 2 * H;                       // output rows
    const int O8 = (NO + OB - 1) / OB * OB;
    const int Z8 = (Zc + OB - 1) / OB * OB;
    constexpr int O8_FIX = (128 + 2 * H + OB - 1) / OB * OB;
    const int SC = FIXED ? 128 + 2 * H : Z8 + 2 * H, SR = O8 + 2 * H;  // S: [SR][SC]
    const int TS = FIXED ? O8_FIX + 2 : O8 + 2, TR = Z8 + 2 * H;        // Tt: [TR][TS], even
    extern __shared__ __align__(16) float sm[];
    float *S = sm;
    float *Tt = S + SR * SC;
    float *tp = Tt + TR * TS;
    for (int i = threadIdx.x; i < SR * SC + TR * TS; i += blockDim.x) sm[i] = 0.f;
    const int grp = g.group[ga];
    const float *A = g.att ? g.A + (size_t)ga * g.Lp * g.nya * nz : nullptr;
    const int x0 = x0_, x1 = x1_;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
    const int cz_lo = max(0, H - z0), cz_hi = min(Z8 + 2 * H, nz - z0 + H);
    const int ncol = cz_hi - cz_lo;
    const bool att_inside = A && !g.att_first;  // "pa": A multiplies before the blur
    __syncthreads();
    if (!att_inside) {
        for (int i = threadIdx.x; i < N * ncol; i += blockDim.x) {
            int y = i / ncol, c = cz_lo + i % ncol;
            S[(2 * H + y) * SC + c] = P[(size_t)y * nz + (z0 - H + c)];
        }
    }
    float th[6];
#pragma unroll
    for (int k = 0; k < 6; k++) th[k] = g.theta_fwd[6 * ga + k];
    int parity = 0;
    // plane whose taps the end of the previous plane stored in tp[parity] (-1: none); the
    // taps of plane xp + 1 are loaded during plane xp, so the y blur does not wait for them
    int taps_of = -1;
#ifdef GB_PHASE_TIMING
    unsigned long long tacc[16] = {};
    const long long t_start = clock64();
    tacc[10] = x1 - x0;
#endif
    long long t0 = GB_B1NOW();
    for (int xp = x0; xp < x1; ++xp) {
        t0 = GB_B1NOW();
        // rows of this plane the gather can sample (object square + 1.5 px margin)
        int ra, rb;
        if (!plane_rows(g, th, xp, g.ya_lo, g.ya_hi, 1.5f, ra, rb)) {
            if (threadIdx.x == 0) wr[xp] = make_int2(0, 0);
            continue;
        }
        if (threadIdx.x == 0) wr[xp] = make_int2(ra - g.ya_lo, rb + 1 - g.ya_lo);
        const int o_lo = ra - (g.pad - H), o_hi = rb - (g.pad - H) + 1;  // output rows
        const int b_lo = o_lo / OB, b_hi = (o_hi + OB - 1) / OB;
        float *tap = tp + parity * 2 * K;
        if (taps_of != xp && threadIdx.x < K) {
            tap[threadIdx.x] = g.taps_r[((size_t)grp * g.Lp + xp) * g.K + threadIdx.x];
            tap[K + threadIdx.x] =
                g.psf2d ? g.taps_z[((size_t)grp * g.Lp + xp) * g.K + threadIdx.x] : 0.f;
        }
        const float *Ap = A ? A + (size_t)xp * g.nya * nz : nullptr;
        if (att_inside) {
            for (int i = threadIdx.x; i < N * ncol; i += blockDim.x) {
                int y = i / ncol, c = cz_lo + i % ncol;
                int z = z0 - H + c;
                S[(2 * H + y) * SC + c] = __fmul_rn(
                    P[(size_t)y * nz + z], Ap[(size_t)(g.pad + y - g.ya_lo) * nz + z]);
            }
        }
        {
            long long t1 = GB_B1NOW();
            GB_B1T(1, t1 - t0);
            t0 = t1;
        }
        __syncthreads();
        {
            long long t1 = GB_B1NOW();
            GB_B1T(2, t1 - t0);
            t0 = t1;
        }
        // the next plane's taps: loaded now, stored after this plane's z pass into the other
        // buffer (free: every warp has passed this plane's first barrier)
        const bool pre = xp + 1 < x1 && threadIdx.x < K;
        float nt_r = 0.f, nt_z = 0.f;
        if (pre) {
            nt_r = g.taps_r[((size_t)grp * g.Lp + xp + 1) * g.K + threadIdx.x];
            if (g.psf2d) nt_z = g.taps_z[((size_t)grp * g.Lp + xp + 1) * g.K + threadIdx.x];
        }
        int tier = kTiers - 1;
        if constexpr (FIXED) tier = g.tier ? g.tier[grp * g.Lp + xp] : kTiers - 1;
        // y blur over column pairs in blocks of OB rows (8-row blocks measured faster than 4:
        // fewer shared-memory loads per output outweigh the coarser task balance); the z blur
        // below uses blocks of OP = OB / 2 z values
        constexpr int OP = OB / 2;
        tier_dispatch<K>(tier, [&](auto kk) {
            constexpr int KK = decltype(kk)::value;
            blur_first2<K, KK, OB>(S, Tt, tap, SC, TS, cz_lo, cz_hi, b_lo, b_hi, warp, lane,
                                   nwarp);
        });
        GB_B1T(8, rb - ra + 1);
        GB_B1T(9, (rb - ra + 1) * tier_taps(K, tier));
        {
            long long t1 = GB_B1NOW();
            GB_B1T(3, t1 - t0);
            t0 = t1;
        }
        __syncthreads();
        {
            long long t1 = GB_B1NOW();
            GB_B1T(4, t1 - t0);
            t0 = t1;
        }
        {
            float *Wp = Ws + (size_t)xp * g.nya * nz;
            const bool amul = Ap && g.att_first;
            // warp-tasks (RP row pairs, 32 consecutive z): lane = (row pair lane % RP, z block
            // lane / RP of OP values).  Each A load and W store instruction of a warp then
            // touches RP row pairs x 128 contiguous bytes (4 cache lines per row), not one
            // 16-byte piece in each of 16 rows; the float2 reads of Tt stay free of bank
            // conflicts within each half warp (z blocks OP * TS floats apart)
            constexpr int RP = OP, ZQ = 32 / RP;
            static_assert(ZQ * OP == 32, "a warp task spans 32 z values");
            const int nrg = ((b_hi - b_lo) * OB + 2 * RP - 1) / (2 * RP);
            const int nzb = Z8 / OP, nzg = (nzb + ZQ - 1) / ZQ;
            const int pr = lane % RP, zq = lane / RP;
            tier_dispatch<K>(tier, [&](auto kk) {
                constexpr int KK = decltype(kk)::value;
                float w[KK];
                load_taps<K, KK>(tap + K, w);
                for (int p = warp; p < nrg * nzg; p += nwarp) {
                    const int rg = p % nrg, zb = (p / nrg) * ZQ + zq;
                    const int o_row = b_lo * OB + rg * 2 * RP + 2 * pr;  // rows o_row, o_row + 1
                    if (o_row >= b_hi * OB || zb >= nzb) continue;
                    const int y = g.pad - H + o_row;
                    const bool st0 = y >= ra && y <= rb, st1 = y + 1 >= ra && y + 1 <= rb;
                    const int zl0 = zb * OP;
                    const bool full = VEC && (zl0 + OP <= Zc);
                    const size_t rowoff = (size_t)(y - g.ya_lo) * nz + z0 + zl0;
                    float a0[OP], a1[OP];
                    if (amul) {  // issue the A loads before the blur arithmetic
#pragma unroll
                        for (int j = 0; j < OP; j++) a0[j] = a1[j] = 0.f;
                        if (full) {
                            if (st0) ldg_vec<OP>(Ap + rowoff, a0);
                            if (st1) ldg_vec<OP>(Ap + rowoff + nz, a1);
                        } else {
#pragma unroll
                            for (int j = 0; j < OP; j++) {
                                if (zl0 + j >= Zc) continue;
                                if (st0) a0[j] = Ap[rowoff + j];
                                if (st1) a1[j] = Ap[rowoff + nz + j];
                            }
                        }
                    }
                    float2 o[OP];
                    if (g.psf2d) {
                        blur_second2<K, KK, OP, false>(Tt, w, TS, zl0, o_row, o);
                    } else {
#pragma unroll
                        for (int j = 0; j < OP; j++)
                            o[j] = *reinterpret_cast<const float2 *>(Tt + (zl0 + j + H) * TS + o_row);
                    }
                    if (!st0 && !st1) continue;
                    if (amul) {
#pragma unroll
                        for (int j = 0; j < OP; j++) {
                            o[j].x = __fmul_rn(o[j].x, a0[j]);
                            o[j].y = __fmul_rn(o[j].y, a1[j]);
                        }
                    }
                    if (full) {
                        float v0[OP], v1[OP];
#pragma unroll
                        for (int j = 0; j < OP; j++) {
                            v0[j] = o[j].x;
                            v1[j] = o[j].y;
                        }
                        if (st0) st_vec<OP>(Wp + rowoff, v0);
                        if (st1) st_vec<OP>(Wp + rowoff + nz, v1);
                    } else {
#pragma unroll
                        for (int j = 0; j < OP; j++) {
                            if (zl0 + j >= Zc) continue;
                            if (st0) Wp[rowoff + j] = o[j].x;
                            if (st1) Wp[rowoff + nz + j] = o[j].y;
                        }
                    }
                }
            });
        }
        if (pre) {
            float *nt = tp + (parity ^ 1) * 2 * K;
            nt[threadIdx.x] = nt_r;
            nt[K + threadIdx.x] = nt_z;
        }
        taps_of = xp + 1;
        {
            long long t1 = GB_B1NOW();
            GB_B1T(5, t1 - t0);
            GB_B1T(6, 1);
        }
        parity ^= 1;
    }
#ifdef GB_PHASE_TIMING
    const int trow = (blockIdx.x * gridDim.y + blockIdx.y) * nwarp + warp;
    if (lane == 0 && trow < 4096) {
        tacc[7] = clock64() - t_start;
        for (int k = 0; k < 16; k++) g_b1_phase_cycles[trow * 16 + k] = tacc[k];
    }
#endif
}

// Grid (work item, z slab) over the angle slots of one group.
template <int K, bool VEC, bool FIXED>
__global__ void __launch_bounds__(512, 1)
    k_b1_psf(SpectDev g, const float *__restrict__ proj, const int *__restrict__ alist,
             const int4 *__restrict__ items, int Zt, float *__restrict__ W) {
    const int4 item = items[blockIdx.x];  // (slot in group, first plane, end plane)
    const int slot = item.x;
    b1_psf_item<K, VEC, FIXED>(g, proj + (size_t)slot * g.N * g.nz, alist[slot],
                               g.wrange + (size_t)slot * g.Lp, item.y, item.z, blockIdx.y * Zt,
                               Zt, W + (size_t)slot * g.Lp * g.nya * g.nz);
}

// Persistent batch form of B1: one CTA per SM dequeues the group's work items of every
// entry (N <= 128, nz <= 128: one fixed z slab), largest first.
template <int K>
__global__ void __launch_bounds__(512, 1) k_b1_psf_batch(const __grid_constant__ B1Batch p) {
    __shared__ int s_item;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(p.counter, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= p.n_items) return;
        const int4 item = p.items[it];  // (slot in group, first plane, end plane, entry)
        const int e = item.w, slot = item.x;
        const SpectDev &g = p.g[e];
        b1_psf_item<K, true, true>(g, p.proj[e] + (size_t)slot * g.N * g.nz, p.alist[e][slot],
                                   g.wrange + (size_t)slot * g.Lp, item.y, item.z, 0, g.nz,
                                   p.W[e] + (size_t)slot * g.Lp * g.nya * g.nz);
    }
}

#ifdef GB_PHASE_TIMING
extern "C" int gb_debug_b1_phase_cycles(unsigned long long *out, int n) {
    return (int)cudaMemcpyFromSymbol(out, g_b1_phase_cycles, sizeof(unsigned long long) * (size_t)n);
}
extern "C" int gb_debug_b1_phase_reset(void) {
    static unsigned long long zero[4096 * 16];
    return (int)cudaMemcpyToSymbol(g_b1_phase_cycles, zero, sizeof(zero));
}
#endif

// -------------------------------------------------------------- B1 (no PSF)
// W[slot][xp][y][z] = P[y - pad][z] * A (rows [pad, pad+N) are the stored rows).
// Without PSF: W[xp][y][z] = A (.) P; a thread per (row, z) or, with nz % 4 == 0, per
// (row, z quad) (16-byte loads and stores).
template <bool VEC>
__global__ void __launch_bounds__(256)
    k_b1_nopsf(SpectDev g, const float *__restrict__ proj, const int *__restrict__ alist,
               float *__restrict__ W) {
    constexpr int V = VEC ? 4 : 1;
    const int slot = blockIdx.z, xp = blockIdx.y;
    const int nzv = g.nz / V;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.nya * nzv) return;
    const int r = i / nzv, z = (i % nzv) * V;
    const int y = g.ya_lo + r;
    const int ga = alist[slot];
    if (i == 0) g.wrange[(size_t)slot * g.Lp + xp] = make_int2(0, g.nya);
    float *wp = W + (((size_t)slot * g.Lp + xp) * g.nya + r) * g.nz + z;
    const bool in = y >= g.pad && y < g.pad + g.N;
    const float *pp = proj + ((size_t)slot * g.N + (y - g.pad)) * g.nz + z;
    const float *ap = g.att ? g.A + (((size_t)ga * g.Lp + xp) * g.nya + r) * g.nz + z : nullptr;
    if constexpr (VEC) {
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (in) {
            v = *reinterpret_cast<const float4 *>(pp);
            if (g.att) v = mul4(v, __ldg(reinterpret_cast<const float4 *>(ap)));
        }
        *reinterpret_cast<float4 *>(wp) = v;
    } else {
        float v = 0.f;
        if (in) {
            v = *pp;
            if (g.att) v = __fmul_rn(v, __ldg(ap));
        }
        *wp = v;
    }
}

template <int K>
static cudaError_t launch_b1_psf_k(const SpectDev &g, const float *proj, const int *alist,
                                   const int4 *items, int n_items, int Zt, float *W,
                                   cudaStream_t st) {
    size_t smem = b1_psf_smem_bytes(K, g.N, Zt);
    dim3 grid(n_items, (g.nz + Zt - 1) / Zt);
    const bool fx = b1_fixed(K, g.N, Zt);
    if (g.nz % 4 == 0) {
        if (fx)
            k_b1_psf<K, true, true><<<grid, 512, smem, st>>>(g, proj, alist, items, Zt, W);
        else
            k_b1_psf<K, true, false><<<grid, 512, smem, st>>>(g, proj, alist, items, Zt, W);
    } else {
        if (fx)
            k_b1_psf<K, false, true><<<grid, 512, smem, st>>>(g, proj, alist, items, Zt, W);
        else
            k_b1_psf<K, false, false><<<grid, 512, smem, st>>>(g, proj, alist, items, Zt, W);
    }
    return cudaGetLastError();
}

template <int K>
static cudaError_t setup_b1_k(size_t smem) {
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(k_b1_psf<K, true, true>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
        cudaSuccess)
        return e;
    if ((e = cudaFuncSetAttribute(k_b1_psf<K, true, false>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
        cudaSuccess)
        return e;
    if ((e = cudaFuncSetAttribute(k_b1_psf<K, false, true>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
        cudaSuccess)
        return e;
    return cudaFuncSetAttribute(k_b1_psf<K, false, false>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

cudaError_t setup_b1(int K, size_t smem) {
    switch (K) {
#define GB_SETUP_CASE(KK) \
    case KK:              \
        return setup_b1_k<KK>(smem);
        GB_FOR_EACH_K(GB_SETUP_CASE)
#undef GB_SETUP_CASE
        default:
            return cudaErrorInvalidValue;
    }
}

cudaError_t setup_b1_batch(int K) {
    switch (K) {
#define GB_SETUP_CASE(KK)                                                                  \
    case KK:                                                                               \
        return cudaFuncSetAttribute(k_b1_psf_batch<KK>,                                    \
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,           \
                                    (int)b1_psf_smem_bytes(KK, 128, 128));
        GB_FOR_EACH_K(GB_SETUP_CASE)
#undef GB_SETUP_CASE
        default:
            return cudaErrorInvalidValue;
    }
}

cudaError_t launch_b1_batch(int K, const B1Batch &p, int grid, cudaStream_t st) {
    switch (K) {
#define GB_LAUNCH_CASE(KK)                                                                 \
    case KK:                                                                               \
        k_b1_psf_batch<KK><<<grid, 512, b1_psf_smem_bytes(KK, 128, 128), st>>>(p);         \
        return cudaGetLastError();
        GB_FOR_EACH_K(GB_LAUNCH_CASE)
#undef GB_LAUNCH_CASE
        default:
            return cudaErrorInvalidValue;
    }
}

static bool b1_fixed(int K, int N, int Zt) {
    int OB = (K <= 31) ? 8 : 4;
    return N <= 128 && (Zt + OB - 1) / OB * OB <= 128;
}

size_t b1_psf_smem_bytes(int K, int N, int Zt) {
    int H = K / 2, OB = (K <= 31) ? 8 : 4;
    int O8 = (N + 2 * H + OB - 1) / OB * OB;
    int Z8 = (Zt + OB - 1) / OB * OB;
    const bool fx = b1_fixed(K, N, Zt);
    size_t SC = fx ? 128 + 2 * H : Z8 + 2 * H;
    size_t TS = fx ? (128 + 2 * H + OB - 1) / OB * OB + 2 : O8 + 2;  // even: float2 pairs
    return sizeof(float) * ((size_t)(O8 + 2 * H) * SC + (size_t)(Z8 + 2 * H) * TS + 4 * K);
}

cudaError_t launch_b1(const SpectDev &g, const float *proj, const int *alist, int n_slots,
                      const int4 *items, int n_items, int Zt, float *W, cudaStream_t st) {
    if (!g.psf) {
        // a user projection pointer may not be 16-byte aligned: scalar kernel then
        if (g.nz % 4 == 0 && ((uintptr_t)proj & 15) == 0) {
            dim3 grid((g.nya * (g.nz / 4) + 255) / 256, g.Lp, n_slots);
            k_b1_nopsf<true><<<grid, 256, 0, st>>>(g, proj, alist, W);
        } else {
            dim3 grid((g.nya * g.nz + 255) / 256, g.Lp, n_slots);
            k_b1_nopsf<false><<<grid, 256, 0, st>>>(g, proj, alist, W);
        }
        return cudaGetLastError();
    }
    switch (g.K) {
#define GB_B1_CASE(KK) \
    case KK:           \
        return launch_b1_psf_k<KK>(g, proj, alist, items, n_items, Zt, W, st);
        GB_FOR_EACH_K(GB_B1_CASE)
#undef GB_B1_CASE
        default:
            return cudaErrorInvalidValue;
    }
}

// ------------------------------------------------------------- RDP helpers
// sum_s w_rs phi1(f_r, f_s) over the 26 neighbours with replicate boundary, in the
// loop order of NearestNeighbourPrior._pair_contribution (nearest_neighbour.py:56-72);
// phi1 of RelativeDifferencePrior (nearest_neighbour.py:176-177).
__device__ __forceinline__ float rdp_sum(const float *__restrict__ f, int nx, int ny, int nz,
                                         int x, int y, int z, float fr, const UpdateArgs &u) {
    float acc = 0.f;
    int n = 0;
    const float two_d = 2.f * u.rdelta;
#pragma unroll
    for (int i = -1; i <= 1; i++) {
        int xi = min(max(x + i, 0), nx - 1);
#pragma unroll
        for (int j = -1; j <= 1; j++) {
            int yj = min(max(y + j, 0), ny - 1);
#pragma unroll
            for (int k = -1; k <= 1; k++) {
                if (i == 0 && j == 0 && k == 0) continue;
                int zk = min(max(z + k, 0), nz - 1);
                float fs = __ldg(f + ((size_t)xi * ny + yj) * nz + zk);
                float d = __fsub_rn(fr, fs);
                float ad = fabsf(d);
                float num = __fmul_rn(
                    d, __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(u.gamma, ad), __fmul_rn(3.f, fs)), fr),
                                 two_d));
                float den = __fadd_rn(__fadd_rn(__fadd_rn(fr, fs), __fmul_rn(u.gamma, ad)), u.rdelta);
                float phi = __fdiv_rn(num, __fmul_rn(den, den));
                acc = __fadd_rn(acc, __fmul_rn(phi, u.w26[n]));
                n++;
            }
        }
    }
    return acc;
}

// rdp_sum for the four voxels z..z+3 of a z quad (z % 4 == 0, nz % 4 == 0), used by the
// fused BSREM step: each (x, y) neighbour row is loaded once (z-1, the quad, z+4,
// clamped), every voxel adds its 26 terms in rdp_sum's order, and the term arithmetic
// uses FMAs and the fast division (about 2 ulp; exact division for denominators below
// 2^-100, where the fast reciprocal would overflow).  The result differs from rdp_sum by
// rounding only (well inside the 1e-5 agreement with the reference).
__device__ __forceinline__ void rdp_sum4(const float *__restrict__ f, int nx, int ny, int nz,
                                         int x, int y, int z, const float (&fr)[4],
                                         const UpdateArgs &u, float (&acc)[4]) {
#pragma unroll
    for (int v = 0; v < 4; v++) acc[v] = 0.f;
    int n = 0;
    const float two_d = 2.f * u.rdelta;
#pragma unroll
    for (int i = -1; i <= 1; i++) {
        const int xi = min(max(x + i, 0), nx - 1);
#pragma unroll
        for (int j = -1; j <= 1; j++) {
            const int yj = min(max(y + j, 0), ny - 1);
            const float *p = f + ((size_t)xi * ny + yj) * nz;
            const float4 c = __ldg(reinterpret_cast<const float4 *>(p + z));
            const float row[6] = {__ldg(p + max(z - 1, 0)), c.x, c.y, c.z, c.w,
                                  __ldg(p + min(z + 4, nz - 1))};
#pragma unroll
            for (int k = -1; k <= 1; k++) {
                if (i == 0 && j == 0 && k == 0) continue;
#pragma unroll
                for (int v = 0; v < 4; v++) {
                    const float fs = row[1 + v + k], r = fr[v];
                    const float d = r - fs, ad = fabsf(d);
                    const float num = d * (fmaf(u.gamma, ad, fmaf(3.f, fs, r)) + two_d);
                    const float den = fmaf(u.gamma, ad, r + fs) + u.rdelta;
                    const float den2 = den * den;
                    const float phi =
                        den2 > 7.8886e-31f ? __fdividef(num, den2) : __fdiv_rn(num, den2);
                    acc[v] = fmaf(phi, u.w26[n], acc[v]);
                }
                n++;
            }
        }
    }
}

__global__ void k_rdp(const float *__restrict__ f, float *__restrict__ grad, int nx, int ny,
                      int nz, UpdateArgs u, float scale) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)nx * ny * nz) return;
    int z = i % nz, y = (i / nz) % ny, x = i / ((size_t)nz * ny);
    float s = rdp_sum(f, nx, ny, nz, x, y, z, f[i], u);
    float v = __fmul_rn(scale, s);
    if (u.fov) v = __fmul_rn(v, u.fov[i]);
    grad[i] = v;
}

// Second derivative of the RDP applied to x (nearest_neighbour.py:89-110, 173-177):
// out_r = beta s FOV_r sum_s w_rs (phi2_1(f_r, f_s) x_r + phi2_2(f_r, f_s) x_s) with
// phi2_1 = 2 (2 f_s + delta)^2 / D^3, phi2_2 = -2 (2 f_r + delta)(2 f_s + delta) / D^3,
// D = gamma |f_r - f_s| + f_r + f_s + delta, replicate boundary.
__global__ void k_rdp_hvp(const float *__restrict__ f, const float *__restrict__ xin,
                          float *__restrict__ out, int nx, int ny, int nz, UpdateArgs u,
                          float scale) {
    size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (size_t)nx * ny * nz) return;
    const int z = idx % nz, y = (idx / nz) % ny, x = idx / ((size_t)nz * ny);
    const float fr = f[idx], xr = xin[idx];
    float diag = 0.f, off = 0.f;
    int n = 0;
    for (int i = -1; i <= 1; i++) {
        const int xi = min(max(x + i, 0), nx - 1);
        for (int j = -1; j <= 1; j++) {
            const int yj = min(max(y + j, 0), ny - 1);
            for (int k = -1; k <= 1; k++) {
                if (i == 0 && j == 0 && k == 0) continue;
                const int zk = min(max(z + k, 0), nz - 1);
                const size_t o = ((size_t)xi * ny + yj) * nz + zk;
                const float fs = __ldg(f + o), xs = __ldg(xin + o);
                const float D = u.gamma * fabsf(fr - fs) + fr + fs + u.rdelta;
                const float D3 = D * D * D;
                const float as = 2.f * fs + u.rdelta, ar = 2.f * fr + u.rdelta;
                diag += u.w26[n] * (2.f * as * as / D3);
                off += u.w26[n] * (-2.f * ar * as / D3) * xs;
                n++;
            }
        }
    }
    float v = scale * (diag * xr + off);
    if (u.fov) v *= u.fov[idx];
    out[idx] = v;
}

cudaError_t launch_rdp_hvp(const float *f, const float *x, float *out, int nx, int ny, int nz,
                           const UpdateArgs &u, float beta_scale, cudaStream_t st) {
    size_t n = (size_t)nx * ny * nz;
    k_rdp_hvp<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(f, x, out, nx, ny, nz, u,
                                                          u.beta * beta_scale);
    return cudaGetLastError();
}

cudaError_t launch_rdp(const float *f, float *grad, int nx, int ny, int nz, const UpdateArgs &u,
                       float beta_scale, cudaStream_t st) {
    size_t n = (size_t)nx * ny * nz;
    k_rdp<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(f, grad, nx, ny, nz, u,
                                                      u.beta * beta_scale);
    return cudaGetLastError();
}

// Update epilogue shared by the gather kernel and the standalone update kernel.
// PRIOR = false compiles out the RDP term (callers that never see BSREM with a prior).
template <bool PRIOR = true>
__device__ __forceinline__ void apply_update(int mode, const UpdateArgs &u, size_t i, int x,
                                             int y, int z, int nx, int ny, int nz, float bp,
                                             float *out) {
    if (u.acc) bp = __fadd_rn(u.acc[i], bp);
    if (mode == B2_WRITE) {
        out[i] = bp;
    } else if (mode == B2_ADD) {
        out[i] = __fadd_rn(out[i], bp);
    } else if (mode == B2_OSEM) {
        float f = u.f[i], nb = u.nbp[i];
        float grad = __fsub_rn(bp, nb);
        float pre = __fmul_rn(f, __frcp_rn(__fadd_rn(nb, kDelta)));
        float fn = __fadd_rn(f, __fmul_rn(pre, grad));
        u.f[i] = fn <= 0.f ? 0.f : fn;
    } else {  // B2_BSREM
        float f = u.f_in[i], nb = u.nbp[i];
        float grad = __fsub_rn(bp, nb);
        if (PRIOR && u.prior) {
            float v = __fmul_rn(__fmul_rn(u.beta, u.w_m),
                                rdp_sum(u.f_in, nx, ny, nz, x, y, z, f, u));
            if (u.fov) v = __fmul_rn(v, u.fov[i]);
            grad = __fsub_rn(grad, v);
        }
        float pre = __fmul_rn(
            f, __fdiv_rn(u.relax, __fadd_rn(__fmul_rn(u.w_m, u.nbp_sum[i]), kDelta)));
        float fn = __fadd_rn(f, __fmul_rn(pre, grad));
        u.f_out[i] = fn <= u.floor_v ? u.floor_v : fn;
    }
}

// apply_update for the z quad z..z+3 (z % 4 == 0, nz % 4 == 0).  PRIOR (BSREM with the
// RDP prior): the prior term comes from rdp_sum4, one neighbourhood load for the four
// voxels; a separate instantiation, so the other modes keep their register count.
template <bool PRIOR>
__device__ __forceinline__ void apply_update4(int mode, const UpdateArgs &u, size_t i, int x,
                                              int y, int z, int nx, int ny, int nz, float4 bp4,
                                              float *out) {
    const float bp[4] = {bp4.x, bp4.y, bp4.z, bp4.w};
    if constexpr (!PRIOR) {
        apply_update(mode, u, i, x, y, z, nx, ny, nz, bp[0], out);
        apply_update(mode, u, i + 1, x, y, z + 1, nx, ny, nz, bp[1], out);
        apply_update(mode, u, i + 2, x, y, z + 2, nx, ny, nz, bp[2], out);
        apply_update(mode, u, i + 3, x, y, z + 3, nx, ny, nz, bp[3], out);
        return;
    }
    float f[4], rdp[4];
#pragma unroll
    for (int v = 0; v < 4; v++) f[v] = u.f_in[i + v];
    rdp_sum4(u.f_in, nx, ny, nz, x, y, z, f, u, rdp);
#pragma unroll
    for (int v = 0; v < 4; v++) {
        float b = bp[v];
        if (u.acc) b = __fadd_rn(u.acc[i + v], b);
        const float nb = u.nbp[i + v];
        float grad = __fsub_rn(b, nb);
        float pv = __fmul_rn(__fmul_rn(u.beta, u.w_m), rdp[v]);
        if (u.fov) pv = __fmul_rn(pv, u.fov[i + v]);
        grad = __fsub_rn(grad, pv);
        const float pre = __fmul_rn(
            f[v], __fdiv_rn(u.relax, __fadd_rn(__fmul_rn(u.w_m, u.nbp_sum[i + v]), kDelta)));
        const float fn = __fadd_rn(f[v], __fmul_rn(pre, grad));
        u.f_out[i + v] = fn <= u.floor_v ? u.floor_v : fn;
    }
}

// ------------------------------------------------------------- B2 gather
// Reference back-projector: for every object voxel, bilinear sample of W at the
// back-rotation (angle 270 - beta) of each angle of the group, summed.  Threads own
// (x, y, z quad); two angles are sampled before accumulating to keep loads in flight.
__device__ __forceinline__ float4 b2_gather_sum4(const SpectDev &g, const float *__restrict__ W,
                                                  const int *__restrict__ alist, int n_slots,
                                                  int x, int y, int z) {
    const int nz = g.nz;
    const float lr = g.lin[x + g.pad], lc = g.lin[y + g.pad];
    const size_t slab = (size_t)g.Lp * g.nya * nz;
    float4 bp = make_float4(0.f, 0.f, 0.f, 0.f);
    int s = 0;
    for (; s + 1 < n_slots; s += 2) {
        float ix, iy, ix2, iy2;
        rot_coords(g.theta_bwd + 6 * alist[s], lr, lc, g.half, ix, iy);
        rot_coords(g.theta_bwd + 6 * alist[s + 1], lr, lc, g.half, ix2, iy2);
        Bilin b1 = bilin(ix, iy), b2 = bilin(ix2, iy2);
        float4 v1, v2;
        sample4_ranged(W + s * slab, g.Lp, g.nya, nz, g.ya_lo, g.wrange + (size_t)s * g.Lp, b1,
                       z, v1);
        sample4_ranged(W + (s + 1) * slab, g.Lp, g.nya, nz, g.ya_lo,
                       g.wrange + (size_t)(s + 1) * g.Lp, b2, z, v2);
        bp.x = __fadd_rn(__fadd_rn(bp.x, v1.x), v2.x);
        bp.y = __fadd_rn(__fadd_rn(bp.y, v1.y), v2.y);
        bp.z = __fadd_rn(__fadd_rn(bp.z, v1.z), v2.z);
        bp.w = __fadd_rn(__fadd_rn(bp.w, v1.w), v2.w);
    }
    if (s < n_slots) {
        float ix, iy;
        rot_coords(g.theta_bwd + 6 * alist[s], lr, lc, g.half, ix, iy);
        Bilin b1 = bilin(ix, iy);
        float4 v1;
        sample4_ranged(W + s * slab, g.Lp, g.nya, nz, g.ya_lo, g.wrange + (size_t)s * g.Lp, b1,
                       z, v1);
        bp.x = __fadd_rn(bp.x, v1.x);
        bp.y = __fadd_rn(bp.y, v1.y);
        bp.z = __fadd_rn(bp.z, v1.z);
        bp.w = __fadd_rn(bp.w, v1.w);
    }
    return bp;
}

// The back-rotation samples of a block's (x, y) rows are the same for every z quad of a
// row: the block computes them once per (row, slot) into shared memory, and each thread
// then reads its row's entries (broadcast loads) instead of repeating the rotation, the
// bilinear weights and the row-range tests per thread.  An entry holds the W slab offset
// of the north-west corner (z excluded), the mask of the corners inside the rows B1
// wrote (bit 0 nw, 1 ne, 2 sw, 3 se) and the four bilinear weights.  Sums and products
// are the ones of b2_gather_sum4, in the same order.
struct __align__(16) B2Tap {
    int off, mask, pad0, pad1;
    float nw, ne, sw, se;
};
constexpr int kB2Taps = 512;  // entries of one block's table (16 KB)

__device__ __forceinline__ void b2_make_tap(const SpectDev &g, const int *__restrict__ alist,
                                            int s, int x, int y, B2Tap &t) {
    float ix, iy;
    rot_coords(g.theta_bwd + 6 * alist[s], g.lin[x + g.pad], g.lin[y + g.pad], g.half, ix, iy);
    const Bilin b = bilin(ix, iy);
    const int r = b.r0, c = b.c0 - g.ya_lo;
    const int2 *wr = g.wrange + (size_t)s * g.Lp;
    const bool r0 = (unsigned)r < (unsigned)g.Lp, r1 = (unsigned)(r + 1) < (unsigned)g.Lp;
    const int2 g0 = r0 ? wr[r] : make_int2(0, 0);
    const int2 g1 = r1 ? wr[r + 1] : make_int2(0, 0);
    int m = 0;
    if (r0 && c >= g0.x && c < g0.y) m |= 1;
    if (r0 && c + 1 >= g0.x && c + 1 < g0.y) m |= 2;
    if (r1 && c >= g1.x && c < g1.y) m |= 4;
    if (r1 && c + 1 >= g1.x && c + 1 < g1.y) m |= 8;
    t.off = (r * g.nya + c) * g.nz;  // the slab has fewer than 2^31 elements (b2_tab_fits)
    t.mask = m;
    t.pad0 = t.pad1 = 0;
    t.nw = b.nw;
    t.ne = b.ne;
    t.sw = b.sw;
    t.se = b.se;
}

__device__ __forceinline__ bool b2_tab_fits(const SpectDev &g, int n_rows, int n_slots) {
    return n_rows * n_slots <= kB2Taps && (long long)g.Lp * g.nya * g.nz < (1LL << 31);
}

__device__ __forceinline__ float4 b2_tap_sample(const float *__restrict__ Ws, const B2Tap &t,
                                                int nya, int nz, int z) {
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    if (t.mask == 0) return zero;
    const float *p = Ws + t.off + z;
    const int rs = nya * nz;
    const float4 vnw = (t.mask & 1) ? __ldg(reinterpret_cast<const float4 *>(p)) : zero;
    const float4 vne = (t.mask & 2) ? __ldg(reinterpret_cast<const float4 *>(p + nz)) : zero;
    const float4 vsw = (t.mask & 4) ? __ldg(reinterpret_cast<const float4 *>(p + rs)) : zero;
    const float4 vse = (t.mask & 8) ? __ldg(reinterpret_cast<const float4 *>(p + rs + nz)) : zero;
    Bilin b;
    b.nw = t.nw;
    b.ne = t.ne;
    b.sw = t.sw;
    b.se = t.se;
    float4 o;
    o.x = bilin_combine(b, vnw.x, vne.x, vsw.x, vse.x);
    o.y = bilin_combine(b, vnw.y, vne.y, vsw.y, vse.y);
    o.z = bilin_combine(b, vnw.z, vne.z, vsw.z, vse.z);
    o.w = bilin_combine(b, vnw.w, vne.w, vsw.w, vse.w);
    return o;
}

// Sum over the slots of one row's table entries; U slots are sampled before accumulating
// (loads in flight), the additions run in slot order.
template <int U>
__device__ __forceinline__ float4 b2_gather_sum4_tab(const float *__restrict__ W, size_t slab,
                                                      const B2Tap *tab, int n_slots, int nya,
                                                      int nz, int z) {
    float4 bp = make_float4(0.f, 0.f, 0.f, 0.f);
    int s = 0;
    for (; s + U <= n_slots; s += U) {
        float4 v[U];
#pragma unroll
        for (int k = 0; k < U; k++) {
            const B2Tap t = tab[s + k];
            v[k] = b2_tap_sample(W + (s + k) * slab, t, nya, nz, z);
        }
#pragma unroll
        for (int k = 0; k < U; k++) {
            bp.x = __fadd_rn(bp.x, v[k].x);
            bp.y = __fadd_rn(bp.y, v[k].y);
            bp.z = __fadd_rn(bp.z, v[k].z);
            bp.w = __fadd_rn(bp.w, v[k].w);
        }
    }
    for (; s < n_slots; s++) {
        const B2Tap t = tab[s];
        const float4 v = b2_tap_sample(W + s * slab, t, nya, nz, z);
        bp.x = __fadd_rn(bp.x, v.x);
        bp.y = __fadd_rn(bp.y, v.y);
        bp.z = __fadd_rn(bp.z, v.z);
        bp.w = __fadd_rn(bp.w, v.w);
    }
    return bp;
}

constexpr int kB2Unroll = 2;

template <bool PRIOR>
__global__ void __launch_bounds__(256)
    k_b2_gather4(SpectDev g, const float *__restrict__ W, const int *__restrict__ alist,
                 int n_slots, float *__restrict__ out, int mode, UpdateArgs u) {
    __shared__ B2Tap tab[kB2Taps];
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int x = blockIdx.z;
    const int N = g.N, nz = g.nz;
    const int n_rows = blockDim.y;  // a block covers rows y of one plane x
    const bool use_tab = b2_tab_fits(g, n_rows, n_slots);
    if (use_tab) {
        const int nt = blockDim.x * blockDim.y, tid = threadIdx.y * blockDim.x + threadIdx.x;
        for (int e = tid; e < n_rows * n_slots; e += nt) {
            const int yr = blockIdx.y * blockDim.y + e / n_slots;
            if (yr < N) b2_make_tap(g, alist, e % n_slots, x, yr, tab[e]);
        }
        __syncthreads();
    }
    if (4 * q >= nz || y >= N) return;
    const int z = 4 * q;
    const float4 bp = use_tab ? b2_gather_sum4_tab<kB2Unroll>(
                                    W, (size_t)g.Lp * g.nya * nz, tab + threadIdx.y * n_slots,
                                    n_slots, g.nya, nz, z)
                              : b2_gather_sum4(g, W, alist, n_slots, x, y, z);
    const size_t i = ((size_t)x * N + y) * nz + z;
    apply_update4<PRIOR>(mode, u, i, x, y, z, N, N, nz, bp, out);
}

// Entry of a block of the batched gather / scatter kernels (the entries' blocks are
// contiguous ranges of the grid, in entry order).
__device__ __forceinline__ int batch_entry(const int *block_off, int b) {
    int e = 0;
    while (e + 1 < kMaxBatch && b >= block_off[e + 1]) e++;
    return e;
}

int b2_gather_blocks(const SpectDev &g) {
    return (int)(((long long)g.N * g.N * (g.nz / 4) + 255) / 256);
}

// Batched reference back-projector with its epilogue: a thread per (x, y, z quad) of an
// entry's object (nz % 4 == 0), flat over the entry's voxels.
__global__ void __launch_bounds__(256) k_b2_gather_batch(const __grid_constant__ B2Batch p) {
    __shared__ B2Tap tab[kB2Taps];
    const int e = batch_entry(p.block_off, blockIdx.x);
    const SpectDev &g = p.g[e];
    const long long q0 = (long long)(blockIdx.x - p.block_off[e]) * 256;
    const long long q = q0 + threadIdx.x;
    const int N = g.N, nz = g.nz, nq = nz / 4, ns = p.n_slots[e];
    const long long total = (long long)N * N * nq;
    // rows (x N + y) of the block's voxels
    const long long row0 = q0 / nq;
    const int n_rows = (int)((min(q0 + 255, total - 1)) / nq - row0) + 1;
    const bool use_tab = b2_tab_fits(g, n_rows, ns);
    if (use_tab) {
        for (int k = threadIdx.x; k < n_rows * ns; k += 256) {
            const long long row = row0 + k / ns;
            b2_make_tap(g, p.alist[e], k % ns, (int)(row / N), (int)(row % N), tab[k]);
        }
        __syncthreads();
    }
    if (q >= total) return;
    const int z = 4 * (int)(q % nq), y = (int)((q / nq) % N), x = (int)(q / ((long long)nq * N));
    const float4 bp =
        use_tab ? b2_gather_sum4_tab<kB2Unroll>(p.W[e], (size_t)g.Lp * g.nya * nz,
                                               tab + (int)(q / nq - row0) * ns, ns, g.nya, nz, z)
                : b2_gather_sum4(g, p.W[e], p.alist[e], ns, x, y, z);
    const size_t i = ((size_t)x * N + y) * nz + z;
    UpdateArgs u{};
    u.f = p.out[e];
    u.nbp = p.nbp[e];
    u.acc = p.acc[e];
    apply_update4<false>(p.mode[e], u, i, x, y, z, N, N, nz, bp, p.out[e]);
}

cudaError_t launch_b2_gather_batch(const B2Batch &p, int n_blocks, cudaStream_t st) {
    if (n_blocks <= 0) return cudaSuccess;
    k_b2_gather_batch<<<n_blocks, 256, 0, st>>>(p);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(256)
    k_b2_gather(SpectDev g, const float *__restrict__ W, const int *__restrict__ alist,
                int n_slots, float *__restrict__ out, int mode, UpdateArgs u) {
    const int z = blockIdx.x * 32 + threadIdx.x;
    const int y = blockIdx.y * 8 + threadIdx.y;
    const int x = blockIdx.z;
    const int N = g.N, nz = g.nz;
    if (z >= nz || y >= N) return;
    const float lr = g.lin[x + g.pad], lc = g.lin[y + g.pad];
    const size_t slab = (size_t)g.Lp * g.nya * nz;
    float bp = 0.f;
    for (int s = 0; s < n_slots; s++) {
        const float *th = g.theta_bwd + 6 * alist[s];
        float ix, iy;
        rot_coords(th, lr, lc, g.half, ix, iy);
        Bilin b = bilin(ix, iy);
        // W rows = padded x (row offset 0), cols = padded y - ya_lo
        bp = __fadd_rn(bp, sample_ranged(W + s * slab, g.Lp, g.nya, nz, g.ya_lo,
                                         g.wrange + (size_t)s * g.Lp, b, z));
    }
    const size_t i = ((size_t)x * N + y) * nz + z;
    apply_update(mode, u, i, x, y, z, N, N, nz, bp, out);
}

cudaError_t launch_b2_gather(const SpectDev &g, const float *W, const int *alist, int n_slots,
                             float *out, int mode, const UpdateArgs &u, cudaStream_t st) {
    dim3 block(32, 8);
    if (g.nz % 4 == 0) {
        // blocks of 256 threads shaped to the z quads of a row: when the quads of a row
        // divide a warp (1, 2, 4, 8 or 16), a warp takes whole rows and no lane idles
        const int qx = g.nz / 4;
        const bool packed = qx < 32 && 32 % qx == 0;
        const dim3 b4(packed ? qx : 32, packed ? 256 / qx : 8);
        dim3 grid((qx + b4.x - 1) / b4.x, (g.N + b4.y - 1) / b4.y, g.N);
        block = b4;
        if (mode == B2_BSREM && u.prior)
            k_b2_gather4<true><<<grid, block, 0, st>>>(g, W, alist, n_slots, out, mode, u);
        else
            k_b2_gather4<false><<<grid, block, 0, st>>>(g, W, alist, n_slots, out, mode, u);
    } else {
        dim3 grid((g.nz + 31) / 32, (g.N + 7) / 8, g.N);
        k_b2_gather<<<grid, block, 0, st>>>(g, W, alist, n_slots, out, mode, u);
    }
    return cudaGetLastError();
}

// ------------------------------------------------------------ B2 scatter
// Exact adjoint of the forward rotation: every W element is scattered to the four
// object voxels the forward sample at the same position gathered from.  VEC: a thread
// takes a z quad and each corner gets one 16-byte vector atomic (nz % 4 == 0, out 16-byte
// aligned); the per-element products are the same as one element at a time.
template <bool VEC>
__global__ void __launch_bounds__(256)
    k_b2_scatter(SpectDev g, const float *__restrict__ W, const int *__restrict__ alist,
                 float *__restrict__ out) {
    constexpr int V = VEC ? 4 : 1;
    const int slot = blockIdx.z, xp = blockIdx.y;
    const int nzv = g.nz / V;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.nya * nzv) return;
    const int r = i / nzv, z = (i % nzv) * V;
    const int yp = g.ya_lo + r;
    const int2 rg = g.wrange[(size_t)slot * g.Lp + xp];
    if (r < rg.x || r >= rg.y) return;
    const float *wp = W + (((size_t)slot * g.Lp + xp) * g.nya + r) * g.nz + z;
    float v[V];
    if constexpr (VEC) {
        const float4 t = *reinterpret_cast<const float4 *>(wp);
        v[0] = t.x;
        v[1] = t.y;
        v[2] = t.z;
        v[3] = t.w;
        if (t.x == 0.f && t.y == 0.f && t.z == 0.f && t.w == 0.f) return;
    } else {
        v[0] = *wp;
        if (v[0] == 0.f) return;
    }
    const float *th = g.theta_fwd + 6 * alist[slot];
    float ix, iy;
    rot_coords(th, g.lin[xp], g.lin[yp], g.half, ix, iy);
    Bilin b = bilin(ix, iy);
    const int N = g.N, nz = g.nz;
    const int r0 = b.r0 - g.pad, c0 = b.c0 - g.pad;
    const float wt[4] = {b.nw, b.ne, b.sw, b.se};
#pragma unroll
    for (int q = 0; q < 4; q++) {
        int rr = r0 + (q >> 1), cc = c0 + (q & 1);
        if ((unsigned)rr >= (unsigned)N || (unsigned)cc >= (unsigned)N) continue;
        float *o = out + ((size_t)rr * N + cc) * nz + z;
        if constexpr (VEC)
            atomicAdd(reinterpret_cast<float4 *>(o),
                      make_float4(__fmul_rn(wt[q], v[0]), __fmul_rn(wt[q], v[1]),
                                  __fmul_rn(wt[q], v[2]), __fmul_rn(wt[q], v[3])));
        else
            atomicAdd(o, __fmul_rn(wt[q], v[0]));
    }
}

int b2_scatter_blocks(const SpectDev &g, int n_slots) {
    return n_slots * g.Lp * ((g.nya * (g.nz / 4) + 255) / 256);
}

// Batched exact adjoint: the blocks of an entry cover (slot, plane, 256 (row, z quad) of
// the plane), as k_b2_scatter's grid does; nz % 4 == 0 and 16-byte aligned objects.
__global__ void __launch_bounds__(256) k_b2_scatter_batch(const __grid_constant__ B2Batch p) {
    const int e = batch_entry(p.block_off, blockIdx.x);
    const SpectDev &g = p.g[e];
    const int per_plane = (g.nya * (g.nz / 4) + 255) / 256;
    const int b = blockIdx.x - p.block_off[e];
    const int slot = b / (per_plane * g.Lp), xp = (b / per_plane) % g.Lp;
    const int i = (b % per_plane) * 256 + threadIdx.x;
    const int nzv = g.nz / 4;
    if (slot >= p.n_slots[e] || i >= g.nya * nzv) return;
    const int r = i / nzv, z = (i % nzv) * 4;
    const int2 rg = g.wrange[(size_t)slot * g.Lp + xp];
    if (r < rg.x || r >= rg.y) return;
    const float4 t = *reinterpret_cast<const float4 *>(
        p.W[e] + (((size_t)slot * g.Lp + xp) * g.nya + r) * g.nz + z);
    if (t.x == 0.f && t.y == 0.f && t.z == 0.f && t.w == 0.f) return;
    float ix, iy;
    rot_coords(g.theta_fwd + 6 * p.alist[e][slot], g.lin[xp], g.lin[g.ya_lo + r], g.half, ix, iy);
    const Bilin bl = bilin(ix, iy);
    const int N = g.N, nz = g.nz;
    const int r0 = bl.r0 - g.pad, c0 = bl.c0 - g.pad;
    const float wt[4] = {bl.nw, bl.ne, bl.sw, bl.se};
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const int rr = r0 + (q >> 1), cc = c0 + (q & 1);
        if ((unsigned)rr >= (unsigned)N || (unsigned)cc >= (unsigned)N) continue;
        atomicAdd(reinterpret_cast<float4 *>(p.out[e] + ((size_t)rr * N + cc) * nz + z),
                  make_float4(__fmul_rn(wt[q], t.x), __fmul_rn(wt[q], t.y), __fmul_rn(wt[q], t.z),
                              __fmul_rn(wt[q], t.w)));
    }
}

cudaError_t launch_b2_scatter_batch(const B2Batch &p, int n_blocks, cudaStream_t st) {
    if (n_blocks <= 0) return cudaSuccess;
    k_b2_scatter_batch<<<n_blocks, 256, 0, st>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_b2_scatter(const SpectDev &g, const float *W, const int *alist, int n_slots,
                              float *out, cudaStream_t st) {
    if (g.nz % 4 == 0 && ((uintptr_t)out & 15) == 0) {
        dim3 grid((g.nya * (g.nz / 4) + 255) / 256, g.Lp, n_slots);
        k_b2_scatter<true><<<grid, 256, 0, st>>>(g, W, alist, out);
    } else {
        dim3 grid((g.nya * g.nz + 255) / 256, g.Lp, n_slots);
        k_b2_scatter<false><<<grid, 256, 0, st>>>(g, W, alist, out);
    }
    return cudaGetLastError();
}

}  // namespace gb
