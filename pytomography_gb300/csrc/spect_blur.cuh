// Register-tiled per-plane blur passes shared by the forward (k_fwd_psf) and the
// back-projection (k_b1_psf) kernels.
//
// Tap tiers: a plane whose kernel is narrow (its outer taps are exactly zero, or below
// the plan's truncation threshold) runs a shorter unrolled loop.  A plane of bucket K
// (half width H) uses KK = 2h+1 taps with h = round(H * {0.2, 0.35, 0.5, 0.65, 0.8, 1})
// (tiers 0..5; h = 3, 5, 7, 9, 11, 14 for K = 29); the taps used are the centred KK of
// the K stored.
#pragma once
#include <cuda_runtime.h>

#include <type_traits>

namespace gb {

constexpr int kTiers = 6;

__host__ __device__ constexpr int tier_half(int K, int tier) {
    return tier >= kTiers - 1
               ? K / 2
               : ((K / 2) * (tier == 0 ? 4 : tier == 1 ? 7 : tier == 2 ? 10 : tier == 3 ? 13 : 16) +
                  10) / 20;
}

__host__ __device__ constexpr int tier_taps(int K, int tier) { return 2 * tier_half(K, tier) + 1; }

// Calls f(std::integral_constant<int, KK>) with the tap count of the plane's tier.
template <int K, typename F>
__device__ __forceinline__ void tier_dispatch(int tier, F &&f) {
    switch (tier) {
        case 0: f(std::integral_constant<int, tier_taps(K, 0)>{}); break;
        case 1: f(std::integral_constant<int, tier_taps(K, 1)>{}); break;
        case 2: f(std::integral_constant<int, tier_taps(K, 2)>{}); break;
        case 3: f(std::integral_constant<int, tier_taps(K, 3)>{}); break;
        case 4: f(std::integral_constant<int, tier_taps(K, 4)>{}); break;
        default: f(std::integral_constant<int, K>{}); break;
    }
}

// Scalar passes for CTAs whose register budget holds no tap registers (768-thread forward);
// the taps are read from shared memory (a broadcast load) inside the tap loop.
//
// First pass: blur along the S row axis for output row blocks [b_lo, b_hi) and columns
// [c_lo, c_hi); writes Tt[c][block * OB + j] (transposed).  Warp-tasks are (32-column
// chunk, row block), lanes take consecutive columns.
template <int K, int KK, int OB>
__device__ __forceinline__ void blur_first_st(const float *__restrict__ S, float *__restrict__ Tt,
                                              const float *__restrict__ tap, int SC, int TS,
                                              int c_lo, int c_hi, int b_lo, int b_hi, int warp,
                                              int lane, int nwarp) {
    constexpr int OFF = (K - KK) / 2;
    const int nb = b_hi - b_lo;
    const int ncc = (c_hi - c_lo + 31) >> 5;
    for (int p = warp; p < ncc * nb; p += nwarp) {
        const int cc = p % ncc, yb = b_lo + p / ncc;
        const int c = c_lo + (cc << 5) + lane;
        if (c >= c_hi) continue;
        const float *sp = S + (yb * OB + OFF) * SC + c;
        float win[OB + KK - 1];
#pragma unroll
        for (int i = 0; i < OB + KK - 1; i++) win[i] = sp[i * SC];
        float o[OB];
#pragma unroll
        for (int j = 0; j < OB; j++) o[j] = 0.f;
#pragma unroll
        for (int t = 0; t < KK; t++) {
            const float wt = tap[OFF + t];
#pragma unroll
            for (int j = 0; j < OB; j++) o[j] = fmaf(wt, win[j + t], o[j]);
        }
        float *tq = Tt + c * TS + yb * OB;
#pragma unroll
        for (int j = 0; j < OB; j++) tq[j] = o[j];
    }
}

// Second pass of one task: blur along the Tt row axis for OB consecutive outputs starting
// at Tt row `row0` (taps of the full bucket start there), column `col`; ACC: o += blur
// instead of o = blur.
template <int K, int KK, int OB, bool ACC>
__device__ __forceinline__ void blur_second_st(const float *__restrict__ Tt,
                                               const float *__restrict__ wsm, int TS, int row0,
                                               int col, float (&o)[OB]) {
    constexpr int OFF = (K - KK) / 2;
    const float *tq = Tt + (row0 + OFF) * TS + col;
    float win[OB + KK - 1];
#pragma unroll
    for (int i = 0; i < OB + KK - 1; i++) win[i] = tq[i * TS];
    if (!ACC) {
#pragma unroll
        for (int j = 0; j < OB; j++) o[j] = 0.f;
    }
#pragma unroll
    for (int t = 0; t < KK; t++) {
        const float wt = wsm[OFF + t];
#pragma unroll
        for (int j = 0; j < OB; j++) o[j] = fmaf(wt, win[j + t], o[j]);
    }
}

// Column-pair variants (fma.rn.f32x2): a thread owns two neighbouring columns and every
// tap is one packed FMA over both.  Each component is the same fmaf chain, in the same tap
// order, as the scalar passes above (identical results) with half the FMA and shared-load
// instructions.  Row strides and the first column must be even (8-byte float2 access).

// First pass over column pairs [c_lo & ~1, (c_hi + 1) & ~1): the extra edge column reads
// S zeros or samples outside the z range the second pass uses.  Warp-tasks are (64-column
// chunk, row block); the transposed output of the two columns goes out as float2 pairs.
template <int K, int KK, int OB>
__device__ __forceinline__ void blur_first2(const float *__restrict__ S, float *__restrict__ Tt,
                                            const float *__restrict__ tap, int SC, int TS,
                                            int c_lo, int c_hi, int b_lo, int b_hi, int warp,
                                            int lane, int nwarp) {
    static_assert(OB % 2 == 0, "pair stores need an even row block");
    constexpr int OFF = (K - KK) / 2;
    float w[KK];
#pragma unroll
    for (int t = 0; t < KK; t++) w[t] = tap[OFF + t];
    const int c0 = c_lo & ~1, c1 = (c_hi + 1) & ~1;
    const int nb = b_hi - b_lo;
    const int ncc = (c1 - c0 + 63) >> 6;
    const int SC2 = SC >> 1;
    for (int p = warp; p < ncc * nb; p += nwarp) {
        const int cc = p % ncc, yb = b_lo + p / ncc;
        const int c = c0 + (cc << 6) + 2 * lane;
        if (c >= c1) continue;
        const float2 *sp = reinterpret_cast<const float2 *>(S + (yb * OB + OFF) * SC + c);
        float2 win[OB + KK - 1];
#pragma unroll
        for (int i = 0; i < OB + KK - 1; i++) win[i] = sp[i * SC2];
        float2 o[OB];
#pragma unroll
        for (int j = 0; j < OB; j++) o[j] = make_float2(0.f, 0.f);
#pragma unroll
        for (int t = 0; t < KK; t++) {
            const float2 wt = make_float2(w[t], w[t]);
#pragma unroll
            for (int j = 0; j < OB; j++) o[j] = __ffma2_rn(wt, win[j + t], o[j]);
        }
        float *tq = Tt + c * TS + yb * OB;
#pragma unroll
        for (int j = 0; j < OB; j += 2) {
            *reinterpret_cast<float2 *>(tq + j) = make_float2(o[j].x, o[j + 1].x);
            *reinterpret_cast<float2 *>(tq + TS + j) = make_float2(o[j].y, o[j + 1].y);
        }
    }
}

// blur_first2 reading each tap from shared memory (a broadcast load) inside the tap loop
// instead of holding all taps in registers.
template <int K, int KK, int OB>
__device__ __forceinline__ void blur_first2_st(const float *__restrict__ S,
                                               float *__restrict__ Tt,
                                               const float *__restrict__ tap, int SC, int TS,
                                               int c_lo, int c_hi, int b_lo, int b_hi, int warp,
                                               int lane, int nwarp) {
    static_assert(OB % 2 == 0, "pair stores need an even row block");
    constexpr int OFF = (K - KK) / 2;
    const int c0 = c_lo & ~1, c1 = (c_hi + 1) & ~1;
    const int nb = b_hi - b_lo;
    const int ncc = (c1 - c0 + 63) >> 6;
    const int SC2 = SC >> 1;
    for (int p = warp; p < ncc * nb; p += nwarp) {
        const int cc = p % ncc, yb = b_lo + p / ncc;
        const int c = c0 + (cc << 6) + 2 * lane;
        if (c >= c1) continue;
        const float2 *sp = reinterpret_cast<const float2 *>(S + (yb * OB + OFF) * SC + c);
        float2 win[OB + KK - 1];
#pragma unroll
        for (int i = 0; i < OB + KK - 1; i++) win[i] = sp[i * SC2];
        float2 o[OB];
#pragma unroll
        for (int j = 0; j < OB; j++) o[j] = make_float2(0.f, 0.f);
#pragma unroll
        for (int t = 0; t < KK; t++) {
            const float wv = tap[OFF + t];
            const float2 wt = make_float2(wv, wv);
#pragma unroll
            for (int j = 0; j < OB; j++) o[j] = __ffma2_rn(wt, win[j + t], o[j]);
        }
        float *tq = Tt + c * TS + yb * OB;
#pragma unroll
        for (int j = 0; j < OB; j += 2) {
            *reinterpret_cast<float2 *>(tq + j) = make_float2(o[j].x, o[j + 1].x);
            *reinterpret_cast<float2 *>(tq + TS + j) = make_float2(o[j].y, o[j + 1].y);
        }
    }
}

// Second pass of one task over the column pair (col, col + 1), col even; ACC: o += blur.
template <int K, int KK, int OB, bool ACC>
__device__ __forceinline__ void blur_second2(const float *__restrict__ Tt,
                                             const float (&w)[KK], int TS, int row0, int col,
                                             float2 (&o)[OB]) {
    constexpr int OFF = (K - KK) / 2;
    const float2 *tq = reinterpret_cast<const float2 *>(Tt + (row0 + OFF) * TS + col);
    const int TS2 = TS >> 1;
    float2 win[OB + KK - 1];
#pragma unroll
    for (int i = 0; i < OB + KK - 1; i++) win[i] = tq[i * TS2];
    if (!ACC) {
#pragma unroll
        for (int j = 0; j < OB; j++) o[j] = make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int t = 0; t < KK; t++) {
        const float2 wt = make_float2(w[t], w[t]);
#pragma unroll
        for (int j = 0; j < OB; j++) o[j] = __ffma2_rn(wt, win[j + t], o[j]);
    }
}

template <int K, int KK>
__device__ __forceinline__ void load_taps(const float *__restrict__ tap, float (&w)[KK]) {
    constexpr int OFF = (K - KK) / 2;
#pragma unroll
    for (int t = 0; t < KK; t++) w[t] = tap[OFF + t];
}

}  // namespace gb
