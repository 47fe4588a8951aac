// Register-tiled per-plane blur passes shared by the forward (k_fwd_psf) and the
// back-projection (k_b1_psf) kernels.
//
// Tap tiers: a plane whose kernel is narrow (its outer taps are exactly zero, or below
// the plan's truncation threshold) runs a shorter unrolled loop.  A plane of bucket K
// (half width H) uses KK = 2h+1 taps with h = H/2, 3H/4 or H (tiers 0, 1, 2); the taps
// used are the centred KK of the K stored.
#pragma once
#include <cuda_runtime.h>

namespace gb {

__host__ __device__ constexpr int tier_half(int K, int tier) {
    return tier == 0 ? (K / 2) / 2 : (tier == 1 ? (3 * (K / 2)) / 4 : K / 2);
}

// First pass: blur along the S row axis for output row blocks [b_lo, b_hi) and columns
// [c_lo, c_hi); writes Tt[c][block * OB + j] (transposed).  Warp-tasks are (32-column
// chunk, row block), lanes take consecutive columns.
template <int K, int KK, int OB>
__device__ __forceinline__ void blur_first(const float *__restrict__ S, float *__restrict__ Tt,
                                           const float *__restrict__ tap, int SC, int TS,
                                           int c_lo, int c_hi, int b_lo, int b_hi, int warp,
                                           int lane, int nwarp) {
    constexpr int OFF = (K - KK) / 2;
    float w[KK];
#pragma unroll
    for (int t = 0; t < KK; t++) w[t] = tap[OFF + t];
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
        for (int t = 0; t < KK; t++)
#pragma unroll
            for (int j = 0; j < OB; j++) o[j] = fmaf(w[t], win[j + t], o[j]);
        float *tq = Tt + c * TS + yb * OB;
#pragma unroll
        for (int j = 0; j < OB; j++) tq[j] = o[j];
    }
}

// Second pass of one task: blur along the Tt row axis for OB consecutive outputs
// starting at Tt row `row0` (taps of the full bucket start there), column `col`.
template <int K, int KK, int OB>
__device__ __forceinline__ void blur_second(const float *__restrict__ Tt,
                                            const float (&w)[KK], int TS, int row0, int col,
                                            float (&o)[OB]) {
    constexpr int OFF = (K - KK) / 2;
    const float *tq = Tt + (row0 + OFF) * TS + col;
    float win[OB + KK - 1];
#pragma unroll
    for (int i = 0; i < OB + KK - 1; i++) win[i] = tq[i * TS];
#pragma unroll
    for (int j = 0; j < OB; j++) o[j] = 0.f;
#pragma unroll
    for (int t = 0; t < KK; t++)
#pragma unroll
        for (int j = 0; j < OB; j++) o[j] = fmaf(w[t], win[j + t], o[j]);
}

template <int K, int KK>
__device__ __forceinline__ void load_taps(const float *__restrict__ tap, float (&w)[KK]) {
    constexpr int OFF = (K - KK) / 2;
#pragma unroll
    for (int t = 0; t < KK; t++) w[t] = tap[OFF + t];
}

}  // namespace gb
