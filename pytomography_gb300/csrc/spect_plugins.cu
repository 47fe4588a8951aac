// Per-angle SPECT obj2obj plugins on an already rotated object: the attenuation factor
// and the depth-dependent separable PSF, each as its own kernel.
//
// These are the plugin calls SPECTAttenuationTransform.forward/backward
// (transforms/SPECT/attenuation.py:72-115) and SPECTPSFTransform.forward/backward
// (transforms/SPECT/psf.py:199-231 -> Seperable1DBlurNet.forward, :27-41) make inside the
// reference's per-angle loop (projectors/SPECT/spect_system_matrix.py:145-154, 188-198).
// The fused projector applies the same two operators inside its plane sweep; these
// kernels serve callers that drive the plugins one angle at a time.
//
// Attenuation: every thread owns one (y, z quad) ray of the rotated frame and walks it
// from the detector side (x = L - 1) towards x = 0, sampling the rotated mu map on the
// fly (bilinear, kornia convention) and keeping the reverse cumulative sum of mu*dx in
// registers; a warp covers 32 consecutive z quads of one row, so the scan front of a
// warp is one coalesced 512-byte row segment per plane.  Nothing is stored between
// calls: the factor exp(-(sum_{k>=x} mu_k dx - mu_x dx / 2)) is formed as the walk
// passes plane x and multiplied into the output at once.
//
// PSF: one CTA per (plane, 16-row tile, 32-column z tile).  The input tile with its
// K/2 halo is staged in shared memory, blurred along y into a second buffer (z halo
// included), then along z into the output; zero padding ('same' convolution) outside
// the plane.
#include "common.cuh"
#include "spect_kernels.cuh"

namespace gb {

struct Theta6 {
    float v[6];
};

// ------------------------------------------------------------- attenuation
template <bool VEC>
__global__ void __launch_bounds__(256)
    k_att_apply(const float *__restrict__ mu, int N, int nz, int pad, int L, float half, Theta6 th,
                const float *__restrict__ lin, float dx, const float *in, float *out) {
    constexpr int W = VEC ? 4 : 1;   // z values per thread
    constexpr int PU = VEC ? 4 : 8;  // planes sampled per step (loads in flight together)
    const int nzw = nz / W;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= L * nzw) return;
    const int y = i / nzw, z = (i % nzw) * W;
    const float lc = lin[y];
    const size_t plane = (size_t)L * nz;
    const size_t off = (size_t)y * nz + z;
    float run[W];
#pragma unroll
    for (int w = 0; w < W; w++) run[w] = 0.f;
    for (int x0 = L - 1; x0 >= 0; x0 -= PU) {
        float v[PU][W];
#pragma unroll
        for (int u = 0; u < PU; u++) {
            const int xp = max(x0 - u, 0);
            float ix, iy;
            rot_coords(th.v, lin[xp], lc, half, ix, iy);
            const Bilin b = bilin(ix, iy);
            if constexpr (VEC) {
                float4 s4;
                sample4(mu, N, N, nz, pad, pad, b, z, s4);
                v[u][0] = __fmul_rn(s4.x, dx);
                v[u][1] = __fmul_rn(s4.y, dx);
                v[u][2] = __fmul_rn(s4.z, dx);
                v[u][3] = __fmul_rn(s4.w, dx);
            } else {
                v[u][0] = __fmul_rn(sample(mu, N, N, nz, pad, pad, b, z), dx);
            }
        }
#pragma unroll
        for (int u = 0; u < PU; u++) {
            const int xp = x0 - u;
            if (xp < 0) break;
            const size_t o = (size_t)xp * plane + off;
            if constexpr (VEC) {
                const float4 a = *reinterpret_cast<const float4 *>(in + o);
                float e[4];
#pragma unroll
                for (int w = 0; w < 4; w++) {
                    run[w] = __fadd_rn(run[w], v[u][w]);
                    e[w] = expf(-__fsub_rn(run[w], __fmul_rn(v[u][w], 0.5f)));
                }
                *reinterpret_cast<float4 *>(out + o) =
                    make_float4(__fmul_rn(a.x, e[0]), __fmul_rn(a.y, e[1]), __fmul_rn(a.z, e[2]),
                                __fmul_rn(a.w, e[3]));
            } else {
                run[0] = __fadd_rn(run[0], v[u][0]);
                const float e = expf(-__fsub_rn(run[0], __fmul_rn(v[u][0], 0.5f)));
                out[o] = __fmul_rn(in[o], e);
            }
        }
    }
}

// --------------------------------------------------------------------- PSF
constexpr int kPsfTY = 16;  // output rows per CTA
constexpr int kPsfTZ = 32;  // output z per CTA
constexpr int kPsfMaxK = 63;

// Dynamic shared memory: S [(TY + 2Hy)][(TZ + 2Hz)], U [TY][(TZ + 2Hz)], taps [ky + kz].
__global__ void __launch_bounds__(256)
    k_psf_apply(const float *__restrict__ in, float *__restrict__ out, int ny, int nz,
                const float *__restrict__ taps_y, const float *__restrict__ taps_z, int ky,
                int kz) {
    extern __shared__ float sm[];
    const int x = blockIdx.z;
    const int y0 = blockIdx.x * kPsfTY, z0 = blockIdx.y * kPsfTZ;
    const int hy = ky / 2, hz = taps_z ? kz / 2 : 0;
    const int SR = kPsfTY + 2 * hy, SC = kPsfTZ + 2 * hz;
    float *S = sm;
    float *U = S + SR * SC;
    float *wy = U + kPsfTY * SC;
    float *wz = wy + ky;
    const float *P = in + (size_t)x * ny * nz;
    for (int t = threadIdx.x; t < ky; t += blockDim.x) wy[t] = taps_y[(size_t)x * ky + t];
    if (taps_z)
        for (int t = threadIdx.x; t < kz; t += blockDim.x) wz[t] = taps_z[(size_t)x * kz + t];
    for (int e = threadIdx.x; e < SR * SC; e += blockDim.x) {
        const int r = e / SC, c = e % SC;
        const int y = y0 - hy + r, z = z0 - hz + c;
        S[e] = (y >= 0 && y < ny && z >= 0 && z < nz) ? P[(size_t)y * nz + z] : 0.f;
    }
    __syncthreads();
    // blur along y (rows of S): U[r][c] = sum_t wy[t] S[r + t][c]
    for (int e = threadIdx.x; e < kPsfTY * SC; e += blockDim.x) {
        const int r = e / SC, c = e % SC;
        float acc = 0.f;
        for (int t = 0; t < ky; t++) acc = fmaf(wy[t], S[(r + t) * SC + c], acc);
        U[e] = acc;
    }
    __syncthreads();
    // blur along z, write the tile
    float *Q = out + (size_t)x * ny * nz;
    for (int e = threadIdx.x; e < kPsfTY * kPsfTZ; e += blockDim.x) {
        const int r = e / kPsfTZ, c = e % kPsfTZ;
        const int y = y0 + r, z = z0 + c;
        if (y >= ny || z >= nz) continue;
        float acc;
        if (taps_z) {
            acc = 0.f;
            for (int t = 0; t < kz; t++) acc = fmaf(wz[t], U[r * SC + c + t], acc);
        } else {
            acc = U[r * SC + c];
        }
        Q[(size_t)y * nz + z] = acc;
    }
}

}  // namespace gb

using namespace gb;

extern "C" gb_status gb_spect_attenuation_apply(const float *mu, int32_t n, int32_t nz,
                                                int32_t pad, float dx, const float *theta,
                                                const float *lin, const float *in, float *out,
                                                gb_stream_t stream) {
    clear_error();
    GB_CHECK_ARG(mu && theta && lin && in && out, "null argument");
    GB_CHECK_ARG(n > 0 && nz > 0 && pad >= 0, "invalid shape (n=%d, nz=%d, pad=%d)", n, nz, pad);
    const int L = n + 2 * pad;
    Theta6 th;
    for (int k = 0; k < 6; k++) th.v[k] = theta[k];
    const float half = (float)(L - 1) / 2.0f;
    const bool vec = nz % 4 == 0 && ((uintptr_t)in & 15) == 0 && ((uintptr_t)out & 15) == 0 &&
                     ((uintptr_t)mu & 15) == 0;
    cudaStream_t st = as_stream(stream);
    if (vec) {
        const int total = L * (nz / 4);
        k_att_apply<true><<<(total + 255) / 256, 256, 0, st>>>(mu, n, nz, pad, L, half, th, lin,
                                                               dx, in, out);
    } else {
        const int total = L * nz;
        k_att_apply<false><<<(total + 255) / 256, 256, 0, st>>>(mu, n, nz, pad, L, half, th, lin,
                                                                dx, in, out);
    }
    GB_LAUNCH_CHECK();
    return GB_OK;
}

extern "C" gb_status gb_spect_psf_apply(const float *in, float *out, int32_t nplanes, int32_t ny,
                                        int32_t nz, const float *taps_y, int32_t ky,
                                        const float *taps_z, int32_t kz, gb_stream_t stream) {
    clear_error();
    GB_CHECK_ARG(in && out && taps_y, "null argument");
    GB_CHECK_ARG(in != out, "the PSF reads neighbouring rows: in and out must differ");
    GB_CHECK_ARG(nplanes > 0 && ny > 0 && nz > 0, "invalid shape (%d, %d, %d)", nplanes, ny, nz);
    GB_CHECK_ARG(ky > 0 && ky % 2 == 1 && (!taps_z || (kz > 0 && kz % 2 == 1)),
                 "tap counts must be odd (ky=%d, kz=%d)", ky, kz);
    if (ky > kPsfMaxK || (taps_z && kz > kPsfMaxK)) {
        set_error("PSF kernels of more than %d taps are not supported (ky=%d, kz=%d)", kPsfMaxK,
                  ky, kz);
        return GB_ERR_UNSUPPORTED;
    }
    GB_CHECK_ARG(nplanes <= 65535, "at most 65535 planes per call (got %d)", nplanes);
    const int hy = ky / 2, hz = taps_z ? kz / 2 : 0;
    const int SC = kPsfTZ + 2 * hz;
    const size_t smem =
        sizeof(float) * ((size_t)(kPsfTY + 2 * hy) * SC + (size_t)kPsfTY * SC + ky + (taps_z ? kz : 0));
    dim3 grid((ny + kPsfTY - 1) / kPsfTY, (nz + kPsfTZ - 1) / kPsfTZ, nplanes);
    k_psf_apply<<<grid, 256, smem, as_stream(stream)>>>(in, out, ny, nz, taps_y, taps_z, ky,
                                                        taps_z ? kz : 0);
    GB_LAUNCH_CHECK();
    return GB_OK;
}
