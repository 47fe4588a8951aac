// Object-space operators either side of the projectors:
//   * the separable Gaussian filter (GaussianFilter, transforms/shared/filters.py:8-80):
//     'same' zero-padded correlation along x, then y, then z with per-axis taps;
//   * the kernel-method basis K (KEMTransform.forward, transforms/shared/kem.py:111-128):
//     out[v] = sum over the size^3 offsets (a, b, c), in (a, b, c) loop order, of
//     kern[(a, b, c)][v] * in[clamp(x + a), clamp(y + b), clamp(z + c)] (replicate
//     boundary, utils/misc.py:40-57).
// Both are memory-bound streaming passes; neighbour reads hit L1/L2.
#include "common.cuh"

namespace gb {

// one axis of the separable filter: out = taps (*) in along `ax`
__global__ void __launch_bounds__(256)
    k_conv_axis(const float *__restrict__ in, float *__restrict__ out, int nx, int ny, int nz,
                int ax, const float *__restrict__ taps, int K) {
    const long long n = (long long)nx * ny * nz;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int z = (int)(i % nz);
    const int y = (int)((i / nz) % ny);
    const int x = (int)(i / ((long long)ny * nz));
    const int len = ax == 0 ? nx : (ax == 1 ? ny : nz);
    const int pos = ax == 0 ? x : (ax == 1 ? y : z);
    const long long stride = ax == 0 ? (long long)ny * nz : (ax == 1 ? nz : 1);
    const int h = K / 2;
    float acc = 0.f;
    for (int t = 0; t < K; t++) {
        const int q = pos + t - h;
        if (q >= 0 && q < len) acc = fmaf(__ldg(taps + t), __ldg(in + i + (q - pos) * stride), acc);
    }
    out[i] = acc;
}

__global__ void __launch_bounds__(256)
    k_kem(const float *__restrict__ in, float *__restrict__ out, const float *__restrict__ kern,
          int nx, int ny, int nz, int size) {
    const long long n = (long long)nx * ny * nz;
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const int z = (int)(v % nz);
    const int y = (int)((v / nz) % ny);
    const int x = (int)(v / ((long long)ny * nz));
    const int h = size / 2;
    float acc = 0.f;
    long long t = 0;
    for (int a = -h; a <= h; a++) {
        const int xa = min(max(x + a, 0), nx - 1);
        for (int b = -h; b <= h; b++) {
            const int yb = min(max(y + b, 0), ny - 1);
            const float *row = in + ((long long)xa * ny + yb) * nz;
            for (int c = -h; c <= h; c++, t++) {
                const int zc = min(max(z + c, 0), nz - 1);
                acc += __ldg(kern + t * n + v) * __ldg(row + zc);
            }
        }
    }
    out[v] = acc;
}

}  // namespace gb

using namespace gb;

extern "C" {

gb_status gb_filter3d(const float *in, float *out, float *scratch, int32_t nx, int32_t ny,
                      int32_t nz, const float *taps_x, int32_t kx, const float *taps_y,
                      int32_t ky, const float *taps_z, int32_t kz, gb_stream_t stream) {
    clear_error();
    GB_CHECK_ARG(in && out && scratch && taps_x && taps_y && taps_z, "null argument");
    GB_CHECK_ARG(nx > 0 && ny > 0 && nz > 0, "shape must be positive");
    GB_CHECK_ARG(kx > 0 && ky > 0 && kz > 0 && (kx & 1) && (ky & 1) && (kz & 1),
                 "tap counts must be odd and positive");
    GB_CHECK_ARG(out != in && scratch != in && scratch != out,
                 "in, out and scratch must be distinct buffers");
    const long long n = (long long)nx * ny * nz;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    cudaStream_t st = as_stream(stream);
    k_conv_axis<<<blocks, 256, 0, st>>>(in, out, nx, ny, nz, 0, taps_x, kx);
    GB_LAUNCH_CHECK();
    k_conv_axis<<<blocks, 256, 0, st>>>(out, scratch, nx, ny, nz, 1, taps_y, ky);
    GB_LAUNCH_CHECK();
    k_conv_axis<<<blocks, 256, 0, st>>>(scratch, out, nx, ny, nz, 2, taps_z, kz);
    GB_LAUNCH_CHECK();
    return GB_OK;
}

gb_status gb_kem_apply(const float *in, float *out, const float *kern, int32_t nx, int32_t ny,
                       int32_t nz, int32_t size, gb_stream_t stream) {
    clear_error();
    GB_CHECK_ARG(in && out && kern, "null argument");
    GB_CHECK_ARG(in != out, "in and out must be distinct buffers");
    GB_CHECK_ARG(nx > 0 && ny > 0 && nz > 0, "shape must be positive");
    GB_CHECK_ARG(size > 0 && (size & 1), "kernel size must be odd and positive");
    const long long n = (long long)nx * ny * nz;
    k_kem<<<(unsigned)((n + 255) / 256), 256, 0, as_stream(stream)>>>(in, out, kern, nx, ny, nz,
                                                                      size);
    GB_LAUNCH_CHECK();
    return GB_OK;
}

}  // extern "C"
