// StarGuide detector window (StarGuideSystemMatrix, projectors/SPECT/starguide_system_matrix.py:
// 30-140): after the rotate -> attenuate -> PSF -> sum projection in the unpadded frame, every
// detector row is translated along y by its offset (kornia Translate: the output at column
// y is the input at column y - shift, linear interpolation, zero outside, :214-230), cropped
// to `width` columns starting at int(ny / 2) - width / 2 (:80-82) and scaled by the
// detector's acquisition time (:84).  Translation along y commutes with the sum along x,
// so it runs once per detector row here instead of once per object plane.  The back
// projection does the reverse (:100-110): scale, zero-pad to ny columns, translate by
// -shift, then the usual back projection.
#include "common.cuh"

namespace gb {

__device__ __forceinline__ float lerp_row(const float *__restrict__ row, int ny, int nz, float s,
                                          int z) {
    const float fl = floorf(s);
    const int y0 = (int)fl;
    const float w = s - fl;
    float v = 0.f;
    if (y0 >= 0 && y0 < ny) v += (1.f - w) * row[(size_t)y0 * nz + z];
    if (y0 + 1 >= 0 && y0 + 1 < ny) v += w * row[(size_t)(y0 + 1) * nz + z];
    return v;
}

// out [n][width][nz] = scale[i] * translate(full[i], shift[i]) on the window columns
__global__ void k_sg_crop(const float *__restrict__ full, float *__restrict__ out, int n, int ny,
                          int nz, int width, const float *__restrict__ shift,
                          const float *__restrict__ scale) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (long long)n * width * nz) return;
    const int z = (int)(q % nz);
    const int c = (int)((q / nz) % width);
    const int i = (int)(q / ((long long)nz * width));
    const int c0 = ny / 2 - width / 2;
    const float *row = full + (size_t)i * ny * nz;
    out[q] = scale[i] * lerp_row(row, ny, nz, (float)(c + c0) - shift[i], z);
}

// full [n][ny][nz] = translate(pad(scale[i] * proj[i]), -shift[i])
__global__ void k_sg_expand(const float *__restrict__ proj, float *__restrict__ full, int n,
                            int ny, int nz, int width, const float *__restrict__ shift,
                            const float *__restrict__ scale) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (long long)n * ny * nz) return;
    const int z = (int)(q % nz);
    const int y = (int)((q / nz) % ny);
    const int i = (int)(q / ((long long)nz * ny));
    const int c0 = ny / 2 - width / 2;
    // padded row p[y'] = proj[y' - c0] for y' in [c0, c0 + width); sample at y + shift
    const float s = (float)y + shift[i] - (float)c0;
    full[q] = scale[i] * lerp_row(proj + (size_t)i * width * nz, width, nz, s, z);
}

}  // namespace gb

using namespace gb;

extern "C" {

gb_status gb_starguide_window(const float *full, float *out, int32_t n, int32_t ny, int32_t nz,
                              int32_t width, const float *shift, const float *scale,
                              gb_stream_t stream) {
    clear_error();
    GB_CHECK_ARG(full && out && shift && scale, "null argument");
    GB_CHECK_ARG(n >= 0 && ny > 0 && nz > 0 && width > 0 && width <= ny, "invalid window shape");
    const long long total = (long long)n * width * nz;
    if (total == 0) return GB_OK;
    k_sg_crop<<<(unsigned)((total + 255) / 256), 256, 0, as_stream(stream)>>>(full, out, n, ny, nz,
                                                                              width, shift, scale);
    GB_LAUNCH_CHECK();
    return GB_OK;
}

gb_status gb_starguide_window_adjoint(const float *proj, float *full, int32_t n, int32_t ny,
                                      int32_t nz, int32_t width, const float *shift,
                                      const float *scale, gb_stream_t stream) {
    clear_error();
    GB_CHECK_ARG(full && proj && shift && scale, "null argument");
    GB_CHECK_ARG(n >= 0 && ny > 0 && nz > 0 && width > 0 && width <= ny, "invalid window shape");
    GB_CHECK_ARG((ny - width) % 2 == 0, "ny - width must be even (the window is zero-padded "
                                        "symmetrically)");
    const long long total = (long long)n * ny * nz;
    if (total == 0) return GB_OK;
    k_sg_expand<<<(unsigned)((total + 255) / 256), 256, 0, as_stream(stream)>>>(
        proj, full, n, ny, nz, width, shift, scale);
    GB_LAUNCH_CHECK();
    return GB_OK;
}

}  // extern "C"
