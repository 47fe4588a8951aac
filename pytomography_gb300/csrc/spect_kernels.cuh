// SPECT rotate+sum kernels for sm_103a (GB300).
//
// Frames and layouts
//   object f      [N][N][nz]   unpadded, z fastest
//   padded frame  Lp = N + 2*pad rows (x) and cols (y); f_pad[r][c] = f[r-pad][c-pad]
//   projections   [n_sel][N][nz]
//   A (attenuation factors, per angle, rotated padded frame)  [n_angles][Lp][nya][nz],
//                 rows y in [ya_lo, ya_hi) only (the rows the PSF halo can reach)
//   W (back-projection stack of one angle group)              [G][Lp][nya][nz]
//
// Rotation convention (kornia, align_corners=True; utils/spatial.py:8-34,
// transforms/shared/spatial.py:21-53): an output voxel (row xp, col yp) samples
//   col = (th0*lin[yp] + th1*lin[xp] + th2 + 1) * (Lp-1)/2
//   row = (th3*lin[yp] + th4*lin[xp] + th5 + 1) * (Lp-1)/2
// bilinearly with zero padding; the arithmetic below keeps the operation order of
// the grid_sample CPU kernel (no FMA contraction) so the taps are reproducible.
#pragma once
#include <cuda.h>  // CUtensorMap
#include <cuda_runtime.h>
#include <stdint.h>

namespace gb {

constexpr float kDelta = 1e-11f;  // pytomography.delta (src/pytomography/__init__.py:21)

struct SpectDev {
    int *err;               // device error word (bounded waits that gave up), or null
    int2 *wrange;           // [G][Lp] W column range written per (slot, plane), or null
    int N, nz, pad, Lp;
    int n_angles;
    int ya_lo, ya_hi, nya;  // stored row range of A and W
    float half;             // (Lp - 1) / 2
    const float *lin;       // [Lp]
    const float *theta_fwd; // [n_angles][6]
    const float *theta_bwd; // [n_angles][6]
    const float *A;         // [n_angles][Lp][nya][nz] or null
    const float *taps_r;    // [n_groups][Lp][K]
    const float *taps_z;    // [n_groups][Lp][K]
    const int *group;       // [n_angles]
    const signed char *tier;  // [n_groups][Lp] tap tier of each plane, or null (full taps)
    int K;                  // taps per row (odd)
    int att;                // attenuation present
    int att_first;          // forward order: attenuation before PSF ("ap")
    int psf;                // PSF present
    int psf2d;              // PSF blurs z as well
    unsigned long long *phase;  // diagnostic builds: per-CTA forward phase cycles, or null
    unsigned wait_polls;        // polls of a bounded mbarrier wait before it gives up
    int dbg_skip_first_copy;    // test hook: the forward never issues its first TMA copy
};

// Polls of a bounded wait (each suspends for at most 20 us): about 1.3 s.
constexpr unsigned kWaitPolls = 1u << 16;

// Epilogue of the gather back-projector.
enum B2Mode : int {
    B2_WRITE = 0,   // out = bp
    B2_ADD = 1,     // out += bp
    B2_OSEM = 2,    // f += f/(nbp+d) * ((bp + acc) - nbp); clamp <= 0 -> 0
    B2_BSREM = 3,   // out = in + in*relax/(w*nbp_sum+d) * ((bp+acc) - nbp - rdp); clamp floor
};

struct UpdateArgs {
    float *f;              // OSEM: object updated in place
    const float *nbp;      // H_m^T 1
    const float *acc;      // partial back projection of earlier angle groups (or null)
    const float *f_in;     // BSREM input object
    float *f_out;          // BSREM output object
    const float *nbp_sum;  // BSREM: sum_k H_k^T 1
    float relax, w_m;      // BSREM relaxation and subset weight
    int prior;             // BSREM: RDP present
    float beta, gamma, rdelta;
    const float *fov;      // RDP FOV scale or null
    float w26[26];         // RDP neighbour weights, loop order i,j,k in {-1,0,1}
    float floor_v;         // BSREM clamp value
};

__device__ __forceinline__ void rot_coords(const float *__restrict__ th, float lin_row,
                                           float lin_col, float half, float &ix, float &iy) {
    float gx = __fadd_rn(__fadd_rn(__fmul_rn(th[0], lin_col), __fmul_rn(th[1], lin_row)), th[2]);
    float gy = __fadd_rn(__fadd_rn(__fmul_rn(th[3], lin_col), __fmul_rn(th[4], lin_row)), th[5]);
    ix = __fmul_rn(__fadd_rn(gx, 1.f), half);
    iy = __fmul_rn(__fadd_rn(gy, 1.f), half);
}

struct Bilin {
    int r0, c0;
    float nw, ne, sw, se;
};

__device__ __forceinline__ Bilin bilin(float ix, float iy) {
    Bilin b;
    float fx = floorf(ix), fy = floorf(iy);
    float w = __fsub_rn(ix, fx), e = __fsub_rn(1.f, w);
    float n = __fsub_rn(iy, fy), s = __fsub_rn(1.f, n);
    b.c0 = (int)fx;
    b.r0 = (int)fy;
    b.nw = __fmul_rn(s, e);
    b.ne = __fmul_rn(s, w);
    b.sw = __fmul_rn(n, e);
    b.se = __fmul_rn(n, w);
    return b;
}

// ((vnw*nw + vne*ne) + vsw*sw) + vse*se, the grid_sample summation order, with fused
// multiply-adds (rounding differs from the unfused CPU order by at most an ulp or two).
__device__ __forceinline__ float bilin_combine(const Bilin &b, float vnw, float vne, float vsw,
                                               float vse) {
    return fmaf(vse, b.se, fmaf(vsw, b.sw, fmaf(vne, b.ne, vnw * b.nw)));
}

// Bilinear sample of a [rows][cols][nz] array whose (row, col) origin is shifted by
// (row_off, col_off): value at (r, c) = src[r - row_off][c - col_off] when inside.
__device__ __forceinline__ float sample(const float *__restrict__ src, int rows, int cols,
                                        int nz, int row_off, int col_off, const Bilin &b,
                                        int z) {
    int r = b.r0 - row_off, c = b.c0 - col_off;
    bool r0 = (unsigned)r < (unsigned)rows, r1 = (unsigned)(r + 1) < (unsigned)rows;
    bool c0 = (unsigned)c < (unsigned)cols, c1 = (unsigned)(c + 1) < (unsigned)cols;
    if (!((r0 || r1) && (c0 || c1))) return 0.f;
    const float *p = src + ((long long)r * cols + c) * nz + z;
    float vnw = (r0 && c0) ? __ldg(p) : 0.f;
    float vne = (r0 && c1) ? __ldg(p + nz) : 0.f;
    float vsw = (r1 && c0) ? __ldg(p + (long long)cols * nz) : 0.f;
    float vse = (r1 && c1) ? __ldg(p + (long long)cols * nz + nz) : 0.f;
    return bilin_combine(b, vnw, vne, vsw, vse);
}

// Four consecutive z values (z % 4 == 0, nz % 4 == 0) of the bilinear sample; returns
// false (and zeros) when no tap is inside the array.
__device__ __forceinline__ bool sample4(const float *__restrict__ src, int rows, int cols, int nz,
                                        int row_off, int col_off, const Bilin &b, int z,
                                        float4 &out) {
    // branch-free: the four (predicated) loads of a sample can be in flight together
    int r = b.r0 - row_off, c = b.c0 - col_off;
    bool r0 = (unsigned)r < (unsigned)rows, r1 = (unsigned)(r + 1) < (unsigned)rows;
    bool c0 = (unsigned)c < (unsigned)cols, c1 = (unsigned)(c + 1) < (unsigned)cols;
    const float *p = src + ((long long)r * cols + c) * nz + z;
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 vnw = (r0 && c0) ? __ldg(reinterpret_cast<const float4 *>(p)) : zero;
    float4 vne = (r0 && c1) ? __ldg(reinterpret_cast<const float4 *>(p + nz)) : zero;
    float4 vsw = (r1 && c0) ? __ldg(reinterpret_cast<const float4 *>(p + (long long)cols * nz)) : zero;
    float4 vse = (r1 && c1) ? __ldg(reinterpret_cast<const float4 *>(p + (long long)cols * nz + nz))
                            : zero;
    out.x = bilin_combine(b, vnw.x, vne.x, vsw.x, vse.x);
    out.y = bilin_combine(b, vnw.y, vne.y, vsw.y, vse.y);
    out.z = bilin_combine(b, vnw.z, vne.z, vsw.z, vse.z);
    out.w = bilin_combine(b, vnw.w, vne.w, vsw.w, vse.w);
    return (r0 || r1) && (c0 || c1);
}

// Same as sample4 for the back-projection stack W of one angle slot: plane r holds data
// only in columns [wr[r].x, wr[r].y); everything else reads as zero.
__device__ __forceinline__ bool sample4_ranged(const float *__restrict__ src, int rows, int cols,
                                               int nz, int col_off, const int2 *__restrict__ wr,
                                               const Bilin &b, int z, float4 &out) {
    int r = b.r0, c = b.c0 - col_off;
    out = make_float4(0.f, 0.f, 0.f, 0.f);
    bool r0 = (unsigned)r < (unsigned)rows, r1 = (unsigned)(r + 1) < (unsigned)rows;
    int2 g0 = r0 ? wr[r] : make_int2(0, 0);
    int2 g1 = r1 ? wr[r + 1] : make_int2(0, 0);
    bool a00 = r0 && c >= g0.x && c < g0.y, a01 = r0 && c + 1 >= g0.x && c + 1 < g0.y;
    bool a10 = r1 && c >= g1.x && c < g1.y, a11 = r1 && c + 1 >= g1.x && c + 1 < g1.y;
    if (!(a00 || a01 || a10 || a11)) return false;
    const float *p = src + ((long long)r * cols + c) * nz + z;
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 vnw = a00 ? __ldg(reinterpret_cast<const float4 *>(p)) : zero;
    float4 vne = a01 ? __ldg(reinterpret_cast<const float4 *>(p + nz)) : zero;
    float4 vsw = a10 ? __ldg(reinterpret_cast<const float4 *>(p + (long long)cols * nz)) : zero;
    float4 vse = a11 ? __ldg(reinterpret_cast<const float4 *>(p + (long long)cols * nz + nz)) : zero;
    out.x = bilin_combine(b, vnw.x, vne.x, vsw.x, vse.x);
    out.y = bilin_combine(b, vnw.y, vne.y, vsw.y, vse.y);
    out.z = bilin_combine(b, vnw.z, vne.z, vsw.z, vse.z);
    out.w = bilin_combine(b, vnw.w, vne.w, vsw.w, vse.w);
    return true;
}

__device__ __forceinline__ float sample_ranged(const float *__restrict__ src, int rows, int cols,
                                               int nz, int col_off, const int2 *__restrict__ wr,
                                               const Bilin &b, int z) {
    int r = b.r0, c = b.c0 - col_off;
    bool r0 = (unsigned)r < (unsigned)rows, r1 = (unsigned)(r + 1) < (unsigned)rows;
    int2 g0 = r0 ? wr[r] : make_int2(0, 0);
    int2 g1 = r1 ? wr[r + 1] : make_int2(0, 0);
    bool a00 = r0 && c >= g0.x && c < g0.y, a01 = r0 && c + 1 >= g0.x && c + 1 < g0.y;
    bool a10 = r1 && c >= g1.x && c < g1.y, a11 = r1 && c + 1 >= g1.x && c + 1 < g1.y;
    if (!(a00 || a01 || a10 || a11)) return 0.f;
    const float *p = src + ((long long)r * cols + c) * nz + z;
    float vnw = a00 ? __ldg(p) : 0.f;
    float vne = a01 ? __ldg(p + nz) : 0.f;
    float vsw = a10 ? __ldg(p + (long long)cols * nz) : 0.f;
    float vse = a11 ? __ldg(p + (long long)cols * nz + nz) : 0.f;
    return bilin_combine(b, vnw, vne, vsw, vse);
}

// Rows y in [ylo, yhi) of plane xp whose sample (rotation th) can land within `margin`
// pixels of the object square [pad, pad+N) (Liang-Barsky clip of the sample segment,
// one row of slack on each side).  False when the plane misses the square.
__device__ __forceinline__ bool plane_rows(const SpectDev &g, const float *th, int xp, int ylo,
                                           int yhi, float margin, int &ra, int &rb) {
    const int y0 = ylo, y1 = yhi - 1;
    float ixa, iya, ixb, iyb;
    rot_coords(th, g.lin[xp], g.lin[y0], g.half, ixa, iya);
    rot_coords(th, g.lin[xp], g.lin[y1], g.half, ixb, iyb);
    const float lo = (float)g.pad - 1.f - margin, hi = (float)(g.pad + g.N) + margin;
    float t0 = 0.f, t1 = 1.f;
    const float p[2] = {ixa, iya}, d[2] = {ixb - ixa, iyb - iya};
#pragma unroll
    for (int k = 0; k < 2; k++) {
        if (fabsf(d[k]) < 1e-12f) {
            if (p[k] < lo || p[k] > hi) return false;
        } else {
            float ta = (lo - p[k]) / d[k], tb = (hi - p[k]) / d[k];
            if (ta > tb) {
                float t = ta;
                ta = tb;
                tb = t;
            }
            t0 = fmaxf(t0, ta);
            t1 = fminf(t1, tb);
        }
    }
    if (t0 > t1) return false;
    const float fa = y0 + t0 * (float)(y1 - y0), fb = y0 + t1 * (float)(y1 - y0);
    ra = max(ylo, (int)floorf(fa) - 1);
    rb = min(yhi - 1, (int)ceilf(fb) + 1);
    return ra <= rb;
}

// ---------------------------------------------------------------- TMA / mbarrier
__device__ __forceinline__ unsigned smem_u32(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_inval(unsigned long long *bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Orders this thread's (and, after a CTA barrier, the CTA's) generic-proxy shared-memory
// accesses before subsequent async-proxy (TMA) writes.
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 1-D TMA bulk copy global -> shared, completion counted on `bar` (16-byte aligned
// addresses, size a multiple of 16).
__device__ __forceinline__ void tma_load_1d(void *dst, const void *src, unsigned bytes,
                                            unsigned long long *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// 2-D TMA tensor copy global -> shared of one box of `map` at element coordinates (x, y)
// (x innermost; x * 4 bytes a multiple of 16).  The box lands densely in shared memory
// (128-byte aligned destination); elements outside the tensor read as zero.  Completion is
// counted on `bar` (the full box bytes).
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y,
                                            unsigned long long *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// Wait for phase `parity` of `bar`, giving up after `limit` polls; each poll may suspend
// the thread for up to 20 us while the phase is incomplete (no busy spinning).
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, unsigned parity,
                                                  unsigned limit) {
    for (unsigned i = 0; i < limit; i++) {
        unsigned ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(smem_u32(bar)), "r"(parity), "r"(20000u)
            : "memory");
        if (ok) return true;
    }
    return false;
}

constexpr int GB_ERR_WAIT_TIMEOUT = 1;  // value written to SpectDev::err

__device__ __forceinline__ float4 mul4(float4 a, float4 b) {
    return make_float4(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y), __fmul_rn(a.z, b.z),
                       __fmul_rn(a.w, b.w));
}

}  // namespace gb
