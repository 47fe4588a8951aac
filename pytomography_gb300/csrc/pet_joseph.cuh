// Joseph (1982) line integrals with optional TOF weighting, shared by the listmode and
// sinogram PET projectors.
//
// Reference wrappers: PETLMSystemMatrix (projectors/PET/petlm_system_matrix.py:24-363)
// and PETSinogramSystemMatrix (projectors/PET/pet_sinogram_system_matrix.py:12-296),
// whose arithmetic is delegated to the third-party parallelproj package
// (joseph3d_fwd / joseph3d_back / joseph3d_fwd_tof_lm / joseph3d_back_tof_lm /
// joseph3d_fwd_tof_sino / joseph3d_back_tof_sino).  parallelproj is not vendored and its
// version is not pinned; the model below restates the published Joseph method with
// parallelproj's documented parameters:
//   * voxel centres at origin + i * voxsize, image [nx][ny][nz] (z fastest);
//   * principal axis k = argmax |p1 - p0|; every plane i whose centre lies between the
//     two end points contributes the bilinear interpolation of the two other axes
//     (voxels outside the image count as zero), weighted by vox_k |d| / |d_k|;
//   * TOF: the plane is also weighted by the Gaussian (sigma) integrated over the TOF bin,
//     (erf((s + bw/2)/(sqrt2 sigma)) - erf((s - bw/2)/(sqrt2 sigma))) / 2, where s is the
//     signed distance along the LOR (towards p1) from the bin centre
//     mid + (tof_bin * bw + center_offset) * u; planes with |s| > n_sigmas sigma + bw/2
//     are skipped.  tof_bin is the stored bin minus (num_bins - 1) // 2.
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

namespace gb {

// TOF bin weight table: w(x) = (erfc((x - bw/2) q) - erfc((x + bw/2) q)) / 2 at
// x = m * lim / kTofTab, m = 0 .. kTofTab (+1 guard), q = 1 / (sqrt(2) sigma), computed
// in double on the host; linear interpolation in |s| (error below 1e-7 of the peak
// weight at the benchmark's sigma, bin width and n_sigmas).
constexpr int kTofTab = 4096;

// Host: the table for bin width bw, sigma and n_sigmas, and kTofTab / lim.
inline void tof_weight_table(float bw, float sigma, float n_sigmas, std::vector<float> &tab,
                             float &inv_step);

struct PetDev {
    int n[3];
    int n_vox;  // n[0] * n[1] * n[2]
    float vox[3], org[3];
    const float *lut;  // [n_det][3]
    int n_det;
    int tof;
    float bw, sig, co, nsig;
    int bin_shift;
    const float *tof_tab;  // [kTofTab + 2]
    float tof_inv_step;    // kTofTab / lim
};

__device__ __forceinline__ float pick(float a, float b, float c, int k) {
    return k == 0 ? a : (k == 1 ? b : c);
}
__device__ __forceinline__ int pick(int a, int b, int c, int k) {
    return k == 0 ? a : (k == 1 ? b : c);
}

// Joseph trace of one LOR.  BACK = false: returns sum of weighted samples of cimg.
// BACK = true: adds val * weights into img (atomics; the two corners of a bilinear pair
// that are neighbours in z go out as one 16-byte vector atomic, zeros in the other two
// lanes, when they share an aligned quad inside the image: 3 pairs in 4).
// Along the principal axis k the plane parameter t, the sample coordinates on the two
// other axes (in voxel units) and the TOF distance s are linear in the plane index i and
// are evaluated as base + i * step.  Axis-dependent quantities are selected into
// registers once (no dynamically indexed local arrays).
// DET (back projection only): img is an array of 64-bit integers holding fixed-point sums
// with `scale` units per 1.0; each contribution is rounded to that grid and added with an
// integer atomic, so the sums do not depend on the order of the additions.
template <bool BACK, bool TOF, bool DET = false>
__device__ __forceinline__ float joseph(const PetDev &g, const float *__restrict__ p0,
                                        const float *__restrict__ p1, float *img,
                                        const float *__restrict__ cimg, int tbin, float val,
                                        float scale = 0.f) {
    auto add = [&](int off, float v) {
        if constexpr (DET)
            atomicAdd(reinterpret_cast<unsigned long long *>(img) + off,
                      (unsigned long long)__float2ll_rn(v * scale));
        else
            atomicAdd(img + off, v);
    };
    const float ax = p0[0], ay = p0[1], az = p0[2];
    const float dx = p1[0] - ax, dy = p1[1] - ay, dz = p1[2] - az;
    const float len = sqrtf(dx * dx + dy * dy + dz * dz);
    if (len == 0.f) return 0.f;
    // principal axis from exact (double) differences of the float end points, so that
    // ties such as |dx| == |dy| resolve the same way as in exact arithmetic
    int k = 0;
    {
        const double ex = fabs((double)p1[0] - (double)ax), ey = fabs((double)p1[1] - (double)ay),
                     ez = fabs((double)p1[2] - (double)az);
        if (ey > ex) k = 1;
        if (ez > (k == 0 ? ex : ey)) k = 2;
    }
    const int a = (k + 1) % 3, b = (k + 2) % 3;
    const int nyz = g.n[1] * g.n[2];
    const float dk = pick(dx, dy, dz, k), da = pick(dx, dy, dz, a), db = pick(dx, dy, dz, b);
    const float pk = pick(ax, ay, az, k), pa0 = pick(ax, ay, az, a), pb0 = pick(ax, ay, az, b);
    const float vk = pick(g.vox[0], g.vox[1], g.vox[2], k);
    const float va = pick(g.vox[0], g.vox[1], g.vox[2], a);
    const float vb = pick(g.vox[0], g.vox[1], g.vox[2], b);
    const float ok = pick(g.org[0], g.org[1], g.org[2], k);
    const float oa = pick(g.org[0], g.org[1], g.org[2], a);
    const float ob = pick(g.org[0], g.org[1], g.org[2], b);
    const int nk = pick(g.n[0], g.n[1], g.n[2], k);
    const int na = pick(g.n[0], g.n[1], g.n[2], a);
    const int nb = pick(g.n[0], g.n[1], g.n[2], b);
    const int sk = pick(nyz, g.n[2], 1, k);
    const int sa = pick(nyz, g.n[2], 1, a);
    const int sb = pick(nyz, g.n[2], 1, b);
    const float cf = vk * len / fabsf(dk);
    const float pk1 = pick(p1[0], p1[1], p1[2], k);
    const float lo = fminf(pk, pk1), hi = fmaxf(pk, pk1);
    int i0 = (int)ceilf((lo - ok) / vk);
    int i1 = (int)floorf((hi - ok) / vk);
    i0 = max(i0, 0);
    i1 = min(i1, nk - 1);
    const float idk = 1.f / dk;
    const float t0 = (ok - pk) * idk, dt = vk * idk;  // t(i) = t0 + i dt
    const float iva = 1.f / va, ivb = 1.f / vb;
    const float fa0 = (pa0 - oa + t0 * da) * iva, dfa = dt * da * iva;
    const float fb0 = (pb0 - ob + t0 * db) * ivb, dfb = dt * db * ivb;
    float s0 = 0.f, ds = 0.f, lim = 0.f;
    if (TOF) {
        const float tc = tbin * g.bw + g.co;
        lim = g.nsig * g.sig + g.bw / 2;
        s0 = (t0 - 0.5f) * len - tc;  // s(i) = s0 + i ds: signed distance from the bin centre
        ds = dt * len;
        // planes with |s| <= lim, with one plane of slack; the exact test runs per plane
        float s_a = (((-lim + tc) / len + 0.5f) * dk + pk - ok) / vk;
        float s_b = (((lim + tc) / len + 0.5f) * dk + pk - ok) / vk;
        int ja = (int)floorf(fminf(s_a, s_b)) - 1, jb = (int)ceilf(fmaxf(s_a, s_b)) + 1;
        i0 = max(i0, ja);
        i1 = min(i1, jb);
    }
    float acc = 0.f;
    if constexpr (!BACK) {
        // Forward: the samples of PU consecutive planes are loaded together, then added
        // in plane order, corner by corner (the same sums as one plane at a time).
        constexpr int PU = 4;
        for (int i = i0; i <= i1; i += PU) {
            float wv[PU], wq[PU][4], vv[PU][4];
            bool ok[PU], in[PU][4];
#pragma unroll
            for (int u = 0; u < PU; u++) {
                const int ip = i + u;
                float w = cf;
                ok[u] = ip <= i1;
                if (TOF && ok[u]) {
                    const float as = fabsf(fmaf((float)ip, ds, s0));
                    if (as > lim) {
                        ok[u] = false;
                    } else {
                        const float t = as * g.tof_inv_step;
                        const int m = min((int)t, kTofTab);
                        const float t0w = __ldg(g.tof_tab + m), t1w = __ldg(g.tof_tab + m + 1);
                        w *= fmaf(t - (float)m, t1w - t0w, t0w);
                    }
                }
                wv[u] = w;
                const float fa = fmaf((float)ip, dfa, fa0), fb = fmaf((float)ip, dfb, fb0);
                const float ga = floorf(fa), gb2 = floorf(fb);
                const int ia = (int)ga, ib = (int)gb2;
                const float wa = fa - ga, wb = fb - gb2;
                const int base = ip * sk;
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int ja = ia + (q & 1), jb = ib + (q >> 1);
                    in[u][q] = ok[u] && (unsigned)ja < (unsigned)na && (unsigned)jb < (unsigned)nb;
                    wq[u][q] = ((q & 1) ? wa : 1.f - wa) * ((q >> 1) ? wb : 1.f - wb);
                    vv[u][q] = in[u][q] ? __ldg(cimg + base + ja * sa + jb * sb) : 0.f;
                }
            }
#pragma unroll
            for (int u = 0; u < PU; u++)
#pragma unroll
                for (int q = 0; q < 4; q++)
                    if (in[u][q]) acc += wv[u] * wq[u][q] * vv[u][q];
        }
        return acc;
    }
    // the bilinear pair axis that is z (stride 1), if any: corners along it are neighbours
    const bool zb = sb == 1, za = sa == 1;
    for (int i = i0; i <= i1; i++) {
        float w = cf;
        if (TOF) {
            const float as = fabsf(fmaf((float)i, ds, s0));
            if (as > lim) continue;
            const float u = as * g.tof_inv_step;
            const int m = min((int)u, kTofTab);
            const float t0w = __ldg(g.tof_tab + m), t1w = __ldg(g.tof_tab + m + 1);
            w *= fmaf(u - (float)m, t1w - t0w, t0w);
        }
        const float fa = fmaf((float)i, dfa, fa0), fb = fmaf((float)i, dfb, fb0);
        const float ga = floorf(fa), gb2 = floorf(fb);
        const int ia = (int)ga, ib = (int)gb2;
        const float wa = fa - ga, wb = fb - gb2;
        const int base = i * sk;
        if (BACK && (zb || za)) {
            // rows along the non-z axis, each with a z-neighbour pair
            const int jz = zb ? ib : ia, jo = zb ? ia : ib;
            const int nzz = zb ? nb : na, no = zb ? na : nb, so = zb ? sa : sb;
            const float wz = zb ? wb : wa, wo = zb ? wa : wb;
            const bool ok0 = (unsigned)jz < (unsigned)nzz, ok1 = (unsigned)(jz + 1) < (unsigned)nzz;
#pragma unroll
            for (int q = 0; q < 2; q++) {
                const int r = jo + q;
                if ((unsigned)r >= (unsigned)no) continue;
                const float wr = val * w * (q ? wo : 1.f - wo);
                const float v0 = wr * (1.f - wz), v1 = wr * wz;
                const int off = base + r * so + jz;
                const int qd = off & 3;  // the pair's position in its aligned quad
                if (!DET && ok0 && ok1 && qd < 3 && off - qd + 4 <= g.n_vox) {
                    // both corners in one 16-byte quad: one vector atomic (zeros elsewhere)
                    float4 v4 = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (qd == 0) {
                        v4.x = v0;
                        v4.y = v1;
                    } else if (qd == 1) {
                        v4.y = v0;
                        v4.z = v1;
                    } else {
                        v4.z = v0;
                        v4.w = v1;
                    }
                    atomicAdd(reinterpret_cast<float4 *>(img + (off - qd)), v4);
                } else {
                    if (ok0) add(off, v0);
                    if (ok1) add(off + 1, v1);
                }
            }
            continue;
        }
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int ja = ia + (q & 1), jb = ib + (q >> 1);
            if ((unsigned)ja >= (unsigned)na || (unsigned)jb >= (unsigned)nb) continue;
            const float wq = ((q & 1) ? wa : 1.f - wa) * ((q >> 1) ? wb : 1.f - wb);
            const int off = base + ja * sa + jb * sb;
            if (BACK)
                add(off, val * w * wq);
            else
                acc += w * wq * __ldg(cimg + off);
        }
    }
    return acc;
}

inline void tof_weight_table(float bw, float sigma, float n_sigmas, std::vector<float> &tab,
                             float &inv_step) {
    const double h = 0.5 * bw, q = 1.0 / (std::sqrt(2.0) * sigma);
    const double lim = (double)n_sigmas * sigma + h;
    tab.assign(kTofTab + 2, 0.f);
    for (int m = 0; m <= kTofTab; m++) {
        const double x = lim * m / kTofTab;
        tab[m] = (float)(0.5 * (std::erfc((x - h) * q) - std::erfc((x + h) * q)));
    }
    tab[kTofTab + 1] = tab[kTofTab];
    inv_step = (float)(kTofTab / lim);
}

}  // namespace gb
