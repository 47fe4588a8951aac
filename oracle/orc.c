/*
 * CPU oracle for the GB300 projector hot path.  TEST INFRASTRUCTURE ONLY: this
 * code is the checker for the CUDA path (tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py).  It is never linked into the product library.
 *
 * It restates, in plain C with OpenMP, the algorithms of:
 *   SPECT rotate+sum projector     src/pytomography/projectors/SPECT/spect_system_matrix.py:120-201
 *   kornia-convention rotation     src/pytomography/utils/spatial.py:8-34,
 *                                  src/pytomography/transforms/shared/spatial.py:21-53
 *   padding                        src/pytomography/utils/spatial.py:36-119
 *   attenuation factor             src/pytomography/transforms/SPECT/attenuation.py:11-21,72-115
 *                                  + rev_cumsum src/pytomography/utils/misc.py:8-19
 *   separable Gaussian PSF         src/pytomography/transforms/SPECT/psf.py:15-41,199-231
 *   Joseph (TOF) listmode projector, called at
 *                                  src/pytomography/projectors/PET/petlm_system_matrix.py:102-108,
 *                                  163-170,270-289,330-351 (third-party parallelproj,
 *                                  absent and unpinned; restated from the published Joseph
 *                                  (1982) method and parallelproj's documented parameters).
 *
 * Compiled twice: REAL=double (the float64 oracle) and REAL=float (the reference's
 * working precision, used for the CPU baseline).  Accumulations are done in REAL.
 *
 * Array layouts are C order: object [Lx][Ly][Lz], projections [A][Ly][Lz]
 * (z fastest), PET image [nx][ny][nz], LUT [n_det][3], events [E][3].
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef REAL
#define REAL double
#endif

#define IDX3(a, b, c, nb, nc) (((size_t)(a) * (nb) + (b)) * (nc) + (c))

/* ---------------------------------------------------------------- geometry */

/* pad = ceil((sqrt(2) N - N) / 2)   (spatial.py:36-45) */
int orc_pad_size(int n) { return (int)ceil((sqrt(2.0) * n - n) / 2.0); }

/* kornia sampling matrix for a square H x H image: normalised dst -> src,
 * [[c, -s, 0], [s, c, 0]] for rotation angle `deg` (counter-clockwise positive). */
static void theta_for(double deg, REAL th[6]) {
    double a = deg * M_PI / 180.0;
    double c = cos(a), s = sin(a);
    th[0] = (REAL)c; th[1] = (REAL)(-s); th[2] = 0;
    th[3] = (REAL)s; th[4] = (REAL)c;    th[5] = 0;
}

static REAL lin(int i, int n) { return (REAL)(-1.0 + 2.0 * (double)i / (double)(n - 1)); }

/* Rotate a [H][H][Z] stack in the (row, col) plane about its centre by `deg`
 * (bilinear, zeros outside, align_corners=True), like
 * rotate(x.permute(2,0,1).unsqueeze(0), deg).  dst must not alias src. */
static void rotate_stack(const REAL *src, REAL *dst, int H, int Z, double deg) {
    REAL th[6];
    theta_for(deg, th);
    #pragma omp parallel for collapse(2) schedule(static)
    for (int h = 0; h < H; h++) {
        for (int w = 0; w < H; w++) {
            REAL xn = lin(w, H), yn = lin(h, H);
            REAL gx = th[0] * xn + th[1] * yn + th[2];
            REAL gy = th[3] * xn + th[4] * yn + th[5];
            REAL ix = (gx + 1) / 2 * (REAL)(H - 1);
            REAL iy = (gy + 1) / 2 * (REAL)(H - 1);
            REAL fx = floor(ix), fy = floor(iy);
            int x0 = (int)fx, y0 = (int)fy;
            REAL wx = ix - fx, wy = iy - fy;
            REAL wt[4] = {(1 - wy) * (1 - wx), (1 - wy) * wx, wy * (1 - wx), wy * wx};
            int rr[4] = {y0, y0, y0 + 1, y0 + 1}, cc[4] = {x0, x0 + 1, x0, x0 + 1};
            REAL *o = dst + IDX3(h, w, 0, H, Z);
            for (int z = 0; z < Z; z++) o[z] = 0;
            for (int k = 0; k < 4; k++) {
                if (rr[k] < 0 || rr[k] >= H || cc[k] < 0 || cc[k] >= H) continue;
                const REAL *s = src + IDX3(rr[k], cc[k], 0, H, Z);
                for (int z = 0; z < Z; z++) o[z] += wt[k] * s[z];
            }
        }
    }
}

/* Exact transpose of rotate_stack: scatter dst values back with the same taps. */
static void rotate_stack_T(const REAL *dst, REAL *src, int H, int Z, double deg) {
    REAL th[6];
    theta_for(deg, th);
    memset(src, 0, sizeof(REAL) * (size_t)H * H * Z);
    #pragma omp parallel
    {
        int nt = 1, it = 0;
#ifdef _OPENMP
        nt = omp_get_num_threads(); it = omp_get_thread_num();
#endif
        int z0 = (int)((long)Z * it / nt), z1 = (int)((long)Z * (it + 1) / nt);
        for (int h = 0; h < H; h++) {
            for (int w = 0; w < H; w++) {
                REAL xn = lin(w, H), yn = lin(h, H);
                REAL gx = th[0] * xn + th[1] * yn + th[2];
                REAL gy = th[3] * xn + th[4] * yn + th[5];
                REAL ix = (gx + 1) / 2 * (REAL)(H - 1);
                REAL iy = (gy + 1) / 2 * (REAL)(H - 1);
                REAL fx = floor(ix), fy = floor(iy);
                int x0 = (int)fx, y0 = (int)fy;
                REAL wx = ix - fx, wy = iy - fy;
                REAL wt[4] = {(1 - wy) * (1 - wx), (1 - wy) * wx, wy * (1 - wx), wy * wx};
                int rr[4] = {y0, y0, y0 + 1, y0 + 1}, cc[4] = {x0, x0 + 1, x0, x0 + 1};
                const REAL *o = dst + IDX3(h, w, 0, H, Z);
                for (int k = 0; k < 4; k++) {
                    if (rr[k] < 0 || rr[k] >= H || cc[k] < 0 || cc[k] >= H) continue;
                    REAL *s = src + IDX3(rr[k], cc[k], 0, H, Z);
                    for (int z = z0; z < z1; z++) s[z] += wt[k] * o[z];
                }
            }
        }
    }
}

/* exp(-rev_cumsum(mu_rot * dx)) along axis 0 (attenuation.py:11-21, misc.py:8-19) */
static void atten_factor(const REAL *mu_rot, REAL *A, int H, int Z, REAL dx) {
    #pragma omp parallel for schedule(static)
    for (int w = 0; w < H; w++) {
        for (int z = 0; z < Z; z++) {
            REAL run = 0;
            for (int h = H - 1; h >= 0; h--) {
                REAL v = mu_rot[IDX3(h, w, z, H, Z)] * dx;
                run += v;
                A[IDX3(h, w, z, H, Z)] = exp(-(run - v / 2));
            }
        }
    }
}

/* Per-plane separable blur of a [H][H][Z] stack: along y with taps wr[h][Kr], then
 * (if wz) along z with taps wz[h][Kz]; zero-padded 'same' correlation
 * (psf.py:27-41, 62-83). */
static void psf_blur(REAL *V, int H, int Z, const REAL *wr, int Kr, const REAL *wz, int Kz) {
    #pragma omp parallel
    {
        REAL *tmp = (REAL *)malloc(sizeof(REAL) * (size_t)H * Z);
        #pragma omp for schedule(static)
        for (int h = 0; h < H; h++) {
            REAL *P = V + IDX3(h, 0, 0, H, Z);
            const REAL *kr = wr + (size_t)h * Kr;
            int hr = Kr / 2;
            for (int y = 0; y < H; y++)
                for (int z = 0; z < Z; z++) {
                    REAL acc = 0;
                    for (int t = 0; t < Kr; t++) {
                        int yy = y + t - hr;
                        if (yy >= 0 && yy < H) acc += kr[t] * P[(size_t)yy * Z + z];
                    }
                    tmp[(size_t)y * Z + z] = acc;
                }
            if (wz) {
                const REAL *kz = wz + (size_t)h * Kz;
                int hz = Kz / 2;
                for (int y = 0; y < H; y++)
                    for (int z = 0; z < Z; z++) {
                        REAL acc = 0;
                        for (int t = 0; t < Kz; t++) {
                            int zz = z + t - hz;
                            if (zz >= 0 && zz < Z) acc += kz[t] * tmp[(size_t)y * Z + zz];
                        }
                        P[(size_t)y * Z + z] = acc;
                    }
            } else {
                memcpy(P, tmp, sizeof(REAL) * (size_t)H * Z);
            }
        }
        free(tmp);
    }
}

/* One angle of the projector.
 *   order: string of transform codes in obj2obj order, 'a' = attenuation, 'p' = PSF.
 *   mode 0: forward   obj[Lx][Ly][Lz] -> proj[Ly][Lz]            (SSM:145-154)
 *   mode 1: backward  proj[Ly][Lz]   -> obj (accumulated)        (SSM:188-198)
 *   mode 2: exact adjoint of mode 0  proj -> obj (accumulated)
 *   wr/wz are the PSF taps of this angle, [Lxp][K]. */
int orc_spect_angle(int mode, const REAL *in, REAL *out, const REAL *mu, int N, int Lz,
                    REAL dx, double beta_deg, const char *order, const REAL *wr, int Kr,
                    const REAL *wz, int Kz) {
    int pad = orc_pad_size(N), H = N + 2 * pad;
    size_t P = (size_t)H * H * Lz;
    REAL *V = (REAL *)calloc(P, sizeof(REAL));
    REAL *T = (REAL *)calloc(P, sizeof(REAL));
    REAL *A = NULL;
    int n_t = (int)strlen(order);
    if (!V || !T) return -1;
    if (strchr(order, 'a')) {
        if (!mu) return -2;
        for (int x = 0; x < N; x++)
            for (int y = 0; y < N; y++)
                memcpy(T + IDX3(x + pad, y + pad, 0, H, Lz), mu + IDX3(x, y, 0, N, Lz),
                       sizeof(REAL) * Lz);
        A = (REAL *)malloc(P * sizeof(REAL));
        rotate_stack(T, V, H, Lz, beta_deg - 270.0);
        atten_factor(V, A, H, Lz, dx);
        memset(T, 0, P * sizeof(REAL));
        memset(V, 0, P * sizeof(REAL));
    }
    if (mode == 0) {
        for (int x = 0; x < N; x++)
            for (int y = 0; y < N; y++)
                memcpy(T + IDX3(x + pad, y + pad, 0, H, Lz), in + IDX3(x, y, 0, N, Lz),
                       sizeof(REAL) * Lz);
        rotate_stack(T, V, H, Lz, beta_deg - 270.0);
        for (int t = 0; t < n_t; t++) {
            if (order[t] == 'a') {
                for (size_t i = 0; i < P; i++) V[i] *= A[i];
            } else {
                psf_blur(V, H, Lz, wr, Kr, wz, Kz);
            }
        }
        for (int y = 0; y < N; y++)
            for (int z = 0; z < Lz; z++) {
                REAL acc = 0;
                for (int h = 0; h < H; h++) acc += V[IDX3(h, y + pad, z, H, Lz)];
                out[(size_t)y * Lz + z] = acc;
            }
    } else {
        for (int h = 0; h < H; h++)
            for (int y = 0; y < N; y++)
                memcpy(V + IDX3(h, y + pad, 0, H, Lz), in + (size_t)y * Lz, sizeof(REAL) * Lz);
        for (int t = n_t - 1; t >= 0; t--) {
            if (order[t] == 'a') {
                for (size_t i = 0; i < P; i++) V[i] *= A[i];
            } else {
                psf_blur(V, H, Lz, wr, Kr, wz, Kz);
            }
        }
        if (mode == 1)
            rotate_stack(V, T, H, Lz, 270.0 - beta_deg);
        else
            rotate_stack_T(V, T, H, Lz, beta_deg - 270.0);
        for (int x = 0; x < N; x++)
            for (int y = 0; y < N; y++) {
                REAL *o = out + IDX3(x, y, 0, N, Lz);
                const REAL *s = T + IDX3(x + pad, y + pad, 0, H, Lz);
                for (int z = 0; z < Lz; z++) o[z] += s[z];
            }
    }
    free(V); free(T); free(A);
    return 0;
}

/* The per-angle obj2obj plugins on an object already in the detector frame of one
 * angle, [H][H][Lz] with H = N + 2 pad (pad = 0: the unpadded frame of
 * assume_padded=False):
 *   which 0: attenuation, out = in * exp(-rev_cumsum(mu_rot * dx)), mu [N][N][Lz] zero-padded
 *            by pad and rotated by beta - 270 (attenuation.py:72-115);
 *   which 1: the separable PSF with taps wr [H][Kr] and wz [H][Kz] (wz NULL: '1D')
 *            (psf.py:199-231). */
int orc_spect_plugin(int which, const REAL *in, REAL *out, const REAL *mu, int N, int Lz,
                     int pad, REAL dx, double beta_deg, const REAL *wr, int Kr, const REAL *wz,
                     int Kz) {
    int H = N + 2 * pad;
    size_t P = (size_t)H * H * Lz;
    memcpy(out, in, P * sizeof(REAL));
    if (which == 1) {
        psf_blur(out, H, Lz, wr, Kr, wz, Kz);
        return 0;
    }
    if (!mu) return -2;
    REAL *T = (REAL *)calloc(P, sizeof(REAL));
    REAL *V = (REAL *)calloc(P, sizeof(REAL));
    if (!T || !V) return -1;
    for (int x = 0; x < N; x++)
        for (int y = 0; y < N; y++)
            memcpy(T + IDX3(x + pad, y + pad, 0, H, Lz), mu + IDX3(x, y, 0, N, Lz),
                   sizeof(REAL) * Lz);
    rotate_stack(T, V, H, Lz, beta_deg - 270.0);
    atten_factor(V, T, H, Lz, dx);
    for (size_t i = 0; i < P; i++) out[i] *= T[i];
    free(T); free(V);
    return 0;
}

/* ------------------------------------------------------------------- PET */

/* Joseph ray tracing of one LOR p0 -> p1 through an image with voxel centres at
 * origin + i * vox.  For every plane of the principal axis whose centre lies
 * between p0 and p1, the LOR point is bilinearly interpolated in the two other
 * axes (out-of-image voxels count as zero); the plane value is weighted by the
 * step length cf = vox_k |d| / |d_k| and, with TOF, by the Gaussian integrated
 * over the TOF bin:
 *   w = (erf((s + bw/2)/(sqrt2 sig)) - erf((s - bw/2)/(sqrt2 sig))) / 2,
 * s = signed distance along the LOR (towards p1) between the plane point and
 * the bin centre  mid + (tof_bin * bw + center_offset) * u;  planes with
 * |s| > n_sigmas * sig + bw/2 are skipped.
 * back = 0: returns the line integral of img; back = 1: adds val * weights into img. */
static REAL joseph(int back, const REAL *p0, const REAL *p1, REAL *img, const int *n,
                   const REAL *origin, const REAL *vox, int tof, REAL bw, REAL sig,
                   REAL center_offset, REAL n_sigmas, int tof_bin, REAL val) {
    REAL d[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
    REAL len = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    if (len == 0) return 0;
    /* principal axis from exact differences of the end points (ties such as
     * |dx| == |dy| resolve as in exact arithmetic, whatever REAL is) */
    int k = 0;
    {
        double e[3] = {fabs((double)p1[0] - (double)p0[0]), fabs((double)p1[1] - (double)p0[1]),
                       fabs((double)p1[2] - (double)p0[2])};
        if (e[1] > e[0]) k = 1;
        if (e[2] > e[k]) k = 2;
    }
    int a = (k + 1) % 3, b = (k + 2) % 3;
    REAL cf = vox[k] * len / fabs(d[k]);
    REAL u[3] = {d[0] / len, d[1] / len, d[2] / len};
    REAL mid[3] = {(p0[0] + p1[0]) / 2, (p0[1] + p1[1]) / 2, (p0[2] + p1[2]) / 2};
    REAL tc = tof_bin * bw + center_offset;
    REAL lim = n_sigmas * sig + bw / 2;
    REAL isq = 1 / (sqrt((REAL)2) * sig);
    /* planes with centre between p0_k and p1_k */
    REAL lo = fmin(p0[k], p1[k]), hi = fmax(p0[k], p1[k]);
    int i0 = (int)ceil((lo - origin[k]) / vox[k]);
    int i1 = (int)floor((hi - origin[k]) / vox[k]);
    if (i0 < 0) i0 = 0;
    if (i1 > n[k] - 1) i1 = n[k] - 1;
    REAL acc = 0;
    for (int i = i0; i <= i1; i++) {
        REAL ck = origin[k] + i * vox[k];
        REAL t = (ck - p0[k]) / d[k];
        REAL pa = p0[a] + t * d[a], pb = p0[b] + t * d[b];
        REAL w = cf;
        if (tof) {
            REAL s = (t - (REAL)0.5) * len - tc;
            if (fabs(s) > lim) continue;
            w *= (erf((s + bw / 2) * isq) - erf((s - bw / 2) * isq)) / 2;
        }
        REAL fa = (pa - origin[a]) / vox[a], fb = (pb - origin[b]) / vox[b];
        REAL ga = floor(fa), gb = floor(fb);
        int ia = (int)ga, ib = (int)gb;
        REAL wa = fa - ga, wb = fb - gb;
        for (int q = 0; q < 4; q++) {
            int ja = ia + (q & 1), jb = ib + (q >> 1);
            if (ja < 0 || ja >= n[a] || jb < 0 || jb >= n[b]) continue;
            REAL wq = ((q & 1) ? wa : 1 - wa) * ((q >> 1) ? wb : 1 - wb);
            int id[3];
            id[k] = i; id[a] = ja; id[b] = jb;
            size_t off = IDX3(id[0], id[1], id[2], n[1], n[2]);
            if (back) {
                REAL add = val * w * wq;
                #pragma omp atomic
                img[off] += add;
            } else {
                acc += w * wq * img[off];
            }
        }
    }
    (void)mid; (void)u;
    return acc;
}

/* Listmode projector.  lut [n_det][3] mm; ids [E][ncol] (id1, id2[, tof bin]);
 * tof_bins_centered: bin index already shifted by -(num_bins-1)//2 is applied
 * here as ids[:,2] - bin_shift.  back = 0: proj[E] = H img; back = 1: img += H^T proj. */
int orc_pet_lm(int back, const REAL *lut, const int64_t *ids, int ncol, int64_t E, REAL *img,
               const int *n, const REAL *origin, const REAL *vox, REAL *proj, int tof, REAL bw,
               REAL sig, REAL center_offset, REAL n_sigmas, int bin_shift) {
    #pragma omp parallel for schedule(dynamic, 256)
    for (int64_t e = 0; e < E; e++) {
        const REAL *p0 = lut + 3 * ids[e * ncol + 0];
        const REAL *p1 = lut + 3 * ids[e * ncol + 1];
        int tb = tof ? (int)(ids[e * ncol + 2] - bin_shift) : 0;
        if (back)
            joseph(1, p0, p1, img, n, origin, vox, tof, bw, sig, center_offset, n_sigmas, tb,
                   proj[e]);
        else
            proj[e] = joseph(0, p0, p1, img, n, origin, vox, tof, bw, sig, center_offset,
                             n_sigmas, tb, 0);
    }
    return 0;
}

/* TOF sinogram projector with explicit LOR endpoints xs/xe [E][3]: proj [E][nb], bin t
 * centred as t - bin_shift (joseph3d_fwd_tof_sino / joseph3d_back_tof_sino call sites
 * pet_sinogram_system_matrix.py:213-225, 271-284). */
int orc_pet_lor_tof(int back, const REAL *xs, const REAL *xe, int64_t E, REAL *img,
                    const int *n, const REAL *origin, const REAL *vox, REAL *proj, int nb,
                    REAL bw, REAL sig, REAL center_offset, REAL n_sigmas, int bin_shift) {
    #pragma omp parallel for schedule(dynamic, 64)
    for (int64_t e = 0; e < E; e++) {
        for (int t = 0; t < nb; t++) {
            REAL *pv = proj + e * nb + t;
            if (back)
                joseph(1, xs + 3 * e, xe + 3 * e, img, n, origin, vox, 1, bw, sig, center_offset,
                       n_sigmas, t - bin_shift, *pv);
            else
                *pv = joseph(0, xs + 3 * e, xe + 3 * e, img, n, origin, vox, 1, bw, sig,
                             center_offset, n_sigmas, t - bin_shift, 0);
        }
    }
    return 0;
}

/* Same, with explicit LOR endpoints xs/xe [E][3] (used for sensitivity LOR sets). */
int orc_pet_lor(int back, const REAL *xs, const REAL *xe, int64_t E, REAL *img, const int *n,
                const REAL *origin, const REAL *vox, REAL *proj) {
    #pragma omp parallel for schedule(dynamic, 256)
    for (int64_t e = 0; e < E; e++) {
        if (back)
            joseph(1, xs + 3 * e, xe + 3 * e, img, n, origin, vox, 0, 1, 1, 0, 3, 0, proj[e]);
        else
            proj[e] = joseph(0, xs + 3 * e, xe + 3 * e, img, n, origin, vox, 0, 1, 1, 0, 3, 0, 0);
    }
    return 0;
}
