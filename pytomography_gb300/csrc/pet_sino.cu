// PET sinogram projectors (TOF and non-TOF Joseph, pet_joseph.cuh), the attenuation
// probability sinogram, and listmode -> sinogram binning.
//
// Reference: PETSinogramSystemMatrix (projectors/PET/pet_sinogram_system_matrix.py:12-296):
// the LOR of sinogram element (angle a, radial r, plane p) runs from
// (x1, y1, z1) = (det_xy[a][r][0], plane_z[p][0]) to (x2, y2, z2) = (det_xy[a][r][1],
// plane_z[p][1]) (_get_xyz_sinogram_coordinates, :50-85); subsets are angles i::n
// (:131-144).  TOF sinograms hold every bin of every LOR (bin fastest); one thread traces
// one (LOR, bin) restricted to that bin's TOF window, so the threads of a warp trace the
// bins of the same or neighbouring LORs.  The listmode binning restates
// listmode_to_sinogram / _listmodeTOF_to_sinogramTOF (io/PET/shared.py:175-272).
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "pet_joseph.cuh"

namespace gb {

struct SinoGeom {
    const float *det_xy;   // [A][R][2][2]
    const float *plane_z;  // [P][2]
    int A, R, P;
};

__device__ __forceinline__ void sino_lor(const SinoGeom &sg, int a, int r, int p, float *p0,
                                         float *p1) {
    const float4 xy = *reinterpret_cast<const float4 *>(sg.det_xy + ((size_t)a * sg.R + r) * 4);
    p0[0] = xy.x;
    p0[1] = xy.y;
    p0[2] = sg.plane_z[2 * p];
    p1[0] = xy.z;
    p1[1] = xy.w;
    p1[2] = sg.plane_z[2 * p + 1];
}

// proj [n_sel][R][P](x nb): element q -> (angle slot, r, p[, bin]); angle = first + slot * stride.
// atten: write exp(-sum) (attenuation probability) instead of the sum.
template <bool TOF>
__global__ void __launch_bounds__(256)
    k_sino_fwd(PetDev g, SinoGeom sg, int first, int stride, long long total, int nb,
               const float *__restrict__ img, float *__restrict__ proj, int atten) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= total) return;
    const long long lor = TOF ? q / nb : q;
    const int bin = TOF ? (int)(q - lor * nb) : 0;
    const int p = (int)(lor % sg.P);
    const long long t = lor / sg.P;
    const int r = (int)(t % sg.R), slot = (int)(t / sg.R);
    float p0[3], p1[3];
    sino_lor(sg, first + slot * stride, r, p, p0, p1);
    const float v = joseph<false, TOF>(g, p0, p1, nullptr, img, bin - g.bin_shift, 0.f);
    proj[q] = atten ? expf(-v) : v;
}

template <bool TOF>
__global__ void __launch_bounds__(256)
    k_sino_bwd(PetDev g, SinoGeom sg, int first, int stride, long long total, int nb,
               const float *__restrict__ proj, float *__restrict__ img) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= total) return;
    const float v = proj[q];
    if (v == 0.f) return;
    const long long lor = TOF ? q / nb : q;
    const int bin = TOF ? (int)(q - lor * nb) : 0;
    const int p = (int)(lor % sg.P);
    const long long t = lor / sg.P;
    const int r = (int)(t % sg.R), slot = (int)(t / sg.R);
    float p0[3], p1[3];
    sino_lor(sg, first + slot * stride, r, p, p0, p1);
    joseph<true, TOF>(g, p0, p1, img, nullptr, bin - g.bin_shift, v);
}

// Listmode -> sinogram.  Per event: within-ring ids w = id % ncpr and rings id / ncpr,
// ordered by decreasing within-ring id (ties keep the event's order; a swap mirrors the
// TOF bin to nb - 1 - bin), sinogram bin (angular, radial) = lor_bins[w_hi][w_lo] and
// plane = plane_idx[ring_hi][ring_lo]; out-of-range bins are dropped.  normalization adds
// half a count at the mirrored pair (lor_bins[w_lo][w_hi], plane_idx[ring_lo][ring_hi]) and
// half at the ordered one.
__global__ void k_lm_to_sino(const int *__restrict__ ev, long long E, int ncol,
                             const float *__restrict__ w, const int *__restrict__ lor_bins,
                             const int *__restrict__ plane_idx, int ncpr, int nr, int A, int R,
                             int P, int nb, int normalization, float *__restrict__ sino) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const int id1 = ev[e * ncol], id2 = ev[e * ncol + 1];
    const int w1 = id1 % ncpr, w2 = id2 % ncpr, r1 = id1 / ncpr, r2 = id2 / ncpr;
    const bool sw = w2 > w1;
    const int wa = sw ? w2 : w1, wb = sw ? w1 : w2, ra = sw ? r2 : r1, rb = sw ? r1 : r2;
    int bin = 0;
    if (nb > 0) {
        bin = ev[e * ncol + 2];
        if (sw) bin = nb - 1 - bin;
        if (bin < 0 || bin >= nb) return;
    }
    const float val = w ? w[e] : 1.f;
    auto put = [&](int x, int y, int rx, int ry, float v) {
        if (x < 0 || x >= ncpr || y < 0 || y >= ncpr || rx < 0 || rx >= nr || ry < 0 || ry >= nr)
            return;
        const int ang = lor_bins[2 * (x * ncpr + y)], rad = lor_bins[2 * (x * ncpr + y) + 1];
        const int pl = plane_idx[rx * nr + ry];
        if (ang < 0 || ang >= A || rad < 0 || rad >= R || pl < 0 || pl >= P) return;
        size_t o = ((size_t)ang * R + rad) * P + pl;
        if (nb > 0) o = o * nb + bin;
        atomicAdd(sino + o, v);
    };
    if (normalization) {
        put(wa, wb, ra, rb, 0.5f * val);
        put(wb, wa, rb, ra, 0.5f * val);
    } else {
        put(wa, wb, ra, rb, val);
    }
}

}  // namespace gb

using namespace gb;

struct gb_pet_sino_plan {
    PetDev dev{};
    SinoGeom geom{};
    float *d_det = nullptr, *d_z = nullptr, *d_tof_tab = nullptr;
    int n_subsets = 1;
    int nb = 0;
};

static void sino_free(gb_pet_sino_plan *p) {
    if (!p) return;
    dev_free(p->d_det);
    dev_free(p->d_z);
    dev_free(p->d_tof_tab);
    delete p;
}

static void sino_range(const gb_pet_sino_plan *p, int subset, int &first, int &stride, int &n) {
    if (subset < 0) {
        first = 0;
        stride = 1;
        n = p->geom.A;
    } else {
        first = subset;
        stride = p->n_subsets;
        n = p->geom.A > subset ? (p->geom.A - subset + p->n_subsets - 1) / p->n_subsets : 0;
    }
}

extern "C" {

gb_status gb_pet_sino_plan_create(const gb_pet_sino_desc *d, gb_pet_sino_plan **out) {
    clear_error();
    GB_CHECK_ARG(d && out, "null argument");
    *out = nullptr;
    GB_CHECK_ARG(d->nx > 0 && d->ny > 0 && d->nz > 0, "image shape must be positive");
    GB_CHECK_ARG(d->n_angles > 0 && d->n_radial > 0 && d->n_planes > 0,
                 "sinogram shape must be positive");
    GB_CHECK_ARG(d->det_xy && d->plane_z, "sinogram geometry tables missing");
    GB_CHECK_ARG(!d->tof || (d->tof_sigma > 0 && d->tof_bin_width > 0 && d->tof_num_bins > 0),
                 "invalid TOF parameters");
    auto *p = new gb_pet_sino_plan();
    PetDev &g = p->dev;
    g.n[0] = d->nx; g.n[1] = d->ny; g.n[2] = d->nz;
    g.n_vox = d->nx * d->ny * d->nz;
    g.vox[0] = d->vx; g.vox[1] = d->vy; g.vox[2] = d->vz;
    g.org[0] = d->ox; g.org[1] = d->oy; g.org[2] = d->oz;
    g.tof = d->tof;
    g.bw = d->tof_bin_width;
    g.sig = d->tof_sigma;
    g.co = d->tof_center_offset;
    g.nsig = d->tof_n_sigmas;
    g.bin_shift = (d->tof_num_bins - 1) / 2;
    p->nb = d->tof ? d->tof_num_bins : 0;
    p->geom.A = d->n_angles;
    p->geom.R = d->n_radial;
    p->geom.P = d->n_planes;
    const size_t ndet = (size_t)d->n_angles * d->n_radial * 4, nz2 = (size_t)d->n_planes * 2;
    cudaError_t e;
    if ((e = dev_alloc(&p->d_det, ndet * sizeof(float))) != cudaSuccess ||
        (e = cudaMemcpy(p->d_det, d->det_xy, ndet * sizeof(float), cudaMemcpyHostToDevice)) !=
            cudaSuccess ||
        (e = dev_alloc(&p->d_z, nz2 * sizeof(float))) != cudaSuccess ||
        (e = cudaMemcpy(p->d_z, d->plane_z, nz2 * sizeof(float), cudaMemcpyHostToDevice)) !=
            cudaSuccess) {
        set_error("sinogram table upload failed: %s", cudaGetErrorString(e));
        sino_free(p);
        return e == cudaErrorMemoryAllocation ? GB_ERR_OOM : GB_ERR_CUDA;
    }
    p->geom.det_xy = p->d_det;
    p->geom.plane_z = p->d_z;
    if (d->tof) {
        std::vector<float> tab;
        float inv_step = 0.f;
        tof_weight_table(d->tof_bin_width, d->tof_sigma, d->tof_n_sigmas, tab, inv_step);
        if ((e = dev_alloc(&p->d_tof_tab, tab.size() * sizeof(float))) != cudaSuccess ||
            (e = cudaMemcpy(p->d_tof_tab, tab.data(), tab.size() * sizeof(float),
                            cudaMemcpyHostToDevice)) != cudaSuccess) {
            set_error("TOF table upload failed: %s", cudaGetErrorString(e));
            sino_free(p);
            return GB_ERR_CUDA;
        }
        g.tof_tab = p->d_tof_tab;
        g.tof_inv_step = inv_step;
    }
    *out = p;
    return GB_OK;
}

gb_status gb_pet_sino_plan_destroy(gb_pet_sino_plan *p) {
    clear_error();
    if (p) {
        cudaDeviceSynchronize();
        sino_free(p);
    }
    return GB_OK;
}

gb_status gb_pet_sino_set_subsets(gb_pet_sino_plan *p, int32_t n_subsets) {
    clear_error();
    GB_CHECK_ARG(p && n_subsets >= 1 && n_subsets <= p->geom.A, "n_subsets must be in [1, %d]",
                 p ? p->geom.A : 0);
    p->n_subsets = n_subsets;
    return GB_OK;
}

int32_t gb_pet_sino_subset_size(const gb_pet_sino_plan *p, int32_t subset) {
    if (!p || subset >= p->n_subsets) return -1;
    int first, stride, n;
    sino_range(p, subset, first, stride, n);
    return n;
}

gb_status gb_pet_sino_forward(gb_pet_sino_plan *p, const float *img, float *proj, int32_t subset,
                              int32_t use_tof, gb_stream_t stream) {
    clear_error();
    GB_CHECK_ARG(p && img && proj, "null argument");
    GB_CHECK_ARG(subset < p->n_subsets, "subset out of range");
    int first, stride, n;
    sino_range(p, subset, first, stride, n);
    const bool tof = use_tof && p->nb > 0;
    const long long total = (long long)n * p->geom.R * p->geom.P * (tof ? p->nb : 1);
    if (total == 0) return GB_OK;
    const unsigned blocks = (unsigned)((total + 255) / 256);
    cudaStream_t st = as_stream(stream);
    if (tof)
        k_sino_fwd<true><<<blocks, 256, 0, st>>>(p->dev, p->geom, first, stride, total, p->nb, img,
                                                 proj, 0);
    else
        k_sino_fwd<false><<<blocks, 256, 0, st>>>(p->dev, p->geom, first, stride, total, 1, img,
                                                  proj, 0);
    GB_LAUNCH_CHECK();
    return GB_OK;
}

gb_status gb_pet_sino_backward(gb_pet_sino_plan *p, const float *proj, float *img,
                               int32_t subset, int32_t use_tof, gb_stream_t stream) {
    clear_error();
    GB_CHECK_ARG(p && img && proj, "null argument");
    GB_CHECK_ARG(((uintptr_t)img & 15) == 0, "image buffer must be 16-byte aligned");
    GB_CHECK_ARG(subset < p->n_subsets, "subset out of range");
    int first, stride, n;
    sino_range(p, subset, first, stride, n);
    const bool tof = use_tof && p->nb > 0;
    const long long total = (long long)n * p->geom.R * p->geom.P * (tof ? p->nb : 1);
    cudaStream_t st = as_stream(stream);
    GB_CUDA(cudaMemsetAsync(img, 0,
                            (size_t)p->dev.n[0] * p->dev.n[1] * p->dev.n[2] * sizeof(float), st));
    if (total == 0) return GB_OK;
    const unsigned blocks = (unsigned)((total + 255) / 256);
    if (tof)
        k_sino_bwd<true><<<blocks, 256, 0, st>>>(p->dev, p->geom, first, stride, total, p->nb,
                                                 proj, img);
    else
        k_sino_bwd<false><<<blocks, 256, 0, st>>>(p->dev, p->geom, first, stride, total, 1, proj,
                                                  img);
    GB_LAUNCH_CHECK();
    return GB_OK;
}

gb_status gb_pet_sino_atten(gb_pet_sino_plan *p, const float *mu, float *prob, int32_t subset,
                            gb_stream_t stream) {
    clear_error();
    GB_CHECK_ARG(p && mu && prob, "null argument");
    GB_CHECK_ARG(subset < p->n_subsets, "subset out of range");
    int first, stride, n;
    sino_range(p, subset, first, stride, n);
    const long long total = (long long)n * p->geom.R * p->geom.P;
    if (total == 0) return GB_OK;
    k_sino_fwd<false><<<(unsigned)((total + 255) / 256), 256, 0, as_stream(stream)>>>(
        p->dev, p->geom, first, stride, total, 1, mu, prob, 1);
    GB_LAUNCH_CHECK();
    return GB_OK;
}

gb_status gb_pet_lm_to_sino(const int32_t *events, int64_t n_events, int32_t ncol,
                            const float *weights, const int32_t *lor_bins,
                            const int32_t *plane_index, int32_t n_crystals_per_ring,
                            int32_t n_rings, int32_t n_angles, int32_t n_radial,
                            int32_t n_planes, int32_t tof_num_bins, int32_t normalization,
                            float *sino, gb_stream_t stream) {
    clear_error();
    GB_CHECK_ARG(sino && lor_bins && plane_index, "null argument");
    GB_CHECK_ARG(n_events >= 0 && (n_events == 0 || events), "events missing");
    GB_CHECK_ARG(ncol == 2 || ncol == 3, "events need 2 or 3 columns");
    GB_CHECK_ARG(tof_num_bins == 0 || ncol == 3, "TOF binning needs a TOF bin column");
    GB_CHECK_ARG(n_crystals_per_ring > 0 && n_rings > 0 && n_angles > 0 && n_radial > 0 &&
                     n_planes > 0,
                 "sinogram geometry must be positive");
    cudaStream_t st = as_stream(stream);
    const size_t n_out = (size_t)n_angles * n_radial * n_planes * std::max(1, (int)tof_num_bins);
    GB_CUDA(cudaMemsetAsync(sino, 0, n_out * sizeof(float), st));
    if (n_events == 0) return GB_OK;
    k_lm_to_sino<<<(unsigned)((n_events + 255) / 256), 256, 0, st>>>(
        events, n_events, ncol, weights, lor_bins, plane_index, n_crystals_per_ring, n_rings,
        n_angles, n_radial, n_planes, tof_num_bins, normalization, sino);
    GB_LAUNCH_CHECK();
    return GB_OK;
}

}  // extern "C"
