// PET listmode projectors: TOF and non-TOF Joseph line integrals (pet_joseph.cuh) and
// their adjoints over sorted event tiles, sensitivity back projection over generated
// crystal pairs, and the fused listmode OSEM sub-iteration.
//
// Reference wrapper: PETLMSystemMatrix (projectors/PET/petlm_system_matrix.py:24-363);
// parallelproj call sites petlm_system_matrix.py:102-108, 163-170, 270-289, 330-351
// (TOF bin centring by (num_bins - 1) // 2 at :280).
#include <algorithm>
#include <cmath>
#include <vector>

#include <cub/device/device_radix_sort.cuh>

#include "common.cuh"
#include "pet_joseph.cuh"

namespace gb {

// Event tiles: the events of a list (every event, or one subset i::n) sorted by a
// locality key, packed as {id1, id2, centred TOF bin, j} where j is the event's position
// in the list (event index first + j * stride).  Threads of a warp then trace nearby,
// nearly parallel LORs: their image reads share L1 lines and their back-projection
// atomics share L2 sectors.  Outputs indexed by j keep the list order.
//
// mode 0: out[k or j] = H img;  mode 1 (ratio): out[k] = num[e] / (H img + s[e] + delta)
template <bool TOF>
__global__ void __launch_bounds__(256)
    k_pet_fwd(PetDev g, const int4 *__restrict__ rec, long long first, long long stride,
              long long n, const float *__restrict__ img, float *__restrict__ out, int ratio,
              const float *__restrict__ sadd, const float *__restrict__ gnum, int gnum_len) {
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int4 r = rec[k];
    const float *p0 = g.lut + 3 * (long long)r.x;
    const float *p1 = g.lut + 3 * (long long)r.y;
    float v = joseph<false, TOF>(g, p0, p1, nullptr, img, r.z, 0.f);
    if (ratio) {  // internal ratio array, tile order
        const long long e = first + (long long)r.w * stride;
        float pr = sadd ? v + sadd[e] : v;
        float num = gnum_len > 1 ? gnum[e] : gnum[0];
        out[k] = num / (pr + 1e-11f);
    } else {
        out[r.w] = v;
    }
}

// proj in tile order (sorted = 1, the fused step's ratio array) or list order (0)
template <bool TOF>
__global__ void __launch_bounds__(256)
    k_pet_bwd(PetDev g, const int4 *__restrict__ rec, long long n,
              const float *__restrict__ proj, int sorted, float *__restrict__ img) {
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int4 r = rec[k];
    const float v = proj[sorted ? k : (long long)r.w];
    if (v == 0.f) return;
    const float *p0 = g.lut + 3 * (long long)r.x;
    const float *p1 = g.lut + 3 * (long long)r.y;
    joseph<true, TOF>(g, p0, p1, img, nullptr, r.z, v);
}

// Deterministic back projection: the same traces accumulated as 64-bit fixed-point sums.
template <bool TOF>
__global__ void __launch_bounds__(256)
    k_pet_bwd_det(PetDev g, const int4 *__restrict__ rec, long long n,
                  const float *__restrict__ proj, const float *__restrict__ scale,
                  unsigned long long *__restrict__ acc) {
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int4 r = rec[k];
    const float v = proj[(long long)r.w];
    if (v == 0.f) return;
    const float *p0 = g.lut + 3 * (long long)r.x;
    const float *p1 = g.lut + 3 * (long long)r.y;
    joseph<true, TOF, true>(g, p0, p1, reinterpret_cast<float *>(acc), nullptr, r.z, v, *scale);
}

// Largest |proj| of the list (atomicMax on the bit patterns of non-negative floats, which
// order like the values; the result does not depend on the order).
__global__ void k_abs_max(const int4 *__restrict__ rec, long long n, const float *__restrict__ proj,
                          unsigned *__restrict__ out) {
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    float m = 0.f;
    if (k < n) m = fabsf(proj[(long long)rec[k].w]);
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0.f) atomicMax(out, __float_as_uint(m));
}

// Fixed-point scale: a power of two such that n events of magnitude <= max|proj|, each
// adding at most cf_max (the longest plane step) to a voxel, stay below 2^61.
__global__ void k_det_scale(const unsigned *__restrict__ maxbits, long long n, float cf_max,
                            float *__restrict__ scale) {
    const double bound = (double)__uint_as_float(*maxbits) * (double)n * (double)cf_max;
    int e = 0;
    if (bound > 0.0) frexp(bound, &e);  // bound < 2^e
    *scale = (float)ldexp(1.0, max(-100, min(100, 61 - e)));
}

__global__ void k_det_to_float(const unsigned long long *__restrict__ acc,
                               const float *__restrict__ scale, float *__restrict__ img,
                               long long n) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    img[i] = (float)((double)(long long)acc[i] / (double)*scale);
}

// Locality key of list event j: principal axis (2 bits), transaxial direction in 8 bins
// over [0, pi) (3 bits) and the Morton code of the TOF-window centre (the LOR midpoint
// without TOF) in cells of 8 voxels, 6 bits per axis (18 bits).
__device__ __forceinline__ unsigned morton3(unsigned x, unsigned y, unsigned z) {
    unsigned m = 0;
#pragma unroll
    for (int b = 0; b < 6; b++)
        m |= (((x >> b) & 1u) << (3 * b)) | (((y >> b) & 1u) << (3 * b + 1)) |
             (((z >> b) & 1u) << (3 * b + 2));
    return m;
}

__global__ void k_pet_keys(PetDev g, const int *__restrict__ ev, int ncol, long long first,
                           long long stride, long long n, unsigned *__restrict__ keys,
                           int *__restrict__ vals) {
    long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int *r = ev + (first + j * stride) * ncol;
    const float *p0 = g.lut + 3 * (long long)r[0];
    const float *p1 = g.lut + 3 * (long long)r[1];
    const float d[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
    const float len = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    const float ad0 = fabsf(d[0]), ad1 = fabsf(d[1]), ad2 = fabsf(d[2]);
    const unsigned axis = ad2 > fmaxf(ad0, ad1) ? 2u : (ad1 > ad0 ? 1u : 0u);
    float phi = atan2f(d[1], d[0]);
    if (phi < 0.f) phi += 3.14159265f;
    const unsigned dir = min(7u, (unsigned)(phi * (8.f / 3.14159265f)));
    const float tc = (g.tof && len > 0.f) ? ((r[2] - g.bin_shift) * g.bw + g.co) / len : 0.f;
    unsigned cell[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const float c = 0.5f * (p0[a] + p1[a]) + tc * d[a];
        const float u = (c - (g.org[a] - 0.5f * g.vox[a])) / (8.f * g.vox[a]);
        cell[a] = (unsigned)min(63, max(0, (int)floorf(u)));
    }
    keys[j] = ((axis * 8u + dir) << 18) | morton3(cell[0], cell[1], cell[2]);
    vals[j] = (int)j;
}

__global__ void k_pet_pack(const int *__restrict__ ev, int ncol, int bin_shift, int tof,
                           long long first, long long stride, long long n,
                           const int *__restrict__ order, int4 *__restrict__ rec) {
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int j = order[k];
    const int *r = ev + (first + (long long)j * stride) * ncol;
    rec[k] = make_int4(r[0], r[1], tof ? r[2] - bin_shift : 0, j);
}

// Sensitivity: non-TOF back projection of (w * exp(-H mu) + delta) over a LOR set given
// either as explicit pairs [n][2] or, when pairs is null, as every crystal pair i < j in
// lexicographic order (torch.combinations order), pair index first + p.
__device__ __forceinline__ void pair_from_index(long long p, int n, int &i, int &j) {
    // p = i (2n - i - 1) / 2 + (j - i - 1)
    double nn = 2.0 * n - 1.0;
    double ii = floor((nn - sqrt(nn * nn - 8.0 * (double)p)) / 2.0);
    long long ib = (long long)ii;
    auto start = [&](long long q) { return q * (2LL * n - q - 1) / 2; };
    while (ib > 0 && start(ib) > p) ib--;
    while (start(ib + 1) <= p) ib++;
    i = (int)ib;
    j = (int)(p - start(ib) + ib + 1);
}

__global__ void __launch_bounds__(256)
    k_pet_sens(PetDev g, const int *__restrict__ pairs, long long first, long long n,
               const float *__restrict__ w, const float *__restrict__ mu, float add,
               float *__restrict__ img) {
    long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    long long q = first + p;
    int i, j;
    if (pairs) {
        i = pairs[2 * q];
        j = pairs[2 * q + 1];
    } else {
        pair_from_index(q, g.n_det, i, j);
    }
    const float *p0 = g.lut + 3 * (long long)i;
    const float *p1 = g.lut + 3 * (long long)j;
    float v = w ? w[q] : 1.f;
    if (mu) v *= expf(-joseph<false, false>(g, p0, p1, nullptr, mu, 0, 0.f));
    v += add;
    joseph<true, false>(g, p0, p1, img, nullptr, 0, v);
}

// Listmode OSEM update: f <- f + f/(nbp + delta) * (bp - nbp); f[f <= 0] = 0
__global__ void k_pet_update(float *__restrict__ f, const float *__restrict__ bp,
                             const float *__restrict__ nbp, long long n) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float fv = f[i], nb = nbp[i];
    float pre = __fmul_rn(fv, __frcp_rn(__fadd_rn(nb, 1e-11f)));
    float fn = __fadd_rn(fv, __fmul_rn(pre, __fsub_rn(bp[i], nb)));
    f[i] = fn <= 0.f ? 0.f : fn;
}

}  // namespace gb

using namespace gb;

struct gb_pet_plan {
    PetDev dev{};
    float *d_lut = nullptr;
    int *d_ev = nullptr;
    int ncol = 2;
    long long n_events = 0;
    int n_subsets = 1;
    float *d_ratio = nullptr, *d_bp = nullptr;
    long long img_size = 0;
    // event tiles: list 0 = every event, list s + 1 = subset s (i::n_subsets)
    int4 *d_rec = nullptr;
    float *d_tof_tab = nullptr;
    std::vector<long long> list_off;
    // deterministic back projection: fixed-point sums [img_size], the list's max |proj|
    // bits and the fixed-point scale
    unsigned long long *d_acc64 = nullptr;
    unsigned *d_maxbits = nullptr;
    float *d_scale = nullptr;
};

static void pet_free(gb_pet_plan *p) {
    if (!p) return;
    dev_free(p->d_lut);
    dev_free(p->d_ev);
    dev_free(p->d_ratio);
    dev_free(p->d_bp);
    dev_free(p->d_rec);
    dev_free(p->d_tof_tab);
    dev_free(p->d_acc64);
    dev_free(p->d_maxbits);
    dev_free(p->d_scale);
    delete p;
}

static void subset_range(const gb_pet_plan *p, int subset, long long &first, long long &stride,
                         long long &n) {
    if (subset < 0) {
        first = 0;
        stride = 1;
        n = p->n_events;
    } else {
        first = subset;
        stride = p->n_subsets;
        n = p->n_events > subset ? (p->n_events - subset + p->n_subsets - 1) / p->n_subsets : 0;
    }
}

// Sort the events of every list by their locality key (device radix sort, stable, so
// equal keys keep list order) and pack the tiles.
static gb_status build_tiles(gb_pet_plan *p, int n_subsets) {
    const long long E = p->n_events;
    dev_free(p->d_rec);
    p->d_rec = nullptr;
    p->list_off.assign(1, 0);
    if (E == 0) {
        for (int s = 0; s < n_subsets; s++) p->list_off.push_back(0);
        return GB_OK;
    }
    GB_CUDA(dev_alloc(&p->d_rec, (size_t)(2 * E) * sizeof(int4)));
    unsigned *keys = nullptr, *keys2 = nullptr;
    int *vals = nullptr, *vals2 = nullptr;
    void *tmp = nullptr;
    size_t tmp_bytes = 0;
    cudaError_t e = cudaSuccess;
    auto fail = [&](cudaError_t err) {
        dev_free(keys); dev_free(keys2); dev_free(vals); dev_free(vals2); dev_free(tmp);
        set_error("event tile build failed: %s", cudaGetErrorString(err));
        return err == cudaErrorMemoryAllocation ? GB_ERR_OOM : GB_ERR_CUDA;
    };
    if ((e = dev_alloc(&keys, E * sizeof(unsigned))) != cudaSuccess ||
        (e = dev_alloc(&keys2, E * sizeof(unsigned))) != cudaSuccess ||
        (e = dev_alloc(&vals, E * sizeof(int))) != cudaSuccess ||
        (e = dev_alloc(&vals2, E * sizeof(int))) != cudaSuccess)
        return fail(e);
    if ((e = cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys, keys2, vals, vals2,
                                             (int)E, 0, 23)) != cudaSuccess ||
        (e = dev_alloc(&tmp, tmp_bytes)) != cudaSuccess)
        return fail(e);
    long long off = 0;
    for (int li = 0; li <= n_subsets; li++) {
        long long first = 0, stride = 1, n = E;
        if (li > 0) {
            first = li - 1;
            stride = n_subsets;
            n = E > first ? (E - first + stride - 1) / stride : 0;
        }
        if (li > 0) p->list_off.push_back(off);
        if (n == 0) continue;
        const unsigned blocks = (unsigned)((n + 255) / 256);
        k_pet_keys<<<blocks, 256>>>(p->dev, p->d_ev, p->ncol, first, stride, n, keys, vals);
        if ((e = cudaGetLastError()) != cudaSuccess) return fail(e);
        size_t tb = tmp_bytes;
        if ((e = cub::DeviceRadixSort::SortPairs(tmp, tb, keys, keys2, vals, vals2, (int)n, 0,
                                                 23)) != cudaSuccess)
            return fail(e);
        k_pet_pack<<<blocks, 256>>>(p->d_ev, p->ncol, p->dev.bin_shift, p->dev.tof, first, stride,
                                    n, vals2, p->d_rec + off);
        if ((e = cudaGetLastError()) != cudaSuccess) return fail(e);
        off += n;
    }
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return fail(e);
    dev_free(keys); dev_free(keys2); dev_free(vals); dev_free(vals2); dev_free(tmp);
    return GB_OK;
}

// The tiles of a subset (-1 = every event).
static const int4 *list_tiles(const gb_pet_plan *p, int subset) {
    return p->d_rec ? p->d_rec + (subset < 0 ? 0 : p->list_off[subset + 1]) : nullptr;
}

extern "C" {

gb_status gb_pet_plan_create(const gb_pet_desc *d, gb_pet_plan **out) {
    clear_error();
    GB_CHECK_ARG(d && out, "null argument");
    *out = nullptr;
    GB_CHECK_ARG(d->nx > 0 && d->ny > 0 && d->nz > 0, "image shape must be positive");
    GB_CHECK_ARG(d->n_det > 1 && d->lut, "scanner LUT missing");
    GB_CHECK_ARG(d->n_events >= 0 && (d->n_events == 0 || d->events), "events missing");
    GB_CHECK_ARG(!d->tof || (d->tof_sigma > 0 && d->tof_bin_width > 0 && d->tof_num_bins > 0),
                 "invalid TOF parameters");
    auto *p = new gb_pet_plan();
    PetDev &g = p->dev;
    g.n[0] = d->nx; g.n[1] = d->ny; g.n[2] = d->nz;
    g.n_vox = d->nx * d->ny * d->nz;
    g.vox[0] = d->vx; g.vox[1] = d->vy; g.vox[2] = d->vz;
    g.org[0] = d->ox; g.org[1] = d->oy; g.org[2] = d->oz;
    g.n_det = d->n_det;
    g.tof = d->tof;
    g.bw = d->tof_bin_width;
    g.sig = d->tof_sigma;
    g.co = d->tof_center_offset;
    g.nsig = d->tof_n_sigmas;
    g.bin_shift = (d->tof_num_bins - 1) / 2;
    p->ncol = d->tof ? 3 : 2;
    p->n_events = d->n_events;
    p->img_size = (long long)d->nx * d->ny * d->nz;
    cudaError_t e;
    if ((e = dev_alloc(&p->d_lut, (size_t)d->n_det * 3 * sizeof(float))) != cudaSuccess ||
        (e = cudaMemcpy(p->d_lut, d->lut, (size_t)d->n_det * 3 * sizeof(float),
                        cudaMemcpyHostToDevice)) != cudaSuccess) {
        set_error("LUT upload failed: %s", cudaGetErrorString(e));
        pet_free(p);
        return GB_ERR_CUDA;
    }
    g.lut = p->d_lut;
    if (d->tof) {
        // TOF bin weight table over |s| in [0, n_sigmas sigma + bw/2]
        std::vector<float> tab;
        float inv_step = 0.f;
        tof_weight_table(d->tof_bin_width, d->tof_sigma, d->tof_n_sigmas, tab, inv_step);
        if ((e = dev_alloc(&p->d_tof_tab, tab.size() * sizeof(float))) != cudaSuccess ||
            (e = cudaMemcpy(p->d_tof_tab, tab.data(), tab.size() * sizeof(float),
                            cudaMemcpyHostToDevice)) != cudaSuccess) {
            set_error("TOF table upload failed: %s", cudaGetErrorString(e));
            pet_free(p);
            return GB_ERR_CUDA;
        }
        g.tof_tab = p->d_tof_tab;
        g.tof_inv_step = inv_step;
    }
    if (d->n_events > 0) {
        size_t bytes = (size_t)d->n_events * p->ncol * sizeof(int);
        if ((e = dev_alloc(&p->d_ev, bytes)) != cudaSuccess ||
            (e = cudaMemcpy(p->d_ev, d->events, bytes, cudaMemcpyDefault)) != cudaSuccess ||
            (e = dev_alloc(&p->d_ratio, (size_t)d->n_events * sizeof(float))) != cudaSuccess ||
            (e = dev_alloc(&p->d_bp, (size_t)p->img_size * sizeof(float))) != cudaSuccess) {
            set_error("event upload failed: %s", cudaGetErrorString(e));
            pet_free(p);
            return e == cudaErrorMemoryAllocation ? GB_ERR_OOM : GB_ERR_CUDA;
        }
        // validate detector ids once (host copy)
        std::vector<int> h((size_t)d->n_events * p->ncol);
        cudaMemcpy(h.data(), p->d_ev, bytes, cudaMemcpyDeviceToHost);
        for (long long i = 0; i < d->n_events; i++)
            for (int c = 0; c < 2; c++) {
                int v = h[(size_t)i * p->ncol + c];
                if (v < 0 || v >= d->n_det) {
                    set_error("event %lld: detector id %d outside [0, %d)", i, v, d->n_det);
                    pet_free(p);
                    return GB_ERR_ARG;
                }
            }
    }
    gb_status st = build_tiles(p, 1);
    if (st != GB_OK) {
        pet_free(p);
        return st;
    }
    *out = p;
    return GB_OK;
}

gb_status gb_pet_plan_destroy(gb_pet_plan *p) {
    clear_error();
    if (p) {
        cudaDeviceSynchronize();
        pet_free(p);
    }
    return GB_OK;
}

gb_status gb_pet_set_subsets(gb_pet_plan *p, int32_t n_subsets) {
    clear_error();
    GB_CHECK_ARG(p && n_subsets >= 1, "invalid subsets");
    gb_status st = build_tiles(p, n_subsets);
    if (st != GB_OK) return st;
    p->n_subsets = n_subsets;
    return GB_OK;
}

gb_status gb_pet_forward(gb_pet_plan *p, const float *img, float *proj, int32_t subset,
                         gb_stream_t stream) {
    clear_error();
    GB_INJECT_ARG();
    GB_CHECK_ARG(p && img && proj, "null argument");
    GB_CHECK_ARG(subset < p->n_subsets, "subset out of range");
    GB_INJECT_LAUNCH();
    long long first, stride, n;
    subset_range(p, subset, first, stride, n);
    if (n == 0) return GB_OK;
    unsigned blocks = (unsigned)((n + 255) / 256);
    const int4 *rec = list_tiles(p, subset);
    if (p->dev.tof)
        k_pet_fwd<true><<<blocks, 256, 0, as_stream(stream)>>>(p->dev, rec, first, stride, n, img,
                                                               proj, 0, nullptr, nullptr, 0);
    else
        k_pet_fwd<false><<<blocks, 256, 0, as_stream(stream)>>>(p->dev, rec, first, stride, n,
                                                                img, proj, 0, nullptr, nullptr, 0);
    GB_LAUNCH_CHECK();
    return GB_OK;
}

gb_status gb_pet_backward(gb_pet_plan *p, const float *proj, float *img, int32_t subset,
                          gb_stream_t stream) {
    clear_error();
    GB_INJECT_ARG();
    GB_CHECK_ARG(p && img && proj, "null argument");
    GB_CHECK_ARG(((uintptr_t)img & 15) == 0, "image buffer must be 16-byte aligned");
    GB_INJECT_LAUNCH();
    GB_CHECK_ARG(subset < p->n_subsets, "subset out of range");
    long long first, stride, n;
    subset_range(p, subset, first, stride, n);
    cudaStream_t st = as_stream(stream);
    GB_CUDA(cudaMemsetAsync(img, 0, (size_t)p->img_size * sizeof(float), st));
    if (n == 0) return GB_OK;
    unsigned blocks = (unsigned)((n + 255) / 256);
    const int4 *rec = list_tiles(p, subset);
    if (p->d_acc64) {  // deterministic mode
        const float cf_max = 1.7320509f * std::max(p->dev.vox[0], std::max(p->dev.vox[1], p->dev.vox[2]));
        GB_CUDA(cudaMemsetAsync(p->d_maxbits, 0, sizeof(unsigned), st));
        k_abs_max<<<blocks, 256, 0, st>>>(rec, n, proj, p->d_maxbits);
        k_det_scale<<<1, 1, 0, st>>>(p->d_maxbits, n, cf_max, p->d_scale);
        GB_CUDA(cudaMemsetAsync(p->d_acc64, 0, (size_t)p->img_size * sizeof(unsigned long long), st));
        if (p->dev.tof)
            k_pet_bwd_det<true><<<blocks, 256, 0, st>>>(p->dev, rec, n, proj, p->d_scale, p->d_acc64);
        else
            k_pet_bwd_det<false><<<blocks, 256, 0, st>>>(p->dev, rec, n, proj, p->d_scale, p->d_acc64);
        k_det_to_float<<<(unsigned)((p->img_size + 255) / 256), 256, 0, st>>>(
            p->d_acc64, p->d_scale, img, p->img_size);
        GB_LAUNCH_CHECK();
        return GB_OK;
    }
    if (p->dev.tof)
        k_pet_bwd<true><<<blocks, 256, 0, st>>>(p->dev, rec, n, proj, 0, img);
    else
        k_pet_bwd<false><<<blocks, 256, 0, st>>>(p->dev, rec, n, proj, 0, img);
    GB_LAUNCH_CHECK();
    return GB_OK;
}

gb_status gb_pet_set_deterministic(gb_pet_plan *p, int32_t on) {
    clear_error();
    GB_CHECK_ARG(p, "null plan");
    dev_free(p->d_acc64);
    dev_free(p->d_maxbits);
    dev_free(p->d_scale);
    p->d_acc64 = nullptr;
    p->d_maxbits = nullptr;
    p->d_scale = nullptr;
    if (!on) return GB_OK;
    GB_CUDA(dev_alloc(&p->d_acc64, (size_t)p->img_size * sizeof(unsigned long long)));
    GB_CUDA(dev_alloc(&p->d_maxbits, sizeof(unsigned)));
    GB_CUDA(dev_alloc(&p->d_scale, sizeof(float)));
    return GB_OK;
}

gb_status gb_pet_osem_step(gb_pet_plan *p, float *img, const float *numerator,
                           int64_t numerator_len, const float *additive, const float *norm_bp,
                           int32_t subset, gb_stream_t stream) {
    clear_error();
    GB_INJECT_ARG();
    GB_CHECK_ARG(p && img && numerator && norm_bp, "null argument");
    GB_INJECT_LAUNCH();
    GB_CHECK_ARG(numerator_len == 1 || numerator_len == p->n_events,
                 "numerator must hold 1 or n_events values");
    GB_CHECK_ARG(subset < p->n_subsets, "subset out of range");
    long long first, stride, n;
    subset_range(p, subset, first, stride, n);
    cudaStream_t st = as_stream(stream);
    unsigned blocks = (unsigned)((n + 255) / 256);
    const int4 *rec = list_tiles(p, subset);
    if (n > 0) {
        if (p->dev.tof)
            k_pet_fwd<true><<<blocks, 256, 0, st>>>(p->dev, rec, first, stride, n, img,
                                                    p->d_ratio, 1, additive, numerator,
                                                    (int)numerator_len);
        else
            k_pet_fwd<false><<<blocks, 256, 0, st>>>(p->dev, rec, first, stride, n, img,
                                                     p->d_ratio, 1, additive, numerator,
                                                     (int)numerator_len);
        GB_LAUNCH_CHECK();
    }
    GB_CUDA(cudaMemsetAsync(p->d_bp, 0, (size_t)p->img_size * sizeof(float), st));
    if (n > 0) {
        if (p->dev.tof)
            k_pet_bwd<true><<<blocks, 256, 0, st>>>(p->dev, rec, n, p->d_ratio, 1, p->d_bp);
        else
            k_pet_bwd<false><<<blocks, 256, 0, st>>>(p->dev, rec, n, p->d_ratio, 1, p->d_bp);
        GB_LAUNCH_CHECK();
    }
    k_pet_update<<<(unsigned)((p->img_size + 255) / 256), 256, 0, st>>>(img, p->d_bp, norm_bp,
                                                                         p->img_size);
    GB_LAUNCH_CHECK();
    return GB_OK;
}

gb_status gb_pet_sensitivity(gb_pet_plan *p, const int32_t *pairs, int64_t n_pairs,
                             const float *weights, const float *mu, float add, float *img,
                             gb_stream_t stream) {
    clear_error();
    GB_CHECK_ARG(p && img, "null argument");
    GB_CHECK_ARG(((uintptr_t)img & 15) == 0, "image buffer must be 16-byte aligned");
    long long total = (long long)p->dev.n_det * (p->dev.n_det - 1) / 2;
    if (!pairs) n_pairs = total;
    GB_CHECK_ARG(n_pairs >= 0, "negative pair count");
    cudaStream_t st = as_stream(stream);
    GB_CUDA(cudaMemsetAsync(img, 0, (size_t)p->img_size * sizeof(float), st));
    const long long chunk = 1LL << 28;  // launch in chunks of 2^28 LORs
    for (long long first = 0; first < n_pairs; first += chunk) {
        long long n = std::min(chunk, (long long)n_pairs - first);
        k_pet_sens<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(p->dev, pairs, first, n, weights,
                                                                mu, add, img);
        GB_LAUNCH_CHECK();
    }
    return GB_OK;
}

gb_status gb_pet_lor_forward(gb_pet_plan *p, const float *img, float *proj, int32_t subset,
                             int32_t use_tof, gb_stream_t stream) {
    clear_error();
    GB_CHECK_ARG(p && img && proj, "null argument");
    GB_CHECK_ARG(subset < p->n_subsets, "subset out of range");
    long long first, stride, n;
    subset_range(p, subset, first, stride, n);
    if (n == 0) return GB_OK;
    unsigned blocks = (unsigned)((n + 255) / 256);
    const int4 *rec = list_tiles(p, subset);
    if (use_tof && p->dev.tof)
        k_pet_fwd<true><<<blocks, 256, 0, as_stream(stream)>>>(p->dev, rec, first, stride, n, img,
                                                               proj, 0, nullptr, nullptr, 0);
    else
        k_pet_fwd<false><<<blocks, 256, 0, as_stream(stream)>>>(p->dev, rec, first, stride, n,
                                                                img, proj, 0, nullptr, nullptr, 0);
    GB_LAUNCH_CHECK();
    return GB_OK;
}

}  // extern "C"
