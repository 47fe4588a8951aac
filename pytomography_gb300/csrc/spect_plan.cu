// C ABI of the SPECT projector: plan creation (tables, attenuation precompute,
// scratch), subset bookkeeping and the stream-ordered projector / update calls.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "spect_launch.h"

namespace gb {

static thread_local std::string g_err;

void set_error(const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
}
void clear_error() { g_err.clear(); }

int device_sm_count() {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 148;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 148;
    return n;
}

static size_t max_smem_optin() {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return v > 0 ? (size_t)v : 227 * 1024;
}

}  // namespace gb

using namespace gb;

struct gb_spect_plan {
    SpectDev dev{};
    int N = 0, nz = 0, pad = 0, Lp = 0, n_angles = 0;
    float dx = 0, dy = 0, dz = 0;
    int H = 0;
    int sm_count = 148;
    // device tables
    float *d_lin = nullptr, *d_theta_fwd = nullptr, *d_theta_bwd = nullptr;
    float *d_taps_r = nullptr, *d_taps_z = nullptr, *d_A = nullptr;
    int *d_group = nullptr;
    // angle lists: [all][subset 0][subset 1]...
    int *d_alist = nullptr;
    int n_subsets = 0;
    std::vector<int> list_off, list_len;
    // scratch
    float *d_partials = nullptr;
    size_t partials_cap = 0;
    float *d_W = nullptr;
    int G = 0;
    float *d_ratio = nullptr, *d_bp = nullptr;
    int Zt_fwd = 0, Zt_b1 = 0;
};

static void free_plan(gb_spect_plan *p) {
    if (!p) return;
    cudaFree(p->d_lin); cudaFree(p->d_theta_fwd); cudaFree(p->d_theta_bwd);
    cudaFree(p->d_taps_r); cudaFree(p->d_taps_z); cudaFree(p->d_A); cudaFree(p->d_group);
    cudaFree(p->d_alist); cudaFree(p->d_partials); cudaFree(p->d_W); cudaFree(p->d_ratio);
    cudaFree(p->d_bp);
    delete p;
}

// Chunks of x planes per angle so that the grid fills the GPU: the PSF kernels run one
// 512-thread CTA per SM, the plain ones many 256-thread blocks per SM.
static int fwd_chunks(const gb_spect_plan *p, int n_sel) {
    int zs = p->dev.psf ? (p->nz + p->Zt_fwd - 1) / p->Zt_fwd : 1;
    int c;
    if (p->dev.psf) {
        c = std::max(1, p->sm_count / std::max(1, n_sel * zs));
    } else {
        int gz = (p->N * p->nz + 255) / 256;
        c = (8 * p->sm_count + n_sel * gz - 1) / std::max(1, n_sel * gz);
    }
    return std::max(1, std::min(c, std::max(1, p->Lp / 4)));
}

static int b1_chunks(const gb_spect_plan *p, int n_sel) {
    int zs = (p->nz + p->Zt_b1 - 1) / p->Zt_b1;
    int c = std::max(1, p->sm_count / std::max(1, n_sel * zs));
    return std::max(1, std::min(c, std::max(1, p->Lp / 4)));
}

static gb_status ensure_partials(gb_spect_plan *p, int n_sel) {
    size_t need = (size_t)n_sel * fwd_chunks(p, n_sel) * p->N * p->nz;
    if (need <= p->partials_cap) return GB_OK;
    cudaFree(p->d_partials);
    p->d_partials = nullptr;
    GB_CUDA(cudaMalloc(&p->d_partials, need * sizeof(float)));
    p->partials_cap = need;
    return GB_OK;
}

static gb_status upload_lists(gb_spect_plan *p, int n_subsets) {
    std::vector<int> all;
    p->list_off.clear();
    p->list_len.clear();
    p->list_off.push_back(0);
    p->list_len.push_back(p->n_angles);
    for (int a = 0; a < p->n_angles; a++) all.push_back(a);
    for (int s = 0; s < n_subsets; s++) {
        p->list_off.push_back((int)all.size());
        int len = 0;
        for (int a = s; a < p->n_angles; a += n_subsets) {
            all.push_back(a);
            len++;
        }
        p->list_len.push_back(len);
    }
    cudaFree(p->d_alist);
    p->d_alist = nullptr;
    GB_CUDA(cudaMalloc(&p->d_alist, all.size() * sizeof(int)));
    GB_CUDA(cudaMemcpy(p->d_alist, all.data(), all.size() * sizeof(int), cudaMemcpyHostToDevice));
    p->n_subsets = n_subsets;
    for (size_t i = 0; i < p->list_len.size(); i++) {
        gb_status st = ensure_partials(p, p->list_len[i]);
        if (st != GB_OK) return st;
    }
    return GB_OK;
}

static bool select_list(const gb_spect_plan *p, int subset, const int **alist, int *n) {
    if (subset < 0) {
        *alist = p->d_alist;
        *n = p->n_angles;
        return true;
    }
    if (subset >= p->n_subsets) return false;
    *alist = p->d_alist + p->list_off[subset + 1];
    *n = p->list_len[subset + 1];
    return true;
}

// z-slab width for the PSF kernels: the largest multiple of the output block that fits
// shared memory (and, for the forward, the 32 accumulator registers per thread).
static int choose_zt(int K, int N, int nz, bool fwd) {
    int OB = (K <= 31) ? 8 : 4;
    size_t cap = max_smem_optin();
    int best = OB;
    for (int zt = OB; zt < nz + OB; zt += OB) {
        int z = std::min(zt, (nz + OB - 1) / OB * OB);
        size_t sm = fwd ? fwd_psf_smem_bytes(K, N, z) : b1_psf_smem_bytes(K, N, z);
        if (sm > cap) break;
        if (fwd) {
            int N8 = (N + OB - 1) / OB * OB;
            if ((long)N8 * (z / OB) > 512L * (32 / OB)) break;
        }
        best = z;
        if (z >= nz) break;
    }
    return std::min(best, nz);
}

extern "C" {

const char *gb_last_error(void) { return g_err.c_str(); }
const char *gb_version(void) { return "gbtomo 0.1.0 (sm_103a)"; }

gb_status gb_spect_plan_create(const gb_spect_desc *d, gb_spect_plan **out) {
    clear_error();
    GB_CHECK_ARG(d && out, "null descriptor or output");
    *out = nullptr;
    GB_CHECK_ARG(d->nx > 0 && d->ny > 0 && d->nz > 0, "object shape must be positive");
    if (d->nx != d->ny) {
        set_error("rotate+sum needs nx == ny (got %d, %d)", d->nx, d->ny);
        return GB_ERR_SHAPE;
    }
    GB_CHECK_ARG(d->n_angles > 0, "n_angles must be positive");
    GB_CHECK_ARG(d->theta_fwd && d->theta_bwd && d->lin, "missing rotation tables");
    std::string order = d->order ? d->order : "";
    if (!(order == "" || order == "a" || order == "p" || order == "ap" || order == "pa")) {
        set_error("unsupported transform order '%s' (supported: '', a, p, ap, pa)", order.c_str());
        return GB_ERR_UNSUPPORTED;
    }
    auto *p = new gb_spect_plan();
    p->N = d->nx;
    p->nz = d->nz;
    p->pad = (int)std::ceil((std::sqrt(2.0) * d->nx - d->nx) / 2.0);
    p->Lp = p->N + 2 * p->pad;
    p->n_angles = d->n_angles;
    p->dx = d->dx; p->dy = d->dy; p->dz = d->dz;
    p->sm_count = device_sm_count();
    const bool att = order.find('a') != std::string::npos;
    const bool psf = order.find('p') != std::string::npos;
    if (att && !d->mu) {
        set_error("attenuation requested without a mu map");
        free_plan(p);
        return GB_ERR_ARG;
    }
    int K = 1;
    if (psf) {
        if (!d->psf_taps_r || !d->psf_group || d->psf_n_groups <= 0 || d->psf_k <= 0 ||
            (d->psf_k % 2) == 0 || (d->psf_2d && !d->psf_taps_z)) {
            set_error("invalid PSF tables");
            free_plan(p);
            return GB_ERR_ARG;
        }
        K = psf_bucket(d->psf_k);
        if (K < 0) {
            set_error("PSF kernel of %d taps exceeds the compiled maximum (45)", d->psf_k);
            free_plan(p);
            return GB_ERR_UNSUPPORTED;
        }
        for (int a = 0; a < d->n_angles; a++)
            if (d->psf_group[a] < 0 || d->psf_group[a] >= d->psf_n_groups) {
                set_error("psf_group[%d] out of range", a);
                free_plan(p);
                return GB_ERR_ARG;
            }
    }
    p->H = psf ? K / 2 : 0;
    SpectDev &g = p->dev;
    g.N = p->N; g.nz = p->nz; g.pad = p->pad; g.Lp = p->Lp;
    g.ya_lo = std::max(0, p->pad - p->H);
    g.ya_hi = std::min(p->Lp, p->pad + p->N + p->H);
    g.nya = g.ya_hi - g.ya_lo;
    g.half = (float)(p->Lp - 1) / 2.0f;
    g.K = K;
    g.att = att;
    g.psf = psf;
    g.att_first = att && (!psf || order == "ap");
    g.psf2d = psf ? (d->psf_2d ? 1 : 0) : 0;

#define FAIL_CUDA(call)                                                                   \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            set_error("%s failed: %s", #call, cudaGetErrorString(e_));                    \
            free_plan(p);                                                                 \
            return e_ == cudaErrorMemoryAllocation ? GB_ERR_OOM : GB_ERR_CUDA;            \
        }                                                                                 \
    } while (0)

    const int n = d->n_angles, Lp = p->Lp;
    FAIL_CUDA(cudaMalloc(&p->d_lin, Lp * sizeof(float)));
    FAIL_CUDA(cudaMemcpy(p->d_lin, d->lin, Lp * sizeof(float), cudaMemcpyHostToDevice));
    FAIL_CUDA(cudaMalloc(&p->d_theta_fwd, 6 * n * sizeof(float)));
    FAIL_CUDA(cudaMemcpy(p->d_theta_fwd, d->theta_fwd, 6 * n * sizeof(float), cudaMemcpyHostToDevice));
    FAIL_CUDA(cudaMalloc(&p->d_theta_bwd, 6 * n * sizeof(float)));
    FAIL_CUDA(cudaMemcpy(p->d_theta_bwd, d->theta_bwd, 6 * n * sizeof(float), cudaMemcpyHostToDevice));
    std::vector<int> grp(n, 0);
    if (psf) std::copy(d->psf_group, d->psf_group + n, grp.begin());
    FAIL_CUDA(cudaMalloc(&p->d_group, n * sizeof(int)));
    FAIL_CUDA(cudaMemcpy(p->d_group, grp.data(), n * sizeof(int), cudaMemcpyHostToDevice));
    if (psf) {
        // centre the caller's k taps inside K, drop taps below psf_trunc_rel * row max
        const int ng = d->psf_n_groups, kin = d->psf_k, off = (K - kin) / 2;
        std::vector<float> tr((size_t)ng * Lp * K, 0.f), tz((size_t)ng * Lp * K, 0.f);
        for (int gi = 0; gi < ng; gi++)
            for (int x = 0; x < Lp; x++) {
                for (int which = 0; which < 2; which++) {
                    const float *src = which == 0 ? d->psf_taps_r : d->psf_taps_z;
                    if (!src) continue;
                    std::vector<float> &dst = which == 0 ? tr : tz;
                    const float *row = src + ((size_t)gi * Lp + x) * kin;
                    float mx = 0.f;
                    for (int t = 0; t < kin; t++) mx = std::max(mx, std::fabs(row[t]));
                    for (int t = 0; t < kin; t++) {
                        float v = row[t];
                        if (d->psf_trunc_rel > 0.f && std::fabs(v) < d->psf_trunc_rel * mx) v = 0.f;
                        dst[((size_t)gi * Lp + x) * K + off + t] = v;
                    }
                }
            }
        FAIL_CUDA(cudaMalloc(&p->d_taps_r, tr.size() * sizeof(float)));
        FAIL_CUDA(cudaMemcpy(p->d_taps_r, tr.data(), tr.size() * sizeof(float), cudaMemcpyHostToDevice));
        FAIL_CUDA(cudaMalloc(&p->d_taps_z, tz.size() * sizeof(float)));
        FAIL_CUDA(cudaMemcpy(p->d_taps_z, tz.data(), tz.size() * sizeof(float), cudaMemcpyHostToDevice));
        p->Zt_fwd = choose_zt(K, p->N, p->nz, true);
        p->Zt_b1 = choose_zt(K, p->N, p->nz, false);
        size_t sf = fwd_psf_smem_bytes(K, p->N, p->Zt_fwd), sb = b1_psf_smem_bytes(K, p->N, p->Zt_b1);
        if (sf > max_smem_optin() || sb > max_smem_optin()) {
            set_error("PSF tiles need %zu / %zu bytes of shared memory (max %zu)", sf, sb,
                      max_smem_optin());
            free_plan(p);
            return GB_ERR_UNSUPPORTED;
        }
        FAIL_CUDA(setup_fwd(K, sf));
        FAIL_CUDA(setup_b1(K, sb));
    } else {
        p->Zt_fwd = p->Zt_b1 = p->nz;
    }
    g.lin = p->d_lin;
    g.theta_fwd = p->d_theta_fwd;
    g.theta_bwd = p->d_theta_bwd;
    g.group = p->d_group;
    g.taps_r = p->d_taps_r;
    g.taps_z = p->d_taps_z;
    if (att) {
        size_t na = (size_t)n * Lp * g.nya * p->nz;
        FAIL_CUDA(cudaMalloc(&p->d_A, na * sizeof(float)));
        g.A = p->d_A;
        FAIL_CUDA(launch_atten(g, d->mu, d->dx, n, p->d_A, 0));
        FAIL_CUDA(cudaStreamSynchronize(0));
    }
    // scratch: W for one angle group, likelihood ratio of all angles, multi-group bp
    p->G = std::min(n, 16);
    FAIL_CUDA(cudaMalloc(&p->d_W, (size_t)p->G * Lp * g.nya * p->nz * sizeof(float)));
    FAIL_CUDA(cudaMalloc(&p->d_ratio, (size_t)n * p->N * p->nz * sizeof(float)));
    FAIL_CUDA(cudaMalloc(&p->d_bp, (size_t)p->N * p->N * p->nz * sizeof(float)));
#undef FAIL_CUDA
    gb_status st = upload_lists(p, 1);
    if (st != GB_OK) {
        free_plan(p);
        return st;
    }
    *out = p;
    return GB_OK;
}

gb_status gb_spect_plan_destroy(gb_spect_plan *p) {
    clear_error();
    if (p) {
        cudaDeviceSynchronize();
        free_plan(p);
    }
    return GB_OK;
}

gb_status gb_spect_set_subsets(gb_spect_plan *p, int32_t n_subsets) {
    clear_error();
    GB_CHECK_ARG(p, "null plan");
    GB_CHECK_ARG(n_subsets >= 1 && n_subsets <= p->n_angles, "n_subsets must be in [1, %d]",
                 p->n_angles);
    return upload_lists(p, n_subsets);
}

int32_t gb_spect_subset_size(const gb_spect_plan *p, int32_t subset) {
    if (!p) return -1;
    const int *al;
    int n;
    if (!select_list(p, subset, &al, &n)) return -1;
    return n;
}

static gb_status run_forward(gb_spect_plan *p, const float *obj, int subset, float *out,
                             int ratio, const float *gproj, const float *sadd, float *pred,
                             cudaStream_t st, const int **alist_out, int *n_out) {
    const int *alist;
    int n;
    if (!select_list(p, subset, &alist, &n)) {
        set_error("subset %d out of range (n_subsets=%d)", subset, p->n_subsets);
        return GB_ERR_STATE;
    }
    int ch = fwd_chunks(p, n);
    gb_status s = ensure_partials(p, n);
    if (s != GB_OK) return s;
    GB_CUDA(launch_fwd(p->dev, obj, alist, n, ch, p->Zt_fwd, p->d_partials, st));
    GB_CUDA(launch_reduce(n, ch, p->N * p->nz, p->d_partials, out, ratio, gproj, sadd, alist,
                          pred, st));
    if (alist_out) *alist_out = alist;
    if (n_out) *n_out = n;
    return GB_OK;
}

gb_status gb_spect_forward(gb_spect_plan *p, const float *obj, float *proj, int32_t subset,
                           gb_stream_t stream) {
    clear_error();
    GB_CHECK_ARG(p && obj && proj, "null argument");
    return run_forward(p, obj, subset, proj, 0, nullptr, nullptr, nullptr, as_stream(stream),
                       nullptr, nullptr);
}

// Back-project `proj` (rows = the angles of alist) in groups of G angles.
static gb_status run_backward(gb_spect_plan *p, const float *proj, const int *alist, int n,
                              int adjoint, float *out, int final_mode, UpdateArgs u,
                              cudaStream_t st) {
    const size_t NZ = (size_t)p->N * p->nz;
    const int n_groups = (n + p->G - 1) / p->G;
    if (adjoint) GB_CUDA(cudaMemsetAsync(out, 0, (size_t)p->N * NZ * sizeof(float), st));
    for (int gi = 0; gi < n_groups; gi++) {
        int a0 = gi * p->G, na = std::min(p->G, n - a0);
        GB_CUDA(launch_b1(p->dev, proj + a0 * NZ, alist + a0, na, b1_chunks(p, na), p->Zt_b1,
                          p->d_W, st));
        if (adjoint) {
            GB_CUDA(launch_b2_scatter(p->dev, p->d_W, alist + a0, na, out, st));
            continue;
        }
        const bool last = gi == n_groups - 1;
        UpdateArgs ua{};
        if (!last || final_mode == B2_WRITE) {
            // accumulate into `out` (plain backward) or the bp scratch (fused updates)
            float *dst = final_mode == B2_WRITE ? out : p->d_bp;
            GB_CUDA(launch_b2_gather(p->dev, p->d_W, alist + a0, na, dst,
                                     gi == 0 ? B2_WRITE : B2_ADD, ua, st));
        } else {
            u.acc = n_groups > 1 ? p->d_bp : nullptr;
            GB_CUDA(launch_b2_gather(p->dev, p->d_W, alist + a0, na, out, final_mode, u, st));
        }
    }
    return GB_OK;
}

gb_status gb_spect_backward(gb_spect_plan *p, const float *proj, float *obj, int32_t subset,
                            int32_t adjoint, gb_stream_t stream) {
    clear_error();
    GB_CHECK_ARG(p && proj && obj, "null argument");
    const int *alist;
    int n;
    if (!select_list(p, subset, &alist, &n)) {
        set_error("subset %d out of range (n_subsets=%d)", subset, p->n_subsets);
        return GB_ERR_STATE;
    }
    UpdateArgs u{};
    return run_backward(p, proj, alist, n, adjoint ? 1 : 0, obj, B2_WRITE, u, as_stream(stream));
}

gb_status gb_spect_osem_step(gb_spect_plan *p, float *obj, const float *g, const float *s,
                             const float *nbp, int32_t subset, float *pred,
                             gb_stream_t stream) {
    clear_error();
    GB_CHECK_ARG(p && obj && g && nbp, "null argument");
    cudaStream_t st = as_stream(stream);
    const int *alist;
    int n;
    gb_status r = run_forward(p, obj, subset, p->d_ratio, 1, g, s, pred, st, &alist, &n);
    if (r != GB_OK) return r;
    UpdateArgs u{};
    u.f = obj;
    u.nbp = nbp;
    return run_backward(p, p->d_ratio, alist, n, 0, obj, B2_OSEM, u, st);
}

static void rdp_weights(float dx, float dy, float dz, float w[26]) {
    int n = 0;
    for (int i = -1; i <= 1; i++)
        for (int j = -1; j <= 1; j++)
            for (int k = -1; k <= 1; k++) {
                if (i == 0 && j == 0 && k == 0) continue;
                double dd = std::sqrt((double)(dx * i) * (dx * i) + (double)(dy * j) * (dy * j) +
                                      (double)(dz * k) * (dz * k));
                w[n++] = (float)(dx / dd);
            }
}

gb_status gb_spect_bsrem_step(gb_spect_plan *p, const float *in, float *out, const float *g,
                              const float *s, const float *nbp, const float *nbp_sum,
                              float relax, float w_m, const gb_rdp_desc *prior, float floor_v,
                              int32_t subset, gb_stream_t stream) {
    clear_error();
    GB_CHECK_ARG(p && in && out && g && nbp && nbp_sum, "null argument");
    GB_CHECK_ARG(in != out, "BSREM needs distinct input and output objects");
    cudaStream_t st = as_stream(stream);
    const int *alist;
    int n;
    gb_status r = run_forward(p, in, subset, p->d_ratio, 1, g, s, nullptr, st, &alist, &n);
    if (r != GB_OK) return r;
    UpdateArgs u{};
    u.f_in = in;
    u.f_out = out;
    u.nbp = nbp;
    u.nbp_sum = nbp_sum;
    u.relax = relax;
    u.w_m = w_m;
    u.floor_v = floor_v;
    if (prior) {
        u.prior = 1;
        u.beta = prior->beta;
        u.gamma = prior->gamma;
        u.rdelta = prior->delta;
        u.fov = prior->fov_scale;
        rdp_weights(p->dx, p->dy, p->dz, u.w26);
    }
    return run_backward(p, p->d_ratio, alist, n, 0, out, B2_BSREM, u, st);
}

gb_status gb_rdp_gradient(const float *f, float *grad, int32_t nx, int32_t ny, int32_t nz,
                          float dx, float dy, float dz, const gb_rdp_desc *prior,
                          float beta_scale, gb_stream_t stream) {
    clear_error();
    GB_CHECK_ARG(f && grad && prior, "null argument");
    GB_CHECK_ARG(nx > 0 && ny > 0 && nz > 0, "shape must be positive");
    UpdateArgs u{};
    u.prior = 1;
    u.beta = prior->beta;
    u.gamma = prior->gamma;
    u.rdelta = prior->delta;
    u.fov = prior->fov_scale;
    rdp_weights(dx, dy, dz, u.w26);
    GB_CUDA(launch_rdp(f, grad, nx, ny, nz, u, beta_scale, as_stream(stream)));
    return GB_OK;
}

}  // extern "C"
