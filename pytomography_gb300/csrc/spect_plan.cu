// C ABI of the SPECT projector: plan creation (tables, attenuation precompute,
// scratch), subset bookkeeping and the stream-ordered projector / update calls.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <mutex>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "spect_blur.cuh"
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

// ---------------------------------------------------------------- fault injection
static std::atomic<int> g_fault_countdown[FAULT_SITES];
static std::once_flag g_fault_env_once;

static int fault_site_of(const std::string &name) {
    if (name == "alloc") return FAULT_ALLOC;
    if (name == "launch") return FAULT_LAUNCH;
    if (name == "arg") return FAULT_ARG;
    return -1;
}

// GBTOMO_INJECT="site:n[,site:n...]" arms the sites at the first check of the process.
static void fault_env_init() {
    const char *env = std::getenv("GBTOMO_INJECT");
    if (!env) return;
    std::string spec(env);
    size_t pos = 0;
    while (pos < spec.size()) {
        size_t end = spec.find(',', pos);
        if (end == std::string::npos) end = spec.size();
        const std::string item = spec.substr(pos, end - pos);
        const size_t colon = item.find(':');
        const int site = fault_site_of(item.substr(0, colon));
        const int n = colon == std::string::npos ? 1 : std::atoi(item.c_str() + colon + 1);
        if (site >= 0 && n > 0) g_fault_countdown[site].store(n);
        pos = end + 1;
    }
}

namespace {
struct DevicePool {
    cudaMemPool_t pool = nullptr;
    cudaStream_t st = nullptr;  // allocation / release stream (non-blocking, library-owned)
    bool tried = false;
};
std::mutex g_pool_mutex;
DevicePool g_pools[64];

// The pool of the current device, created on first use; null when the device has no
// memory-pool support (plain cudaMalloc / cudaFree are used then, for every block).
DevicePool *device_pool() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(g_pool_mutex);
    DevicePool &d = g_pools[dev];
    if (!d.tried) {
        d.tried = true;
        int supported = 0;
        cudaDeviceGetAttribute(&supported, cudaDevAttrMemoryPoolsSupported, dev);
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        if (supported && cudaMemPoolCreate(&d.pool, &props) == cudaSuccess &&
            cudaStreamCreateWithFlags(&d.st, cudaStreamNonBlocking) == cudaSuccess) {
            unsigned long long keep = kPoolKeepBytes;
            cudaMemPoolSetAttribute(d.pool, cudaMemPoolAttrReleaseThreshold, &keep);
        } else {
            if (d.pool) cudaMemPoolDestroy(d.pool);
            d.pool = nullptr;
            d.st = nullptr;
            cudaGetLastError();
        }
    }
    return d.pool ? &d : nullptr;
}
}  // namespace

cudaError_t dev_alloc(void **p, size_t bytes) {
    if (fault_injected(FAULT_ALLOC)) return cudaErrorMemoryAllocation;
    DevicePool *d = device_pool();
    if (!d) return cudaMalloc(p, bytes);
    cudaError_t e = cudaMallocFromPoolAsync(p, bytes, d->pool, d->st);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(d->st);  // the block is then usable from every stream
}

cudaError_t release_pool_memory() {
    DevicePool *d = device_pool();
    if (!d) return cudaSuccess;
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return e;
    return cudaMemPoolTrimTo(d->pool, 0);
}

void dev_free(void *p) {
    if (!p) return;
    DevicePool *d = device_pool();
    if (!d) {
        cudaFree(p);
        return;
    }
    cudaDeviceSynchronize();
    cudaFreeAsync(p, d->st);
}

bool fault_injected(FaultSite site) {
    std::call_once(g_fault_env_once, fault_env_init);
    int c = g_fault_countdown[site].load();
    while (c > 0) {
        if (g_fault_countdown[site].compare_exchange_weak(c, c - 1)) return c == 1;
    }
    return false;
}

int device_sm_count() {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 148;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 148;
    return n;
}

// Dynamic shared memory a PSF kernel may use: the device's opt-in maximum per block less
// 1 KB for the kernels' static shared variables (mbarrier, work-queue slot).
static size_t max_smem_optin() {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return (v > 0 ? (size_t)v : 227 * 1024) - 1024;
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
    signed char *d_tier = nullptr;
    int *d_group = nullptr;
    std::vector<signed char> h_tier;  // tap tier per (PSF group, plane)
    std::vector<int> h_group;         // PSF group per angle
    // angle lists: [all][subset 0][subset 1]..., with their work items
    int *d_alist = nullptr;
    int4 *d_items = nullptr;
    int *d_ioff = nullptr;
    int n_subsets = 0;
    std::vector<std::vector<int>> explicit_subsets;  // caller's subset lists, if set
    struct List {
        int alist_off = 0, n = 0;
        int fitem_off = 0, n_fitems = 0;  // forward items in d_items
        int ioff_off = 0;                 // n + 1 item offsets per slot in d_ioff
        std::vector<int> gitem_off, n_gitems;  // B1 items of each angle group
        int f_half = 0, b_half = 0;  // first forward / group-0 B1 item of slot n / 2
    };
    std::vector<List> lists;
    std::vector<float> h_theta_fwd, h_lin;
    // scratch
    float *d_partials = nullptr;
    size_t partials_cap = 0;
    float *d_W = nullptr;
    int G = 0;
    float *d_ratio = nullptr, *d_bp = nullptr;
    int2 *d_wrange = nullptr;
    int *d_err = nullptr;
    int Zt_fwd = 0, Zt_b1 = 0;
    int fwd_tpb = 512;  // forward CTA size: 512 or 768 threads (one CTA per SM)
    int fwd_variant = 1;  // 1: k_fwd_psf; 2: k_fwd_psf2
    int fwd_items = 1, b1_items = 1;  // work items per resident CTA slot and z slab
    unsigned lists_version = 0;       // bumped whenever the subset / work lists change
    // fused OSEM step in two angle halves on two streams (the second half's forward and
    // the first half's back projection overlap; fork / join by events)
    int osem_split = 0;  // measured slower at 128^3 x 12 angles: off by default
    cudaStream_t st2 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
};

static void free_plan(gb_spect_plan *p) {
    if (!p) return;
    dev_free(p->d_lin); dev_free(p->d_theta_fwd); dev_free(p->d_theta_bwd);
    dev_free(p->d_taps_r); dev_free(p->d_taps_z); dev_free(p->d_A); dev_free(p->d_group);
    dev_free(p->d_tier);
    dev_free(p->dev.phase);
    dev_free(p->d_alist); dev_free(p->d_items); dev_free(p->d_ioff);
    dev_free(p->d_partials); dev_free(p->d_W); dev_free(p->d_ratio);
    dev_free(p->d_bp);
    dev_free(p->d_wrange);
    dev_free(p->d_err);
    if (p->st2) cudaStreamDestroy(p->st2);
    if (p->ev_fork) cudaEventDestroy(p->ev_fork);
    if (p->ev_join) cudaEventDestroy(p->ev_join);
    delete p;
}

// Rows of plane xp whose rotated sample can reach the object square (host, double
// precision; only used to estimate work, the kernels decide exactly).
static bool host_plane_rows(const gb_spect_plan *p, int a, int xp, int ylo, int yhi,
                            double margin, int &ra, int &rb) {
    const float *th = p->h_theta_fwd.data() + 6 * a;
    const double half = (p->Lp - 1) / 2.0;
    auto coords = [&](int y, double &ix, double &iy) {
        double gx = (double)th[0] * p->h_lin[y] + (double)th[1] * p->h_lin[xp] + th[2];
        double gy = (double)th[3] * p->h_lin[y] + (double)th[4] * p->h_lin[xp] + th[5];
        ix = (gx + 1) * half;
        iy = (gy + 1) * half;
    };
    const int y0 = ylo, y1 = yhi - 1;
    double pa[2], pb[2];
    coords(y0, pa[0], pa[1]);
    coords(y1, pb[0], pb[1]);
    const double lo = p->pad - 1 - margin, hi = p->pad + p->N + margin;
    double t0 = 0, t1 = 1;
    for (int k = 0; k < 2; k++) {
        double d = pb[k] - pa[k];
        if (std::fabs(d) < 1e-12) {
            if (pa[k] < lo || pa[k] > hi) return false;
        } else {
            double ta = (lo - pa[k]) / d, tb = (hi - pa[k]) / d;
            if (ta > tb) std::swap(ta, tb);
            t0 = std::max(t0, ta);
            t1 = std::min(t1, tb);
        }
    }
    if (t0 > t1) return false;
    ra = std::max(ylo, (int)std::floor(y0 + t0 * (y1 - y0)) - 1);
    rb = std::min(yhi - 1, (int)std::ceil(y0 + t1 * (y1 - y0)) + 1);
    return ra <= rb;
}

// Estimated cost (SM cycles) of every plane of angle a, linear models fitted to per-CTA
// cycle counts on GB300 (object sizes 64-128, 60-120 angles, three subsets each): a fixed
// cost per occupied plane (barriers, pipeline drain), a cost per sampled row and a cost
// per blurred output row and tap (the plane's tap tier sets the taps).
//   forward: 6360 + 106 rows + 2.76 (output rows x taps); a plane no sample reaches: 100
//   B1:      5370 +  67 rows + 2.37 (rows x taps);        a plane no sample reaches: 835
// (B1's model was refitted by least squares, with a constant per CTA that the split does
// not need, after its z-pass tasks changed shape; the forward's refit the same way moved
// the launch from 0.1622 to 0.1641 ms and was not kept.)
// (The forward skips empty planes with a support test; B1 also records their empty row
// range.)
static std::vector<double> plane_work(const gb_spect_plan *p, int a, bool fwd) {
    std::vector<double> w(p->Lp, fwd ? 100.0 : 835.0);
    const int H = p->H, K = p->dev.K;
    const int ylo = std::max(0, p->pad - H), yhi = std::min(p->Lp, p->pad + p->N + H);
    const int grp = p->h_group.empty() ? 0 : p->h_group[a];
    for (int xp = 0; xp < p->Lp; xp++) {
        int ra, rb;
        if (!host_plane_rows(p, a, xp, ylo, yhi, fwd ? 0.5 : 1.5, ra, rb)) continue;
        const int tier = p->h_tier.empty() ? kTiers - 1 : p->h_tier[(size_t)grp * p->Lp + xp];
        const double kk = tier_taps(K, tier);
        const double rows = rb - ra + 1;
        if (fwd) {
            const int o = std::min(p->N, rb + H - p->pad + 1) - std::max(0, ra - H - p->pad);
            w[xp] = 6360.0 + 106.0 * rows + 2.76 * kk * std::max(0, o);
        } else {
            w[xp] = 5370.0 + 67.0 * rows + 2.37 * kk * rows;
        }
    }
    return w;
}

// Split [0, Lp) into c contiguous plane ranges of about equal work: each boundary is put
// where the running sum comes closest to its share.
static void split_planes(const std::vector<double> &w, int c, int slot,
                         std::vector<int4> &out) {
    const int L = (int)w.size();
    double total = 0;
    for (double v : w) total += v;
    int x = 0;
    double acc = 0;
    int prev = 0;
    for (int k = 1; k <= c; k++) {
        int end = L;
        if (k < c) {
            const double target = total * k / c;
            while (x < L - (c - k) && acc + 0.5 * w[x] <= target) acc += w[x++];
            end = std::max(x, prev + 1);
            while (x < end) acc += w[x++];
        }
        out.push_back(make_int4(slot, prev, end, 0));
        prev = end;
    }
}

// Chunks per angle for the plain (no PSF) forward: many 256-thread blocks per SM (a
// thread per z quad when nz % 4 == 0).
static int nopsf_chunks(const gb_spect_plan *p, int n_sel) {
    int gz = (p->N * (p->nz % 4 == 0 ? p->nz / 4 : p->nz) + 255) / 256;
    int c = (8 * p->sm_count + n_sel * gz - 1) / std::max(1, n_sel * gz);
    return std::max(1, std::min(c, std::max(1, p->Lp / 4)));
}

// Per-angle chunk counts: about one wave of items (n angles x chunks x z-slabs), each
// angle's share proportional to its estimated work (largest remainder), at least one.
static std::vector<int> chunk_counts(const gb_spect_plan *p, const std::vector<double> &work,
                                     int zslabs, int per_sm = 1) {
    const int n = (int)work.size();
    const int T = std::max(n, p->sm_count * per_sm / std::max(1, zslabs));
    const int cmax = std::max(1, p->Lp / 4);
    double total = 0;
    for (double v : work) total += v;
    std::vector<int> c(n, 1);
    if (total <= 0) return c;
    std::vector<std::pair<double, int>> rem;
    int used = 0;
    for (int i = 0; i < n; i++) {
        const double share = T * work[i] / total;
        c[i] = std::max(1, std::min(cmax, (int)share));
        used += c[i];
        rem.push_back({share - (int)share, i});
    }
    std::sort(rem.begin(), rem.end(), [](auto &a, auto &b) { return a.first > b.first; });
    for (size_t k = 0; used < T && k < rem.size(); k++)
        if (c[rem[k].second] < cmax) {
            c[rem[k].second]++;
            used++;
        }
    return c;
}

static double sum_of(const std::vector<double> &v) {
    double t = 0;
    for (double x : v) t += x;
    return t;
}

static gb_status upload_lists(gb_spect_plan *p, int n_subsets) {
    std::vector<int> all;
    std::vector<int4> items;
    std::vector<int> ioff;
    p->lists.clear();
    std::vector<std::vector<int>> angle_lists;
    {
        std::vector<int> l;
        for (int a = 0; a < p->n_angles; a++) l.push_back(a);
        angle_lists.push_back(l);
    }
    if (!p->explicit_subsets.empty()) {
        n_subsets = (int)p->explicit_subsets.size();
        for (const auto &l : p->explicit_subsets) angle_lists.push_back(l);
    } else {
        for (int s = 0; s < n_subsets; s++) {
            std::vector<int> l;
            for (int a = s; a < p->n_angles; a += n_subsets) l.push_back(a);
            angle_lists.push_back(l);
        }
    }
    const bool psf = p->dev.psf;
    const int zs_f = psf ? (p->nz + p->Zt_fwd - 1) / p->Zt_fwd : 1;
    const int zs_b = psf ? (p->nz + p->Zt_b1 - 1) / p->Zt_b1 : 1;
    std::vector<std::vector<double>> wf(p->n_angles), wb(p->n_angles);
    if (psf)
        for (int a = 0; a < p->n_angles; a++) {
            wf[a] = plane_work(p, a, true);
            wb[a] = plane_work(p, a, false);
        }
    size_t max_items = 0;
    for (const auto &l : angle_lists) {
        gb_spect_plan::List L;
        L.alist_off = (int)all.size();
        L.n = (int)l.size();
        all.insert(all.end(), l.begin(), l.end());
        // forward items
        L.fitem_off = (int)items.size();
        L.ioff_off = (int)ioff.size();
        if (psf) {
            std::vector<double> wa(L.n);
            for (int i = 0; i < L.n; i++) wa[i] = sum_of(wf[l[i]]);
            std::vector<int> cnt = chunk_counts(p, wa, zs_f, p->fwd_items);
            for (int i = 0; i < L.n; i++) {
                ioff.push_back((int)items.size() - L.fitem_off);
                if (i == L.n / 2) L.f_half = (int)items.size() - L.fitem_off;
                split_planes(wf[l[i]], cnt[i], i, items);
            }
        } else {
            int c = nopsf_chunks(p, L.n);
            for (int i = 0; i < L.n; i++) {
                ioff.push_back((int)items.size() - L.fitem_off);
                for (int k = 0; k < c; k++)
                    items.push_back(make_int4(i, k * p->Lp / c, (k + 1) * p->Lp / c, 0));
            }
        }
        L.n_fitems = (int)items.size() - L.fitem_off;
        ioff.push_back(L.n_fitems);
        max_items = std::max(max_items, (size_t)L.n_fitems);
        // B1 items per angle group
        for (int a0 = 0; a0 < L.n; a0 += p->G) {
            int na = std::min(p->G, L.n - a0);
            L.gitem_off.push_back((int)items.size());
            if (psf) {
                std::vector<double> wa(na);
                for (int i = 0; i < na; i++) wa[i] = sum_of(wb[l[a0 + i]]);
                std::vector<int> cnt = chunk_counts(p, wa, zs_b, p->b1_items);
                for (int i = 0; i < na; i++) {
                    if (a0 == 0 && i == L.n / 2) L.b_half = (int)items.size() - L.gitem_off.back();
                    split_planes(wb[l[a0 + i]], cnt[i], i, items);
                }
            }
            L.n_gitems.push_back((int)items.size() - L.gitem_off.back());
        }
        p->lists.push_back(L);
    }
    dev_free(p->d_alist);
    dev_free(p->d_items);
    dev_free(p->d_ioff);
    p->d_alist = nullptr;
    p->d_items = nullptr;
    p->d_ioff = nullptr;
    GB_CUDA(dev_alloc(&p->d_alist, all.size() * sizeof(int)));
    GB_CUDA(cudaMemcpy(p->d_alist, all.data(), all.size() * sizeof(int), cudaMemcpyHostToDevice));
    GB_CUDA(dev_alloc(&p->d_items, std::max<size_t>(1, items.size()) * sizeof(int4)));
    if (!items.empty())
        GB_CUDA(cudaMemcpy(p->d_items, items.data(), items.size() * sizeof(int4),
                           cudaMemcpyHostToDevice));
    GB_CUDA(dev_alloc(&p->d_ioff, ioff.size() * sizeof(int)));
    GB_CUDA(cudaMemcpy(p->d_ioff, ioff.data(), ioff.size() * sizeof(int), cudaMemcpyHostToDevice));
    p->n_subsets = n_subsets;
    p->lists_version++;
    size_t need = max_items * p->N * p->nz;
    if (need > p->partials_cap) {
        dev_free(p->d_partials);
        p->d_partials = nullptr;
        GB_CUDA(dev_alloc(&p->d_partials, need * sizeof(float)));
        p->partials_cap = need;
    }
    return GB_OK;
}

// List index of a subset (-1 = every angle), or -1 when out of range.
static int list_index(const gb_spect_plan *p, int subset) {
    if (subset < 0) return 0;
    if (subset >= p->n_subsets) return -1;
    return subset + 1;
}

static bool select_list(const gb_spect_plan *p, int subset, const int **alist, int *n) {
    int li = list_index(p, subset);
    if (li < 0) return false;
    *alist = p->d_alist + p->lists[li].alist_off;
    *n = p->lists[li].n;
    return true;
}

// z-slab width for the PSF kernels: the largest multiple of the output block that fits
// shared memory (and, for the forward, the 32 accumulator registers per thread of a
// `tpb`-thread CTA: 512 or 768 threads, one CTA per SM).
static int choose_zt(int K, int N, int nz, bool fwd, int tpb = 512) {
    int OB = (K <= 31) ? 8 : 4;
    size_t cap = max_smem_optin();
    int best = 0;
    for (int zt = OB; zt < nz + OB; zt += OB) {
        int z = std::min(zt, (nz + OB - 1) / OB * OB);
        size_t sm = fwd ? fwd_psf_smem_bytes(K, N, z, tpb) : b1_psf_smem_bytes(K, N, z);
        if (sm > cap) break;
        if (fwd && tpb > 512) {  // 768 threads: 24 warps x (3 or 6) linear warp-tasks
            const int N8 = (N + OB - 1) / OB * OB, n_yc = (N8 + 31) / 32;
            if ((long)n_yc * (z / OB) > 24L * (OB == 8 ? 3 : 6)) break;
        } else if (fwd) {  // phase-3 tasks of k_fwd_psf: 16 warps x (16 / OB) row-pair tasks
            const int N8 = (N + OB - 1) / OB * OB, NT = 16 / OB, n_yc = (N8 + 63) / 64;
            if (n_yc <= NT) {
                if (z / OB > (tpb / 32) * (NT / n_yc)) break;
            } else if ((long)(N8 / 2) * (z / OB) > (long)tpb * NT) {
                break;
            }
        }
        best = z;
        if (z >= nz) break;
    }
    return std::min(best, nz);
}

extern "C" {

const char *gb_last_error(void) { return g_err.c_str(); }

gb_status gb_inject_fault(const char *site, int32_t nth) {
    clear_error();
    std::call_once(g_fault_env_once, fault_env_init);
    GB_CHECK_ARG(site, "null site");
    const int s = fault_site_of(site);
    GB_CHECK_ARG(s >= 0, "unknown fault site '%s' (alloc, launch, arg)", site);
    GB_CHECK_ARG(nth >= 0, "nth must be >= 0");
    g_fault_countdown[s].store(nth);
    return GB_OK;
}
const char *gb_version(void) { return "gbtomo 0.1.0 (sm_103a)"; }

gb_status gb_release_pool_memory(void) {
    clear_error();
    GB_CUDA(release_pool_memory());
    return GB_OK;
}

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
    p->pad = d->no_pad ? 0 : (int)std::ceil((std::sqrt(2.0) * d->nx - d->nx) / 2.0);
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
        K = psf_bucket(std::max(d->psf_k, d->psf_k_min));
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
    g.n_angles = p->n_angles;
    g.ya_lo = std::max(0, p->pad - p->H);
    g.ya_hi = std::min(p->Lp, p->pad + p->N + p->H);
    g.nya = g.ya_hi - g.ya_lo;
    g.half = (float)(p->Lp - 1) / 2.0f;
    g.K = K;
    g.att = att;
    g.psf = psf;
    g.att_first = att && (!psf || order == "ap");
    g.psf2d = psf ? (d->psf_2d ? 1 : 0) : 0;
    g.wait_polls = kWaitPolls;
    g.dbg_skip_first_copy = 0;

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
    p->h_theta_fwd.assign(d->theta_fwd, d->theta_fwd + 6 * n);
    p->h_lin.assign(d->lin, d->lin + Lp);
    FAIL_CUDA(dev_alloc(&p->d_lin, Lp * sizeof(float)));
    FAIL_CUDA(cudaMemcpy(p->d_lin, d->lin, Lp * sizeof(float), cudaMemcpyHostToDevice));
    FAIL_CUDA(dev_alloc(&p->d_theta_fwd, 6 * n * sizeof(float)));
    FAIL_CUDA(cudaMemcpy(p->d_theta_fwd, d->theta_fwd, 6 * n * sizeof(float), cudaMemcpyHostToDevice));
    FAIL_CUDA(dev_alloc(&p->d_theta_bwd, 6 * n * sizeof(float)));
    FAIL_CUDA(cudaMemcpy(p->d_theta_bwd, d->theta_bwd, 6 * n * sizeof(float), cudaMemcpyHostToDevice));
    std::vector<int> grp(n, 0);
    if (psf) std::copy(d->psf_group, d->psf_group + n, grp.begin());
    p->h_group = grp;
    FAIL_CUDA(dev_alloc(&p->d_group, n * sizeof(int)));
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
        // tap tier of every plane: the narrowest unrolled loop that holds its nonzero taps
        std::vector<signed char> tier((size_t)ng * Lp, kTiers - 1);
        const int Hk = K / 2;
        for (int gi = 0; gi < ng; gi++)
            for (int x = 0; x < Lp; x++) {
                int h = 0;
                for (int which = 0; which < 2; which++) {
                    const std::vector<float> &tab = which == 0 ? tr : tz;
                    for (int t = 0; t < K; t++)
                        if (tab[((size_t)gi * Lp + x) * K + t] != 0.f) h = std::max(h, std::abs(t - Hk));
                }
                int t = 0;
                while (t < kTiers - 1 && h > tier_half(K, t)) t++;
                tier[(size_t)gi * Lp + x] = (signed char)t;
            }
        p->h_tier = tier;
        FAIL_CUDA(dev_alloc(&p->d_tier, tier.size()));
        FAIL_CUDA(cudaMemcpy(p->d_tier, tier.data(), tier.size(), cudaMemcpyHostToDevice));
        FAIL_CUDA(dev_alloc(&p->d_taps_r, tr.size() * sizeof(float)));
        FAIL_CUDA(cudaMemcpy(p->d_taps_r, tr.data(), tr.size() * sizeof(float), cudaMemcpyHostToDevice));
        FAIL_CUDA(dev_alloc(&p->d_taps_z, tz.size() * sizeof(float)));
        FAIL_CUDA(cudaMemcpy(p->d_taps_z, tz.data(), tz.size() * sizeof(float), cudaMemcpyHostToDevice));
        p->Zt_fwd = choose_zt(K, p->N, p->nz, true);
        p->Zt_b1 = choose_zt(K, p->N, p->nz, false);
        if (!p->Zt_fwd || !p->Zt_b1) {
            set_error("PSF tiles of %d taps at %d rows do not fit shared memory (max %zu)", K,
                      p->N, max_smem_optin());
            free_plan(p);
            return GB_ERR_UNSUPPORTED;
        }
        // the limit is a property of the kernel, shared by every plan of this tap bucket:
        // raise it to the device maximum (each launch still asks only for its own tile)
        FAIL_CUDA(setup_fwd(K, max_smem_optin(), 512));
        FAIL_CUDA(setup_b1(K, max_smem_optin()));
    } else {
        p->Zt_fwd = p->Zt_b1 = p->nz;
    }
    g.lin = p->d_lin;
    g.theta_fwd = p->d_theta_fwd;
    g.theta_bwd = p->d_theta_bwd;
    g.group = p->d_group;
    g.taps_r = p->d_taps_r;
    g.taps_z = p->d_taps_z;
    g.tier = p->d_tier;
    if (att) {
        size_t na = (size_t)n * Lp * g.nya * p->nz;
        FAIL_CUDA(dev_alloc(&p->d_A, na * sizeof(float)));
        g.A = p->d_A;
        FAIL_CUDA(launch_atten(g, d->mu, d->dx, n, p->d_A, 0));
        FAIL_CUDA(cudaStreamSynchronize(0));
    }
    // scratch: W for one angle group, likelihood ratio of all angles, multi-group bp
    p->G = std::min(n, 16);
    FAIL_CUDA(dev_alloc(&p->d_W, (size_t)p->G * Lp * g.nya * p->nz * sizeof(float)));
    FAIL_CUDA(dev_alloc(&p->d_ratio, (size_t)n * p->N * p->nz * sizeof(float)));
    FAIL_CUDA(dev_alloc(&p->d_bp, (size_t)p->N * p->N * p->nz * sizeof(float)));
    FAIL_CUDA(dev_alloc(&p->d_wrange, (size_t)p->G * Lp * sizeof(int2)));
    FAIL_CUDA(cudaMemset(p->d_wrange, 0, (size_t)p->G * Lp * sizeof(int2)));
    FAIL_CUDA(dev_alloc(&p->d_err, sizeof(int)));
    FAIL_CUDA(cudaMemset(p->d_err, 0, sizeof(int)));
    FAIL_CUDA(cudaStreamCreateWithFlags(&p->st2, cudaStreamNonBlocking));
    FAIL_CUDA(cudaEventCreateWithFlags(&p->ev_fork, cudaEventDisableTiming));
    FAIL_CUDA(cudaEventCreateWithFlags(&p->ev_join, cudaEventDisableTiming));
    g.wrange = p->d_wrange;
    g.err = p->d_err;
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

gb_status gb_spect_device_status(gb_spect_plan *p, int32_t *code) {
    clear_error();
    GB_CHECK_ARG(p && code, "null argument");
    GB_CUDA(cudaMemcpy(code, p->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    return GB_OK;
}

gb_status gb_spect_clear_device_status(gb_spect_plan *p) {
    clear_error();
    GB_CHECK_ARG(p, "null plan");
    GB_CUDA(cudaMemset(p->d_err, 0, sizeof(int)));
    return GB_OK;
}

gb_status gb_spect_set_debug(gb_spect_plan *p, int32_t skip_first_copy, int32_t wait_polls) {
    clear_error();
    GB_CHECK_ARG(p, "null plan");
    GB_CHECK_ARG(wait_polls >= 0, "wait_polls must be >= 0");
    p->dev.dbg_skip_first_copy = skip_first_copy ? 1 : 0;
    p->dev.wait_polls = wait_polls ? (unsigned)wait_polls : kWaitPolls;
    return GB_OK;
}

gb_status gb_spect_set_subsets(gb_spect_plan *p, int32_t n_subsets) {
    clear_error();
    GB_CHECK_ARG(p, "null plan");
    GB_CHECK_ARG(n_subsets >= 1 && n_subsets <= p->n_angles, "n_subsets must be in [1, %d]",
                 p->n_angles);
    p->explicit_subsets.clear();
    return upload_lists(p, n_subsets);
}

gb_status gb_spect_set_subset_lists(gb_spect_plan *p, int32_t n_subsets, const int32_t *angle_idx,
                                    const int32_t *counts) {
    clear_error();
    GB_CHECK_ARG(p && angle_idx && counts, "null argument");
    GB_CHECK_ARG(n_subsets >= 1, "n_subsets must be positive");
    std::vector<std::vector<int>> lists(n_subsets);
    long long off = 0;
    for (int s = 0; s < n_subsets; s++) {
        GB_CHECK_ARG(counts[s] >= 1, "subset %d is empty", s);
        for (int k = 0; k < counts[s]; k++) {
            const int a = angle_idx[off + k];
            GB_CHECK_ARG(a >= 0 && a < p->n_angles, "angle index %d outside [0, %d)", a,
                         p->n_angles);
            lists[s].push_back(a);
        }
        off += counts[s];
    }
    p->explicit_subsets = lists;
    return upload_lists(p, n_subsets);
}

int32_t gb_spect_subset_size(const gb_spect_plan *p, int32_t subset) {
    if (!p) return -1;
    const int *al;
    int n;
    if (!select_list(p, subset, &al, &n)) return -1;
    return n;
}

gb_status gb_spect_get_tuning(const gb_spect_plan *p, gb_spect_tuning *out) {
    clear_error();
    GB_CHECK_ARG(p && out, "null argument");
    out->fwd_tpb = p->fwd_tpb;
    out->fwd_variant = p->fwd_variant;
    out->osem_split = p->osem_split;
    out->fwd_zt = p->Zt_fwd;
    out->fwd_items = p->fwd_items;
    out->b1_zt = p->Zt_b1;
    out->b1_items = p->b1_items;
    return GB_OK;
}

// Check a tuning against the plan's limits and fill in the z slabs left at 0.
static gb_status resolve_tuning(const gb_spect_plan *p, gb_spect_tuning &t) {
    const int K = p->dev.K, OB = (K <= 31) ? 8 : 4;
    GB_CHECK_ARG(t.fwd_tpb == 512 || t.fwd_tpb == 768, "fwd_tpb must be 512 or 768");
    if (t.fwd_variant == 0) t.fwd_variant = p->fwd_variant;
    GB_CHECK_ARG(t.fwd_variant == 1 || t.fwd_variant == 2, "fwd_variant must be 1 or 2");
    GB_CHECK_ARG(t.osem_split == 0 || t.osem_split == 1, "osem_split must be 0 or 1");
    if (t.fwd_variant == 2 && !fwd2_eligible(p->dev, max_smem_optin())) {
        set_error("forward variant 2 needs attenuation before a 2-D PSF of at most 29 taps, "
                  "N and nz <= 128 and nz %% 4 == 0");
        return GB_ERR_UNSUPPORTED;
    }
    GB_CHECK_ARG(t.fwd_items >= 1 && t.fwd_items <= 2 && t.b1_items >= 1 && t.b1_items <= 2,
                 "items per SM must be 1 or 2");
    const int zf = choose_zt(K, p->N, p->nz, true, t.fwd_tpb);
    const int zb = choose_zt(K, p->N, p->nz, false);
    if (!zf || !zb) {
        set_error("the %d-thread forward tile does not fit shared memory", t.fwd_tpb);
        return GB_ERR_UNSUPPORTED;
    }
    if (t.fwd_zt == 0 || t.fwd_variant == 2) t.fwd_zt = t.fwd_variant == 2 ? p->nz : zf;
    if (t.b1_zt == 0) t.b1_zt = zb;
    GB_CHECK_ARG(t.fwd_variant == 2 ||
                     (t.fwd_zt > 0 && t.fwd_zt <= zf && (t.fwd_zt % OB == 0 || t.fwd_zt == p->nz)),
                 "fwd_zt must be a multiple of %d in (0, %d]", OB, zf);
    GB_CHECK_ARG(t.b1_zt > 0 && t.b1_zt <= zb && (t.b1_zt % OB == 0 || t.b1_zt == p->nz),
                 "b1_zt must be a multiple of %d in (0, %d]", OB, zb);
    return GB_OK;
}

gb_status gb_spect_set_tuning(gb_spect_plan *p, const gb_spect_tuning *tuning) {
    clear_error();
    GB_CHECK_ARG(p && tuning, "null argument");
    if (!p->dev.psf) return GB_OK;  // the plain kernels have no tiles
    gb_spect_tuning t = *tuning;
    gb_status st = resolve_tuning(p, t);
    if (st != GB_OK) return st;
    const int K = p->dev.K;
    GB_CUDA(setup_fwd(K, max_smem_optin(), t.fwd_tpb));
    GB_CUDA(setup_b1(K, max_smem_optin()));
    if (t.fwd_variant == 2) GB_CUDA(setup_fwd2(K));
    p->fwd_tpb = t.fwd_tpb;
    p->fwd_variant = t.fwd_variant;
    p->osem_split = t.osem_split;
    p->Zt_fwd = t.fwd_zt;
    p->fwd_items = t.fwd_items;
    p->Zt_b1 = t.b1_zt;
    p->b1_items = t.b1_items;
    return upload_lists(p, std::max(1, p->n_subsets));
}

static gb_status run_forward(gb_spect_plan *p, const float *obj, int subset, float *out,
                             int ratio, const float *gproj, const float *sadd, float *pred,
                             cudaStream_t st) {
    const int li = list_index(p, subset);
    if (li < 0) {
        set_error("subset %d out of range (n_subsets=%d)", subset, p->n_subsets);
        return GB_ERR_STATE;
    }
    const gb_spect_plan::List &L = p->lists[li];
    const int *alist = p->d_alist + L.alist_off;
    GB_CUDA(launch_fwd(p->dev, obj, alist, p->d_items + L.fitem_off, L.n_fitems, p->Zt_fwd,
                       p->fwd_tpb, p->fwd_variant, p->d_partials, st));
    GB_CUDA(launch_reduce(L.n, p->d_ioff + L.ioff_off, p->N * p->nz, p->d_partials, out, ratio,
                          gproj, sadd, alist, pred, st));
    return GB_OK;
}

gb_status gb_spect_forward(gb_spect_plan *p, const float *obj, float *proj, int32_t subset,
                           gb_stream_t stream) {
    clear_error();
    GB_INJECT_ARG();
    GB_CHECK_ARG(p && obj && proj, "null argument");
    GB_INJECT_LAUNCH();
    return run_forward(p, obj, subset, proj, 0, nullptr, nullptr, nullptr, as_stream(stream));
}

// Back-project `proj` (rows = the angles of list li) in groups of G angles.
static gb_status run_backward(gb_spect_plan *p, const float *proj, int li, int adjoint,
                              float *out, int final_mode, UpdateArgs u, cudaStream_t st) {
    const gb_spect_plan::List &L = p->lists[li];
    const int *alist = p->d_alist + L.alist_off;
    const int n = L.n;
    const size_t NZ = (size_t)p->N * p->nz;
    const int n_groups = (n + p->G - 1) / p->G;
    if (adjoint) GB_CUDA(cudaMemsetAsync(out, 0, (size_t)p->N * NZ * sizeof(float), st));
    for (int gi = 0; gi < n_groups; gi++) {
        int a0 = gi * p->G, na = std::min(p->G, n - a0);
        GB_CUDA(launch_b1(p->dev, proj + a0 * NZ, alist + a0, na, p->d_items + L.gitem_off[gi],
                          L.n_gitems[gi], p->Zt_b1, p->d_W, st));
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
    GB_INJECT_ARG();
    GB_CHECK_ARG(p && proj && obj, "null argument");
    GB_INJECT_LAUNCH();
    const int li = list_index(p, subset);
    if (li < 0) {
        set_error("subset %d out of range (n_subsets=%d)", subset, p->n_subsets);
        return GB_ERR_STATE;
    }
    UpdateArgs u{};
    return run_backward(p, proj, li, adjoint ? 1 : 0, obj, B2_WRITE, u, as_stream(stream));
}

// Autotuner: time each candidate tile configuration of the forward kernel, then of the
// back-projection kernel, on a temporary object of ones and keep the fastest.  The
// candidates are the CTA size (512 threads, or 768 threads with the taps in shared memory),
// the widest z slab and half of it, and one or two work items per CTA slot.
gb_status gb_spect_autotune(gb_spect_plan *p, int32_t subset, int32_t reps,
                            gb_spect_tuning *out, gb_stream_t stream) {
    clear_error();
    GB_CHECK_ARG(p, "null plan");
    GB_CHECK_ARG(reps >= 1 && reps <= 1000, "reps must be in [1, 1000]");
    const int li = list_index(p, subset);
    if (li < 0) {
        set_error("subset %d out of range (n_subsets=%d)", subset, p->n_subsets);
        return GB_ERR_STATE;
    }
    if (!p->dev.psf) return out ? gb_spect_get_tuning(p, out) : GB_OK;
    cudaStream_t st = as_stream(stream);
    const int K = p->dev.K, OB = (K <= 31) ? 8 : 4;
    const size_t vol = (size_t)p->N * p->N * p->nz;
    const size_t npr = (size_t)p->lists[li].n * p->N * p->nz;
    float *obj = nullptr, *proj = nullptr, *back = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    gb_status rc = GB_OK;
    gb_spect_tuning best{};
    gb_spect_get_tuning(p, &best);
    auto cleanup = [&]() {
        dev_free(obj);
        dev_free(proj);
        dev_free(back);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    };
#define TUNE_CUDA(call)                                                                \
    do {                                                                               \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess) {                                                       \
            set_error("%s failed: %s", #call, cudaGetErrorString(e_));                 \
            cleanup();                                                                 \
            return e_ == cudaErrorMemoryAllocation ? GB_ERR_OOM : GB_ERR_CUDA;         \
        }                                                                              \
    } while (0)
    TUNE_CUDA(dev_alloc(&obj, vol * sizeof(float)));
    TUNE_CUDA(dev_alloc(&proj, npr * sizeof(float)));
    TUNE_CUDA(dev_alloc(&back, vol * sizeof(float)));
    {
        std::vector<float> ones(vol, 1.0f);
        TUNE_CUDA(cudaMemcpy(obj, ones.data(), vol * sizeof(float), cudaMemcpyHostToDevice));
    }
    TUNE_CUDA(cudaEventCreate(&e0));
    TUNE_CUDA(cudaEventCreate(&e1));
    // mean time of one call over `reps` after one untimed call; < 0 on failure
    auto time_ms = [&](auto &&call) -> float {
        if (call() != GB_OK) return -1.f;
        cudaEventRecord(e0, st);
        for (int r = 0; r < reps; r++)
            if (call() != GB_OK) return -1.f;
        cudaEventRecord(e1, st);
        if (cudaEventSynchronize(e1) != cudaSuccess) return -1.f;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        return ms / reps;
    };
    auto fwd_call = [&]() {
        return run_forward(p, obj, subset, proj, 0, nullptr, nullptr, nullptr, st);
    };
    auto bwd_call = [&]() { return run_backward(p, proj, li, 0, back, B2_WRITE, UpdateArgs{}, st); };
    // forward candidates
    float best_ms = 1e30f;
    gb_spect_tuning fbest = best;
    for (int tpb : {512, 768}) {
        const int zmax = choose_zt(K, p->N, p->nz, true, tpb);
        if (!zmax) continue;
        for (int zt : {zmax, (zmax / 2) / OB * OB}) {
            if (zt < 2 * OB || (zt != zmax && zt >= p->nz)) continue;
            for (int items : {1, 2}) {
                gb_spect_tuning t = best;
                t.fwd_variant = 1;
                t.fwd_tpb = tpb;
                t.fwd_zt = zt;
                t.fwd_items = items;
                if (gb_spect_set_tuning(p, &t) != GB_OK) continue;
                const float ms = time_ms(fwd_call);
                if (ms >= 0.f && ms < best_ms) {
                    best_ms = ms;
                    fbest = t;
                }
            }
        }
    }
    if (fwd2_eligible(p->dev, max_smem_optin()))
        for (int items : {1, 2}) {
            gb_spect_tuning t = best;
            t.fwd_variant = 2;
            t.fwd_tpb = 512;
            t.fwd_items = items;
            if (gb_spect_set_tuning(p, &t) != GB_OK) continue;
            const float ms = time_ms(fwd_call);
            if (ms >= 0.f && ms < best_ms) {
                best_ms = ms;
                fbest = t;
            }
        }
    best.fwd_tpb = fbest.fwd_tpb;
    best.fwd_zt = fbest.fwd_zt;
    best.fwd_items = fbest.fwd_items;
    best.fwd_variant = fbest.fwd_variant;
    // back-projection candidates (with the chosen forward tiles)
    best_ms = 1e30f;
    gb_spect_tuning bbest = best;
    const int zbmax = choose_zt(K, p->N, p->nz, false);
    for (int zt : {zbmax, (zbmax / 2) / OB * OB}) {
        if (zt < 2 * OB || (zt != zbmax && zt >= p->nz)) continue;
        for (int items : {1, 2}) {
            gb_spect_tuning t = best;
            t.b1_zt = zt;
            t.b1_items = items;
            if (gb_spect_set_tuning(p, &t) != GB_OK) continue;
            const float ms = time_ms(bwd_call);
            if (ms >= 0.f && ms < best_ms) {
                best_ms = ms;
                bbest = t;
            }
        }
    }
    best.b1_zt = bbest.b1_zt;
    best.b1_items = bbest.b1_items;
#undef TUNE_CUDA
    cudaError_t le = cudaGetLastError();
    cleanup();
    if (le != cudaSuccess) {
        set_error("autotune launch failed: %s", cudaGetErrorString(le));
        return GB_ERR_CUDA;
    }
    rc = gb_spect_set_tuning(p, &best);
    if (rc == GB_OK && out) *out = best;
    return rc;
}

// The fused OSEM sub-iteration in two halves of the subset's angles (one angle group):
// half A's forward, reduction and B1 on the caller's stream, half B's on the plan's second
// stream, then the gather with the update on the caller's stream.  Both forwards start
// together (one wave of CTAs between them); each half's B1 starts as soon as its own
// ratio rows exist, filling the SMs the slower forward CTAs leave idle.  The kernels and
// their work items are the single-stream step's, so results are identical.
static gb_status osem_split_step(gb_spect_plan *p, const gb_spect_plan::List &L, float *obj,
                                 const float *g, const float *s, const float *nbp, float *pred,
                                 cudaStream_t st) {
    const int *alist = p->d_alist + L.alist_off;
    const int h = L.n / 2;
    const size_t NZ = (size_t)p->N * p->nz;
    const int4 *fit = p->d_items + L.fitem_off;
    const int *ioff = p->d_ioff + L.ioff_off;
    const int4 *bit = p->d_items + L.gitem_off[0];
    cudaStream_t s2 = p->st2;
    GB_CUDA(cudaEventRecord(p->ev_fork, st));
    GB_CUDA(cudaStreamWaitEvent(s2, p->ev_fork, 0));
    GB_CUDA(launch_fwd(p->dev, obj, alist, fit, L.f_half, p->Zt_fwd, p->fwd_tpb, p->fwd_variant,
                       p->d_partials, st));
    GB_CUDA(launch_fwd(p->dev, obj, alist, fit + L.f_half, L.n_fitems - L.f_half, p->Zt_fwd,
                       p->fwd_tpb, p->fwd_variant, p->d_partials + (size_t)L.f_half * NZ, s2));
    GB_CUDA(launch_reduce(h, ioff, (int)NZ, p->d_partials, p->d_ratio, 1, g, s, alist, pred, st));
    GB_CUDA(launch_reduce(L.n - h, ioff + h, (int)NZ, p->d_partials, p->d_ratio + h * NZ, 1, g, s,
                          alist + h, pred ? pred + h * NZ : nullptr, s2));
    GB_CUDA(launch_b1(p->dev, p->d_ratio, alist, L.n, bit, L.b_half, p->Zt_b1, p->d_W, st));
    GB_CUDA(launch_b1(p->dev, p->d_ratio, alist, L.n, bit + L.b_half, L.n_gitems[0] - L.b_half,
                      p->Zt_b1, p->d_W, s2));
    GB_CUDA(cudaEventRecord(p->ev_join, s2));
    GB_CUDA(cudaStreamWaitEvent(st, p->ev_join, 0));
    UpdateArgs u{};
    u.f = obj;
    u.nbp = nbp;
    GB_CUDA(launch_b2_gather(p->dev, p->d_W, alist, L.n, obj, B2_OSEM, u, st));
    return GB_OK;
}

gb_status gb_spect_osem_step(gb_spect_plan *p, float *obj, const float *g, const float *s,
                             const float *nbp, int32_t subset, float *pred,
                             gb_stream_t stream) {
    clear_error();
    GB_INJECT_ARG();
    GB_CHECK_ARG(p && obj && g && nbp, "null argument");
    GB_INJECT_LAUNCH();
    cudaStream_t st = as_stream(stream);
    const int li = list_index(p, subset);
    if (li >= 0 && p->osem_split && p->dev.psf && p->lists[li].n >= 4 && p->lists[li].n <= p->G)
        return osem_split_step(p, p->lists[li], obj, g, s, nbp, pred, st);
    gb_status r = run_forward(p, obj, subset, p->d_ratio, 1, g, s, pred, st);
    if (r != GB_OK) return r;
    UpdateArgs u{};
    u.f = obj;
    u.nbp = nbp;
    return run_backward(p, p->d_ratio, li, 0, obj, B2_OSEM, u, st);
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
    GB_INJECT_LAUNCH();
    cudaStream_t st = as_stream(stream);
    gb_status r = run_forward(p, in, subset, p->d_ratio, 1, g, s, nullptr, st);
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
    return run_backward(p, p->d_ratio, list_index(p, subset), 0, out, B2_BSREM, u, st);
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

#ifdef GB_PHASE_TIMING
// Diagnostic builds: per-warp phase cycle counts of the plan's forward launches
// ([4096][16], layout in spect_fwd_psf.cuh), attached on first use.
extern "C" int gb_debug_fwd_phase_cycles(gb_spect_plan *p, unsigned long long *out, int n) {
    if (!p->dev.phase) return -1;
    return (int)cudaMemcpy(out, p->dev.phase, sizeof(unsigned long long) * (size_t)n,
                           cudaMemcpyDeviceToHost);
}
extern "C" int gb_debug_fwd_phase_reset(gb_spect_plan *p) {
    if (!p->dev.phase) {
        cudaError_t e = dev_alloc(&p->dev.phase, sizeof(unsigned long long) * 4096 * 16);
        if (e != cudaSuccess) return (int)e;
    }
    return (int)cudaMemset(p->dev.phase, 0, sizeof(unsigned long long) * 4096 * 16);
}
#endif

gb_status gb_rdp_hessian_vector(const float *f, const float *x, float *out, int32_t nx,
                                int32_t ny, int32_t nz, float dx, float dy, float dz,
                                const gb_rdp_desc *prior, float beta_scale, gb_stream_t stream) {
    clear_error();
    GB_CHECK_ARG(f && x && out && prior, "null argument");
    GB_CHECK_ARG(nx > 0 && ny > 0 && nz > 0, "shape must be positive");
    GB_CHECK_ARG(out != f && out != x, "out must not alias f or x");
    UpdateArgs u{};
    u.prior = 1;
    u.beta = prior->beta;
    u.gamma = prior->gamma;
    u.rdelta = prior->delta;
    u.fov = prior->fov_scale;
    rdp_weights(dx, dy, dz, u.w26);
    GB_CUDA(launch_rdp_hvp(f, x, out, nx, ny, nz, u, beta_scale, as_stream(stream)));
    return GB_OK;
}

}  // extern "C"

namespace gb {

bool plan_forward_args(const gb_spect_plan *p, int subset, FwdArgs *a) {
    const int li = p ? list_index(p, subset) : -1;
    if (li < 0) return false;
    const gb_spect_plan::List &L = p->lists[li];
    a->g = p->dev;
    a->alist = p->d_alist + L.alist_off;
    a->n_sel = L.n;
    a->items = p->d_items + L.fitem_off;
    a->n_items = L.n_fitems;
    a->ioff = p->d_ioff + L.ioff_off;
    a->Zt = p->Zt_fwd;
    a->tpb = p->fwd_tpb;
    a->variant = p->fwd_variant;
    return true;
}

}  // namespace gb

// ======================================================================== batches
// Several entries (reconstructions, or objects sharing one plan) projected by one persistent
// launch per phase.  The work items of all entries are split by the plans' plane-cost
// model into about kBatchWaves waves and ordered largest first, so small and large problems
// fill the GPU together; partial sums are reduced per (entry, angle) in plane order.

namespace gb {
constexpr int kBatchWaves = 2;
}

struct gb_spect_batch {
    int n = 0;
    gb_spect_plan *plans[kMaxBatch] = {};
    int K = 0, G = 16;
    int n_lists = 0;  // 1 + n_subsets of the plans at creation
    unsigned versions[kMaxBatch] = {};  // the plans' list versions at creation
    int *d_alists = nullptr;            // every list's angles of every entry
    int2 *wrange[kMaxBatch] = {};
    float *W[kMaxBatch] = {};
    float *ratio[kMaxBatch] = {};
    float *bp[kMaxBatch] = {};
    int slots_cap[kMaxBatch] = {};  // W slots of each entry
    CUtensorMap tm[kMaxBatch];  // 64-byte aligned type
    struct Lists {
        int4 *fitems = nullptr;
        int n_fitems = 0;
        int2 *rows = nullptr;
        int *row_off = nullptr, *row_items = nullptr;
        int n_rows = 0;
        std::vector<int4 *> bitems;  // per angle group
        std::vector<int> n_bitems;
        int n_groups = 0;
        int n_sel[kMaxBatch] = {};
        const int *alist[kMaxBatch] = {};  // device angle list of each entry
    };
    std::vector<Lists> lists;
    float *partials = nullptr;
    int nz_max = 0;
    int *counters = nullptr;  // [2]: forward and B1 queues
};

static void free_batch(gb_spect_batch *b) {
    if (!b) return;
    for (int e = 0; e < kMaxBatch; e++) {
        dev_free(b->wrange[e]);
        dev_free(b->W[e]);
        dev_free(b->ratio[e]);
        dev_free(b->bp[e]);
    }
    for (auto &L : b->lists) {
        dev_free(L.fitems);
        dev_free(L.rows);
        dev_free(L.row_off);
        dev_free(L.row_items);
        for (int4 *p : L.bitems) dev_free(p);
    }
    dev_free(b->partials);
    dev_free(b->counters);
    dev_free(b->d_alists);
    delete b;
}

template <typename T>
static gb_status upload_vec(T **dst, const std::vector<T> &v) {
    GB_CUDA(dev_alloc(dst, std::max<size_t>(1, v.size()) * sizeof(T)));
    if (!v.empty()) GB_CUDA(cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return GB_OK;
}

// Work items of the entries' angles (entry e: angles al[e][s0 .. s0 + n[e])), split by the
// cost model into about kBatchWaves waves and sorted by cost, largest first; slot indices
// are relative to s0.  order[k] = index of the k-th item in (entry, slot, plane) order.
static void batch_items(const gb_spect_batch *b, const std::vector<std::vector<int>> &al,
                        const std::vector<int> &s0, const std::vector<int> &n, bool fwd,
                        std::vector<int4> &items, std::vector<int> &order) {
    std::vector<std::vector<double>> w;
    std::vector<int> ent, slot;
    double total = 0;
    for (int e = 0; e < b->n; e++)
        for (int i = 0; i < n[e]; i++) {
            w.push_back(plane_work(b->plans[e], al[e][s0[e] + i], fwd));
            ent.push_back(e);
            slot.push_back(i);
            total += sum_of(w.back());
        }
    const int sms = b->plans[0]->sm_count;
    const double target = total / std::max(1, kBatchWaves * sms);
    std::vector<int4> raw;
    std::vector<double> cost;
    for (size_t k = 0; k < w.size(); k++) {
        const int Lp = (int)w[k].size();
        const int c = std::max(1, std::min(std::max(1, Lp / 4),
                                           (int)std::lround(sum_of(w[k]) / std::max(target, 1.0))));
        std::vector<int4> part;
        split_planes(w[k], c, slot[k], part);
        for (int4 it : part) {
            it.w = ent[k];
            double cst = 0;
            for (int x = it.y; x < it.z; x++) cst += w[k][x];
            raw.push_back(it);
            cost.push_back(cst);
        }
    }
    std::vector<int> idx(raw.size());
    for (size_t k = 0; k < idx.size(); k++) idx[k] = (int)k;
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int c) { return cost[a] > cost[c]; });
    items.resize(raw.size());
    order.assign(raw.size(), 0);
    for (size_t k = 0; k < idx.size(); k++) {
        items[k] = raw[idx[k]];
        order[idx[k]] = (int)k;
    }
}

static bool batch_list_ok(const gb_spect_batch *b) {
    for (int e = 0; e < b->n; e++)
        if (b->plans[e]->lists_version != b->versions[e]) return false;
    return true;
}

// SpectDev of entry e with its own W row ranges
static SpectDev batch_dev(const gb_spect_batch *b, int e) {
    SpectDev g = b->plans[e]->dev;
    g.wrange = b->wrange[e];
    return g;
}

static gb_status batch_forward(gb_spect_batch *b, int li, const float *const *objects, int ratio,
                               float *const *out, const float *const *gproj,
                               const float *const *sadd, cudaStream_t st) {
    const gb_spect_batch::Lists &L = b->lists[li];
    FwdBatch fp;
    std::memset(&fp, 0, sizeof(fp));
    for (int e = 0; e < b->n; e++) {
        fp.tm[e] = b->tm[e];
        fp.g[e] = batch_dev(b, e);
        fp.f[e] = objects[e];
        fp.alist[e] = L.alist[e];
    }
    fp.items = L.fitems;
    fp.n_items = L.n_fitems;
    fp.counter = b->counters;
    fp.partials = b->partials;
    fp.nz_max = b->nz_max;
    GB_CUDA(cudaMemsetAsync(b->counters, 0, sizeof(int), st));
    const int grid = std::max(1, std::min(L.n_fitems, b->plans[0]->sm_count));
    cudaError_t err = cudaErrorInvalidValue;
    switch (b->K) {
#define GB_BATCH_CASE(KK)                                  \
    case KK:                                               \
        err = launch_fwd_psf_batch_##KK(fp, grid, st);     \
        break;
        GB_FOR_EACH_K(GB_BATCH_CASE)
#undef GB_BATCH_CASE
    }
    GB_CUDA(err);
    ReduceBatch rp;
    std::memset(&rp, 0, sizeof(rp));
    for (int e = 0; e < b->n; e++) {
        rp.out[e] = out[e];
        rp.gproj[e] = gproj ? gproj[e] : nullptr;
        rp.sadd[e] = sadd ? sadd[e] : nullptr;
        rp.alist[e] = L.alist[e];
        rp.NZ[e] = b->plans[e]->N * b->plans[e]->nz;
    }
    rp.rows = L.rows;
    rp.row_off = L.row_off;
    rp.row_items = L.row_items;
    rp.partials = b->partials;
    rp.nz_max = b->nz_max;
    rp.ratio = ratio;
    GB_CUDA(launch_reduce_batch(rp, L.n_rows, st));
    return GB_OK;
}

// Back projection of proj[e] (rows = the list's angles) in groups of G angles.
// kind 0: reference operator into out[e]; 1: exact adjoint into out[e];
// 2: fused OSEM update of out[e] (the objects) with norm_bp[e].
static gb_status batch_backward(gb_spect_batch *b, int li, const float *const *proj, int kind,
                                float *const *out, const float *const *norm_bp, cudaStream_t st) {
    const gb_spect_batch::Lists &L = b->lists[li];
    if (kind == 1)
        for (int e = 0; e < b->n; e++) {
            const gb_spect_plan *p = b->plans[e];
            GB_CUDA(cudaMemsetAsync(out[e], 0, (size_t)p->N * p->N * p->nz * sizeof(float), st));
        }
    for (int gi = 0; gi < L.n_groups; gi++) {
        B1Batch bp1;
        std::memset(&bp1, 0, sizeof(bp1));
        B2Batch bp2;
        std::memset(&bp2, 0, sizeof(bp2));
        int blocks = 0;
        for (int e = 0; e < b->n; e++) {
            const gb_spect_plan *p = b->plans[e];
            const int a0 = gi * b->G, na = std::max(0, std::min(b->G, L.n_sel[e] - a0));
            bp1.g[e] = bp2.g[e] = batch_dev(b, e);
            bp1.proj[e] = proj[e] + (size_t)a0 * p->N * p->nz;
            bp1.alist[e] = bp2.alist[e] = L.alist[e] + a0;
            bp1.W[e] = b->W[e];
            bp2.W[e] = b->W[e];
            bp2.n_slots[e] = na;
            bp2.block_off[e] = blocks;
            const bool last = na > 0 && a0 + na == L.n_sel[e];
            if (kind == 2) {
                bp2.out[e] = last ? out[e] : b->bp[e];
                bp2.nbp[e] = norm_bp[e];
                bp2.acc[e] = (last && gi > 0) ? b->bp[e] : nullptr;
                bp2.mode[e] = last ? B2_OSEM : (gi == 0 ? B2_WRITE : B2_ADD);
            } else {
                bp2.out[e] = out[e];
                bp2.mode[e] = gi == 0 ? B2_WRITE : B2_ADD;
            }
            if (na > 0)
                blocks += kind == 1 ? b2_scatter_blocks(bp2.g[e], na) : b2_gather_blocks(bp2.g[e]);
        }
        for (int e = b->n; e <= kMaxBatch; e++) bp2.block_off[e] = blocks;
        bp1.items = L.bitems[gi];
        bp1.n_items = L.n_bitems[gi];
        bp1.counter = b->counters + 1;
        GB_CUDA(cudaMemsetAsync(b->counters + 1, 0, sizeof(int), st));
        if (L.n_bitems[gi] > 0)
            GB_CUDA(launch_b1_batch(b->K, bp1, std::min(L.n_bitems[gi], b->plans[0]->sm_count),
                                    st));
        if (kind == 1)
            GB_CUDA(launch_b2_scatter_batch(bp2, blocks, st));
        else
            GB_CUDA(launch_b2_gather_batch(bp2, blocks, st));
    }
    return GB_OK;
}

extern "C" {

gb_status gb_spect_batch_create(gb_spect_plan *const *plans, int32_t n, gb_spect_batch **out) {
    clear_error();
    GB_CHECK_ARG(plans && out, "null argument");
    *out = nullptr;
    GB_CHECK_ARG(n >= 1 && n <= kMaxBatch, "a batch holds 1 to %d entries (got %d)", kMaxBatch, n);
    auto *b = new gb_spect_batch();
    b->n = n;
    for (int e = 0; e < n; e++) {
        gb_spect_plan *p = plans[e];
        if (!p) {
            free_batch(b);
            set_error("null plan %d", e);
            return GB_ERR_ARG;
        }
        const char *why = nullptr;
        if (!p->dev.psf) why = "has no PSF";
        else if (p->N > 128 || p->nz > 128) why = "is larger than 128 x 128 x 128";
        else if (p->nz % 4 != 0) why = "has nz not divisible by 4";
        else if (e > 0 && p->dev.K != b->plans[0]->dev.K) why = "has another PSF tap bucket";
        else if (e > 0 && p->lists.size() != b->plans[0]->lists.size()) why = "has another subset count";
        if (why) {
            set_error("plan %d %s: batches need PSF plans of one tap bucket (psf_k_min), one "
                      "subset count, N and nz <= 128 and nz %% 4 == 0", e, why);
            free_batch(b);
            return GB_ERR_UNSUPPORTED;
        }
        b->plans[e] = p;
    }
    b->K = b->plans[0]->dev.K;
    if (fwd_psf_smem_bytes(b->K, 128, 128, 512) > max_smem_optin() ||
        b1_psf_smem_bytes(b->K, 128, 128) > max_smem_optin()) {
        set_error("the %d-tap batch tiles do not fit shared memory", b->K);
        free_batch(b);
        return GB_ERR_UNSUPPORTED;
    }
    b->n_lists = (int)b->plans[0]->lists.size();
#define BFAIL(st_)                   \
    do {                             \
        gb_status s_ = (st_);        \
        if (s_ != GB_OK) {           \
            free_batch(b);           \
            return s_;               \
        }                            \
    } while (0)
#define BCUDA(call)                                                                      \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess) {                                                         \
            set_error("%s failed: %s", #call, cudaGetErrorString(e_));                   \
            free_batch(b);                                                               \
            return e_ == cudaErrorMemoryAllocation ? GB_ERR_OOM : GB_ERR_CUDA;           \
        }                                                                                \
    } while (0)
    switch (b->K) {
#define GB_SETUP_CASE(KK)                       \
    case KK:                                    \
        BCUDA(setup_fwd_psf_batch_##KK());      \
        break;
        GB_FOR_EACH_K(GB_SETUP_CASE)
#undef GB_SETUP_CASE
    }
    BCUDA(setup_b1_batch(b->K));
    size_t max_items = 1;
    for (int e = 0; e < n; e++) b->nz_max = std::max(b->nz_max, b->plans[e]->N * b->plans[e]->nz);
    b->lists.resize(b->n_lists);
    std::vector<int> all_angles;
    std::vector<std::vector<size_t>> alist_off(b->n_lists, std::vector<size_t>(n));
    for (int e = 0; e < n; e++) b->versions[e] = b->plans[e]->lists_version;
    for (int li = 0; li < b->n_lists; li++) {
        gb_spect_batch::Lists &L = b->lists[li];
        std::vector<std::vector<int>> al(n);
        std::vector<int> s0(n, 0), cnt(n);
        for (int e = 0; e < n; e++) {
            const gb_spect_plan *p = b->plans[e];
            const gb_spect_plan::List &pl = p->lists[li];
            std::vector<int> h(pl.n);
            BCUDA(cudaMemcpy(h.data(), p->d_alist + pl.alist_off, pl.n * sizeof(int),
                             cudaMemcpyDeviceToHost));
            al[e] = h;
            cnt[e] = pl.n;
            L.n_sel[e] = pl.n;
            alist_off[li][e] = all_angles.size();
            all_angles.insert(all_angles.end(), h.begin(), h.end());
            b->slots_cap[e] = std::max(b->slots_cap[e], std::min(b->G, pl.n));
            L.n_groups = std::max(L.n_groups, (pl.n + b->G - 1) / b->G);
        }
        // forward items and the reduction rows
        std::vector<int4> fit;
        std::vector<int> order;
        batch_items(b, al, s0, cnt, true, fit, order);
        std::vector<int2> rows;
        std::vector<int> row_off{0}, row_items;
        {
            // the unsorted items come in (entry, slot, plane) order: group them by row
            std::vector<int4> raw(fit.size());
            for (size_t k = 0; k < order.size(); k++) raw[k] = fit[order[k]];
            size_t k = 0;
            for (int e = 0; e < n; e++)
                for (int s = 0; s < cnt[e]; s++) {
                    rows.push_back(make_int2(e, s));
                    while (k < raw.size() && raw[k].w == e && raw[k].x == s)
                        row_items.push_back(order[k++]);
                    row_off.push_back((int)row_items.size());
                }
        }
        L.n_fitems = (int)fit.size();
        L.n_rows = (int)rows.size();
        max_items = std::max(max_items, fit.size());
        BFAIL(upload_vec(&L.fitems, fit));
        BFAIL(upload_vec(&L.rows, rows));
        BFAIL(upload_vec(&L.row_off, row_off));
        BFAIL(upload_vec(&L.row_items, row_items));
        // B1 items per angle group
        for (int gi = 0; gi < L.n_groups; gi++) {
            std::vector<int> gs0(n), gcnt(n);
            for (int e = 0; e < n; e++) {
                gs0[e] = gi * b->G;
                gcnt[e] = std::max(0, std::min(b->G, cnt[e] - gs0[e]));
            }
            std::vector<int4> bit;
            std::vector<int> border;
            batch_items(b, al, gs0, gcnt, false, bit, border);
            int4 *d = nullptr;
            gb_status st = upload_vec(&d, bit);
            L.bitems.push_back(d);
            L.n_bitems.push_back((int)bit.size());
            BFAIL(st);
        }
    }
    BFAIL(upload_vec(&b->d_alists, all_angles));
    for (int li = 0; li < b->n_lists; li++)
        for (int e = 0; e < n; e++) b->lists[li].alist[e] = b->d_alists + alist_off[li][e];
    for (int e = 0; e < n; e++) {
        const gb_spect_plan *p = b->plans[e];
        const size_t slab = (size_t)p->Lp * p->dev.nya * p->nz;
        BCUDA(dev_alloc(&b->W[e], (size_t)b->slots_cap[e] * slab * sizeof(float)));
        BCUDA(dev_alloc(&b->wrange[e], (size_t)b->slots_cap[e] * p->Lp * sizeof(int2)));
        BCUDA(cudaMemset(b->wrange[e], 0, (size_t)b->slots_cap[e] * p->Lp * sizeof(int2)));
        size_t max_sel = 1;
        bool multi = false;
        for (const auto &L : b->lists) {
            max_sel = std::max(max_sel, (size_t)L.n_sel[e]);
            multi = multi || L.n_sel[e] > b->G;
        }
        BCUDA(dev_alloc(&b->ratio[e], max_sel * p->N * p->nz * sizeof(float)));
        if (multi) BCUDA(dev_alloc(&b->bp[e], (size_t)p->N * p->N * p->nz * sizeof(float)));
        const int HP = (b->K / 2 + 3) / 4 * 4;
        BCUDA(make_att_tmap(p->dev, fwd_s_cols(128, HP), &b->tm[e]));
    }
    BCUDA(dev_alloc(&b->partials, max_items * b->nz_max * sizeof(float)));
    BCUDA(dev_alloc(&b->counters, 2 * sizeof(int)));
#undef BFAIL
#undef BCUDA
    *out = b;
    return GB_OK;
}

gb_status gb_spect_batch_destroy(gb_spect_batch *b) {
    clear_error();
    if (b) {
        cudaDeviceSynchronize();
        free_batch(b);
    }
    return GB_OK;
}

static gb_status batch_list(const gb_spect_batch *b, int subset, int *li) {
    if (!batch_list_ok(b)) {
        set_error("a plan's subsets or tiles changed after the batch was created; create it "
                  "again");
        return GB_ERR_STATE;
    }
    *li = subset < 0 ? 0 : subset + 1;
    if (*li >= b->n_lists) {
        set_error("subset %d out of range (n_subsets=%d)", subset, b->n_lists - 1);
        return GB_ERR_STATE;
    }
    return GB_OK;
}

gb_status gb_spect_batch_forward(gb_spect_batch *b, const float *const *objects,
                                 float *const *proj, int32_t subset, gb_stream_t stream) {
    clear_error();
    GB_INJECT_ARG();
    GB_CHECK_ARG(b && objects && proj, "null argument");
    for (int e = 0; e < b->n; e++) GB_CHECK_ARG(objects[e] && proj[e], "null buffer of entry %d", e);
    GB_INJECT_LAUNCH();
    int li;
    gb_status s = batch_list(b, subset, &li);
    if (s != GB_OK) return s;
    return batch_forward(b, li, objects, 0, proj, nullptr, nullptr, as_stream(stream));
}

gb_status gb_spect_batch_backward(gb_spect_batch *b, const float *const *proj,
                                  float *const *objects, int32_t subset, int32_t adjoint,
                                  gb_stream_t stream) {
    clear_error();
    GB_INJECT_ARG();
    GB_CHECK_ARG(b && proj && objects, "null argument");
    for (int e = 0; e < b->n; e++) {
        GB_CHECK_ARG(proj[e] && objects[e], "null buffer of entry %d", e);
        GB_CHECK_ARG(!adjoint || ((uintptr_t)objects[e] & 15) == 0,
                     "object %d must be 16-byte aligned (vector atomics)", e);
    }
    GB_INJECT_LAUNCH();
    int li;
    gb_status s = batch_list(b, subset, &li);
    if (s != GB_OK) return s;
    return batch_backward(b, li, proj, adjoint ? 1 : 0, objects, nullptr, as_stream(stream));
}

gb_status gb_spect_batch_osem_step(gb_spect_batch *b, float *const *objects,
                                   const float *const *projections, const float *const *additive,
                                   const float *const *norm_bp, int32_t subset,
                                   gb_stream_t stream) {
    clear_error();
    GB_INJECT_ARG();
    GB_CHECK_ARG(b && objects && projections && norm_bp, "null argument");
    for (int e = 0; e < b->n; e++)
        GB_CHECK_ARG(objects[e] && projections[e] && norm_bp[e], "null buffer of entry %d", e);
    GB_INJECT_LAUNCH();
    int li;
    gb_status s = batch_list(b, subset, &li);
    if (s != GB_OK) return s;
    cudaStream_t st = as_stream(stream);
    s = batch_forward(b, li, objects, 1, b->ratio, projections, additive, st);
    if (s != GB_OK) return s;
    return batch_backward(b, li, b->ratio, 2, objects, norm_bp, st);
}

}  // extern "C"
