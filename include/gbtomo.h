/*
 * gbtomo — C ABI of the GB300 projector hot path (libgbtomo.so).
 *
 * Plain pointers and sizes only.  Every float pointer named "device" is a CUDA
 * device pointer on the current device; streams are passed as opaque
 * `gb_stream_t` (a cudaStream_t; NULL = legacy default stream).  All calls are
 * stream-ordered and allocate nothing: plans own every table and scratch buffer
 * they need, allocated at plan creation.  Calls on one plan must be ordered on a
 * single stream (they share the plan's scratch).  Errors are negative status codes;
 * gb_last_error() returns the message of the calling thread's last failure.
 *
 * The reference interfaces each entry point replaces are cited beside it
 * (paths inside the PyTomography 3.3.2 source tree).
 */
#ifndef GBTOMO_H
#define GBTOMO_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t gb_status;
typedef void *gb_stream_t;

#define GB_OK 0
#define GB_ERR_ARG (-1)          /* invalid argument / null pointer */
#define GB_ERR_SHAPE (-2)        /* unsupported or inconsistent shape */
#define GB_ERR_OOM (-3)          /* device allocation failed at plan creation */
#define GB_ERR_CUDA (-4)         /* a CUDA runtime call or launch failed */
#define GB_ERR_UNSUPPORTED (-5)  /* configuration outside what the kernels implement */
#define GB_ERR_STATE (-6)        /* call out of order (e.g. subsets not set) */

/* Message of the calling thread's last failed call ("" if none). */
const char *gb_last_error(void);
/* Library version string. */
const char *gb_version(void);

/* Device memory of plans and batches comes from a library-owned stream-ordered pool on each
 * device, which keeps up to 16 GiB of freed blocks reserved for the next plan (no
 * counterpart in the reference, whose tensors come from PyTorch's caching allocator).
 * Returns the current device's reserved but unused blocks to the driver, after waiting for
 * the device, so that other allocators can use them; blocks of live plans stay. */
gb_status gb_release_pool_memory(void);

/* Host-side fault injection for tests of the error paths (no counterpart in the reference,
 * which has no native code).  Arms `site` ("alloc": a device allocation at plan creation,
 * subset setup or tuning returns GB_ERR_OOM; "launch": a projector / update entry point
 * returns GB_ERR_CUDA before launching anything; "arg": such an entry point returns
 * GB_ERR_ARG) so that its nth check from now on fails, once; nth = 0 disarms it.  The
 * environment variable GBTOMO_INJECT ("alloc:1,launch:2") arms sites the same way when the
 * library first checks one.  Nothing here touches the GPU. */
gb_status gb_inject_fault(const char *site, int32_t nth);

/* ------------------------------------------------------------------ SPECT */

typedef struct gb_spect_plan gb_spect_plan;

/* Geometry and plugin configuration of a SPECT rotate+sum system matrix.
 * Mirrors SPECTObjectMeta / SPECTProjMeta (metadata/SPECT/spect_metadata.py:8-64),
 * SPECTAttenuationTransform (transforms/SPECT/attenuation.py:24-115) and
 * SPECTPSFTransform (transforms/SPECT/psf.py:101-231) after configure(). */
typedef struct gb_spect_desc {
    int32_t nx, ny, nz;       /* object shape [nx][ny][nz], z fastest; nx == ny */
    float dx, dy, dz;         /* voxel size (cm) */
    int32_t n_angles;         /* number of projection angles */
    /* Normalised sampling matrices [n_angles][6] (host) of the kornia-convention
     * in-plane rotation used by the forward projector (angle beta - 270) and the
     * back-projector (angle 270 - beta): src = theta . (lin[col], lin[row], 1). */
    const float *theta_fwd;
    const float *theta_bwd;
    const float *lin;         /* host [n_pad]: linspace(-1, 1, n_pad), n_pad = nx + 2*pad */
    const float *mu;          /* device [nx][ny][nz] attenuation map (cm^-1), or NULL */
    const char *order;        /* obj2obj transforms in application order: any of "", "a",
                                 "p", "ap", "pa" (a = attenuation, p = PSF) */
    int32_t psf_2d;           /* 1: blur along y and z ('2D'); 0: along y only ('1D') */
    int32_t psf_n_groups;     /* number of distinct detector radii */
    const int32_t *psf_group; /* host [n_angles]: PSF table index of each angle */
    int32_t psf_k;            /* taps per table row (odd); shorter kernels are zero-padded */
    const float *psf_taps_r;  /* host [n_groups][n_pad][psf_k]: y-direction taps per plane */
    const float *psf_taps_z;  /* host [n_groups][n_pad][psf_k]: z-direction taps per plane */
    float psf_trunc_rel;      /* taps below this fraction of a plane's largest tap are
                                 dropped (0 keeps every tap) */
    int32_t no_pad;           /* 1: rotate in the unpadded nx x nx frame (n_pad = nx), as the
                                 StarGuide system matrix does (transforms configured with
                                 assume_padded=False); 0: the padded frame of SPECTSystemMatrix */
    int32_t psf_k_min;        /* 0, or a tap count the plan's PSF bucket must hold at least:
                                 plans run together by gb_spect_batch_create share one bucket */
} gb_spect_desc;

/* Create / destroy a plan.  Creation uploads the geometry tables and precomputes the
 * attenuation factors exp(-rev_cumsum(mu_rot*dx)) of every angle in the rotated
 * padded frame (attenuation.py:11-21, utils/misc.py:8-19).  Replaces
 * SPECTSystemMatrix.__init__ + Transform.configure
 * (projectors/SPECT/spect_system_matrix.py:26-36, projectors/system_matrix.py:46-52). */
gb_status gb_spect_plan_create(const gb_spect_desc *desc, gb_spect_plan **plan);
gb_status gb_spect_plan_destroy(gb_spect_plan *plan);

/* Device-side error word of the plan (synchronous read): 0, or 1 when a kernel's
 * bounded wait on its TMA copies gave up (the kernel then returned without output).
 * No counterpart in the reference (which has no device code). */
gb_status gb_spect_device_status(gb_spect_plan *plan, int32_t *code);
/* Reset the device error word to 0. */
gb_status gb_spect_clear_device_status(gb_spect_plan *plan);
/* Test hook of the bounded waits (no counterpart in the reference): skip_first_copy = 1
 * makes the fused forward projector (attenuation before PSF, nz % 4 == 0) leave its first
 * attenuation copy of every work item unissued, so its wait for that copy runs out after
 * wait_polls polls (each at most 20 us; 0 restores the default of 65536) and the kernel
 * returns with the error word set to 1.  Nothing is left in flight. */
gb_status gb_spect_set_debug(gb_spect_plan *plan, int32_t skip_first_copy, int32_t wait_polls);

/* Interleaved angle subsets indices[i::n_subsets]
 * (spect_system_matrix.py:58-71).  n_subsets >= 1. */
gb_status gb_spect_set_subsets(gb_spect_plan *plan, int32_t n_subsets);
/* Explicit subsets: subset s holds the counts[s] angle indices that follow those of the
 * earlier subsets in angle_idx (host arrays), in projection-row order.  Replaces the
 * interleaved subsets until gb_spect_set_subsets is called again; used for the StarGuide
 * subsets of whole angle groups (starguide_system_matrix.py:166-179). */
gb_status gb_spect_set_subset_lists(gb_spect_plan *plan, int32_t n_subsets,
                                    const int32_t *angle_idx, const int32_t *counts);
/* Number of angles in a subset (-1 = all angles). */
int32_t gb_spect_subset_size(const gb_spect_plan *plan, int32_t subset);

/* Tile configuration of a plan's PSF kernels.  Plan creation picks the widest tiles that
 * fit shared memory; gb_spect_autotune times candidates on the device and keeps the
 * fastest.  No counterpart in the reference (which has no device code). */
typedef struct gb_spect_tuning {
    int32_t fwd_tpb;   /* threads per forward CTA: 512 or 768 (one CTA per SM) */
    int32_t fwd_zt;    /* forward z-slab width; 0 = the widest that fits */
    int32_t fwd_items; /* forward work items per resident CTA slot and z slab: 1 or 2 */
    int32_t b1_zt;     /* back-projection (rotated frame) z-slab width; 0 = widest */
    int32_t b1_items;  /* back-projection work items per SM and z slab: 1 or 2 */
    int32_t fwd_variant; /* forward kernel: 1 (samples gathered per plane, y blur first) or 2
                            (corner rows staged through a cp.async ring, z blur first;
                            attenuation before a 2-D PSF of at most 29 taps, N and
                            nz <= 128); 0 keeps the plan's current one */
    int32_t osem_split;  /* 1: gb_spect_osem_step runs the two halves of a subset's angles on
                            two streams (fork / join by events, same kernels and results);
                            0: one stream */
} gb_spect_tuning;
gb_status gb_spect_get_tuning(const gb_spect_plan *plan, gb_spect_tuning *out);
/* Apply a tuning (rebuilds the work lists of the current subsets; may allocate: call at
 * set-up, outside stream capture).  GB_ERR_UNSUPPORTED when a tile does not fit. */
gb_status gb_spect_set_tuning(gb_spect_plan *plan, const gb_spect_tuning *tuning);
/* Time the candidate tunings on `subset` (reps launches each, on a temporary object of
 * ones), apply the fastest forward and back-projection tiles and return them in *out
 * (may be NULL).  Allocates temporaries: call at set-up, outside stream capture.  A plan
 * without PSF has nothing to tune and returns its tuning unchanged. */
gb_status gb_spect_autotune(gb_spect_plan *plan, int32_t subset, int32_t reps,
                            gb_spect_tuning *out, gb_stream_t stream);

/* Forward projection H_m f -> proj [n_sel][ny][nz] (device).
 * Replaces SPECTSystemMatrix.forward (spect_system_matrix.py:120-157).
 * subset = -1 projects every angle. */
gb_status gb_spect_forward(gb_spect_plan *plan, const float *object, float *proj,
                           int32_t subset, gb_stream_t stream);

/* Same projection as gb_spect_forward, for callers that must not allocate device memory
 * while they run (code on a pool-restricted stream, processes whose device memory belongs
 * to another allocator, services that budget every allocation up front).  No counterpart in the reference.  Its partial sums use a fixed
 * 16 MiB device array compiled into the library instead of the plan's scratch; calls
 * needing more than 4,194,304 floats of partials (the plan's work items for the subset,
 * at least one per angle, times nx * nz) return GB_ERR_SHAPE.  Calls share that array: overlapping calls on the GPU race.  The first
 * call on a device looks the array up (cudaGetSymbolAddress); make it before any stream
 * capture. */
gb_status gb_spect_forward_static(gb_spect_plan *plan, const float *object, float *proj,
                                  int32_t subset, gb_stream_t stream);

/* Back projection proj [n_sel][ny][nz] -> object [nx][ny][nz] (device, overwritten).
 * adjoint = 0: the reference back-projector, which rotates back with bilinear
 *              interpolation by +(270 - beta)
 *              (SPECTSystemMatrix.backward, spect_system_matrix.py:159-201);
 * adjoint = 1: the exact transpose of gb_spect_forward (same taps, scattered). */
gb_status gb_spect_backward(gb_spect_plan *plan, const float *proj, float *object,
                            int32_t subset, int32_t adjoint, gb_stream_t stream);

/* One fused OSEM sub-iteration, in place on `object`:
 *   f <- f + f/(normBP_m + delta) * (H_m^T (g_m / (H_m f + s_m + delta)) - normBP_m),
 *   f[f <= 0] = 0.
 * projections / additive are the FULL [n_angles][ny][nz] arrays (additive may be NULL);
 * norm_bp is H_m^T 1 of this subset.  Replaces one pass of
 * PreconditionedGradientAscentAlgorithm.__call__ with OSEM
 * (algorithms/preconditioned_gradient_ascent.py:103-122, 319-329) and
 * PoissonLogLikelihood.compute_gradient (likelihoods/poisson_log_likelihood.py:16-36).
 * predicted (optional, device [n_sel][ny][nz]) receives H_m f + s_m. */
gb_status gb_spect_osem_step(gb_spect_plan *plan, float *object, const float *projections,
                             const float *additive, const float *norm_bp, int32_t subset,
                             float *predicted, gb_stream_t stream);

/* ------------------------------------------------- per-angle obj2obj plugins
 * The two plugins of the reference's per-angle loop
 * (projectors/SPECT/spect_system_matrix.py:145-154 and 188-198), applied to an object
 * that the caller has already padded and rotated into the detector frame of one angle:
 * [L][ny][nz] device arrays, x (the first axis) towards the detector.  They need no plan.
 *
 * Attenuation, SPECTAttenuationTransform.forward / backward
 * (transforms/SPECT/attenuation.py:72-115 with get_prob_of_detection_matrix, :11-21, and
 * rev_cumsum, utils/misc.py:8-19):
 *   out[x][y][z] = in[x][y][z] * exp(-(sum_{k>=x} t_k - t_x / 2)),  t_k = mu_rot[k][y][z] * dx,
 * where mu_rot is mu ([n][n][nz], device, cm^-1) zero-padded by `pad` in x and y
 * (L = n + 2 pad) and sampled at the kornia-convention rotation `theta` (host [6], the
 * forward-projector matrix of the angle, as gb_spect_desc.theta_fwd) over the grid `lin`
 * (device [L], linspace(-1, 1, L)).  The factor is recomputed from mu on every call.
 * Backward is the same diagonal operator.  in may equal out. */
gb_status gb_spect_attenuation_apply(const float *mu, int32_t n, int32_t nz, int32_t pad,
                                     float dx, const float *theta, const float *lin,
                                     const float *in, float *out, gb_stream_t stream);
/* Depth-dependent separable PSF, SPECTPSFTransform.forward / backward
 * (transforms/SPECT/psf.py:199-231 -> Seperable1DBlurNet.forward, :27-41): per plane x,
 * a 'same' zero-padded correlation along y with taps_y[x] ([nplanes][ky], device), then
 * along z with taps_z[x] ([nplanes][kz], device; NULL = the '1D' model, no z blur).
 * Backward is the same (symmetric taps).  Odd tap counts up to 63; in and out must
 * differ. */
gb_status gb_spect_psf_apply(const float *in, float *out, int32_t nplanes, int32_t ny,
                             int32_t nz, const float *taps_y, int32_t ky, const float *taps_z,
                             int32_t kz, gb_stream_t stream);

/* ---------------------------------------------------------------- batches
 * Several independent projection problems in one launch per phase: the reconstructions of
 * a serving batch (each with its own plan: size, angles, attenuation, PSF), or several
 * objects on one shared plan (a batch of the autograd path).  Replaces the reference's
 * per-reconstruction, per-angle Python loops (projectors/SPECT/spect_system_matrix.py:
 * 145-154, 188-198, driven by algorithms/preconditioned_gradient_ascent.py:80-129).
 *
 * A batch holds 1 to 32 entries, entry e projecting with plans[e] (plans may repeat).  The
 * plans must have a PSF of one tap bucket (create them with a common psf_k_min), one
 * subset count (subsets set before the batch is created), N <= 128, nz <= 128 and
 * nz % 4 == 0.  The work items of every entry's angles are split by the plans' plane-cost
 * model into about two waves of the GPU and dequeued, largest first, by one persistent CTA
 * per SM; the per-(entry, angle) sums are reduced in plane order, so results do not depend
 * on the queue order.  Creation allocates the batch's scratch (W stacks, ratio rows,
 * partial sums); the calls allocate nothing.  Host arrays hold one device pointer per
 * entry.  Calls on one batch must be ordered on one stream. */
typedef struct gb_spect_batch gb_spect_batch;
gb_status gb_spect_batch_create(gb_spect_plan *const *plans, int32_t n, gb_spect_batch **batch);
gb_status gb_spect_batch_destroy(gb_spect_batch *batch);
/* proj[e] [n_sel][ny][nz] = H_{e,m} objects[e] for every entry (subset -1: all angles). */
gb_status gb_spect_batch_forward(gb_spect_batch *batch, const float *const *objects,
                                 float *const *proj, int32_t subset, gb_stream_t stream);
/* objects[e] (overwritten) = H_{e,m}^T proj[e]: adjoint = 0 the reference back-projector,
 * 1 the exact transpose of gb_spect_batch_forward (objects 16-byte aligned). */
gb_status gb_spect_batch_backward(gb_spect_batch *batch, const float *const *proj,
                                  float *const *objects, int32_t subset, int32_t adjoint,
                                  gb_stream_t stream);
/* One fused OSEM sub-iteration of every entry, as gb_spect_osem_step with subset `subset`:
 * objects[e] updated in place, projections[e] / additive[e] (additive may be NULL, or hold
 * NULL entries) the full [n_angles][ny][nz] arrays, norm_bp[e] the entry's H_m^T 1. */
gb_status gb_spect_batch_osem_step(gb_spect_batch *batch, float *const *objects,
                                   const float *const *projections, const float *const *additive,
                                   const float *const *norm_bp, int32_t subset,
                                   gb_stream_t stream);

/* Relative-difference prior with Euclidean neighbour weights
 * (priors/nearest_neighbour.py:156-183, 207-220). */
typedef struct gb_rdp_desc {
    float beta, gamma, delta;  /* delta: pytomography.delta at prior construction */
    const float *fov_scale;    /* device [nx][ny][nz] or NULL (all ones) */
} gb_rdp_desc;

/* One fused BSREM sub-iteration (PGA:436-474):
 *   out = in + in * relax / (w_m * sum_k normBP_k + delta)
 *              * (H_m^T (g_m/(H_m in + s_m + delta)) - normBP_m - grad V(in) * w_m),
 *   out[out <= floor] = floor,
 * grad V from the RDP prior (prior may be NULL: no prior).  in and out must differ. */
gb_status gb_spect_bsrem_step(gb_spect_plan *plan, const float *object_in, float *object_out,
                              const float *projections, const float *additive,
                              const float *norm_bp, const float *norm_bp_sum, float relax,
                              float subset_weight, const gb_rdp_desc *prior, float floor_value,
                              int32_t subset, gb_stream_t stream);

/* RDP gradient beta * scale * sum_s w_rs phi1(f_r, f_s) * fov_scale
 * (nearest_neighbour.py:44-75 with phi1 of :176-177), replicate boundary. */
gb_status gb_rdp_gradient(const float *object, float *grad, int32_t nx, int32_t ny,
                          int32_t nz, float dx, float dy, float dz, const gb_rdp_desc *prior,
                          float beta_scale, gb_stream_t stream);
/* RDP second derivative at f applied to x (the derivative_order=2 operator of
 * NearestNeighbourPrior.__call__, nearest_neighbour.py:89-110 with phi2_1 / phi2_2 of
 * :179-183): out_r = beta * scale * fov_r * sum_s w_rs (phi2_1(f_r, f_s) x_r +
 * phi2_2(f_r, f_s) x_s); used by the uncertainty estimate.  out must not alias f or x. */
gb_status gb_rdp_hessian_vector(const float *f, const float *x, float *out, int32_t nx,
                                int32_t ny, int32_t nz, float dx, float dy, float dz,
                                const gb_rdp_desc *prior, float beta_scale, gb_stream_t stream);

/* -------------------------------------------------------------------- PET */

typedef struct gb_pet_plan gb_pet_plan;

/* Listmode geometry and events.  Mirrors PETLMProjMeta / PETTOFMeta
 * (metadata/PET/petlm_metadata.py:6-39, metadata/PET/pet_tof_metadata.py:5-37) and the
 * PETLMSystemMatrix constructor (projectors/PET/petlm_system_matrix.py:24-57). */
typedef struct gb_pet_desc {
    int32_t nx, ny, nz;        /* image shape [nx][ny][nz], z fastest */
    float vx, vy, vz;          /* voxel size (mm) */
    float ox, oy, oz;          /* centre of voxel (0,0,0) (mm): (-shape/2 + 0.5) * voxel */
    int32_t n_det;             /* crystals in the scanner LUT */
    const float *lut;          /* host [n_det][3] crystal centres (mm) */
    int32_t tof;               /* 1: events carry a TOF bin in column 2 */
    int32_t tof_num_bins;
    float tof_bin_width;       /* mm */
    float tof_sigma;           /* mm */
    float tof_center_offset;   /* mm */
    float tof_n_sigmas;
    int64_t n_events;
    const int32_t *events;     /* host or device [n_events][2 or 3]: id1, id2 (, tof bin) */
} gb_pet_desc;

/* Replaces PETLMSystemMatrix.__init__ (petlm_system_matrix.py:24-57) minus the
 * sensitivity image (gb_pet_sensitivity).  Events are copied to the device once. */
gb_status gb_pet_plan_create(const gb_pet_desc *desc, gb_pet_plan **plan);
gb_status gb_pet_plan_destroy(gb_pet_plan *plan);
/* Interleaved event subsets indices[i::n_subsets] (petlm_system_matrix.py:176-189). */
gb_status gb_pet_set_subsets(gb_pet_plan *plan, int32_t n_subsets);

/* TOF (or non-TOF) Joseph forward projection of the subset's events -> proj [n_sel].
 * Replaces parallelproj.joseph3d_fwd_tof_lm / joseph3d_fwd as called by
 * PETLMSystemMatrix.forward (petlm_system_matrix.py:243-297). */
gb_status gb_pet_forward(gb_pet_plan *plan, const float *img, float *proj, int32_t subset,
                         gb_stream_t stream);
/* Adjoint: image (overwritten) = H_m^T proj.  Replaces joseph3d_back_tof_lm /
 * joseph3d_back in PETLMSystemMatrix.backward (petlm_system_matrix.py:299-363).
 * img must be 16-byte aligned (vector atomics). */
gb_status gb_pet_backward(gb_pet_plan *plan, const float *proj, float *img, int32_t subset,
                          gb_stream_t stream);
/* Deterministic back projection for reproducibility (no counterpart in the reference):
 * with on = 1, gb_pet_backward accumulates every contribution as a 64-bit fixed-point
 * integer (scale 2^k with k chosen on the device from the largest |proj| of the call so
 * that no sum can overflow) and converts the sums to float at the end; the results are
 * then bit-identical from run to run, whatever the order of the atomic additions, and
 * agree with the float path to rounding.  Allocates an int64 image (call at set-up);
 * on = 0 frees it and restores the float-atomic path. */
gb_status gb_pet_set_deterministic(gb_pet_plan *plan, int32_t on);
/* Non-TOF line integrals of `img` along the subset's events (attenuation path,
 * petlm_system_matrix.py:91-110); use_tof selects the TOF kernel instead. */
gb_status gb_pet_lor_forward(gb_pet_plan *plan, const float *img, float *proj, int32_t subset,
                             int32_t use_tof, gb_stream_t stream);
/* Sensitivity image: non-TOF back projection of (weights * exp(-H mu) + add) over the
 * LOR set `pairs` [n_pairs][2] (device), or over every crystal pair i < j when pairs is
 * NULL (petlm_system_matrix.py:112-174).  weights / mu may be NULL; img must be 16-byte
 * aligned. */
gb_status gb_pet_sensitivity(gb_pet_plan *plan, const int32_t *pairs, int64_t n_pairs,
                             const float *weights, const float *mu, float add, float *img,
                             gb_stream_t stream);
/* One fused listmode OSEM sub-iteration in place on img:
 * f += f/(nbp+delta) * (H_m^T (numerator / (H_m f + s_m + delta)) - nbp), clamp at 0.
 * numerator holds 1 value (listmode: projections = [1.]) or n_events values; additive
 * (full [n_events], device) may be NULL; norm_bp is the subset's normalisation image. */
gb_status gb_pet_osem_step(gb_pet_plan *plan, float *img, const float *numerator,
                           int64_t numerator_len, const float *additive, const float *norm_bp,
                           int32_t subset, gb_stream_t stream);

/* ------------------------------------------------------------ PET sinogram
 * Replaces the projection arithmetic of PETSinogramSystemMatrix
 * (projectors/PET/pet_sinogram_system_matrix.py:12-296): the LOR of sinogram element
 * (angle a, radial r, plane p) runs from (det_xy[a][r][0], plane_z[p][0]) to
 * (det_xy[a][r][1], plane_z[p][1]) (_get_xyz_sinogram_coordinates, :50-85). */
typedef struct gb_pet_sino_plan gb_pet_sino_plan;

typedef struct gb_pet_sino_desc {
    int32_t nx, ny, nz;        /* image shape [nx][ny][nz], z fastest */
    float vx, vy, vz;          /* voxel size (mm) */
    float ox, oy, oz;          /* centre of voxel (0,0,0) (mm) */
    int32_t n_angles, n_radial, n_planes;  /* sinogram [n_angles][n_radial][n_planes] */
    const float *det_xy;       /* host [n_angles][n_radial][2][2]: (x, y) of crystals 1, 2 */
    const float *plane_z;      /* host [n_planes][2]: z of crystals 1, 2 */
    int32_t tof;               /* 1: TOF sinograms (bin fastest) are available */
    int32_t tof_num_bins;
    float tof_bin_width;       /* mm */
    float tof_sigma;           /* mm */
    float tof_center_offset;   /* mm */
    float tof_n_sigmas;
} gb_pet_sino_desc;

gb_status gb_pet_sino_plan_create(const gb_pet_sino_desc *desc, gb_pet_sino_plan **plan);
gb_status gb_pet_sino_plan_destroy(gb_pet_sino_plan *plan);
/* Angle subsets i::n_subsets (pet_sinogram_system_matrix.py:131-144). */
gb_status gb_pet_sino_set_subsets(gb_pet_sino_plan *plan, int32_t n_subsets);
/* Angles in a subset (-1 = all angles). */
int32_t gb_pet_sino_subset_size(const gb_pet_sino_plan *plan, int32_t subset);
/* proj [n_sel][n_radial][n_planes] (x tof_num_bins, bin fastest, when use_tof on a TOF
 * plan) = H img: joseph3d_fwd / joseph3d_fwd_tof_sino (:203-235). */
gb_status gb_pet_sino_forward(gb_pet_sino_plan *plan, const float *img, float *proj,
                              int32_t subset, int32_t use_tof, gb_stream_t stream);
/* img = H^T proj (overwrites img): joseph3d_back / joseph3d_back_tof_sino (:263-292);
 * use_tof = 0 on a TOF plan is the reference's force_nonTOF.  img must be 16-byte
 * aligned. */
gb_status gb_pet_sino_backward(gb_pet_sino_plan *plan, const float *proj, float *img,
                               int32_t subset, int32_t use_tof, gb_stream_t stream);
/* prob [n_sel][n_radial][n_planes] = exp(-H mu), the attenuation probability sinogram
 * (_compute_atteunation_probability_projection, :87-109). */
gb_status gb_pet_sino_atten(gb_pet_sino_plan *plan, const float *mu, float *prob,
                            int32_t subset, gb_stream_t stream);
/* Listmode -> sinogram histogram (io/PET/shared.py:175-272), all pointers device:
 * events [n_events][ncol] (id1, id2[, TOF bin]); weights [n_events] or NULL; lor_bins
 * [ncpr][ncpr][2] (angular, radial) and plane_index [n_rings][n_rings] from
 * sinogram_coordinates; tof_num_bins = 0 for a non-TOF sinogram; normalization averages the
 * ordered and the mirrored binning.  sino [n_angles][n_radial][n_planes](x tof_num_bins) is
 * overwritten. */
gb_status gb_pet_lm_to_sino(const int32_t *events, int64_t n_events, int32_t ncol,
                            const float *weights, const int32_t *lor_bins,
                            const int32_t *plane_index, int32_t n_crystals_per_ring,
                            int32_t n_rings, int32_t n_angles, int32_t n_radial,
                            int32_t n_planes, int32_t tof_num_bins, int32_t normalization,
                            float *sino, gb_stream_t stream);

/* --------------------------------------------------------- StarGuide window */
/* Detector window of the StarGuide system matrix (projectors/SPECT/
 * starguide_system_matrix.py:30-110) applied to projections of a no_pad plan (all device):
 * out [n][width][nz] = scale[i] * full[i] translated along y by shift[i] pixels (output
 * column y reads input column y - shift, linear interpolation, zero outside) on the
 * columns int(ny/2) - width/2 ... + width - 1.  The reference uses width 16, shift =
 * offset / dx and scale = time / 1000. */
gb_status gb_starguide_window(const float *full, float *out, int32_t n, int32_t ny, int32_t nz,
                              int32_t width, const float *shift, const float *scale,
                              gb_stream_t stream);
/* The back-projection side: full [n][ny][nz] = the window of scale[i] * proj[i]
 * zero-padded to ny columns ((ny - width) even), translated by -shift[i]. */
gb_status gb_starguide_window_adjoint(const float *proj, float *full, int32_t n, int32_t ny,
                                      int32_t nz, int32_t width, const float *shift,
                                      const float *scale, gb_stream_t stream);

/* ---------------------------------------------------- object-space operators */
/* Separable Gaussian filter, GaussianFilter.forward (transforms/shared/filters.py:47-63):
 * 'same' zero-padded correlation along x, then y, then z with odd tap counts.  All
 * pointers device; in, out and scratch ([nx][ny][nz] each) must be distinct. */
gb_status gb_filter3d(const float *in, float *out, float *scratch, int32_t nx, int32_t ny,
                      int32_t nz, const float *taps_x, int32_t kx, const float *taps_y,
                      int32_t ky, const float *taps_z, int32_t kz, gb_stream_t stream);
/* Kernel-method basis, KEMTransform.forward (transforms/shared/kem.py:111-128):
 * out[v] = sum_t kern[t][v] * in[clamp(v + offset_t)] over the size^3 offsets in
 * (a, b, c) loop order, replicate boundary.  kern [size^3][nx][ny][nz] device. */
gb_status gb_kem_apply(const float *in, float *out, const float *kern, int32_t nx, int32_t ny,
                       int32_t nz, int32_t size, gb_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* GBTOMO_H */
