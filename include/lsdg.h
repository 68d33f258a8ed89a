/*
 * lsdg.h -- C-ABI of the GB300-native LSD-SLAM per-pixel hot path.
 *
 * Two parts, both computed by hand-written CUDA kernels for sm_103a on one GPU:
 *   - direct image alignment: the per-point warp, photometric residual, Jacobian and
 *     Huber-weighted normal equations inside a Levenberg-Marquardt loop over the image
 *     pyramid (SE3Tracker::trackFrame, Sim3Tracker::trackFrameSim3, calculateWarpUpdate);
 *   - the semi-dense inverse-depth filter (DepthMap::updateKeyframe -> observeDepth,
 *     DepthMap::createKeyFrame -> propagateDepth, regularizeDepthMap).
 *
 * Where the reference meets this path: lib/App/InputThread.cpp:71 hands every undistorted
 * 8-bit frame to SlamSystem::nextImage, whose tracking / mapping / constraint-search threads call
 * the four methods above (they live in the lsd-slam fips import, fips.yml:2-4).  The results
 * leave through OutputIOWrapper (lib/Pangolin_IOWrapper/PangolinOutputIOWrapper.cpp:42-97), which
 * reads per pyramid level row-major float arrays idepth(lvl), idepthVar(lvl), image(lvl) with
 * idepth <= 0 meaning "no depth" (lib/Pangolin_IOWrapper/Keyframe.h:95).  lsdg_frame_get_depth and
 * lsdg_depth_get return exactly that layout.
 *
 * Conventions
 *   - images: row-major float32, pixel centres at integer coordinates; width and height must be
 *     multiples of 2^(levels-1).
 *   - pinhole back-projection X = (x - cx) / fx * z (Keyframe.h:86-89,134-136), z = 1 / idepth.
 *   - pyramid level l+1 is the 2x2 mean of level l; fx_{l+1} = fx_l / 2,
 *     cx_{l+1} = (cx_l + 0.5) / 2 - 0.5.
 *   - a pose is 12 doubles, row-major [R | t] (3x4).  "a_to_b" maps a point in camera a's
 *     coordinates into camera b's.  A Sim3 pose is 13 doubles: [R | t] followed by the scale s
 *     (x_b = s R x_a + t).
 *   - every call returns lsdg_status; lsdg_last_error gives a message.  Nothing aborts and no
 *     C++ exception crosses this boundary.  Host pointers are caller-owned and only read or
 *     written during the call.  All device memory is owned by the context.
 *   - calls on one context run in order on the context's CUDA stream and are synchronous unless
 *     documented otherwise.  Use one context per calling thread (the reference runs tracking,
 *     mapping and constraint search on separate threads).
 *
 * There is no CPU fallback: every compute entry point launches CUDA kernels and fails with
 * LSDG_CUDA_ERROR when no usable GPU is present.
 */
#ifndef LSDG_H_
#define LSDG_H_

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define LSDG_API __attribute__((visibility("default")))
#else
#define LSDG_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define LSDG_MAX_LEVELS 6
#define LSDG_NE_SIZE 32      /* normal-equation record, see lsdg_se3_normal_equations */
#define LSDG_NE_SIZE_SIM3 40 /* Sim3 record, see lsdg_sim3_normal_equations */

typedef enum lsdg_status {
  LSDG_OK = 0,
  LSDG_INVALID_ARG = 1,
  LSDG_TRACKING_LOST = 2, /* the pose is still written; quality numbers are in the stats */
  LSDG_DIVERGED = 3,
  LSDG_TIMEOUT = 4, /* a bounded device-side wait ran out; the context stays usable */
  LSDG_CUDA_ERROR = 5,
  LSDG_OUT_OF_MEMORY = 6,
  LSDG_NOT_SUPPORTED = 7
} lsdg_status;

typedef struct lsdg_intrinsics {
  float fx, fy, cx, cy; /* level 0 */
} lsdg_intrinsics;

/* Tuning table shared by the kernels and the CPU oracle.  The upstream constants are not
 * available (the lsd-slam import is not vendored), so this table is the project's own; each
 * value's meaning is documented here and lsdg_default_params fills it. */
typedef struct lsdg_params {
  int32_t levels; /* pyramid levels, 1..LSDG_MAX_LEVELS (default 5) */

  /* ---- direct alignment (SE3 and Sim3) ---- */
  int32_t max_iterations[LSDG_MAX_LEVELS]; /* LM iterations per level, index = level */
  float photometric_variance; /* sigma_I^2 of a residual (intensity units^2) */
  float huber_delta;          /* Huber threshold on the variance-normalised residual */
  float min_z;                /* warped points with z <= min_z are not used (m) */
  float border_margin;        /* a point takes part in a level only if its first warp of that level
                                 lands this many pixels inside the image (px) */
  float lm_lambda_initial;    /* LM damping at the start of each level: A_ii = H_ii (1 + lambda) */
  float lm_lambda_up;         /* lambda *= up after a rejected step */
  float lm_lambda_down;       /* lambda *= down after an accepted step */
  float step_eps;             /* level l ends when the undamped Gauss-Newton step of the current
                                 linearisation is below step_eps * 2^l in every twist coordinate */
  float stall_eps;            /* ... or when a step is rejected while that undamped step is below
                                 stall_eps * 2^l (the level's noise floor is reached) */
  float min_good_ratio;       /* inliers / used points below which tracking is lost */
  float min_usage;            /* used points / keyframe points below which tracking is lost */
  float sim3_depth_variance;  /* floor of the inverse-depth residual variance (Sim3) */
  float sim3_depth_weight;    /* weight of the inverse-depth residual relative to photometric */

  /* ---- depth filter: observeDepth ---- */
  float min_grad;          /* keyframe gradient magnitude needed to observe a pixel */
  float min_idepth;        /* search range limits (1/m) */
  float max_idepth;
  float epipolar_var;      /* sigma_l^2: variance of the epipolar line position (px^2) */
  float image_var;         /* sigma_i^2: image noise variance for the photometric disparity error */
  float min_grad_along_epl2; /* minimum squared cosine between gradient and epipolar line */
  float max_ssd;           /* mean squared difference per sample above which a match fails */
  float unique_ratio;      /* the best SSD must be below second-best / unique_ratio */
  float search_sigmas;     /* search +- this many standard deviations around a hypothesis */
  float max_search_len;    /* longest epipolar segment searched (px) */
  float min_search_len;    /* shortest epipolar segment searched (px) */
  float fuse_chi2;         /* (d_obs - d)^2 / (var + var_obs) above this: inconsistent */
  float min_epl_length;    /* epipolar disparity below this many pixels per unit of inverse depth
                              (1/m) means no usable baseline: the observation is skipped */
  int32_t validity_init;   /* validity of a new hypothesis */
  int32_t validity_max;
  int32_t validity_penalty; /* subtracted on an inconsistent observation */
  int32_t blacklist_limit; /* pixels with this many failed matches are no longer observed */

  /* ---- propagateDepth ---- */
  float prediction_var;    /* added to the propagated variance (1/m^2) */
  float propagate_max_photo_diff; /* |I_new - I_old| above this drops a propagated hypothesis */

  /* ---- regularizeDepthMap + hole filling ---- */
  int32_t reg_radius;       /* window half-size */
  float reg_chi2;           /* neighbour compatible if (d_n - d)^2 <= reg_chi2 (var_n + var) */
  int32_t reg_min_support;  /* a hypothesis with fewer compatible neighbours is removed */
  int32_t fill_min_support; /* a hole with at least this many valid neighbours is filled */
  float fill_var_factor;    /* variance of a filled pixel = factor * neighbours' harmonic mean */

  /* inverse-depth refinement (lsdg_energy_refine) */
  float refine_prior_weight; /* weight of the Gaussian prior (rho - rho0)^2 / var of each point; 0 = none */
  int32_t reserved[7];
} lsdg_params;

typedef struct lsdg_track_stats {
  int32_t status;                       /* lsdg_status of this alignment */
  int32_t passes[LSDG_MAX_LEVELS];      /* residual passes run per level (1 + iterations) */
  int32_t total_passes;
  int32_t n_points;                     /* keyframe points at level 0 */
  int32_t n_valid;                      /* points that warped into the image (last pass, level 0) */
  int32_t n_good;                       /* inliers (|r / sigma| <= huber_delta) */
  float mean_energy;                    /* mean Huber energy of the last accepted pass */
  float good_ratio;                     /* n_good / n_valid */
  float usage;                          /* n_valid / n_points */
  double hessian[28];                   /* upper triangle of J^T W J at the result (21 SE3, 28 Sim3) */
} lsdg_track_stats;

typedef struct lsdg_ctx lsdg_ctx;
typedef struct lsdg_frame lsdg_frame;
typedef struct lsdg_batch lsdg_batch;
typedef struct lsdg_depthmap lsdg_depthmap;
typedef struct lsdg_energy lsdg_energy;
typedef struct lsdg_undistorter lsdg_undistorter;

/* Input camera calibration (what libvideoio's UndistorterFactory reads from the file given with
 * -c/--calib, tools/LSD.cpp:62,88; the sample is d2_camera.xml).  Models:
 *   LSDG_CALIB_PINHOLE: no distortion (u = f x + w/2 + cx, v = f y + h/2 + cy);
 *   LSDG_CALIB_FRAME ("<projection>frame</projection>"): with r^2 = x^2 + y^2,
 *     x' = x (1 + k1 r^2 + k2 r^4 + k3 r^6 + k4 r^8) + p1 (r^2 + 2 x^2) + 2 p2 x y
 *     y' = y (1 + k1 r^2 + k2 r^4 + k3 r^6 + k4 r^8) + p2 (r^2 + 2 y^2) + 2 p1 x y
 *     u = w/2 + cx + x' f + x' b1 + y' b2,   v = h/2 + cy + y' f
 *   with (u, v) measured from the image's top-left corner (pixel centres at +0.5). */
#define LSDG_CALIB_PINHOLE 0
#define LSDG_CALIB_FRAME 1
typedef struct lsdg_calibration {
  int32_t model;
  int32_t width, height;   /* raw input size */
  double f, cx, cy;        /* focal length; principal point offset from the image centre (pixels) */
  double b1, b2;           /* affinity and skew */
  double k1, k2, k3, k4;   /* radial */
  double p1, p2;           /* tangential */
} lsdg_calibration;

/* Wire formats of the viewer path, byte-compatible with the reference's structs:
 * InputPointDense (lib/Pangolin_IOWrapper/Keyframe.h:16-21): what publishKeyframe copies per pixel,
 * Keyframe::MyVertex (Keyframe.h:50-54): one point of the keyframe's cloud, colour stored B, G, R, A. */
typedef struct lsdg_input_point_dense {
  float idepth;
  float idepth_var;
  uint8_t color[4];
} lsdg_input_point_dense;

typedef struct lsdg_cloud_vertex {
  float point[3];
  uint8_t color[4];
} lsdg_cloud_vertex;

/* Keyframe::computeVbo's filter constants (Keyframe.h:78-82); lsdg_cloud_default_params gives
 * scaled_th 1e-3, abs_th 1e-1, min_near_support 9 (the sparsify factor is 1 there: no sampling). */
typedef struct lsdg_cloud_params {
  float scaled_th;        /* drop a point when idepth_var * depth^4 > scaled_th */
  float abs_th;           /* ... or when idepth_var * depth^4 * scale^2 > abs_th */
  int32_t min_near_support; /* 3x3 neighbours (centre included) within sqrt(2 var) of its idepth */
  int32_t reserved;
} lsdg_cloud_params;

/* ------------------------------------------------------------------------------------------ */
/* Context                                                                                     */
/* ------------------------------------------------------------------------------------------ */

/* Fill the default tuning table (host only, needs no GPU). */
LSDG_API void lsdg_default_params(lsdg_params* params);

/* ABI version of this header (host only). */
LSDG_API int32_t lsdg_abi_version(void);

/* Create a context on CUDA device `device` with its own stream.  params may be NULL (defaults). */
LSDG_API lsdg_status lsdg_create(lsdg_ctx** out, const lsdg_params* params, int device);
LSDG_API lsdg_status lsdg_destroy(lsdg_ctx* ctx);
LSDG_API lsdg_status lsdg_set_params(lsdg_ctx* ctx, const lsdg_params* params);
LSDG_API const char* lsdg_last_error(const lsdg_ctx* ctx);
/* The context's cudaStream_t (for callers that time or order work around the library). */
LSDG_API void* lsdg_stream(lsdg_ctx* ctx);
LSDG_API lsdg_status lsdg_sync(lsdg_ctx* ctx);
/* Number of kernel launches this context has issued so far (all entry points). */
LSDG_API int64_t lsdg_launch_count(const lsdg_ctx* ctx);

/* ------------------------------------------------------------------------------------------ */
/* Frames (upstream Frame: intensity + gradient pyramid, optional keyframe depth)              */
/* ------------------------------------------------------------------------------------------ */

LSDG_API lsdg_status lsdg_frame_create(lsdg_ctx* ctx, int width, int height, const lsdg_intrinsics* intr,
                              lsdg_frame** out);
LSDG_API lsdg_status lsdg_frame_destroy(lsdg_ctx* ctx, lsdg_frame* frame);
/* Upload a float32 image (host) and build the {I, gx, gy} pyramid on the device. */
LSDG_API lsdg_status lsdg_frame_upload(lsdg_ctx* ctx, lsdg_frame* frame, const float* image);
/* Same for an 8-bit image, the type InputThread hands to SlamSystem::nextImage
 * (lib/App/InputThread.cpp:58-71). */
LSDG_API lsdg_status lsdg_frame_upload_u8(lsdg_ctx* ctx, lsdg_frame* frame, const uint8_t* image);
/* Set level-0 inverse depth and its variance (host arrays, idepth <= 0 = none) and build the
 * depth pyramid and the tracking reference points (SoA float4 {X, Y, Z, I} + float var). */
LSDG_API lsdg_status lsdg_frame_set_depth(lsdg_ctx* ctx, lsdg_frame* frame, const float* idepth,
                                 const float* idepth_var);
/* Read back one pyramid level as float4 {I, gx, gy, 0} per pixel (4 * w_l * h_l floats). */
LSDG_API lsdg_status lsdg_frame_get_level(lsdg_ctx* ctx, const lsdg_frame* frame, int level, float* out);
/* Read back one level of the depth pyramid (Frame::idepth(lvl) / idepthVar(lvl) layout). */
LSDG_API lsdg_status lsdg_frame_get_depth(lsdg_ctx* ctx, const lsdg_frame* frame, int level, float* idepth,
                                 float* idepth_var);
/* Read back the tracking reference points of one level: xyzi = 4 floats per point, var = 1. */
LSDG_API lsdg_status lsdg_frame_get_points(lsdg_ctx* ctx, const lsdg_frame* frame, int level, float* xyzi,
                                  float* var, int capacity, int* count);

/* ------------------------------------------------------------------------------------------ */
/* SE3 direct alignment                                                                        */
/* ------------------------------------------------------------------------------------------ */

/* calculateWarpUpdate at a fixed pose: one residual pass of `reference`'s level-`level` points
 * warped into `frame` by ref_to_frame.  out[LSDG_NE_SIZE] =
 *   [0..20]  upper triangle of sum w J^T J (row-major: 00 01 .. 05 11 .. 55)
 *   [21..26] sum w J^T r
 *   [27]     sum of Huber energies
 *   [28]     points used (warped into the image)
 *   [29]     inliers, [30] outliers, [31] points that left the image or went behind the camera.
 * J is d r / d xi for the left increment exp(xi) * ref_to_frame, xi = (v, omega). */
LSDG_API lsdg_status lsdg_se3_normal_equations(lsdg_ctx* ctx, const lsdg_frame* reference,
                                      const lsdg_frame* frame, int level,
                                      const double ref_to_frame[12], double out[LSDG_NE_SIZE]);

/* SE3Tracker::trackFrame: align `frame` to the keyframe `reference` (which carries depth),
 * coarse to fine, starting from frame_to_ref_init.  Writes the refined frame_to_ref and stats.
 * Returns LSDG_TRACKING_LOST (pose still written) when the quality tests fail. */
LSDG_API lsdg_status lsdg_track_se3(lsdg_ctx* ctx, const lsdg_frame* reference, const lsdg_frame* frame,
                           const double frame_to_ref_init[12], double frame_to_ref_out[12],
                           lsdg_track_stats* stats);

/* ------------------------------------------------------------------------------------------ */
/* Sim3 direct alignment of two keyframes (constraint search)                                   */
/* ------------------------------------------------------------------------------------------ */

/* A Sim3 pose is 13 doubles {R (9, row-major), t (3), s}: x_b = s R x_a + t. */

/* One Sim3 residual pass at a fixed pose (both frames need depth).  out[LSDG_NE_SIZE_SIM3] =
 *   [0..27] upper triangle of sum w J^T J (7x7), [28..34] sum w J^T r, [35] energy, [36] points
 *   used, [37] inliers, [38] outliers, [39] points that left the image.  J is d r / d xi for the
 *   left increment exp(xi) * ref_to_frame, xi = (v, omega, log-scale); each point contributes its
 *   photometric residual and, where frame's depth map has the four bilinear corners, the
 *   inverse-depth residual 1/z' - D_frame(u'). */
LSDG_API lsdg_status lsdg_sim3_normal_equations(lsdg_ctx* ctx, const lsdg_frame* reference, const lsdg_frame* frame,
                                                int level, const double ref_to_frame[13],
                                                double out[LSDG_NE_SIZE_SIM3]);

/* Sim3Tracker::trackFrameSim3: align keyframe `frame` (with depth) to keyframe `reference`,
 * 7 parameters, the same LM rules as lsdg_track_se3 with a 7x7 FP64 solve. */
LSDG_API lsdg_status lsdg_track_sim3(lsdg_ctx* ctx, const lsdg_frame* reference, const lsdg_frame* frame,
                                     const double frame_to_ref_init[13], double frame_to_ref_out[13],
                                     lsdg_track_stats* stats);

/* ------------------------------------------------------------------------------------------ */
/* Batched alignment: many independent pairs of mixed size, one persistent launch              */
/* ------------------------------------------------------------------------------------------ */

/* Create a batch of n pairs; pair i has size widths[i] x heights[i] and intrinsics intr[i]. */
LSDG_API lsdg_status lsdg_batch_create(lsdg_ctx* ctx, int n, const int* widths, const int* heights,
                              const lsdg_intrinsics* intr, lsdg_batch** out);
LSDG_API lsdg_status lsdg_batch_destroy(lsdg_ctx* ctx, lsdg_batch* batch);
/* Host -> device copies (asynchronous on the context stream; the host arrays must stay valid
 * until the next lsdg_sync / lsdg_batch_read).  Each array holds the pairs' planes back to back
 * in pair order (pair i: widths[i] * heights[i] floats).  init is 12 doubles per pair. */
LSDG_API lsdg_status lsdg_batch_load(lsdg_ctx* ctx, lsdg_batch* batch, const float* ref_images,
                            const float* ref_idepth, const float* ref_idepth_var,
                            const float* new_images, const double* frame_to_ref_init);
/* Device-only step on the loaded inputs: both pyramids of every pair, the reference points and
 * the persistent LM tracker over all pairs and levels.  Asynchronous; replayed from a CUDA graph
 * after the first call. */
LSDG_API lsdg_status lsdg_batch_run(lsdg_ctx* ctx, lsdg_batch* batch);
/* Device -> host results (synchronises the context stream).  LSDG_TIMEOUT: the step's keyframe
 * build ran out of one of its bounded waits (the poses of that step are not to be used; the
 * context stays usable). */
LSDG_API lsdg_status lsdg_batch_read(lsdg_ctx* ctx, lsdg_batch* batch, double* frame_to_ref_out,
                            lsdg_track_stats* stats);
/* Pipelined form: lsdg_batch_submit_* enqueues one step (the upload of its inputs on the batch's
 * copy stream into whichever of the batch's two input slots the previous step is not using, the
 * step's graph behind the upload, the read-back of its poses and stats behind the graph on a
 * read-back stream) and returns; lsdg_batch_collect waits for the oldest submitted step and copies
 * its results out (LSDG_TIMEOUT as for lsdg_batch_read).  At
 * most two steps are in flight (a third submit fails with LSDG_INVALID_ARG); results come back in
 * submission order.  For the copies to overlap the tracking, the host arrays must be pinned
 * (page-locked) and stay untouched until the step is collected.  The synchronous calls
 * (load / run / read / track) refuse while steps are in flight. */
LSDG_API lsdg_status lsdg_batch_submit_se3(lsdg_ctx* ctx, lsdg_batch* batch, const float* ref_images,
                                           const float* ref_idepth, const float* ref_idepth_var,
                                           const float* new_images, const double* frame_to_ref_init);
/* Same as lsdg_batch_submit_se3 with 8-bit images (row-major w x h bytes per frame, the camera's
 * own format: upstream frames are built from 8-bit images and their level-0 float plane is the
 * byte value, so results are identical to submitting the images as floats).  The bytes cross the
 * bus, the conversion to float runs on the device behind the copy. */
LSDG_API lsdg_status lsdg_batch_submit_se3_u8(lsdg_ctx* ctx, lsdg_batch* batch, const uint8_t* ref_images,
                                              const float* ref_idepth, const float* ref_idepth_var,
                                              const uint8_t* new_images, const double* frame_to_ref_init);
LSDG_API lsdg_status lsdg_batch_submit_sim3(lsdg_ctx* ctx, lsdg_batch* batch, const float* ref_images,
                                            const float* ref_idepth, const float* ref_idepth_var,
                                            const float* new_images, const float* new_idepth,
                                            const float* new_idepth_var, const double* frame_to_ref_init);
LSDG_API lsdg_status lsdg_batch_collect(lsdg_ctx* ctx, lsdg_batch* batch, double* frame_to_ref_out,
                                        lsdg_track_stats* stats);
/* Fill the batch from frames already on the device (device-to-device copies of their level-0
 * planes): pair i tracks frames[i] against refs[i] (refs need depth; frames too for a Sim3 batch),
 * sizes as the batch was created with.  The constraint search's candidates are resident keyframes,
 * so nothing crosses the host bus but the initial poses.  Then lsdg_batch_run / lsdg_batch_read. */
LSDG_API lsdg_status lsdg_batch_load_frames(lsdg_ctx* ctx, lsdg_batch* batch, const lsdg_frame* const* refs,
                                            const lsdg_frame* const* frames, const double* frame_to_ref_init);
/* A batch of Sim3 constraint trackings (a new keyframe against its candidates): both keyframes of
 * every pair carry depth; poses are 13 doubles.  lsdg_batch_run and lsdg_batch_read work on it as on
 * an SE3 batch. */
LSDG_API lsdg_status lsdg_batch_create_sim3(lsdg_ctx* ctx, int n, const int* widths, const int* heights,
                                            const lsdg_intrinsics* intr, lsdg_batch** out);
LSDG_API lsdg_status lsdg_batch_load_sim3(lsdg_ctx* ctx, lsdg_batch* batch, const float* ref_images,
                                          const float* ref_idepth, const float* ref_idepth_var,
                                          const float* new_images, const float* new_idepth,
                                          const float* new_idepth_var, const double* frame_to_ref_init);
LSDG_API lsdg_status lsdg_batch_track_sim3(lsdg_ctx* ctx, lsdg_batch* batch, const float* ref_images,
                                           const float* ref_idepth, const float* ref_idepth_var,
                                           const float* new_images, const float* new_idepth,
                                           const float* new_idepth_var, const double* frame_to_ref_init,
                                           double* frame_to_ref_out, lsdg_track_stats* stats);
/* load + run + read. */
LSDG_API lsdg_status lsdg_batch_track_se3(lsdg_ctx* ctx, lsdg_batch* batch, const float* ref_images,
                                 const float* ref_idepth, const float* ref_idepth_var,
                                 const float* new_images, const double* frame_to_ref_init,
                                 double* frame_to_ref_out, lsdg_track_stats* stats);
/* Device time of the last run's two phases (pyramids + points; the persistent tracker), read from
 * CUDA events the captured graph records on the context stream.  Synchronises. */
LSDG_API lsdg_status lsdg_batch_timing(lsdg_ctx* ctx, lsdg_batch* batch, float* build_ms, float* track_ms);
/* The launch shape the autotuner picked for this batch (threads per CTA, CTAs per cluster, clusters
 * in the persistent grid) and the kernel launches one lsdg_batch_run issues. */
LSDG_API lsdg_status lsdg_batch_shape(lsdg_ctx* ctx, lsdg_batch* batch, int* threads, int* minblocks, int* cluster,
                                      int* clusters, int* launches_per_run);
/* The coarse phase of the batch's plan: levels [top, split] run first with each pair on a cluster of
 * `cluster` CTAs of `threads`, then the finer levels with the shape lsdg_batch_shape reports
 * (split = -1: a single launch over all levels). */
LSDG_API lsdg_status lsdg_batch_split(lsdg_ctx* ctx, lsdg_batch* batch, int* split, int* threads, int* minblocks,
                                      int* cluster);
/* TEST HOOK -- not part of the tracking API; the library's own tests call it, applications never
 * should.  It exercises the batch build's bounded wait: in the following steps band 0 of keyframe
 * `frame` publishes no point counts, so the other bands of that keyframe wait until their limit and
 * the step reports LSDG_TIMEOUT from lsdg_batch_read / _collect (the context stays usable; -1 turns
 * it off).  The step's graph is captured again and the tile shape is tuned again at the next run. */
LSDG_API lsdg_status lsdg_batch_test_withhold(lsdg_ctx* ctx, lsdg_batch* batch, int frame);
/* Read back the tracking reference points the batch's last step built for pair `pair`'s keyframe at
 * one level (the layout of lsdg_frame_get_points; synchronises the context stream). */
LSDG_API lsdg_status lsdg_batch_get_points(lsdg_ctx* ctx, lsdg_batch* batch, int pair, int level, float* xyzi,
                                           float* var, int capacity, int* count);
/* Residual passes the last lsdg_batch_run executed, summed over pairs and levels, and the
 * algorithmic bytes those passes read (points + frame levels + sums). */
LSDG_API lsdg_status lsdg_batch_work(lsdg_ctx* ctx, lsdg_batch* batch, int64_t* passes,
                            double* pass_bytes, double* unique_bytes);

/* ------------------------------------------------------------------------------------------ */
/* Semi-dense inverse-depth filter (upstream DepthMap)                                         */
/* ------------------------------------------------------------------------------------------ */

#define LSDG_MAX_REFS 16

/* A keyframe depth map: the keyframe image (level 0 with gradients) and the per-pixel state
 * {idepth, var, idepth_smoothed, var_smoothed, validity, blacklist} in HBM. */
LSDG_API lsdg_status lsdg_depth_create(lsdg_ctx* ctx, int width, int height, const lsdg_intrinsics* intr,
                                       lsdg_depthmap** out);
LSDG_API lsdg_status lsdg_depth_destroy(lsdg_ctx* ctx, lsdg_depthmap* dm);
/* Keyframe image and initial hypotheses (idepth <= 0 or var <= 0: none; others start with
 * validity = params.validity_init). */
LSDG_API lsdg_status lsdg_depth_set_keyframe(lsdg_ctx* ctx, lsdg_depthmap* dm, const float* image,
                                             const float* idepth, const float* idepth_var);
/* Upload n_refs (<= LSDG_MAX_REFS) reference images, back to back (asynchronous). */
LSDG_API lsdg_status lsdg_depth_load_refs(lsdg_ctx* ctx, lsdg_depthmap* dm, int n_refs, const float* ref_images);
/* DepthMap::updateKeyframe on the loaded references: observeDepth of every pixel against
 * references 0..n_refs-1 in order (epipolar search + fusion), then, if regularize != 0,
 * regularizeDepthMap.  key_to_ref: 12 doubles per reference.  Asynchronous. */
LSDG_API lsdg_status lsdg_depth_update_loaded(lsdg_ctx* ctx, lsdg_depthmap* dm, int n_refs,
                                              const double* key_to_ref, int regularize);
/* load_refs + update_loaded, synchronous. */
LSDG_API lsdg_status lsdg_depth_update(lsdg_ctx* ctx, lsdg_depthmap* dm, int n_refs, const float* ref_images,
                                       const double* key_to_ref, int regularize);
/* The same with 8-bit reference frames (the InputThread's format, lib/App/InputThread.cpp:59-62):
 * n_refs * w * h bytes, converted to intensity planes on the device. */
LSDG_API lsdg_status lsdg_depth_update_u8(lsdg_ctx* ctx, lsdg_depthmap* dm, int n_refs, const uint8_t* ref_images,
                                          const double* key_to_ref, int regularize);
/* regularizeDepthMap (+ hole filling and removal of unsupported hypotheses), synchronous. */
LSDG_API lsdg_status lsdg_depth_regularize(lsdg_ctx* ctx, lsdg_depthmap* dm);
/* DepthMap::createKeyFrame: propagateDepth of every hypothesis into the new keyframe (nearest
 * hypothesis wins a pixel), which then becomes this depth map's keyframe; regularize != 0 runs
 * regularizeDepthMap on it.  Synchronous. */
LSDG_API lsdg_status lsdg_depth_create_keyframe(lsdg_ctx* ctx, lsdg_depthmap* dm, const float* new_image,
                                                const double key_to_new[12], int regularize);
/* propagateDepth for callers that cannot allocate device memory when a keyframe changes: an
 * application that reserves all GPU memory at start-up and forbids allocation in its real-time
 * mapping thread, one that records the mapping step inside its own stream capture (allocation
 * cannot be captured), or one that cannot accept the device-wide synchronisation an allocation may
 * imply.  No counterpart in the reference: upstream DepthMap allocates its own buffers.
 *
 * Same computation as lsdg_depth_create_keyframe's propagation (without regularisation), but no
 * context and no allocation: inputs and outputs are the caller's device buffers (width * height
 * elements each, row-major), the work is enqueued on the caller's `stream` (cudaStream_t; NULL = the
 * legacy default stream) and the call returns without synchronising.  old_* is the old keyframe's raw
 * state (idepth, var, validity), new_* receive the new keyframe's state.  The current device of the
 * calling thread must own `stream` and the buffers.
 *
 * The only scratch, a 64-bit z-buffer of one entry per pixel, is a device array inside the library
 * that every GPU which loads the library holds until the process exits: at most 1280 x 960 =
 * 1,228,800 pixels (9.8 MB); larger sizes return LSDG_INVALID_ARG.  The first call on a device looks
 * up that array's device address (cudaGetSymbolAddress), so make the first call on each device before
 * any stream capture.  The looked-up address is kept per device number for the life of the
 * process: it belongs to the device's primary context (the one the CUDA runtime uses), so do not call
 * this from another context on the same device, nor after cudaDeviceReset.  All calls share the
 * array: calls that overlap on the GPU (different streams, or different host threads, on one device)
 * race on it -- serialise them.  Errors are reported by the return value only (there is no context
 * for lsdg_last_error); a CUDA error already pending on the calling thread when the call starts is
 * left in place and the call returns LSDG_CUDA_ERROR without enqueuing anything. */
LSDG_API lsdg_status lsdg_depth_propagate_noalloc(void* stream, int width, int height, const lsdg_intrinsics* intr,
                                                  const lsdg_params* params, const double old_to_new[12],
                                                  const float* old_image, const float* new_image,
                                                  const float* old_idepth, const float* old_var,
                                                  const int32_t* old_validity, float* new_idepth, float* new_var,
                                                  float* new_idepth_smoothed, float* new_var_smoothed,
                                                  int32_t* new_validity, int32_t* new_blacklist);

/* Read the state (any pointer may be NULL).  idepth / idepth_smoothed <= 0 means no depth
 * (the layout Frame::idepth(0) / idepthVar(0) hands to the viewer). */
LSDG_API lsdg_status lsdg_depth_get(lsdg_ctx* ctx, lsdg_depthmap* dm, float* idepth, float* idepth_var,
                                    float* idepth_smoothed, float* var_smoothed, int32_t* validity,
                                    int32_t* blacklist);

/* ------------------------------------------------------------------------------------------ */
/* Differentiable photometric energy (forward / adjoint) and inverse-depth refinement          */
/* ------------------------------------------------------------------------------------------ */

/* The energy of a keyframe level's points against a frame, as a function of the pose and of every
 * point's inverse depth rho_i (no upstream counterpart; the residual model is the tracker's):
 *   p_i = q_i / rho_i (q_i = ((x - cx)/fx, (y - cy)/fy, 1) from the point's pixel), p'_i = M p_i + t,
 *   r_i = I_frame(pi(p'_i)) - I_keyframe(x_i, y_i)   (Catmull-Rom sampling of the frame level),
 *   E   = sum_i h(r_i^2 / s_i),  h(e2) = e2 if sqrt(e2) <= huber_delta else delta (2 sqrt(e2) - delta),
 * s_i = photometric_variance or a per-point value (lsdg_energy_set_sigma2).  A point takes part when
 * z' > min_z and its projection lies inside border_margin.  The pose is [M | t] (ref_to_frame, M = R,
 * or sR for dof 7) perturbed by a left increment exp(xi): the gradient with respect to xi at 0 is
 * 2 x the sum w J^T r of lsdg_se3_normal_equations (same points, same weights).
 *
 * The object follows the contract of an autograd Function: lsdg_energy_forward computes E and saves
 * what the backward needs (frame, pose, dof, the inverse depths' version); lsdg_energy_backward
 * takes dL/dE and returns dL/dxi and dL/drho, recomputing every residual instead of storing it.
 * Changing the inverse depths after the forward makes the backward fail (LSDG_INVALID_ARG), as a
 * modified saved tensor does.
 *
 * The energy binds the keyframe's point set of `level` at creation (a copy: later set_depth calls
 * on the keyframe do not change it); its points are those of lsdg_frame_get_points, in order. */
LSDG_API lsdg_status lsdg_energy_create(lsdg_ctx* ctx, const lsdg_frame* keyframe, int level, lsdg_energy** out);
LSDG_API lsdg_status lsdg_energy_destroy(lsdg_ctx* ctx, lsdg_energy* e);
/* Number of points (the length of every per-point array below). */
LSDG_API lsdg_status lsdg_energy_size(lsdg_ctx* ctx, const lsdg_energy* e, int* n_points);
/* Pixel index (row-major, in the level) of every point. */
LSDG_API lsdg_status lsdg_energy_pixels(lsdg_ctx* ctx, const lsdg_energy* e, int32_t* pixels);
/* Host copies of the points' inverse depths (NULL restores the keyframe's). */
LSDG_API lsdg_status lsdg_energy_set_idepth(lsdg_ctx* ctx, lsdg_energy* e, const float* idepth);
LSDG_API lsdg_status lsdg_energy_get_idepth(lsdg_ctx* ctx, const lsdg_energy* e, float* idepth);
/* Per-point residual variance s_i (NULL: photometric_variance for every point). */
LSDG_API lsdg_status lsdg_energy_set_sigma2(lsdg_ctx* ctx, lsdg_energy* e, const float* sigma2);
/* E at ref_to_frame (12 doubles) with dof 6 (SE3) or 7 (Sim3, M = sR); n_active: points taking part. */
LSDG_API lsdg_status lsdg_energy_forward(lsdg_ctx* ctx, lsdg_energy* e, const lsdg_frame* frame,
                                         const double ref_to_frame[12], int dof, double* energy, int* n_active);
/* Adjoint of the last forward: grad_xi[dof] = grad_energy * dE/dxi, grad_idepth[i] (host, may be
 * NULL) = grad_energy * dE/drho_i (0 for points that do not take part). */
LSDG_API lsdg_status lsdg_energy_backward(lsdg_ctx* ctx, lsdg_energy* e, double grad_energy, double* grad_xi,
                                          float* grad_idepth);
/* Photometric inverse-depth refinement over n_frames frames at fixed poses (ref_to_frame, 12 doubles
 * each, n_frames <= LSDG_MAX_REFS): every point independently runs `steps` damped Newton steps of its
 * energy sum_j h(r_ij^2 / s_i) + refine_prior_weight (rho - rho0)^2 / var_i (rho0: its inverse depth
 * at the call, var_i: the keyframe's variance), with the frames it is seen in fixed by the margin test
 * at rho0, a trial that leaves a frame's sampling box rejected, rho clamped to
 * [min_idepth, max_idepth] and the tracker's lambda schedule.  Every step recomputes the point's
 * residuals in all frames; nothing is stored per residual.  The refined inverse depths replace the
 * energy's (lsdg_energy_get_idepth); energy_before / energy_after: the summed point energies. */
LSDG_API lsdg_status lsdg_energy_refine(lsdg_ctx* ctx, lsdg_energy* e, int n_frames, const lsdg_frame* const* frames,
                                        const double* ref_to_frames, int steps, double* energy_before,
                                        double* energy_after, int* n_refined);
/* Device time (ms) of the last forward, backward and refine kernels, from CUDA events. */
LSDG_API lsdg_status lsdg_energy_timing(lsdg_ctx* ctx, const lsdg_energy* e, float* forward_ms, float* backward_ms,
                                        float* refine_ms);

/* ------------------------------------------------------------------------------------------ */
/* Input step: raw 8-bit frame -> undistorted frame (InputThread, lib/App/InputThread.cpp:59-71)  */
/* ------------------------------------------------------------------------------------------ */

/* Parses a calibration file with <calibration> tags (<projection>, <width>, <height>, <f>, <cx>,
 * <cy>, <b1>, <b2>, <k1>..<k4>, <p1>, <p2>; absent coefficients are 0).  Host only, no GPU. */
LSDG_API lsdg_status lsdg_calibration_load_xml(const char* path, lsdg_calibration* out);

/* An undistorter from `calib` to an ideal pinhole camera of out_w x out_h with intrinsics out_K
 * (NULL: the calibration's size, fx = fy = f, principal point w/2 + cx - 0.5, h/2 + cy - 0.5 in
 * pixel-centre coordinates).  The remap table (source position of every output pixel) is computed
 * once on the device in FP64 and kept as float pairs. */
LSDG_API lsdg_status lsdg_undistorter_create(lsdg_ctx* ctx, const lsdg_calibration* calib, int out_w, int out_h,
                                             const lsdg_intrinsics* out_K, lsdg_undistorter** out);
LSDG_API lsdg_status lsdg_undistorter_destroy(lsdg_ctx* ctx, lsdg_undistorter* u);
/* The output camera (what undistorter->getCamera() / outputImageSize() give the SLAM system). */
LSDG_API lsdg_status lsdg_undistorter_camera(lsdg_ctx* ctx, const lsdg_undistorter* u, int* out_w, int* out_h,
                                             lsdg_intrinsics* out_K);
/* Uploads a raw 8-bit frame (calib width x height), undistorts it on the device (bilinear, rounded to
 * 8 bits like the undistorted CV_8UC1 image the input thread hands over; outside the raw image: 0)
 * into `frame` (out_w x out_h, created with the output camera) and builds its pyramid. */
LSDG_API lsdg_status lsdg_frame_upload_distorted_u8(lsdg_ctx* ctx, lsdg_undistorter* u, lsdg_frame* frame,
                                                    const uint8_t* raw);
/* The undistorted 8-bit image of the last upload (host, out_w x out_h), for the GUI's live view. */
LSDG_API lsdg_status lsdg_undistorter_last_image(lsdg_ctx* ctx, const lsdg_undistorter* u, uint8_t* out);

/* ------------------------------------------------------------------------------------------ */
/* Keyframe point cloud (the viewer's data path, headless)                                      */
/* ------------------------------------------------------------------------------------------ */

LSDG_API void lsdg_cloud_default_params(lsdg_cloud_params* p);

/* PangolinOutputIOWrapper::publishKeyframe's per-pixel copy
 * (lib/Pangolin_IOWrapper/PangolinOutputIOWrapper.cpp:79-89) of the depth map's keyframe:
 * {idepth, idepth_var} = the smoothed state (what Frame::idepth(0) / idepthVar(0) hold), every colour
 * byte = the keyframe intensity converted to uint8 (truncated; values outside [0, 255] saturate).
 * out: host array of w * h. */
LSDG_API lsdg_status lsdg_depth_export_points(lsdg_ctx* ctx, lsdg_depthmap* dm, lsdg_input_point_dense* out);

/* Keyframe::computeVbo (lib/Pangolin_IOWrapper/Keyframe.h:66-143) without OpenGL: the points of a
 * w x h InputPointDense array (host) that pass the variance and neighbour-support filter,
 * back-projected with (fx, fy, cx, cy) and the keyframe's Sim3 scale, in row-major order into `out`
 * (host, capacity w * h vertices); *count = the number of vertices (Keyframe::points).  An array
 * with fewer than 3 rows or columns has no interior pixel: *count = 0, as computeVbo's loop keeps
 * nothing. */
LSDG_API lsdg_status lsdg_cloud_build(lsdg_ctx* ctx, int w, int h, float fx, float fy, float cx, float cy,
                                      float scale, const lsdg_cloud_params* params,
                                      const lsdg_input_point_dense* points, lsdg_cloud_vertex* out,
                                      int* count);

/* The same from the depth map's keyframe straight into a caller-owned DEVICE buffer (the VBO the
 * GL viewer would upload, kept on the GPU): export + filter + back-projection on the device, only the
 * count comes back.  out_device: capacity w * h vertices. */
LSDG_API lsdg_status lsdg_cloud_from_depthmap(lsdg_ctx* ctx, lsdg_depthmap* dm, float scale,
                                              const lsdg_cloud_params* params, lsdg_cloud_vertex* out_device,
                                              int* count);

/* ------------------------------------------------------------------------------------------ */
/* Pose wire formats (host only, no GPU)                                                        */
/* ------------------------------------------------------------------------------------------ */

/* GraphFramePose (lib/Pangolin_IOWrapper/Keyframe.h:23-27): a keyframe id and the 7 floats that
 * publishKeyframeGraph memcpys out of Sophus::Sim3f::data() (PangolinOutputIOWrapper.cpp:161):
 * the RxSO3 quaternion (x, y, z, w), whose squared norm is the scale, then the translation. */
typedef struct lsdg_graph_frame_pose {
  int32_t id;
  float cam_to_world[7];
} lsdg_graph_frame_pose;

/* 13-double Sim3 {R, t, s} <-> the 7-float Sophus layout above. */
LSDG_API void lsdg_sim3_to_sophus7(const double pose13[13], float out7[7]);
LSDG_API void lsdg_sophus7_to_sim3(const float in7[7], double pose13[13]);
/* One line of TextOutputIOWrapper's pose file (lib/Pangolin_IOWrapper/TextOutputIOWrapper.cpp:104-117):
 * "id,x,y,z,px,py,pz\n" with the camera-to-world translation and the translation of the frame's
 * pose relative to its parent, each value as a default C++ stream prints it (6 significant digits).
 * Returns the number of characters written (excluding the terminating 0), or -1 if `len` is short. */
LSDG_API int lsdg_format_pose_row(int id, const double cam_to_world13[13], const double this_to_parent13[13],
                                  char* buf, int len);

/* ------------------------------------------------------------------------------------------ */
/* The full SLAM loop (upstream SlamSystem; host C++ over the calls above)                      */
/* ------------------------------------------------------------------------------------------ */

/* Upstream's SlamSystem is fed by InputThread (lib/App/InputThread.cpp:71
 * `system->nextImage(runningIdx, imageUndist, camera)`), finalised at the end (tools/LSD.cpp:139)
 * and publishes a keyframe graph (PangolinOutputIOWrapper::publishKeyframeGraph,
 * lib/Pangolin_IOWrapper/PangolinOutputIOWrapper.cpp:148-168) and per-frame poses
 * (TextOutputIOWrapper::publishTrackedFrame, lib/Pangolin_IOWrapper/TextOutputIOWrapper.cpp:100-120).
 * lsdg_slam is that loop: tracking and mapping on the caller's thread in lsdg_slam_next_image
 * (trackFrame against the current keyframe, updateKeyframe, keyframe creation by createKeyFrame);
 * Sim3 constraint search of each new keyframe against its predecessor and nearby keyframes (batched,
 * optionally in both directions) and the Sim3 pose-graph optimisation on a worker thread with its
 * own context.  Its policy constants are this project's own (upstream's are not available). */
typedef struct lsdg_slam lsdg_slam;
typedef struct lsdg_slam_params {
  float kf_dist;            /* a new keyframe after this much travel from the current one (m)      */
  float kf_angle_deg;       /* ... or this much rotation (degrees)                                 */
  float kf_min_usage;       /* ... or when fewer of the keyframe's points than this stay in view    */
  int32_t refresh_every;    /* tracking reference refreshed from the depth filter every N frames   */
  int32_t n_candidates;     /* Sim3 constraint candidates per new keyframe (predecessor included)  */
  float cand_radius;        /* candidates: earlier keyframes whose centres lie within this (m)     */
  int32_t optimize_every;   /* pose-graph optimisation after this many keyframes with a loop edge  */
  int32_t final_iterations; /* Gauss-Newton iterations of lsdg_slam_finalize                      */
  float max_track_jump;     /* a tracked pose this far from the constant-velocity guess is lost (m) */
  int32_t both_directions;  /* track every constraint both ways and keep it only when they agree  */
  float consistency_trans;  /* ... translation of Z_ab Z_ba below this fraction of |t_ab|         */
  float consistency_rot;    /* ... rotation below this (rad)                                      */
  float consistency_scale;  /* ... |log scale| below this                                         */
  int32_t async_constraints; /* constraint search on the worker thread (1) or inline (0)          */
  int32_t graph_threads;    /* host threads of the pose graph's Cholesky                           */
  float odometry_scale_weight; /* scale information of a keyframe-to-keyframe odometry edge, as a
                                  fraction of its strongest SE3 direction                          */
  int32_t ref_min_validity; /* tracking reference: only depth whose validity count reaches this    */
  float sim3_info_scale;    /* information of a Sim3 constraint = the tracker's J^T W J times this */
  float ref_max_var;        /* tracking reference: only depth whose variance is below this (0 = all) */
  float epipolar_var;       /* sigma_l^2 of the loop's depth filter (px^2), replacing
                               lsdg_params.epipolar_var (0 = keep it): in the loop the epipolar line
                               comes from a tracked pose, whose error moves the line by more than the
                               exact poses lsdg_params' default assumes */
  int32_t reactivate;       /* before making a keyframe, track the frame against the earlier
                               keyframes near the camera (SlamSystem's re-positioning); one that
                               tracks it well becomes the current keyframe again (its depth map is
                               refined further) and the keyframe left is tied to it in the graph */
  float react_radius;       /* ... candidates: camera centres within this of the camera (m)        */
  float react_angle_deg;    /* ... and viewing directions within this angle (degrees)              */
  float react_min_usage;    /* ... accepted when at least this share of its points stay in view    */
  float react_max_jump;     /* ... and the tracked pose is this close to the graph's prediction (m) */
  int32_t react_min_age;    /* ... candidates: keyframes made at least this many keyframes ago     */
  float react_min_good;     /* ... accepted when at least this share of the points in view are
                               inliers, and when the frame lies within half of kf_dist and of
                               kf_angle_deg of the keyframe (so that it is not left at once)      */
  int32_t retrack_iterations; /* when the current keyframe is left: this many rounds of re-tracking
                                 the frames mapped into it against its refined depth and mapping
                                 them again from its starting depth with the new poses (0 = off) */
  int32_t reserved[1];
} lsdg_slam_params;

typedef struct lsdg_slam_stats {
  int32_t frames, keyframes, lost_frames, sim3_edges, sim3_rejected, graph_optimisations;
  int32_t reactivations;    /* keyframes made current again instead of a new keyframe */
  int32_t reserved[5];
} lsdg_slam_stats;

LSDG_API void lsdg_slam_default_params(lsdg_slam_params* p);
/* A system for width x height 8-bit frames of camera `intr` on `device` (two contexts, a depth map). */
LSDG_API lsdg_status lsdg_slam_create(const lsdg_params* params, const lsdg_slam_params* sp, int device,
                                      int width, int height, const lsdg_intrinsics* intr, lsdg_slam** out);
LSDG_API lsdg_status lsdg_slam_destroy(lsdg_slam* s);
LSDG_API const char* lsdg_slam_last_error(const lsdg_slam* s);
/* The first keyframe, with a known inverse depth and variance (idepth <= 0 = none). */
LSDG_API lsdg_status lsdg_slam_bootstrap(lsdg_slam* s, int id, const uint8_t* image, const float* idepth,
                                         const float* var);
/* SlamSystem::nextImage: track, map, and possibly make a keyframe (which starts its constraint
 * search).  A frame that fails to track keeps the constant-velocity guess and is counted lost. */
LSDG_API lsdg_status lsdg_slam_next_image(lsdg_slam* s, int id, const uint8_t* image);
/* SlamSystem::finalize: waits for the constraint search and optimises the pose graph. */
LSDG_API lsdg_status lsdg_slam_finalize(lsdg_slam* s);
LSDG_API lsdg_status lsdg_slam_get_stats(const lsdg_slam* s, lsdg_slam_stats* out);
/* Camera-to-world Sim3 {R, t, s} (13 doubles) of every frame so far (keyframe pose from the graph
 * times the frame's tracked pose); cam_to_world = NULL returns the count in n. */
LSDG_API lsdg_status lsdg_slam_get_poses(lsdg_slam* s, double* cam_to_world, int capacity, int* n);
/* The keyframe graph as publishKeyframeGraph hands it out (GraphFramePose: id + Sophus 7 floats). */
LSDG_API lsdg_status lsdg_slam_keyframe_graph(lsdg_slam* s, lsdg_graph_frame_pose* out, int capacity, int* n);
/* Keyframe k's level-0 tracking depth (inverse depth and variance, width x height, idepth <= 0 =
 * none) and the id of the frame it was made from: what publishKeyframe hands the viewer
 * (PangolinOutputIOWrapper.cpp:77-89).  The current keyframe's is its latest refresh. */
LSDG_API lsdg_status lsdg_slam_keyframe_depth(lsdg_slam* s, int k, int* frame_id, float* idepth, float* var);
/* One TextOutputIOWrapper pose row per frame (lsdg_format_pose_row) into a file. */
LSDG_API lsdg_status lsdg_slam_write_pose_file(lsdg_slam* s, const char* path);

/* The Sim3 pose graph alone (host only): nodes are camera-to-world Sim3 poses, an edge (i, j, Z, W)
 * says "pose j seen from pose i is Z" with 7x7 information W (twist order v, omega, log-scale; row
 * major); cost sum rho(r^T W r), r = log(Z^-1 T_i^-1 T_j), Huber kernel at 3 sigma; node 0 held. */
typedef struct lsdg_posegraph lsdg_posegraph;
LSDG_API lsdg_status lsdg_posegraph_create(lsdg_posegraph** out);
LSDG_API lsdg_status lsdg_posegraph_destroy(lsdg_posegraph* g);
LSDG_API int lsdg_posegraph_add_node(lsdg_posegraph* g, const double cam_to_world13[13]);
LSDG_API lsdg_status lsdg_posegraph_add_edge(lsdg_posegraph* g, int i, int j, const double z13[13],
                                             const double info[49]);
LSDG_API lsdg_status lsdg_posegraph_optimize(lsdg_posegraph* g, int iterations, double* cost);
LSDG_API lsdg_status lsdg_posegraph_get_pose(const lsdg_posegraph* g, int i, double cam_to_world13[13]);
/* exp / log of sim(3) twists (v, omega, log-scale) <-> 13-double poses. */
LSDG_API void lsdg_sim3_exp13(const double xi[7], double out13[13]);
LSDG_API void lsdg_sim3_log13(const double pose13[13], double xi[7]);

/* ------------------------------------------------------------------------------------------ */
/* Measurement                                                                                 */
/* ------------------------------------------------------------------------------------------ */

/* L2 read bandwidth of an L2-resident working set on the context's GPU (GB/s): a persistent grid
 * re-reads a `bytes` buffer `reps` times with L2-only loads (no counterpart in the reference; the
 * denominator of the L2-side roofline of the tracker, whose re-reads across passes L2 serves).
 * Allocates and frees its buffer; synchronises the context stream. */
LSDG_API lsdg_status lsdg_measure_l2_read(lsdg_ctx* ctx, long bytes, int reps, double* gbps);

/* ------------------------------------------------------------------------------------------ */
/* Autotuner                                                                                   */
/* ------------------------------------------------------------------------------------------ */

/* Entry `index` of the context's tile-shape cache: workload key, threads per CTA, CTAs per SM the
 * register budget allows for, CTAs per cluster, clusters resident at once, and the tracker time
 * that won.  LSDG_INVALID_ARG past the end.  The environment variable
 * LSDG_TRACK_SHAPE="threads,cluster[,minblocks]" pins the shape instead of timing candidates. */
LSDG_API lsdg_status lsdg_tune_info(lsdg_ctx* ctx, int index, char* key, int key_len, int* threads, int* minblocks,
                                    int* cluster, int* max_clusters, float* ms);

#ifdef __cplusplus
}
#endif

#endif /* LSDG_H_ */
