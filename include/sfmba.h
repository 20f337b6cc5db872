/*
 * sfmba.h - C ABI of the GB300 bundle adjuster (libsfmba_gb300.so).
 *
 * This is the drop-in boundary for the `sfm-ba` crate of sfmtory. Each entry
 * point names the Rust item it replaces (paths are inside the sfmtory
 * project). All arrays are plain caller-owned buffers in structure-of-arrays
 * form; no entry point takes ownership of anything and none aborts: every
 * call returns an `sfmba_status` and `sfmba_last_error()` gives the message
 * of the last failure on the calling thread.
 *
 * Differences in shape from the Rust API, all mechanical:
 *   - `Vec<CameraModel>` becomes a model id per camera plus a padded
 *     [num_cameras][8] parameter table in `CameraModel::params()` order.
 *   - `Pose` is 7 doubles: Hamilton quaternion (qw, qx, qy, qz) then t.
 *   - `Vec<bool>` masks become uint8 arrays of full length, or NULL for
 *     "all false" (the Rust code reads missing entries as false).
 *   - `fixed_camera_params: Vec<Vec<bool>>` becomes a padded
 *     [num_cameras][8] uint8 table (entries past a camera's parameter count,
 *     or past the inner Vec's length, are 0).
 *   - `BaOutput` is written into caller buffers named in `sfmba_result`.
 */
#ifndef SFMBA_H
#define SFMBA_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SFMBA_MAX_CAMERA_PARAMS 8
#define SFMBA_POSE_STRIDE 7

/* COLMAP model ids, crates/sfm-core/src/camera.rs:74-83 (`model_id`). */
typedef enum sfmba_camera_model {
    SFMBA_SIMPLE_PINHOLE = 0, /* f, cx, cy                         */
    SFMBA_PINHOLE = 1,        /* fx, fy, cx, cy                    */
    SFMBA_SIMPLE_RADIAL = 2,  /* f, cx, cy, k                      */
    SFMBA_RADIAL = 3,         /* f, cx, cy, k1, k2                 */
    SFMBA_OPENCV = 4,         /* fx, fy, cx, cy, k1, k2, p1, p2    */
    SFMBA_OPENCV_FISHEYE = 5  /* fx, fy, cx, cy, k1, k2, k3, k4    */
} sfmba_camera_model;

/* crates/sfm-ba/src/lib.rs:213-218 (`RobustLoss`). */
typedef enum sfmba_robust_loss {
    SFMBA_LOSS_NONE = 0,
    SFMBA_LOSS_HUBER = 1,
    SFMBA_LOSS_CAUCHY = 2
} sfmba_robust_loss;

/* Arithmetic of the residual/Jacobian/Schur/PCG kernels. The total cost,
 * the step-acceptance test and the dense Cholesky are FP64 in both. */
typedef enum sfmba_precision {
    SFMBA_PRECISION_FP64 = 0,  /* plain all-FP64 path                      */
    SFMBA_PRECISION_MIXED = 1  /* FP32 residual/Jacobian/Schur/PCG kernels  */
} sfmba_precision;

/* How the reduced camera system is solved. */
typedef enum sfmba_solver {
    SFMBA_SOLVER_AUTO = 0,   /* dense Cholesky up to a few thousand unknowns, else PCG */
    SFMBA_SOLVER_DENSE = 1,  /* explicit Schur complement + FP64 blocked Cholesky (LU fallback) */
    SFMBA_SOLVER_PCG = 2     /* matrix-free Schur PCG, block-Jacobi preconditioner */
} sfmba_solver;

typedef enum sfmba_status {
    SFMBA_OK = 0,
    SFMBA_ERR_INVALID_ARGUMENT = 1,
    SFMBA_ERR_CUDA = 2,
    SFMBA_ERR_OUT_OF_MEMORY = 3,
    SFMBA_ERR_NO_DEVICE = 4,
    SFMBA_ERR_UNSUPPORTED = 5,
    SFMBA_ERR_INTERNAL = 6
} sfmba_status;

/* crates/sfm-ba/src/lib.rs:56-96 (`Observation`, `BaInput`). */
typedef struct sfmba_problem {
    int64_t num_images;
    int64_t num_cameras;
    int64_t num_points;
    int64_t num_observations;
    const int32_t *camera_of_image;      /* [num_images]                        */
    const int32_t *camera_model;         /* [num_cameras] sfmba_camera_model    */
    const double *camera_params;         /* [num_cameras][8]                    */
    const double *poses;                 /* [num_images][7] qw qx qy qz tx ty tz */
    const double *points;                /* [num_points][3]                     */
    const int32_t *obs_image;            /* [num_observations]                  */
    const int32_t *obs_point;            /* [num_observations]                  */
    const double *obs_xy;                /* [num_observations][2] pixels        */
    const uint8_t *fixed_poses;          /* [num_images] or NULL                */
    const uint8_t *fixed_cameras;        /* [num_cameras] or NULL               */
    const uint8_t *fixed_camera_params;  /* [num_cameras][8] or NULL            */
} sfmba_problem;

/* crates/sfm-ba/src/lib.rs:220-238 (`BaParams` and its Default), plus the
 * GB300 solver controls. `sfmba_default_options` fills the reference
 * defaults (50 iterations, lambda0 1e-3, Huber at 2 px). */
typedef struct sfmba_options {
    int32_t max_iterations;
    double initial_lambda;
    int32_t robust_loss;          /* sfmba_robust_loss */
    double loss_scale_px;
    int32_t precision;            /* sfmba_precision   */
    int32_t solver;               /* sfmba_solver      */
    int32_t pcg_max_iterations;   /* per damping retry (PCG solver)            */
    double pcg_tolerance;         /* stop PCG at |r| <= tol |b| (default 0.1)  */
    int32_t refinement_steps;     /* FP64 iterative-refinement steps (dense)   */
    double target_cost;           /* > 0: also stop once cost <= target_cost   */
    int32_t dense_max_dim;        /* AUTO picks dense up to this reduced dim   */
    int32_t fp64_polish;          /* mixed path: when the FP32 loop would stop,
                                     continue the same LM loop in FP64 (default 0:
                                     the FP32 path already forms its gradient from
                                     FP64 residuals and stops where FP64 does) */
    int32_t kernel_variant;       /* 0: launch variants of the PCG observation passes
                                     and of the batched Schur reduction picked by the
                                     autotuner; k > 0: force variant k - 1 of each
                                     (point pass min(k, 11), image pass modulo 10,
                                     batched Schur modulo 3; all variants of a
                                     kernel give the same results) */
    int32_t pcg_coarse_clusters;  /* PCG solver: clusters of consecutive images in the
                                     coarse correction of the preconditioner (0: 64,
                                     at most 128; < 0: block-Jacobi alone) */
    int32_t dense_fp64_fma;       /* dense solver and batched windows, mixed path:
                                     0 (default) runs the Cholesky's trailing updates
                                     on the BF16 tensor cores by error-free splitting
                                     (FP64 accuracy); 1 keeps FP64 fused
                                     multiply-adds, as the FP64 path does */
    int32_t reserved[3];
} sfmba_options;

/* crates/sfm-ba/src/lib.rs:240-247 (`BaOutput`). Output buffers are caller
 * owned and may be NULL to skip that copy-out. */
typedef struct sfmba_result {
    double *poses;                /* [num_images][7]  */
    double *points;               /* [num_points][3]  */
    double *camera_params;        /* [num_cameras][8] */
    double initial_cost;
    double final_cost;
    int32_t iterations_run;
    int32_t status;
    int32_t damping_retries;      /* inner retries summed over outer iterations */
    int32_t solver_used;          /* sfmba_solver actually run                 */
    int32_t polish_iteration;     /* outer iteration where the FP64 polish began, -1 if none */
    int32_t reserved_i;
    int64_t linear_iterations;    /* PCG iterations summed over all retries    */
    int64_t reduced_dim;          /* size of the reduced camera system          */
    int64_t valid_observations;   /* observations in front of their camera at the end */
    double seconds;               /* wall time of the call, measured inside     */
    double reserved[4];
} sfmba_result;

/* Reference defaults of BaParams (lib.rs:229-238) and of the GB300 controls. */
void sfmba_default_options(sfmba_options *options);

/* Replaces `pub fn bundle_adjust(input: BaInput, params: &BaParams) -> BaOutput`
 * (crates/sfm-ba/src/lib.rs:747). All pointers are host pointers. */
int sfmba_bundle_adjust(const sfmba_problem *problem, const sfmba_options *options,
                        sfmba_result *result);

/* Same solve with every problem and result pointer in device memory of the
 * current CUDA device; runs on `stream` (a cudaStream_t, or NULL for the
 * library's own stream) and returns after the solve has finished. */
int sfmba_bundle_adjust_device(const sfmba_problem *problem, const sfmba_options *options,
                               sfmba_result *result, void *stream);

/* Replaces `pub fn mean_reprojection_error(input: &BaInput) -> f64`
 * (crates/sfm-ba/src/lib.rs:708-725). Host pointers. */
int sfmba_mean_reprojection_error(const sfmba_problem *problem, double *out_mean_px);

/* The robust cost `bundle_adjust` minimises (lib.rs:727-745, `total_cost`,
 * private in the crate): sum over observations of w * |r|^2. Host pointers. */
int sfmba_total_cost(const sfmba_problem *problem, const sfmba_options *options,
                     double *out_cost);

/* Replaces `pub fn default_fixed_params_mask(&[CameraModel]) -> Vec<Vec<bool>>`
 * (crates/sfm-ba/src/intrinsics.rs:49-61). Writes [num_cameras][8]. */
int sfmba_default_fixed_params_mask(int64_t num_cameras, const int32_t *camera_model,
                                    uint8_t *out_mask);

/* Replaces `pub fn refine_intrinsics(...)` (crates/sfm-ba/src/intrinsics.rs:116-147)
 * with IntrinsicsRefineParams mapped onto sfmba_options (max_iterations,
 * initial_lambda, robust_loss, loss_scale_px). Updates problem->camera_params
 * in place through `camera_params_inout` ([num_cameras][8], host). */
int sfmba_refine_intrinsics(const sfmba_problem *problem, const sfmba_options *options,
                            double *camera_params_inout);

/* Many independent bundle adjustments (local BA windows, as
 * sfm-reconstruction's BaScope::Local issues them one call at a time,
 * crates/sfm-reconstruction/src/lib.rs:1287-1299) solved together, each
 * with its own damping and stopping. Host pointers. */
int sfmba_bundle_adjust_batched(int32_t num_windows, const sfmba_problem *windows,
                                const sfmba_options *options, sfmba_result *results);

/* crates/sfm-reconstruction/src/lib.rs:1722-1768 (`filter_and_reoptimize`,
 * the final intrinsics-guarded pass of the reconstruction): bundle
 * adjustment, then up to two rounds of dropping the observations whose point
 * is behind the camera (z <= 1e-9) or whose reprojection error under the
 * previous output exceeds threshold_px, each followed by an adjustment from
 * that output; a round that drops nothing or leaves fewer than 12
 * observations ends the loop. Everything stays on the GPU between rounds.
 * `result` holds the last adjustment's output and statistics; keep_out
 * ([num_observations] or NULL) is 1 for the observations that adjustment
 * used. Host pointers. */
int sfmba_filter_and_reoptimize(const sfmba_problem *problem, const sfmba_options *options,
                                double threshold_px, sfmba_result *result, uint8_t *keep_out);

/* How the global adjustment treats camera intrinsics
 * (crates/sfm-reconstruction/src/lib.rs:1300-1316, `IntrinsicsMode`). */
typedef enum sfmba_intrinsics_mode {
    SFMBA_INTRINSICS_FIXED = 0,        /* intrinsics held                                   */
    SFMBA_INTRINSICS_FREE = 1,         /* one plain solve with intrinsics free              */
    SFMBA_INTRINSICS_FREE_GUARDED = 2  /* filtered solves, fixed-vs-free comparison         */
} sfmba_intrinsics_mode;

/* The intrinsics handling of the reference's global bundle adjustment
 * (crates/sfm-reconstruction/src/lib.rs:1567-1708, inside
 * `run_bundle_adjustment`), over an already-built problem. The problem's
 * fixed_cameras mask holds the cameras the user fixed; a camera seen by
 * fewer than 5 images is also held when intrinsics are free (:1601-1611,
 * :1638-1657).
 *   FIXED: one adjustment with every camera fixed.
 *   FREE: one adjustment with the free cameras free (:1598-1621).
 *   FREE_GUARDED: `filter_and_reoptimize` (threshold max_reprojection_error_px)
 *     with every camera fixed, then, if some camera has >= 5 images, again
 *     with the free cameras free; the free result is taken iff every camera's
 *     distortion coefficients are below 0.5 in magnitude (:1672-1677) and its
 *     plain mean reprojection error over ALL the problem's observations is
 *     lower than the fixed result's (:1567-1578, :1691-1695).
 * The options (max_iterations, loss, ...) are used as given: the reference's
 * caller picks max_iterations per mode (200 / 50 / 50, :1494-1520).
 * result: the chosen adjustment. keep_out ([num_observations] or NULL): the
 * observations the chosen adjustment used (all 1 without filtering).
 * chose_free_out (or NULL): 1 if the intrinsics-free result was taken.
 * mean_errors_out ([2] or NULL): plain mean reprojection error of the fixed
 * and of the free candidate (NaN for one not run). Host pointers. */
int sfmba_adjust_global(const sfmba_problem *problem, const sfmba_options *options,
                        int32_t intrinsics_mode, double max_reprojection_error_px,
                        sfmba_result *result, uint8_t *keep_out, int32_t *chose_free_out,
                        double *mean_errors_out);

/* crates/sfm-geometry/src/pnp.rs:151-206 (`refine_pose_gauss_newton`) for
 * num independent poses in one call: pose k (poses[k][7], qw qx qy qz tx ty
 * tz, in and out) takes `iterations` Gauss-Newton steps (left rotation
 * increment, additive translation, J^T J + 1e-9 I solved by partial-pivot
 * LU; a singular or non-finite step ends the pose's loop) over its
 * correspondences [offsets[k], offsets[k+1]) of points3d ([N][3], world) and
 * points2d_norm ([N][2], normalised image coordinates); offsets[0] = 0,
 * N = offsets[num]. Host pointers. */
int sfmba_refine_pose_gauss_newton_batched(int32_t num, const int64_t *offsets, const double *points3d,
                                           const double *points2d_norm, int32_t iterations, double *poses);

/* crates/sfm-geometry/src/pnp.rs:211-309 (`pnp_ransac`, with ransac.rs:72-131
 * and pnp.rs:22-130) for num images at once, correspondences laid out as in
 * sfmba_refine_pose_gauss_newton_batched: 6-point DLT hypotheses from the
 * xorshift64 stream seeded 0xFACADE, the adaptive iteration count at
 * confidence 0.999 (at most max_iterations), the local refit over the
 * inliers and two Gauss-Newton polish rounds, each kept only if it loses no
 * inliers; `threshold` in normalised units. found_out[k] = 0 where the
 * reference returns None (then poses_out[k] is unspecified and the mask 0);
 * else poses_out[k][7] and inliers_out[offsets[k] + i] (may be NULL).
 * iterations_out[k] (may be NULL): RANSAC iterations run. Host pointers. */
int sfmba_pnp_ransac_batched(int32_t num, const int64_t *offsets, const double *points3d,
                             const double *points2d_norm, double threshold, int32_t max_iterations,
                             double *poses_out, uint8_t *inliers_out, int32_t *found_out,
                             int64_t *iterations_out);

/* Statistics of cmd_refine (crates/sfm-cli/src/main.rs:1110-1123). */
typedef struct sfmba_refine_report {
    int64_t num_images;
    int64_t num_cameras;
    int64_t num_points3d;
    int64_t num_observations;
    double initial_cost;
    double final_cost;
    int32_t iterations_run;
    int32_t reserved_i;
    double mean_error_before_px;  /* Reconstruction::mean_reprojection_error before */
    double mean_error_after_px;   /* ... and after, with the recomputed point errors */
    double seconds;
    double reserved[4];
} sfmba_refine_report;

/* `sfmtory refine` (crates/sfm-cli/src/main.rs:946-1130) over a COLMAP text
 * model (cameras.txt, images.txt, points3D.txt; crates/sfm-io/src/colmap.rs)
 * in dir_in: one global bundle adjustment on the GPU with image 0 (in id
 * order) anchored, cameras fixed or (refine_intrinsics) free with the
 * principal point masked, every point's stored error recomputed as its mean
 * pixel reprojection error, the refined model written to dir_out (may be
 * dir_in; created if missing). options NULL: the reference's Huber loss and
 * 200 iterations. Fewer than 2 images, no points, no observation linking a
 * track to a registered image's keypoint, a malformed file or an image whose
 * camera is missing are errors (SFMBA_ERR_INVALID_ARGUMENT). */
int sfmba_colmap_refine(const char *dir_in, const char *dir_out, const sfmba_options *options,
                        int32_t refine_intrinsics, sfmba_refine_report *report);

/* crates/sfm-io/src/colmap.rs: read the text model in dir_in and write it to
 * dir_out in the reference's number formats (read_model + write_model). */
int sfmba_colmap_rewrite(const char *dir_in, const char *dir_out);

/* Reads the text model in dir: counts[5] = cameras, images, points3D, track
 * elements, keypoints (may be NULL); mean_error =
 * Reconstruction::mean_reprojection_error (crates/sfm-core/src/model.rs:84-97,
 * may be NULL). */
int sfmba_colmap_model_stats(const char *dir, int64_t *counts, double *mean_error);

/* Residual and Jacobian blocks of individual observations, computed on the
 * GPU by the same device code the solver uses (crates/sfm-ba/src/lib.rs:327-590,
 * `analytic_jacobians`). For observation o: r[o][2], j_pose[o][2][6],
 * j_point[o][2][3], j_camera[o][2][8] (columns past the model's parameter
 * count are 0), valid[o] = point in front of the camera (z > 1e-9).
 * `precision` selects the FP64 or FP32 kernel. Host pointers. */
int sfmba_residuals_jacobians(const sfmba_problem *problem, int32_t precision, double *r,
                              double *j_pose, double *j_point, double *j_camera,
                              uint8_t *valid);

/* A reconstruction in progress as sfm-reconstruction holds it during
 * incremental growth (crates/sfm-reconstruction/src/lib.rs:126-129
 * `PointWork` {xyz, track of (image, keypoint)}, the registered flags, the
 * poses and cameras): input of the local-window builder. Each track element
 * carries its keypoint's pixel (the reference reads it from the image's
 * features, lib.rs:131-134). */
typedef struct sfmba_reconstruction {
    int64_t num_images;
    int64_t num_cameras;
    int64_t num_points;
    const int32_t *camera_of_image;   /* [num_images]                                  */
    const int32_t *camera_model;      /* [num_cameras] sfmba_camera_model              */
    const double *camera_params;      /* [num_cameras][8]                              */
    const double *poses;              /* [num_images][7]; registered images only read  */
    const uint8_t *registered;        /* [num_images]                                  */
    const uint8_t *pose_fixed;        /* [num_images] or NULL: poses the caller pinned
                                         (ImageInput::pose_fixed with an initial pose) */
    const double *points;             /* [num_points][3]                               */
    const int64_t *track_offsets;     /* [num_points+1], track_offsets[0] = 0          */
    const int32_t *track_image;       /* [track_offsets[num_points]]                   */
    const double *track_xy;           /* [track_offsets[num_points]][2] pixels         */
} sfmba_reconstruction;

/* Caller-owned output arrays of one local window, sized by the counts of a
 * sizing call (images I, cameras C, points P, observations O). Any pointer
 * may be NULL to skip that array. */
typedef struct sfmba_window_buffers {
    int32_t *image_ids;            /* [I] reconstruction image of each window image  */
    int32_t *camera_ids;           /* [C] reconstruction camera of each window camera */
    int32_t *point_ids;            /* [P] reconstruction point of each window point  */
    int32_t *camera_of_image;      /* [I]                                             */
    int32_t *camera_model;         /* [C]                                             */
    double *camera_params;         /* [C][8]                                          */
    double *poses;                 /* [I][7]                                          */
    double *points;                /* [P][3]                                          */
    int32_t *obs_image;            /* [O]                                             */
    int32_t *obs_point;            /* [O]                                             */
    double *obs_xy;                /* [O][2]                                          */
    uint8_t *fixed_poses;          /* [I]                                             */
    uint8_t *fixed_cameras;        /* [C] all 1: local bundles hold the intrinsics    */
    uint8_t *fixed_camera_params;  /* [C][8] default_fixed_params_mask                */
} sfmba_window_buffers;

/* BaScope::Local window construction (crates/sfm-reconstruction/src/lib.rs:
 * 1287-1299, :1320, :1336-1473) for num_centers centre images at once: the
 * centre's points (tracks of >= 2 elements) free; the centre and its
 * num_free_neighbours most co-visible registered images (ties by index;
 * LOCAL_BA_NUM_IMAGES = 6 in the reference) free; every other registered
 * image observing those points present and fixed, as are seed_image (-1:
 * none) and the pinned poses; if no pose is fixed, the first window image;
 * compact indices in the reference's order; cameras fixed with the
 * principal point masked. counts_out[k][4] = images, cameras, points,
 * observations of window k, all 0 where the reference makes no solve (fewer
 * than two images or no observation). windows NULL: sizes only; else
 * num_centers buffer sets sized by an earlier sizing call with the same
 * arguments (checked). Host computation; each window can be passed to
 * sfmba_bundle_adjust or, all together, to sfmba_bundle_adjust_batched. */
int sfmba_local_windows(const sfmba_reconstruction *rec, int32_t seed_image, int32_t num_free_neighbours,
                        int32_t num_centers, const int32_t *centers, int64_t *counts_out,
                        sfmba_window_buffers *windows);

/* No counterpart in the reference. The robust cost of sfmba_total_cost for
 * a problem whose arrays are all in device memory, computed without
 * allocating any memory, for callers that cannot let a library allocate
 * (a fixed per-component slice of the GPU, or a thread that must not pay
 * for cudaFree's device-wide synchronisation). The result is written to
 * `out_cost_device` (device memory) on `stream` (NULL: the default stream);
 * the call waits for its stream and returns once the result is there, so it
 * must not be called on a stream that is being captured into a CUDA graph.
 * Scratch is a fixed 32 KB array inside the library, held on every device
 * the library is used on until exit; at most SFMBA_NOALLOC_MAX_OBSERVATIONS
 * observations (larger problems are rejected with
 * SFMBA_ERR_INVALID_ARGUMENT). The first call on a device looks up the
 * array's device address. Indices and model ids are validated as
 * sfmba_total_cost validates them (SFMBA_ERR_INVALID_ARGUMENT, NaN written).
 * Calls share the array: calls that overlap on one GPU race. */
#define SFMBA_NOALLOC_MAX_OBSERVATIONS 16777216
int sfmba_total_cost_noalloc(const sfmba_problem *problem, const sfmba_options *options,
                             double *out_cost_device, void *stream);

/* Benchmarking aid (no counterpart in the reference): throughput of the
 * current GPU's arithmetic units that the dense Cholesky can use, in
 * TFLOP/s: out[0] FP64 fused multiply-add, out[1] the FP64 tensor
 * instruction (mma.sync m8n8k4), out[2] the BF16 tensor instruction
 * (mma.sync m16n8k16, FP32 accumulation). */
int sfmba_measure_peaks(double *out);

/* Test and benchmarking aid (the factorisation of lib.rs:1081-1094 on its
 * own): the blocked Cholesky of the dense solver applied to the symmetric
 * positive-definite n x n matrix A (host, row-major; its lower triangle is
 * read) on the GPU. L (host, n x n) receives the lower factor, zeros above
 * the diagonal. tensor_update != 0 runs the trailing updates on the BF16
 * tensor cores by error-free splitting (the mixed path's choice), 0 with
 * FP64 fused multiply-adds. *seconds (if not NULL): device time of the
 * factorisation. A matrix that is not positive definite gives
 * SFMBA_ERR_INVALID_ARGUMENT. */
int sfmba_dense_cholesky(int64_t n, const double *A, double *L, int32_t tensor_update, double *seconds);

/* Benchmarking aid (no counterpart in the reference): when enabled, every
 * kernel phase of the solves made on this thread is bracketed by CUDA events
 * on its launch stream. Enabling or disabling clears the totals. */
int sfmba_profile_enable(int32_t on);

/* JSON object {phase: {"ms": total device ms, "launches": n}} of the
 * profiled phases since the last sfmba_profile_enable, into buf[len], with
 * "kernel_launches", "host_ms" (wall ms of host-side stages: the batched
 * entry's batch building and copies, and the set-up's stages "setup_layout",
 * "setup_upload", "setup_sort", "setup_partition", "setup_coarse",
 * "setup_chunks", "setup_rest", each waited for on the stream while
 * profiling), "counts", "lm_trace" and "autotune". */
int sfmba_profile_report(char *buf, int64_t len);

/* Message of the last failed call on this thread ("" if none). */
const char *sfmba_last_error(void);

/* Library version string. */
const char *sfmba_version(void);

#ifdef __cplusplus
}
#endif

#endif /* SFMBA_H */
