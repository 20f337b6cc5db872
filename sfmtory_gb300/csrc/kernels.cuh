// Launchers of the GB300 bundle-adjustment kernels. Each launcher picks the
// template instance (precision, image block width D) at run time; templates
// stay inside their .cu file.
#pragma once

#include "common.cuh"

namespace sfmba {

// Device buffers of one solve (all owned by the workspace arena).
// Coarse correction of the PCG preconditioner (k_coarse.cu).
constexpr int kMaxCoarseClusters = 128;
constexpr int kDefaultCoarseClusters = 64;
constexpr int kMinImagesPerCluster = 4;
constexpr int kCoarseChunk = 64;  // points per warp in the coarse assembly
struct CoarseBufs {
    int nc = 0;                       // clusters (0: off)
    int *img_cluster = nullptr;       // [nI]
    int *clu_start = nullptr;         // [nc+1] first image of each cluster (consecutive images)
    int *pair_pt = nullptr;           // points of the point-cluster pairs, grouped by cluster pair
    long long ninc = 0;               // point-cluster incidences (a point's distinct clusters)
    long long *inc_off = nullptr;     // [nP+1] first incidence of each point
    int *inc_cl = nullptr;            // [ninc] cluster of each incidence, increasing within a point
    int *inc_order = nullptr;         // [ninc] incidences by their point's track length (k_coarse_y's thread order)
    int *inc_pt = nullptr;            // [ninc] point of each incidence
    void *ybuf = nullptr;             // [ninc][3*D] Y_c of each incidence, element type of the linearisation
    int ngroups = 0;
    int2 *group_cc = nullptr;         // [ngroups] (c, c'), c <= c'
    int *group_chunk_off = nullptr;   // [ngroups+1]
    int nchunks = 0;
    int4 *chunk = nullptr;            // [nchunks] {group, first, end, 0} into pair_pt
    double *chunk_part = nullptr;     // [nchunks][D*D]
    double *A = nullptr;              // [Nc*Nc] coarse matrix, FP64
    float *X32 = nullptr;             // [2][Np*Np] ping-pong buffers of the block sweep (coarse_padded_size),
                                      // then [Np] doubles: the symmetric scaling
    int *fail = nullptr;              // [2]: the sweep met a non-finite pivot; pivots raised to their floor
    float *Ainv = nullptr;            // [Nc*Nc] symmetric FP32 A^-1, applied per iteration
    void *cc = nullptr;               // [Nc] coarse correction, element type of the PCG vectors
    double *zc = nullptr;             // [Nc] Z^T r
    double *zpart = nullptr;          // [ceil(nI/8)][3][D] per-block restriction sums (cooperative CG kernel)
};

// Free cameras shared by several images, on the PCG solver. The reduced
// system has one slot block per camera (lib.rs:753-787); the PCG's vectors
// are image level, so every image using a shared camera ("linked" image)
// carries a copy of the camera's entries and the first such image (the
// owner) holds the ones the preconditioner and the dot products count. The
// camera's block of the block-Jacobi preconditioner is exact:
//   sum_i (H_i + lambda diag H_i)_cc - sum_p Y_pc^T C_p^-1 Y_pc,
// Y_pc = sum over p's observations in images of camera c of Jx~^T Jc~_cam,
// one (point, camera) incidence each, summed per camera in a fixed order.
struct SharedBufs {
    int nsh = 0;                      // shared free cameras (0: none)
    int *img_owner = nullptr;         // [nI] image holding the camera entries (itself if not linked)
    int *img_shcam = nullptr;         // [nI] shared-camera index of the image, -1 if not linked
    int *sh_img_start = nullptr;      // [nsh+1]
    int *sh_imgs = nullptr;           // images of each shared camera, in image order
    long long ninc = 0;               // (point, shared camera) incidences
    long long *inc_off = nullptr;     // [nP+1] first incidence of each point
    int *inc_sorted = nullptr;        // [ninc] incidences ordered by camera (then point)
    void *inc_W = nullptr;            // [ninc][NS] upper triangle of Y^T C^-1 Y (kernel precision)
    int nchunks = 0;
    int4 *chunk = nullptr;            // [nchunks] {camera, first, end, 0} into inc_sorted
    int *cam_chunk_off = nullptr;     // [nsh+1]
    double *chunk_part = nullptr;     // [nchunks][NS]
};
constexpr int kSharedChunk = 256;     // incidences per warp in the per-camera sums

struct Bufs {
    // sizes
    int nI = 0, nC = 0, nP = 0;
    long long nO = 0;
    int n = 0;        // reduced-system dimension (reference slotting)
    int D = 6;        // image block width: 6 pose columns + widest camera
    int nID = 0;      // nI * D
    int mixed = 0;    // 1: FP32 linearisation/Schur/PCG, 0: FP64
    int uniform_model = -1;  // the model of every camera, -1 when they differ
    int loss = 0;
    double loss_scale = 1.0;
    // problem, solver layout
    const int *cam_model = nullptr;     // [nC]
    const int *cam_of_img = nullptr;    // [nI]
    double *cams = nullptr, *cams_trial = nullptr;      // [nC*8]
    double *poses = nullptr, *poses_trial = nullptr;    // [nI*7]
    double *points = nullptr, *points_trial = nullptr;  // [nP*3]
    float4 *points32 = nullptr;                         // [nP] FP32 copy (mixed)
    int *ob_img = nullptr, *ob_pt = nullptr;            // [nO] point-sorted
    double2 *ob_xy = nullptr;                           // [nO]
    int *pt_start = nullptr;                            // [nP+1]
    int *img_start = nullptr;                           // [nI+1]
    int *img_obs = nullptr;                             // [nO] image-sorted -> point-sorted index
    int *pt_perm = nullptr;       // [nP] solver point index -> caller's point index
    int *pt_old2new = nullptr;    // [nP] caller's point index -> solver point index
    int *img_slot = nullptr;      // [nI*D] slot of column r of image i, -1 if not an unknown
    int *img_active = nullptr;    // [nI] bit r: column r is an unknown
    // Column masks of the PCG vector kernels (both = img_active without
    // shared cameras): pmask - columns an image's own block-Jacobi block and
    // coarse space cover (a linked image's camera columns excluded); dmask -
    // columns counted in dot products (the owner's camera columns included).
    int *img_pmask = nullptr;     // [nI]
    int *img_dmask = nullptr;     // [nI]
    SharedBufs sh;
    int *img_free = nullptr;      // [nI] pose free or camera free
    int *cam_slot = nullptr;      // [nC] first slot of the camera, -1 if fixed
    int *pose_slot = nullptr;     // [nI] first slot of the pose, -1 if fixed
    int *slot_pre_start = nullptr;  // [n+1]
    int *slot_pre = nullptr;        // image-level indices i*D+r mapped onto each slot
    unsigned char *slot_masked = nullptr;  // [n]
    // linearisation (element type float or double by `mixed`)
    void *img_lin = nullptr;      // [nI] ImageLin<T>
    float4 *ob_rs = nullptr;      // [nO] point-major FP64 residual, sqrt(weight), valid at the current parameters (FP32 path)
    float4 *ob_rs_trial = nullptr;  // [nO] the same at the trial parameters (written by the trial cost)
    void *rec = nullptr;          // [nO * stride] records
    unsigned char *ob_valid = nullptr;  // [nO]
    void *pt_C = nullptr;         // [nP*6] symmetric 3x3 (00 01 02 11 12 22)
    void *pt_g = nullptr;         // [nP*3]
    int *pt_nfree = nullptr;      // [nP]
    void *pt_Cinv = nullptr;      // [nP*6]
    void *pt_h = nullptr;         // [nP*3] Cinv g
    unsigned char *pt_ok = nullptr;  // [nP]
    double *img_H = nullptr;      // [nI*D*D]
    double *img_b = nullptr;      // [nI*D]
    double *img_rhs = nullptr;    // [nI*D]
    void *img_delta = nullptr;    // [nI*D] step of the image block (T)
    // dense reduced system
    int2 *pairs = nullptr;        // [npairs] (obs a, obs b), grouped by image pair
    int *group_start = nullptr;   // [ngroups+1]
    int2 *group_ij = nullptr;     // [ngroups]
    int *group_order = nullptr;   // [ngroups] groups by decreasing pair count: the Schur kernels' launch order
    long long npairs = 0;
    int ngroups = 0;
    double *S_img = nullptr;      // [nID*nID]
    double *S = nullptr;          // [n*n] symmetric reduced system
    double *L = nullptr;          // [n*n] Cholesky / LU factors
    double *Linv = nullptr;       // [nblocks*64*64] inverses of diagonal blocks
    // Tensor-core trailing updates of the Cholesky (NULL: FP64 fused
    // multiply-adds): BF16 slices [7][n][64] and exponents [n] of a panel;
    // two of each (alternating by panel) for the single dense system, one
    // for the batched windows.
    uint16_t *oz_slices = nullptr;
    int *oz_exp = nullptr;
    int *lu_perm = nullptr;       // [n]
    double *rhs = nullptr, *delta = nullptr, *diagB = nullptr, *work = nullptr, *work2 = nullptr;  // [n]
    double *ref_res = nullptr, *ref_corr = nullptr;  // [n] refinement residual and correction
    // LM bookkeeping
    LMState *state = nullptr;
    double *partials = nullptr;   // [kCostBlocks*2]
    double *img_rt64 = nullptr;   // [nI][12] FP64 R (row-major) and t of the poses the cost evaluates
    // Double-float copies for the FP32 path's cost (no OPENCV_FISHEYE camera):
    int df_cost = 0;
    float4 *ob_xy_df = nullptr;   // [nO] {x hi, x lo, y hi, y lo}
    float4 *pts_df = nullptr;     // [nP][2] {x hi, x lo, y hi, y lo}, {z hi, z lo, 0, 0}
    float *rt_df = nullptr;       // [nI][24] img_rt64 as pairs
    float *cams_df = nullptr;     // [nC][16] camera parameters as pairs
    long long *count_partials = nullptr;
    // PCG (matrix-free) vectors, [nI*D] each, element type T
    void *pcg_x = nullptr, *pcg_r = nullptr, *pcg_z = nullptr, *pcg_p = nullptr, *pcg_q = nullptr;
    float *pcg_p4 = nullptr;      // FP32: copy of p in planes (plane_index; pad4(D)/4 planes of [nI] float4), point pass
    float4 *img_mv = nullptr;     // FP32 PCG: per-image constants of MvOp in 5 planes of [nI] float4:
                                  //   (R0 R1 R2 R3) (R4 R5 R6 R7) (R8 t0 t1 t2) (f fy k1 k2) (cx cy 0 0)
    CoarseBufs co;                // coarse correction of the preconditioner
    void *pcg_u = nullptr;        // [nP*4] per-point Cinv E^T p
    void *pcg_Minv = nullptr;     // [nI*D*D] block-Jacobi inverse
    float *img_Hf = nullptr;      // FP32 PCG: [nI*D*D] H_i + lambda diag H_i (the CG kernel's B p)
    double *pcg_part = nullptr;   // [3*nI] per-image partial dot products
    double *pcg_blk = nullptr;    // [4*kPcgMaxCoopBlocks] per-block partial sums of the cooperative CG kernel
    double pcg_tol = 1e-6;
    // Work partition of the matrix-free passes (fixed-size observation chunks).
    int *pchunk = nullptr;        // [npchunks+1] point-aligned chunk starts (point-major order)
    int npchunks = 0;
    int *ipart_off = nullptr;     // [nI+1] first partial slot of each image
    void *ipart = nullptr;        // [nparts*D] per-(chunk, image) partial sums
    void *ipart2 = nullptr;       // [nparts*(D(D+1)/2+D)] block partials of the image passes
    int nparts = 0;
    int4 *iachunk = nullptr;      // image-aligned chunks {image, first, end} of the image-block passes
    int *iachunk_off = nullptr;   // [nI+1] first chunk (= partial slot) of each image
    int n_iachunks = 0;
    int4 *obrec = nullptr;        // [nO] point-major {image, point, x, y (float bits)}
    int4 *isrec = nullptr;        // [nO] image-major {image, point, x, y (float bits)}
    // Batched windows: per-image / per-point "take part" flags of the current
    // phase (NULL: everything takes part). Kernels skip the rest.
    unsigned char *img_live = nullptr;  // [nI]
    unsigned char *pt_live = nullptr;   // [nP]
};

// Levenberg-Marquardt state of one window of a batched solve.
struct WinState {
    double lambda, nu;
    double cost, trial_cost, cost_before, initial_cost;
    double lambda_start, nu_start;  // damping at the start of the outer iteration
    long long valid_obs, trial_valid_obs;
    int iterations, retries, retries_outer;
    int accepted;        // accepted in the current retry, not yet committed
    int accepted_outer;  // some retry of this outer iteration was accepted
    int active;          // takes part in the current retry
    int factor_failed, solve_failed;
    int done;            // stopped (or parked until the FP64 polish)
    int wants_polish, polished, polish_iteration;
};

// Window structure of a batched solve. The windows are concatenated into
// one block-diagonal problem (images, cameras, points, slots in window
// order); these arrays map the concatenation back to windows and locate
// each window's dense reduced system.
struct WinBufs {
    int W = 0;
    int max_n = 0;                 // largest window system
    WinState *ws = nullptr;        // [W]
    int *pt_win = nullptr;         // [nP] window of each point (solver order)
    int *img_win = nullptr;        // [nI]
    int *cam_win = nullptr;        // [nC]
    int *slot_win = nullptr;       // [n]
    int *img_base = nullptr;       // [W] first image of the window
    int *nid_w = nullptr;          // [W] images of the window * D
    int *n_w = nullptr;            // [W] reduced-system dimension
    int *slot_base = nullptr;      // [W] first slot
    long long *s_off = nullptr;    // [W] offset of the window's n_w^2 system in S and L
    long long *simg_off = nullptr; // [W] offset of its nid_w^2 image-level blocks in S_img
    long long *linv_off = nullptr; // [W] offset of its diagonal-block inverses in Linv
    long long *obs_off = nullptr;  // [W+1] observation range (point-major order)
    int *counts = nullptr;         // [4] summary read by the host each retry
    int *slot_perm = nullptr;      // [n] position in the window systems -> slot
    int *row_first = nullptr;      // [n] first nonzero column of each permuted row
    double *rhs_p = nullptr;       // [n] right-hand side in permuted order
    int4 *fold_blk = nullptr;      // [n_fold_blk] {window, first row, end row} of the fold kernel
    int n_fold_blk = 0;
    int *lu_list = nullptr;        // [W] windows in the LU fallback
    int *lu_count = nullptr;       // [1]
    // cost blocks: up to kWinCostChunk observations of one window each
    int ncblk = 0;
    int *cblk_win = nullptr;       // [ncblk] window of the block
    long long *cblk_lo = nullptr;  // [ncblk+1] observation range of the block
    int *wblk_start = nullptr;     // [W+1] first block of each window
    double *cpart = nullptr;       // [ncblk] partial cost
    long long *cpart_n = nullptr;  // [ncblk] partial valid count
};

constexpr int kWinCostChunk = 8192;

constexpr int kCostBlocks = 1024;
constexpr int kDotSlots = 16;
constexpr int kCholNB = 64;
constexpr int kChunkObs = 256;  // observations per warp in the matrix-free passes
constexpr int kPcgMaxCoopBlocks = 4096;  // grid of the cooperative CG kernel at most

// Inputs/outputs of the per-observation Jacobian probe (original order).
struct JacProbe {
    long long nO = 0;
    double *poses = nullptr, *cams = nullptr, *points = nullptr, *obs_xy = nullptr;
    int *cam_of_img = nullptr, *cam_model = nullptr, *obs_img = nullptr, *obs_pt = nullptr;
    double *r = nullptr, *jp = nullptr, *jx = nullptr, *jc = nullptr;
    unsigned char *valid = nullptr;
};

// ---- setup (k_setup.cu)
size_t sort_temp_bytes(long long nO, int nP, int nI);
// Visibility order of the points: sorted by the first image observing them
// (ties by index), so points seen by the same cameras sit together. Writes
// perm (new -> old), old2new and the observations' point indices renumbered.
void order_points(const int *obs_point_in, const int *obs_image_in, long long nO, int nP, int nI, int *key,
                  int *key_sorted, int *iota_tmp, int *perm, int *old2new, int *obs_point_out, void *temp,
                  size_t temp_bytes, cudaStream_t s);
void gather_points(const double *src, const int *perm, int nP, double *dst, cudaStream_t s);
void scatter_points(const double *src, const int *old2new, int nP, double *dst, cudaStream_t s);
void sort_observations(const int *obs_point_in, const int *obs_image_in, const double *obs_xy_in,
                       long long nO, int nP, int nI, Bufs &b, void *temp, size_t temp_bytes,
                       int *keys_tmp, int *vals_tmp, int *keys_tmp2, int *vals_tmp2,
                       cudaStream_t s);
size_t pairs_temp_bytes(long long npairs, int nI);
long long count_pairs(const Bufs &b, long long *d_count_scan, void *temp, size_t temp_bytes,
                      cudaStream_t s);
void build_pairs(Bufs &b, const long long *d_count_scan, unsigned *keys_a, unsigned *keys_b,
                 int2 *vals_b, void *temp, size_t temp_bytes, int *d_ngroups, cudaStream_t s);
void validate_problem_device(const int *cam_of_img, const int *cam_model, const int *obs_image,
                             const int *obs_point, long long nO, int nI, int nC, int nP,
                             int *d_bad, cudaStream_t s);

// ---- linearisation and LM bookkeeping (k_lin.cu)
void launch_prepare_images(const Bufs &b, cudaStream_t s);
void launch_linearize(const Bufs &b, cudaStream_t s);
void launch_point_reduce(const Bufs &b, cudaStream_t s);
void launch_diag_fold(const Bufs &b, cudaStream_t s);
void launch_point_inverse(const Bufs &b, cudaStream_t s);
void launch_image_rhs(const Bufs &b, cudaStream_t s);
void launch_gather_delta(const Bufs &b, const double *delta_slot, cudaStream_t s);
void launch_backsub_update(const Bufs &b, const double *delta_slot, cudaStream_t s);
void launch_update_images(const Bufs &b, const double *delta_slot, cudaStream_t s);
// cost of (poses, cams, points) or of the trial buffers, into state->cost/trial_cost
void launch_cost(const Bufs &b, bool trial, bool into_trial, cudaStream_t s);
// FP64 rotation matrix and translation of every pose ([nI][12]) for the cost.
// Double-float copy of the observations for the FP32 path's cost (b.df_cost).
void launch_split_xy_df(const Bufs &b, cudaStream_t s);
// Double-float copies of the points, pose matrices (img_rt64, formed first)
// and camera parameters the cost evaluates (current or trial).
void launch_split_df(const Bufs &b, bool trial, cudaStream_t s);
void launch_pose_rt64(const double *poses, int nI, double *rt, cudaStream_t s);
void launch_mean_error(const Bufs &b, cudaStream_t s);  // -> partials; host finalises
void launch_accept(const Bufs &b, cudaStream_t s);
void launch_commit(const Bufs &b, cudaStream_t s);
void launch_reject(const Bufs &b, cudaStream_t s);
void launch_refresh_points32(const Bufs &b, cudaStream_t s);
void launch_begin_outer(const Bufs &b, cudaStream_t s);
void launch_begin_retry(const Bufs &b, cudaStream_t s);
void launch_count_valid(const Bufs &b, cudaStream_t s);
void launch_jacobian_probe(const JacProbe &q, bool fp32, cudaStream_t s);

// ---- dense reduced system (k_dense.cu)
void launch_schur_pairs(const Bufs &b, cudaStream_t s);
void launch_fold_system(const Bufs &b, cudaStream_t s);
void launch_fold_rhs(const Bufs &b, cudaStream_t s);  // slot-order rhs only
void launch_cholesky(const Bufs &b, cudaStream_t s);
void launch_cholesky_solve(const Bufs &b, const double *rhs, double *x, cudaStream_t s);
void launch_refine(const Bufs &b, cudaStream_t s);
void launch_lu_factor(const Bufs &b, cudaStream_t s);
void launch_lu_solve(const Bufs &b, cudaStream_t s);

// ---- matrix-free observation passes (k_matfree.cu)
void launch_mf_prepare(const Bufs &b, cudaStream_t s);          // packed observation records
void launch_mf_point_reduce(const Bufs &b, cudaStream_t s);     // C_p, g_p, free count
void launch_mf_image_blocks(const Bufs &b, cudaStream_t s);     // H_i, b_i
void launch_image_blocks_records(const Bufs &b, cudaStream_t s);  // H_i, b_i from stored records
void launch_mf_precond(const Bufs &b, cudaStream_t s);          // M^-1, rhs, PCG start vectors
// FP32: H_i, b_i and the preconditioner from one image-aligned pass (the
// MODE-0 and MODE-1 sums together), then both finishes.
void launch_mf_precond_fused(const Bufs &b, cudaStream_t s);
// The two PCG passes in launch variant 0..k{Point,Image}PassVariants-1
// (same results; chosen by the autotuner).
constexpr int kPointPassVariants = 11;  // the last one streams its records by bulk copies (mf_tma.cuh)
constexpr int kImagePassVariants = 10;
constexpr int kPassVariants = 11;  // the most variants of any tuned kernel
void launch_mf_points(const Bufs &b, cudaStream_t s, int variant);  // u = C^-1 E^T p
void launch_mf_images(const Bufs &b, cudaStream_t s, int variant);  // partials of E u
void launch_mf_backsub(const Bufs &b, const double *delta_slot, cudaStream_t s);

// ---- matrix-free Schur PCG, vector side (k_pcg.cu)
// Scalars of a new solve (after launch_mf_precond).
void launch_pcg_start(const Bufs &b, cudaStream_t s);
// One PCG iteration is launch_mf_points, launch_mf_images, then
// launch_pcg_images_finish (q = S p) and launch_pcg_vector (x, r, z, p).
void launch_pcg_images_finish(const Bufs &b, cudaStream_t s);
void launch_pcg_vector(const Bufs &b, cudaStream_t s, int parity, bool coarse = false);  // parity = iteration & 1
// Everything of one PCG iteration after the image pass (q = S p, the
// shared cameras' sums, alpha, x/r/z, the coarse correction, beta, p) as one
// cooperative launch with grid-wide barriers (k_pcg_coop.cu).
void launch_pcg_iteration_vector(const Bufs &b, cudaStream_t s, int parity, bool coarse);
// Work partition of the matrix-free passes (after sort_observations).
void launch_pcg_partition(Bufs &b, cudaStream_t s);
// Scatter the image-level solution to the slot-level delta.
void launch_pcg_finish(const Bufs &b, double *delta_slot, cudaStream_t s);

// ---- shared free cameras on the PCG solver (k_shared.cu)
size_t shared_setup_temp_bytes(int nP, long long ninc);
// Distinct shared cameras per point, scanned into b.sh.inc_off; returns the total.
long long launch_shared_count(const Bufs &b, long long *count, void *temp, size_t temp_bytes, cudaStream_t s);
// Incidences sorted by camera into b.sh.inc_sorted; cam_counts[c] = incidences of camera c.
void launch_shared_sort(const Bufs &b, int *key, int *val, int *key2, int *cam_counts, void *temp,
                        size_t temp_bytes, cudaStream_t s);
// Per damping retry, after the point inverses and the image-block pass:
// the shared cameras' exact preconditioner blocks, their rhs, and the PCG
// start vectors on their columns (after the image blocks' own start).
void launch_shared_precond(const Bufs &b, cudaStream_t s);
// q on the shared cameras' columns: summed over each camera's images and
// copied back to all of them; the owner's p.q partial.
void launch_shared_qreduce(const Bufs &b, cudaStream_t s);

// ---- coarse correction of the PCG preconditioner (k_coarse.cu)
size_t coarse_setup_temp_bytes(int nP, long long npairs_max);
// Pairs count per point (exclusive-scanned into off) and distinct clusters
// per point (scanned into inc_off, total in *ninc); returns the pair total.
long long launch_coarse_count(const Bufs &b, long long *count, long long *off, long long *kcount,
                              long long *inc_off, long long *ninc, void *temp, size_t temp_bytes, cudaStream_t s);
// Emits and sorts the point-cluster pairs; key_counts[c * nc + c'] = group
// sizes; the clusters of every incidence into b.co.inc_cl.
void launch_coarse_group(const Bufs &b, const long long *off, long long npairs, int *key, int *val, int *key2,
                         int *val_sorted, int *key_counts, void *temp, size_t temp_bytes, cudaStream_t s);
// inc_order: the incidences sorted by their point's track length (key, val,
// key2 are scratch of at least ninc entries).
void launch_coarse_inc_order(const Bufs &b, int *key, int *val, int *key2, void *temp, size_t temp_bytes,
                             cudaStream_t s);
// A_c (FP64) for the current damping and point inverses.
void launch_coarse_assemble(const Bufs &b, cudaStream_t s);
// z += Z Ainv Z^T r with the r.z / r.r partials (init: the start of a solve, p = z).
void launch_coarse_correct(const Bufs &b, bool init, cudaStream_t s);
// Ainv = A_c^-1 in FP32 by the block sweep (one cooperative launch); on a
// non-finite pivot co.fail[0] = 1 and Ainv = 0; co.fail[1] counts the
// pivots raised to their floor.
void launch_coarse_invert(const Bufs &b, cudaStream_t s);
// Side of the sweep's square buffers for an Nc x Nc coarse matrix.
int coarse_padded_size(int Nc);

// ---- throughput probes (k_peaks.cu): TFLOP/s of FP64 FMA, FP64 mma.sync
// m8n8k4 and BF16 mma.sync m16n8k16 on the current device.
struct PeakRates {
    double dfma_tflops = 0.0, dmma_tflops = 0.0, bf16_mma_tflops = 0.0;
};
PeakRates measure_peaks(cudaStream_t s, double *sink);

// ---- refine_intrinsics (k_intrinsics.cu)
struct IntrinsicsBufs {
    int nC = 0;
    const double *poses = nullptr, *points = nullptr, *ob_xy = nullptr;
    const int *ob_img = nullptr, *ob_pt = nullptr, *cam_model = nullptr;
    const int *cobs_start = nullptr, *cobs = nullptr;  // observations grouped by camera
    double *cams = nullptr;                             // [nC][8] in / out
};
void launch_refine_intrinsics(const IntrinsicsBufs &q, int max_iterations, double lambda0, int loss, double scale,
                              cudaStream_t s);

// ---- PnP registration and pose refinement (k_pnp.cu)
// Device arrays of the batched RANSAC PnP: P images, image k's
// correspondences [off[k], off[k+1]) of X ([N][3]) and uv ([N][2],
// normalised); B hypotheses per round.
struct PnpBufs {
    int P = 0, B = 0;
    long long max_it = 0;
    double thr = 0.0;
    const long long *off = nullptr;
    const double *X = nullptr, *uv = nullptr;
    const unsigned long long *raw = nullptr;  // [6 * max_it] xorshift64 stream
    void *state = nullptr;                    // [P] per-image RANSAC state
    double *models = nullptr;                 // [P * B][8]
    unsigned char *valid = nullptr;           // [P * B]
    long long *counts = nullptr;              // [P * B]
    int *active = nullptr;                    // [2]: images whose loop goes on, most iterations left
    double *dlt_scratch = nullptr;            // [N][24] DLT rows of the local refit
    long long *slot_scratch = nullptr;        // [N]
    unsigned char *mask = nullptr, *mask_trial = nullptr;  // [N]
    double *poses = nullptr;                  // [P][7] out
    int *found = nullptr;                     // [P] out
};
size_t pnp_state_bytes();
void launch_pnp_init(const PnpBufs &q, cudaStream_t s);
void launch_pnp_round(const PnpBufs &q, long long round_base, cudaStream_t s);
void launch_pnp_finish(const PnpBufs &q, cudaStream_t s);
void launch_pnp_iterations(const PnpBufs &q, long long *iters, cudaStream_t s);
void launch_refine_pose_gn(const long long *off, const double *X, const double *uv, int P, int iterations,
                           double *poses, cudaStream_t s);

// ---- filter_and_reoptimize (k_filter.cu)
// Device arrays of the observation filter: the current observations in set
// 0, the kept ones compacted into set 1 (the caller swaps).
struct FilterBufs {
    const int *cam_of_img = nullptr, *cam_model = nullptr;
    int *img[2] = {nullptr, nullptr}, *pt[2] = {nullptr, nullptr}, *orig[2] = {nullptr, nullptr};
    double *xy[2] = {nullptr, nullptr};
    unsigned char *flag = nullptr;
    int *iota = nullptr;          // 0, 1, 2, ... (the selected positions)
    int *sel = nullptr;
    int *count = nullptr;
    void *temp = nullptr;
    size_t temp_bytes = 0;
};
size_t filter_temp_bytes(long long nO);
// Per-point mean reprojection error over a point-ordered observation list.
void launch_point_errors(const double *poses, const double *cams, const double *points, const int *cam_of_img,
                         const int *cam_model, const int *ob_img, const double *ob_xy, const long long *pt_obs,
                         int nP, double *err_out, int *n_out, cudaStream_t s);
void launch_filter_iota(int *v, long long n, cudaStream_t s);
// flags of the m current observations under (poses, cams, points); kept ones into set 1, count into *f.count
void launch_filter_select(const FilterBufs &f, long long m, const double *poses, const double *cams,
                          const double *points, double threshold, cudaStream_t s);
void launch_filter_keep(const int *orig, long long m, unsigned char *keep, long long nO, cudaStream_t s);

// Damped 3 x 3 point block inverse, C_lambda = C + lambda diag(C) (packed
// c00 c01 c02 c11 c12 c22), and h = C_lambda^-1 g (lib.rs:958-965): false
// when det == 0 or the point has no free block (the reference's `None`).
// FP64 path: in FP64. FP32 path: the adjugate in FP32 (fused multiply-adds)
// where the block is well conditioned (|det| > 1e-4 of the product of its
// diagonal, which bounds det for a positive semi-definite block); a
// near-singular block and the det == 0 decision fall back to FP64 from the
// same FP32 entries, whose products FP64 holds exactly. The FP32 stage and
// the FP64 stage are separate functions so a block of threads can run the
// second for its points side by side (point_inverse_block).
__device__ __forceinline__ bool point_block_inverse_fast(const float *C, const float *g, double lam, bool has_free,
                                                         float *Ci, float *h) {
    const float l = (float)lam;
    const float m00 = fmaf(C[0], l, C[0]), m11 = fmaf(C[3], l, C[3]), m22 = fmaf(C[5], l, C[5]);
    const float m01 = C[1], m02 = C[2], m12 = C[4];
    const float c00 = fmaf(m11, m22, -m12 * m12);
    const float c01 = fmaf(m12, m02, -m01 * m22);
    const float c02 = fmaf(m01, m12, -m11 * m02);
    const float det = fmaf(m00, c00, fmaf(m01, c01, m02 * c02));
    if (!(has_free && fabsf(det) > 1e-4f * fabsf(m00 * m11 * m22) && isfinite(det))) return false;
    const float id = 1.0f / det;
    const float i00 = c00 * id, i01 = c01 * id, i02 = c02 * id;
    const float i11 = fmaf(m00, m22, -m02 * m02) * id;
    const float i12 = fmaf(m02, m01, -m00 * m12) * id;
    const float i22 = fmaf(m00, m11, -m01 * m01) * id;
    Ci[0] = i00; Ci[1] = i01; Ci[2] = i02; Ci[3] = i11; Ci[4] = i12; Ci[5] = i22;
    h[0] = fmaf(i00, g[0], fmaf(i01, g[1], i02 * g[2]));
    h[1] = fmaf(i01, g[0], fmaf(i11, g[1], i12 * g[2]));
    h[2] = fmaf(i02, g[0], fmaf(i12, g[1], i22 * g[2]));
    return true;
}
// The FP64 stage of the FP32 path (a block the FP32 stage declined).
__device__ __forceinline__ bool point_block_inverse_slow(const float *C, const float *g, double lam, bool has_free,
                                                         float *Ci, float *h) {
    if (!has_free) return false;
    const float l = (float)lam;
    const double d00 = fmaf(C[0], l, C[0]), d11 = fmaf(C[3], l, C[3]), d22 = fmaf(C[5], l, C[5]);
    const double d01 = C[1], d02 = C[2], d12 = C[4];
    const double e00 = d11 * d22 - d12 * d12, e01 = d12 * d02 - d01 * d22, e02 = d01 * d12 - d11 * d02;
    const double dd = d00 * e00 + d01 * e01 + d02 * e02;
    if (dd == 0.0) return false;
    const double id = 1.0 / dd;
    const double i00 = e00 * id, i01 = e01 * id, i02 = e02 * id;
    const double i11 = (d00 * d22 - d02 * d02) * id, i12 = (d02 * d01 - d00 * d12) * id;
    const double i22 = (d00 * d11 - d01 * d01) * id;
    Ci[0] = (float)i00; Ci[1] = (float)i01; Ci[2] = (float)i02;
    Ci[3] = (float)i11; Ci[4] = (float)i12; Ci[5] = (float)i22;
    const double g0 = g[0], g1 = g[1], g2 = g[2];
    h[0] = (float)(i00 * g0 + i01 * g1 + i02 * g2);
    h[1] = (float)(i01 * g0 + i11 * g1 + i12 * g2);
    h[2] = (float)(i02 * g0 + i12 * g1 + i22 * g2);
    return true;
}
__device__ __forceinline__ bool point_block_inverse_fp64(const double *C, const double *g, double lam, bool has_free,
                                                         double *Ci, double *h) {
    double m00 = C[0], m01 = C[1], m02 = C[2], m11 = C[3], m12 = C[4], m22 = C[5];
    m00 = m00 + m00 * lam; m11 = m11 + m11 * lam; m22 = m22 + m22 * lam;
    const double c00 = m11 * m22 - m12 * m12;
    const double c01 = m12 * m02 - m01 * m22;
    const double c02 = m01 * m12 - m11 * m02;
    const double det = m00 * c00 + m01 * c01 + m02 * c02;
    if (!has_free || det == 0.0) return false;
    const double id = 1.0 / det;
    const double i00 = c00 * id, i01 = c01 * id, i02 = c02 * id;
    const double i11 = (m00 * m22 - m02 * m02) * id;
    const double i12 = (m02 * m01 - m00 * m12) * id;
    const double i22 = (m00 * m11 - m01 * m01) * id;
    Ci[0] = i00; Ci[1] = i01; Ci[2] = i02; Ci[3] = i11; Ci[4] = i12; Ci[5] = i22;
    const double g0 = g[0], g1 = g[1], g2 = g[2];
    h[0] = i00 * g0 + i01 * g1 + i02 * g2;
    h[1] = i01 * g0 + i11 * g1 + i12 * g2;
    h[2] = i02 * g0 + i12 * g1 + i22 * g2;
    return true;
}

// Threads per block of the point-inverse kernels.
constexpr int kPointInvBlock = 256;

// The damped inverses of a block's points (one thread each; lam_of(p) the
// point's damping, live(p) whether it takes part), None written as zeros
// with pt_ok = 0. On the FP32 path the points the FP32 stage declines are
// collected in shared memory and taken by the block's threads side by side
// in the FP64 stage, so a near-singular point costs one lane's FP64 work
// instead of its whole warp's (GB300 runs FP64 at 1/64 of the FP32 rate);
// every point's result is the same as inverting it alone. Called by every
// thread of a block of kPointInvBlock threads.
template <typename T, typename Lam, typename Live>
__device__ __forceinline__ void point_inverse_block(const T *pt_C, const T *pt_g, const int *pt_nfree, int nP,
                                                    Lam lam_of, Live live, T *pt_Cinv, T *pt_h,
                                                    unsigned char *pt_ok) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    auto finish = [&](int q, bool ok) {
        if (!ok) {
            T *Ci = pt_Cinv + 6 * (size_t)q;
            T *h = pt_h + 3 * (size_t)q;
            for (int k = 0; k < 6; ++k) Ci[k] = T(0);
            h[0] = h[1] = h[2] = T(0);
        }
        pt_ok[q] = ok ? 1 : 0;
    };
    if constexpr (std::is_same<T, float>::value) {
        __shared__ int slow[kPointInvBlock];
        __shared__ int nslow;
        if (threadIdx.x == 0) nslow = 0;
        __syncthreads();
        if (p < nP && live(p)) {
            if (point_block_inverse_fast(pt_C + 6 * (size_t)p, pt_g + 3 * (size_t)p, lam_of(p), pt_nfree[p] > 0,
                                         pt_Cinv + 6 * (size_t)p, pt_h + 3 * (size_t)p))
                pt_ok[p] = 1;
            else
                slow[atomicAdd(&nslow, 1)] = p;
        }
        __syncthreads();
        const int n = nslow;
        for (int k = threadIdx.x; k < n; k += blockDim.x) {
            const int q = slow[k];
            finish(q, point_block_inverse_slow(pt_C + 6 * (size_t)q, pt_g + 3 * (size_t)q, lam_of(q),
                                               pt_nfree[q] > 0, pt_Cinv + 6 * (size_t)q, pt_h + 3 * (size_t)q));
        }
    } else {
        if (p >= nP || !live(p)) return;
        finish(p, point_block_inverse_fp64(pt_C + 6 * (size_t)p, pt_g + 3 * (size_t)p, lam_of(p), pt_nfree[p] > 0,
                                           pt_Cinv + 6 * (size_t)p, pt_h + 3 * (size_t)p));
    }
}

// ---- batched windows (k_batched.cu)
// Summary counts written by launch_wb_summary.
enum { WB_NOT_DONE = 0, WB_RETRY_PENDING = 1, WB_FACTOR_FAILED = 2, WB_WANTS_POLISH = 3 };
void launch_wb_window_of_points(const int *win_of_input_point, const int *perm, int nP, int *pt_win,
                                cudaStream_t s);
void launch_wb_init(const WinBufs &w, double initial_lambda, cudaStream_t s);
// img_live / pt_live for the next phase: windows not done (retry = false) or retrying.
void launch_wb_live(const Bufs &b, const WinBufs &w, bool retry, cudaStream_t s);
void launch_wb_begin_outer(const WinBufs &w, int max_iterations, cudaStream_t s);
void launch_wb_begin_retry(const WinBufs &w, cudaStream_t s);
void launch_wb_point_inverse(const Bufs &b, const WinBufs &w, cudaStream_t s);
// variant: launch shape (k_batched.cu WbSchurShape), 0 .. kWbSchurVariants - 1; all give the same sums
constexpr int kWbSchurVariants = 3;
void launch_wb_schur(const Bufs &b, const WinBufs &w, cudaStream_t s, int variant = 0);
void launch_wb_fold(const Bufs &b, const WinBufs &w, cudaStream_t s);
void launch_wb_cholesky(const Bufs &b, const WinBufs &w, cudaStream_t s);
void launch_wb_solve(const Bufs &b, const WinBufs &w, const double *rhs, double *x, cudaStream_t s);
void launch_wb_refine(const Bufs &b, const WinBufs &w, cudaStream_t s);
// delta (slot order) from the permuted solution of the retrying windows
void launch_wb_scatter(const Bufs &b, const WinBufs &w, cudaStream_t s);
// LU fallback for the n_failed windows whose Cholesky failed in this retry.
void launch_wb_lu(const Bufs &b, const WinBufs &w, int n_failed, cudaStream_t s);
void launch_wb_cost(const Bufs &b, const WinBufs &w, bool trial, cudaStream_t s);
void launch_wb_accept_commit(const Bufs &b, const WinBufs &w, cudaStream_t s);
void launch_wb_reject_failed(const WinBufs &w, cudaStream_t s);
void launch_wb_end_outer(const WinBufs &w, int max_iterations, bool polish_allowed, double target_cost,
                         cudaStream_t s);
void launch_wb_start_polish(const WinBufs &w, cudaStream_t s);
void launch_wb_summary(const WinBufs &w, cudaStream_t s);

}  // namespace sfmba
