// Batched local bundle adjustment: many independent windows concatenated
// into one block-diagonal problem. Observation, point and image kernels are
// shared with the single-problem path; this file holds what is per window:
// the LM state, the damped point inverses, the dense reduced systems (Schur
// reduction into per-window image-level blocks, fold to slot order, blocked
// FP64 Cholesky and triangular solves, refinement), the per-window cost and
// the accept / commit rules (crates/sfm-ba/src/lib.rs:914-1221, applied to
// each window independently as sfm-reconstruction's BaScope::Local calls
// would, lib.rs:1287-1299 there).
#include <cooperative_groups.h>

#include <type_traits>

#include "camera.cuh"
#include "chol_block.cuh"
#include "kernels.cuh"
#include "ozaki.cuh"
#include "schur.cuh"

namespace sfmba {

namespace {

constexpr int NB = kCholNB;
constexpr int LD = NB + 1;

// Which images and points take part in the current phase: outer-iteration
// kernels (linearisation, reductions) run for windows not done, retry
// kernels (point inverse, rhs, back-substitution) for windows retrying.
__global__ void k_wb_live(const WinState *ws, const int *img_win, const int *pt_win, int nI, int nP, int retry,
                          unsigned char *img_live, unsigned char *pt_live) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < nI) {
        const WinState &s = ws[img_win[t]];
        img_live[t] = retry ? (unsigned char)(s.active != 0) : (unsigned char)(s.done == 0);
    }
    if (t < nP) {
        const WinState &s = ws[pt_win[t]];
        pt_live[t] = retry ? (unsigned char)(s.active != 0) : (unsigned char)(s.done == 0);
    }
}

__global__ void k_wb_window_of_points(const int *win_in, const int *perm, int nP, int *pt_win) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < nP) pt_win[p] = win_in[perm[p]];
}

// After the initial cost: damping lambda0, nu = 2 (lib.rs:801-802); a window
// without unknowns returns at once (lib.rs:777-787).
__global__ void k_wb_init(WinState *ws, const int *n_w, int W, double lambda0) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= W) return;
    WinState &s = ws[w];
    s.lambda = lambda0;
    s.nu = 2.0;
    s.initial_cost = s.cost;
    s.cost_before = s.cost;
    s.lambda_start = lambda0;
    s.nu_start = 2.0;
    s.iterations = s.retries = s.retries_outer = 0;
    s.accepted = s.accepted_outer = s.active = 0;
    s.factor_failed = s.solve_failed = 0;
    s.done = n_w[w] == 0 ? 1 : 0;
    s.wants_polish = s.polished = 0;
    s.polish_iteration = -1;
}

__global__ void k_wb_begin_outer(WinState *ws, int W, int max_iterations) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= W) return;
    WinState &s = ws[w];
    s.accepted_outer = 0;
    s.retries_outer = 0;
    if (s.done) return;
    if (s.iterations >= max_iterations) {
        s.done = 1;
        return;
    }
    s.iterations += 1;
    s.cost_before = s.cost;
    s.lambda_start = s.lambda;
    s.nu_start = s.nu;
    if (s.valid_obs == 0) s.done = 1;  // lib.rs:855-857
}

__global__ void k_wb_begin_retry(WinState *ws, int W) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= W) return;
    WinState &s = ws[w];
    s.accepted = 0;
    s.factor_failed = 0;
    s.solve_failed = 0;
    s.active = (!s.done && !s.accepted_outer && s.retries_outer < kMaxDampingRetries) ? 1 : 0;
    if (s.active) {
        s.retries += 1;
        s.retries_outer += 1;
    }
}

// Damped point inverses with the damping of the point's window.
template <typename T>
__global__ void __launch_bounds__(kPointInvBlock)
    k_wb_point_inverse(const T *pt_C, const T *pt_g, const int *pt_nfree, const int *pt_win, const WinState *ws,
                       int nP, T *pt_Cinv, T *pt_h, unsigned char *pt_ok, const unsigned char *pt_live) {
    point_inverse_block<T>(pt_C, pt_g, pt_nfree, nP, [&](int q) { return ws[pt_win[q]].lambda; },
                           [&](int q) { return pt_live[q] != 0; }, pt_Cinv, pt_h, pt_ok);
}

// Launch shapes of the batched Schur reduction, picked by the autotuner in
// solver.cu: warps per block and the minimum resident blocks per SM (the
// register budget of the 7 x 4 tile sums and their Kahan terms). Every shape
// runs one warp per image pair with the same arithmetic, so the sums and
// results are the same. Measured on the 512-window batch (Schur phase of a
// whole FP32 batch): no cap 87 ms (157 registers), 5 blocks/SM 101 ms,
// 6 blocks/SM 123 ms, 8 blocks/SM 198 ms — the spills cost more than the
// extra warps gain; smaller tiles over 16 or 32 lanes (more warps, other
// rounding) took 83-157 ms. FP64: 800-818 ms for every cap (FP64-bound).
template <typename T, int V>
struct WbSchurShape {
    static constexpr bool kF = sizeof(T) == 4;
    static constexpr int kW = kF ? (V == 2 ? 2 : 4) : 2;
    static constexpr int kMinBlocks = kF ? (V == 0 ? 1 : V == 1 ? 5 : 10) : (V == 0 ? 1 : V == 1 ? 6 : 8);
};

// Schur reduction of the image pairs of every retrying window (one warp per
// pair, schur.cuh), written into the window's image-level block matrix.
template <typename T, int D, int V>
__global__ void __launch_bounds__(32 * WbSchurShape<T, V>::kW, WbSchurShape<T, V>::kMinBlocks)
    k_wb_schur_pairs(const T *__restrict__ rec, const int2 *__restrict__ pairs, const int *__restrict__ group_start,
                     const int2 *__restrict__ group_ij, const int *__restrict__ group_order, int ngroups,
                     const int *__restrict__ ob_pt,
                     const T *__restrict__ pt_Cinv, const unsigned char *__restrict__ pt_ok,
                     const double *__restrict__ img_H, const int *__restrict__ img_win,
                     const int *__restrict__ img_base, const int *__restrict__ nid_w,
                     const long long *__restrict__ simg_off, const WinState *__restrict__ ws,
                     double *__restrict__ S_img) {
    constexpr int W = WbSchurShape<T, V>::kW;
    using Tile = SchurTile<T, D>;
    __shared__ T sA[W][32][Tile::LDS];
    __shared__ T sP[W][32][Tile::LDS];
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (blockIdx.x * W + wl >= ngroups) return;
    const int g = group_order[blockIdx.x * W + wl];
    const int2 ij = group_ij[g];
    const int w = img_win[ij.x];
    if (!ws[w].active) return;
    double out[Tile::RH][Tile::CQ];
    schur_group<T, D>(rec, pairs, group_start[g], group_start[g + 1], ob_pt, pt_Cinv, pt_ok, sA[wl], sP[wl], lane,
                      out);
    if (lane >= Tile::LS) return;
    const int li = ij.x - img_base[w], lj = ij.y - img_base[w];
    const int nid = nid_w[w];
    double *Sw = S_img + simg_off[w];
    const int r0 = (lane >> 2) * Tile::RH, c0 = (lane & 3) * Tile::CQ;
#pragma unroll
    for (int a = 0; a < Tile::RH; ++a)
#pragma unroll
        for (int b = 0; b < Tile::CQ; ++b) {
            const int r = r0 + a, c = c0 + b;
            if (r >= D || c >= D) continue;
            const double v = out[a][b];
            if (li == lj) {
                Sw[(size_t)(li * D + r) * nid + li * D + c] = img_H[(size_t)ij.x * D * D + r * D + c] + v;
            } else {
                Sw[(size_t)(li * D + r) * nid + lj * D + c] = v;
                Sw[(size_t)(lj * D + c) * nid + li * D + r] = v;
            }
        }
}

// Window systems are factored in a permuted slot order (slot_perm: position
// -> slot, each image's pose slots followed by its camera's), in which the
// co-visibility of nearby images makes S banded. row_first[a] is the first
// nonzero column of row a of the permuted system; Cholesky keeps L inside
// that envelope, so the factorisation skips the tiles outside it.
__global__ void k_wb_envelope_init(const int *slot_win, const int *slot_base, int n, const WinState *ws,
                                   int *row_first) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    const int w = slot_win[a];
    if (ws[w].active) row_first[a] = a - slot_base[w];
}

__global__ void k_wb_gather_rhs(const int *slot_perm, const int *slot_win, int n, const double *rhs, double *rhs_p,
                                const WinState *ws) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    if (ws[slot_win[a]].active) rhs_p[a] = rhs[slot_perm[a]];
}

__global__ void k_wb_scatter_delta(const int *slot_perm, const int *slot_win, int n, const double *x_p,
                                   double *delta, const WinState *ws) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    const WinState &s = ws[slot_win[a]];
    if (s.active && !s.factor_failed) delta[slot_perm[a]] = x_p[a];
}

// Window w's system in permuted slot order: S[a][b] from its image-level
// blocks, damping with the window's lambda, masks, symmetrisation, and the
// envelope. One block per fold block {window, first row, end row} (about
// 8192 entries each, listed on the host), so windows that are not retrying
// cost one early exit per block.
__global__ void __launch_bounds__(128) k_wb_fold(const int4 *__restrict__ fold_blk, const double *__restrict__ S_img,
                                                 const long long *__restrict__ simg_off,
                                                 const int *__restrict__ nid_w, const int *__restrict__ n_w,
                                                 const int *__restrict__ slot_base, const long long *__restrict__ s_off,
                                                 const int *__restrict__ img_base, int D,
                                                 const int *__restrict__ slot_perm,
                                                 const int *__restrict__ pre_start, const int *__restrict__ pre,
                                                 const unsigned char *__restrict__ masked,
                                                 const double *__restrict__ diagB, const WinState *__restrict__ ws,
                                                 double *__restrict__ S, double *__restrict__ L,
                                                 int *__restrict__ row_first) {
    const int4 fb = fold_blk[blockIdx.x];
    const int w = fb.x;
    if (!ws[w].active) return;
    const int n = n_w[w];
    const int sb = slot_base[w];
    const int nid = nid_w[w];
    const int ub = img_base[w] * D;  // first image-level index of the window
    const double *Sw = S_img + simg_off[w];
    const double lam = ws[w].lambda;
    double *Sd = S + s_off[w], *Ld = L + s_off[w];
    for (int a = fb.y; a < fb.z; ++a) {
        const int ga = slot_perm[sb + a];
        const bool ma = masked[ga];
        const int as = pre_start[ga], ae = pre_start[ga + 1];
        int first = 0x7fffffff;
        for (int b0 = 0; b0 < n; b0 += blockDim.x) {
            const int b = b0 + threadIdx.x;
            if (b < n) {
                const int gb = slot_perm[sb + b];
                double v;
                if (ma || masked[gb]) {
                    v = a == b ? 1.0 : 0.0;
                } else {
                    double vab = 0.0, vba = 0.0;
                    for (int x = as; x < ae; ++x)
                        for (int y = pre_start[gb]; y < pre_start[gb + 1]; ++y) {
                            const int ux = pre[x] - ub, uy = pre[y] - ub;
                            vab += Sw[(size_t)ux * nid + uy];
                            vba += Sw[(size_t)uy * nid + ux];
                        }
                    v = 0.5 * (vab + vba);
                    if (a == b) v += diagB[ga] * lam;
                }
                Sd[(size_t)a * n + b] = v;
                Ld[(size_t)a * n + b] = v;
                if (b < a && v != 0.0 && b < first) first = b;
            }
        }
        first = __reduce_min_sync(0xffffffffu, first);
        if ((threadIdx.x & 31) == 0 && first < a) atomicMin(row_first + sb + a, first);
    }
}

// ---- batched blocked Cholesky (one matrix per window, leading dim n_w)

__global__ void __launch_bounds__(256) k_wb_chol_diag(double *Lall, const long long *s_off, const int *n_w,
                                                       double *Linv_all, const long long *linv_off, int k0,
                                                       WinState *ws) {
    extern __shared__ double sm[];
    double *A = sm;
    double *X = sm + NB * LD;
    __shared__ double buf[NB + 3];
    static_assert(LD == kBlkLD, "tile stride of chol_block_factor_invert");
    const int w = blockIdx.x;
    const int n = n_w[w];
    if (!ws[w].active || ws[w].factor_failed || k0 >= n) return;
    double *L = Lall + s_off[w];
    const int nb = min(NB, n - k0);
    const int tid = threadIdx.x;
    for (int idx = tid; idx < nb * nb; idx += blockDim.x) {
        const int r = idx / nb, c = idx - r * nb;
        A[r * LD + c] = c <= r ? L[(size_t)(k0 + r) * n + k0 + c] : 0.0;
    }
    __syncthreads();
    if (!chol_block_factor_invert(A, X, nb, buf)) {
        if (tid == 0) ws[w].factor_failed = 1;
        return;
    }
    for (int idx = tid; idx < nb * nb; idx += blockDim.x) {
        const int r = idx / nb, c = idx - r * nb;
        if (c <= r) L[(size_t)(k0 + r) * n + k0 + c] = A[r * LD + c];
    }
    double *out = Linv_all + linv_off[w] + (size_t)(k0 / NB) * NB * NB;
    for (int idx = tid; idx < NB * NB; idx += blockDim.x) {
        const int r = idx / NB, c = idx - r * NB;
        out[idx] = (r < nb && c < nb) ? X[r * LD + c] : 0.0;
    }
}

constexpr int PANEL_ROWS = 32;

__global__ void __launch_bounds__(256) k_wb_chol_panel(double *Lall, const long long *s_off, const int *n_w,
                                                        const double *Linv_all, const long long *linv_off, int k0,
                                                        const WinState *ws, const int *row_first,
                                                        const int *slot_base) {
    extern __shared__ double sm[];
    double *Li = sm;
    double *R = sm + NB * LD;
    const int w = blockIdx.y;
    const int n = n_w[w];
    if (!ws[w].active || ws[w].factor_failed || k0 >= n) return;
    double *L = Lall + s_off[w];
    const int nb = min(NB, n - k0);
    const int r0 = k0 + nb + blockIdx.x * PANEL_ROWS;
    const int rows = min(PANEL_ROWS, n - r0);
    if (rows <= 0) return;
    // rows whose envelope starts right of this column block stay zero
    const int *rf = row_first + slot_base[w];
    const bool outside = (int)threadIdx.x >= rows || rf[r0 + threadIdx.x] > k0 + nb - 1;
    if (__syncthreads_and(outside)) return;
    const double *inv = Linv_all + linv_off[w] + (size_t)(k0 / NB) * NB * NB;
    for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) Li[(idx / NB) * LD + idx % NB] = inv[idx];
    for (int idx = threadIdx.x; idx < rows * nb; idx += blockDim.x) {
        const int r = idx / nb, c = idx - r * nb;
        R[r * LD + c] = L[(size_t)(r0 + r) * n + k0 + c];
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < rows * nb; idx += blockDim.x) {
        const int r = idx / nb, c = idx - r * nb;
        double s = 0.0;
        for (int t = 0; t <= c; ++t) s += R[r * LD + t] * Li[c * LD + t];
        L[(size_t)(r0 + r) * n + k0 + c] = s;
    }
}

__global__ void __launch_bounds__(256) k_wb_chol_update(double *Lall, const long long *s_off, const int *n_w, int k0,
                                                         const WinState *ws, const int *row_first,
                                                         const int *slot_base) {
    extern __shared__ double sm[];
    double *Pi = sm;
    double *Pj = sm + NB * LD;
    const int w = blockIdx.y;
    const int n = n_w[w];
    if (!ws[w].active || ws[w].factor_failed || k0 + NB >= n) return;
    double *L = Lall + s_off[w];
    const int t0 = k0 + NB;
    const long long q = blockIdx.x;
    int ti = (int)((sqrt(8.0 * (double)q + 1.0) - 1.0) * 0.5);
    while ((long long)(ti + 1) * (ti + 2) / 2 <= q) ++ti;
    while ((long long)ti * (ti + 1) / 2 > q) --ti;
    const int tj = (int)(q - (long long)ti * (ti + 1) / 2);
    const int ri = t0 + ti * NB, rj = t0 + tj * NB;
    if (ri >= n || rj >= n) return;
    const int mi = min(NB, n - ri), mj = min(NB, n - rj);
    // a panel tile whose rows all start right of this column block is zero
    const int *rf = row_first + slot_base[w];
    const int tr = threadIdx.x;
    const bool nzi = tr < mi && rf[ri + tr] <= k0 + NB - 1;
    const bool nzj = tr < mj && rf[rj + tr] <= k0 + NB - 1;
    const int any_i = __syncthreads_or(nzi);
    const int any_j = __syncthreads_or(nzj);
    if (!any_i || !any_j) return;
    for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) {
        const int r = idx / NB, c = idx - r * NB;
        Pi[r * LD + c] = r < mi ? L[(size_t)(ri + r) * n + k0 + c] : 0.0;
        Pj[r * LD + c] = r < mj ? L[(size_t)(rj + r) * n + k0 + c] : 0.0;
    }
    __syncthreads();
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    double acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
    for (int t = 0; t < NB; ++t) {
        double x[4], y[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) x[a] = Pi[(ty * 4 + a) * LD + t];
#pragma unroll
        for (int b = 0; b < 4; ++b) y[b] = Pj[(tx + 16 * b) * LD + t];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) acc[a][b] += x[a] * y[b];
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const int r = ty * 4 + a;
        if (r >= mi) continue;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int c = tx + 16 * b;
            if (c >= mj) continue;
            if (ti == tj && c > r) continue;
            L[(size_t)(ri + r) * n + rj + c] -= acc[a][b];
        }
    }
}

// Tensor-core form of the two kernels above for the mixed batch (ozaki.cuh):
// slices and exponents of window w's panel rows (global slot index
// slot_base[w] + row; slices [kOzSlices][ntot][64]), then the trailing tiles.
__global__ void __launch_bounds__(256) k_wb_oz_split(const double *Lall, const long long *s_off, const int *n_w,
                                                      int k0, const WinState *ws, const int *slot_base, int ntot,
                                                      __nv_bfloat16 *slices, int *exps) {
    const int w = blockIdx.y;
    const int n = n_w[w];
    if (!ws[w].active || ws[w].factor_failed || k0 >= n) return;
    const int nb = min(NB, n - k0);
    const int r = k0 + nb + blockIdx.x * 8 + (threadIdx.x >> 5);
    if (r >= n) return;
    const int g = slot_base[w] + r;
    oz_split_row(Lall + s_off[w] + (size_t)r * n + k0, nb, threadIdx.x & 31, slices + (size_t)g * kOzK,
                 (size_t)ntot * kOzK, exps + g);
}

__global__ void __launch_bounds__(128, 1) k_wb_oz_update(double *Lall, const long long *s_off, const int *n_w, int k0,
                                                         const WinState *ws, const int *row_first,
                                                         const int *slot_base, int ntot,
                                                         const __nv_bfloat16 *slices, const int *exps) {
    extern __shared__ __align__(16) unsigned char oz_sm[];
    __shared__ double fR[kOzTile], fC[kOzTile];
    const int w = blockIdx.y;
    const int n = n_w[w];
    if (!ws[w].active || ws[w].factor_failed || k0 + NB >= n) return;
    const int t0 = k0 + NB;
    const long long q = blockIdx.x;
    int ti = (int)((sqrt(8.0 * (double)q + 1.0) - 1.0) * 0.5);
    while ((long long)(ti + 1) * (ti + 2) / 2 <= q) ++ti;
    while ((long long)ti * (ti + 1) / 2 > q) --ti;
    const int tj = (int)(q - (long long)ti * (ti + 1) / 2);
    const int ri = t0 + ti * kOzTile, rj = t0 + tj * kOzTile;
    if (ri >= n || rj >= n) return;
    const int mi = min(kOzTile, n - ri), mj = min(kOzTile, n - rj);
    // a panel tile whose rows all start right of this column block is zero
    const int sb = slot_base[w];
    const int *rf = row_first + sb;
    const int tr = threadIdx.x;
    const bool nzi = tr < mi && rf[ri + tr] <= k0 + NB - 1;
    const bool nzj = tr >= kOzTile && tr - kOzTile < mj && rf[rj + tr - kOzTile] <= k0 + NB - 1;
    const int any_i = __syncthreads_or(nzi);
    const int any_j = __syncthreads_or(nzj);
    if (!any_i || !any_j) return;
    oz_tile_update(Lall + s_off[w] + (size_t)ri * n + rj, (size_t)n, mi, mj, ti == tj,
                   slices + (size_t)(sb + ri) * kOzK, slices + (size_t)(sb + rj) * kOzK, (size_t)ntot * kOzK,
                   exps + sb + ri, exps + sb + rj, oz_sm, fR, fC);
}

// Whole triangular solve L L^T x = b of window w in one CTA (windows are at
// most a few hundred unknowns): forward with the diagonal-block inverses,
// then backward; b and x are the window's slices of the slot vectors.
__global__ void __launch_bounds__(256) k_wb_chol_solve(const double *Lall, const long long *s_off, const int *n_w,
                                                        const double *Linv_all, const long long *linv_off,
                                                        const int *slot_base, const double *rhs, double *work,
                                                        double *x, const WinState *ws, const int *row_first) {
    __shared__ double yk[NB];
    __shared__ int blk_first;
    const int w = blockIdx.x;
    if (!ws[w].active || ws[w].factor_failed) return;
    const int n = n_w[w];
    if (n == 0) return;
    const double *L = Lall + s_off[w];
    const double *Linv = Linv_all + linv_off[w];
    double *b = work + slot_base[w];
    double *xo = x + slot_base[w];
    const int *rf = row_first + slot_base[w];
    for (int a = threadIdx.x; a < n; a += blockDim.x) b[a] = rhs[slot_base[w] + a];
    __syncthreads();
    // forward: y_k = Lkk^-1 b_k; b_r -= L[r, k] y_k for r below
    for (int k0 = 0; k0 < n; k0 += NB) {
        const int nb = min(NB, n - k0);
        const double *inv = Linv + (size_t)(k0 / NB) * NB * NB;
        if (threadIdx.x < nb) {
            double s = 0.0;
            for (int t = 0; t <= (int)threadIdx.x; ++t) s += inv[threadIdx.x * NB + t] * b[k0 + t];
            yk[threadIdx.x] = s;
        }
        __syncthreads();
        if (threadIdx.x < nb) b[k0 + threadIdx.x] = yk[threadIdx.x];
        for (int r = k0 + nb + threadIdx.x; r < n; r += blockDim.x) {
            if (rf[r] > k0 + nb - 1) continue;  // L[r, block] is outside the envelope
            double s = 0.0;
            for (int t = 0; t < nb; ++t) s += L[(size_t)r * n + k0 + t] * yk[t];
            b[r] -= s;
        }
        __syncthreads();
    }
    // backward: x_k = Lkk^-T y_k; y_r -= L[k, r]^T x_k for r above
    for (int k0 = ((n - 1) / NB) * NB; k0 >= 0; k0 -= NB) {
        const int nb = min(NB, n - k0);
        const double *inv = Linv + (size_t)(k0 / NB) * NB * NB;
        if (threadIdx.x < nb) {
            double s = 0.0;
            for (int r = threadIdx.x; r < nb; ++r) s += inv[r * NB + threadIdx.x] * b[k0 + r];
            yk[threadIdx.x] = s;
        }
        __syncthreads();
        if (threadIdx.x < nb) xo[k0 + threadIdx.x] = yk[threadIdx.x];
        if (threadIdx.x == 0) blk_first = k0;
        __syncthreads();
        if (threadIdx.x < nb) atomicMin(&blk_first, rf[k0 + threadIdx.x]);
        __syncthreads();
        // L[k0.., r] is zero for columns r left of every row's envelope
        for (int r = blk_first + threadIdx.x; r < k0; r += blockDim.x) {
            double s = 0.0;
            for (int t = 0; t < nb; ++t) s += L[(size_t)(k0 + t) * n + r] * yk[t];
            b[r] -= s;
        }
        __syncthreads();
    }
}

// res = rhs - S x for window w (one CTA per window), the FP64 residual of
// one refinement step.
__global__ void __launch_bounds__(256) k_wb_residual(const double *Sall, const long long *s_off, const int *n_w,
                                                      const int *slot_base, const double *x, const double *rhs,
                                                      double *res, const WinState *ws) {
    const int w = blockIdx.x;
    if (!ws[w].active || ws[w].factor_failed) return;
    const int n = n_w[w];
    const double *S = Sall + s_off[w];
    const double *xw = x + slot_base[w];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int r = warp; r < n; r += blockDim.x >> 5) {
        double s = 0.0;
        for (int c = lane; c < n; c += 32) s += S[(size_t)r * n + c] * xw[c];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        if (lane == 0) res[slot_base[w] + r] = rhs[slot_base[w] + r] - s;
    }
}

__global__ void k_wb_axpy(const int *slot_win, int n, const double *c, double *x, const WinState *ws) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    const WinState &s = ws[slot_win[a]];
    if (s.active && !s.factor_failed) x[a] += c[a];
}

// Per-window FP64 cost in two deterministic passes: blocks of up to
// kWinCostChunk observations (a window's observations are contiguous in
// point-major order) write partial sums, then each window adds its blocks in
// order. trial = 0 -> cost, valid_obs; 1 -> trial_cost, trial_valid_obs of
// the windows whose step was solved.
__global__ void __launch_bounds__(256) k_wb_cost_partials(
    const double *rt, const double *cams, const double *points, const int *cam_of_img, const int *cam_model,
    const int *ob_img, const int *ob_pt, const double2 *ob_xy, const int *cblk_win, const long long *cblk_lo,
    int loss, double scale, int trial, const WinState *ws, double *cpart, long long *cpart_n, float4 *rs_out) {
    __shared__ double ssum[256];
    __shared__ long long scnt[256];
    const int blk = blockIdx.x;
    const int w = cblk_win[blk];
    if (trial && !(ws[w].active && !ws[w].factor_failed)) return;
    double sum = 0.0;
    long long cnt = 0;
    for (long long o = cblk_lo[blk] + threadIdx.x; o < cblk_lo[blk + 1]; o += blockDim.x) {
        const int i = ob_img[o], p = ob_pt[o];
        const int c = cam_of_img[i];
        const double *X = points + 3 * (size_t)p;
        const double2 xy = ob_xy[o];
        double rx, ry;
        const bool ok = residual64_rt(rt + 12 * (size_t)i, cam_model[c], cams + 8 * (size_t)c, X[0], X[1], X[2],
                                      xy.x, xy.y, rx, ry);
        double w = 1.0;
        if (ok) {
            const double n2 = rx * rx + ry * ry;
            if (loss == SFMBA_LOSS_NONE) sum += n2;
            else {
                const double nn = sqrt(n2);
                w = robust_weight<double>(nn, loss, scale);
                sum += w * nn * nn;
            }
            ++cnt;
        }
        // FP64 residual and sqrt(weight) for the next linearisation (FP32 records)
        if (rs_out) rs_out[o] = ok ? make_float4((float)rx, (float)ry, (float)sqrt(w), 1.f) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    ssum[threadIdx.x] = sum;
    scnt[threadIdx.x] = cnt;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if (threadIdx.x < h) {
            ssum[threadIdx.x] += ssum[threadIdx.x + h];
            scnt[threadIdx.x] += scnt[threadIdx.x + h];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        cpart[blk] = ssum[0];
        cpart_n[blk] = scnt[0];
    }
}

// k_wb_cost_partials for the FP32 batch with the projection in double-float
// arithmetic (the pair copies of b.df_cost; robust weights and block sums
// FP64), as the single-problem FP32 cost.
__global__ void __launch_bounds__(256) k_wb_cost_partials_df(
    const float *rt_df, const float *cams_df, const float4 *pts_df, const int *cam_of_img, const int *cam_model,
    const int *ob_img, const int *ob_pt, const float4 *xy_df, const int *cblk_win, const long long *cblk_lo,
    int loss, double scale, int trial, const WinState *ws, double *cpart, long long *cpart_n, float4 *rs_out) {
    __shared__ double ssum[256];
    __shared__ long long scnt[256];
    const int blk = blockIdx.x;
    const int w = cblk_win[blk];
    if (trial && !(ws[w].active && !ws[w].factor_failed)) return;
    dfl sum2 = df_make(0.f);
    double wsum = 0.0;
    long long cnt = 0;
    for (long long o = cblk_lo[blk] + threadIdx.x; o < cblk_lo[blk + 1]; o += blockDim.x) {
        const int i = ob_img[o], p = ob_pt[o];
        const int c = cam_of_img[i];
        dfl rt[12], cp[8];
        const float4 *r4 = reinterpret_cast<const float4 *>(rt_df + 24 * (size_t)i);
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const float4 v = __ldg(r4 + k);
            rt[2 * k] = {v.x, v.y};
            rt[2 * k + 1] = {v.z, v.w};
        }
        const float4 *c4 = reinterpret_cast<const float4 *>(cams_df + 16 * (size_t)c);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float4 v = __ldg(c4 + k);
            cp[2 * k] = {v.x, v.y};
            cp[2 * k + 1] = {v.z, v.w};
        }
        const float4 pa = pts_df[2 * (size_t)p], pb = pts_df[2 * (size_t)p + 1];
        const float4 xy = xy_df[o];
        dfl rx, ry;
        const bool ok = residual_df(rt, cam_model[c], cp, {pa.x, pa.y}, {pa.z, pa.w}, {pb.x, pb.y}, {xy.x, xy.y},
                                    {xy.z, xy.w}, rx, ry);
        float sw = 1.f;
        if (ok) {
            const dfl n2 = rx * rx + ry * ry;
            if (loss == SFMBA_LOSS_NONE) sum2 = sum2 + n2;
            else {
                const double nn = sqrt(df_to_double(n2)), wt = robust_weight<double>(nn, loss, scale);
                wsum += wt * nn * nn;
                sw = (float)sqrt(wt);
            }
            ++cnt;
        }
        if (rs_out) rs_out[o] = ok ? make_float4(rx.hi, ry.hi, sw, 1.f) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    ssum[threadIdx.x] = df_to_double(sum2) + wsum;
    scnt[threadIdx.x] = cnt;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if (threadIdx.x < h) {
            ssum[threadIdx.x] += ssum[threadIdx.x + h];
            scnt[threadIdx.x] += scnt[threadIdx.x + h];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        cpart[blk] = ssum[0];
        cpart_n[blk] = scnt[0];
    }
}

__global__ void k_wb_cost_finalize(const int *wblk_start, const double *cpart, const long long *cpart_n, int W,
                                   int trial, WinState *ws) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= W) return;
    WinState &s = ws[w];
    if (trial && !(s.active && !s.factor_failed)) return;
    double sum = 0.0;
    long long cnt = 0;
    for (int k = wblk_start[w]; k < wblk_start[w + 1]; ++k) {
        sum += cpart[k];
        cnt += cpart_n[k];
    }
    if (trial) {
        s.trial_cost = sum;
        s.trial_valid_obs = cnt;
    } else {
        s.cost = sum;
        s.valid_obs = cnt;
    }
}

// Accept / reject per retrying window (lib.rs:1188-1212); a window decided
// here leaves the retry round.
__global__ void k_wb_accept(WinState *ws, int W) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= W) return;
    WinState &s = ws[w];
    if (!s.active || s.factor_failed) return;
    const double t = s.trial_cost;
    if (isfinite(t) && t < s.cost) {
        s.accepted = 1;
        s.accepted_outer = 1;
        s.cost = t;
        s.valid_obs = s.trial_valid_obs;
        s.lambda = fmax(s.lambda / 3.0, 1e-12);
        s.nu = 2.0;
    } else {
        s.lambda *= s.nu;
        s.nu *= 2.0;
    }
    s.active = 0;
}

// Windows whose Cholesky and LU both failed: grow the damping (lib.rs:1089-1091).
__global__ void k_wb_reject_failed(WinState *ws, int W) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= W) return;
    WinState &s = ws[w];
    if (!s.active || !s.factor_failed) return;
    s.lambda *= s.nu;
    s.nu *= 2.0;
    s.active = 0;
}

// Trial parameters of the windows accepted in this retry become current.
__global__ void k_wb_commit(const WinState *ws, const int *pt_win, const int *img_win, const int *cam_win, int nI,
                            int nC, int nP, const double *poses_trial, const double *cams_trial,
                            const double *points_trial, double *poses, double *cams, double *points,
                            float4 *points32, long long nO, const int *ob_pt, const float4 *rs_trial, float4 *rs) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (rs && t < nO && ws[pt_win[ob_pt[t]]].accepted) rs[t] = rs_trial[t];
    if (t < nP && ws[pt_win[t]].accepted) {
        const double x = points_trial[3 * t], y = points_trial[3 * t + 1], z = points_trial[3 * t + 2];
        points[3 * t] = x; points[3 * t + 1] = y; points[3 * t + 2] = z;
        if (points32) points32[t] = make_float4((float)x, (float)y, (float)z, 0.f);
    }
    if (t < 7LL * nI && ws[img_win[t / 7]].accepted) poses[t] = poses_trial[t];
    if (t < 8LL * nC && ws[cam_win[t / 8]].accepted) cams[t] = cams_trial[t];
}

// End of an outer iteration (lib.rs:1215-1221): a window with no accepted
// retry, or a relative decrease below 1e-6, stops. On the mixed path with
// the FP64 polish it is parked instead (damping of a failed iteration
// restored) until the whole batch continues in FP64.
__global__ void k_wb_end_outer(WinState *ws, int W, int max_iterations, int polish_allowed, double target_cost) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= W) return;
    WinState &s = ws[w];
    if (s.done) return;
    bool stop;
    if (!s.accepted_outer) {
        stop = true;
    } else {
        if (target_cost > 0.0 && s.cost <= target_cost) {
            s.done = 1;
            return;
        }
        const double rel = (s.cost_before - s.cost) / fmax(s.cost_before, 1e-12);
        stop = rel < kFunctionTolerance;
    }
    if (stop && polish_allowed && !s.polished && isfinite(s.cost) && s.iterations < max_iterations) {
        s.wants_polish = 1;
        s.polish_iteration = s.iterations;
        if (!s.accepted_outer) {
            s.lambda = s.lambda_start;
            s.nu = s.nu_start;
        }
        s.done = 1;
        return;
    }
    if (stop || s.iterations >= max_iterations) s.done = 1;
}

__global__ void k_wb_start_polish(WinState *ws, int W) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= W) return;
    WinState &s = ws[w];
    s.polished = 1;
    if (s.wants_polish) {
        s.wants_polish = 0;
        s.done = 0;
    }
}

// Batch summary for the host (one block); clears the per-retry accept flags
// once the commit has consumed them.
__global__ void __launch_bounds__(256) k_wb_summary(WinState *ws, int W, int *counts) {
    __shared__ int red[4][256];
    int c[4] = {0, 0, 0, 0};
    for (int w = threadIdx.x; w < W; w += blockDim.x) {
        WinState &s = ws[w];
        s.accepted = 0;
        c[WB_NOT_DONE] += !s.done;
        c[WB_RETRY_PENDING] += (!s.done && !s.accepted_outer && s.retries_outer < kMaxDampingRetries);
        c[WB_FACTOR_FAILED] += (s.active && s.factor_failed);
        c[WB_WANTS_POLISH] += s.wants_polish;
    }
    for (int k = 0; k < 4; ++k) red[k][threadIdx.x] = c[k];
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if (threadIdx.x < h)
            for (int k = 0; k < 4; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x < 4) counts[threadIdx.x] = red[threadIdx.x][0];
}

// Partial-pivoting LU of the windows whose Cholesky failed (lib.rs:1084-1092),
// on the permuted system, for all of them at once: a compact list of the
// failing windows, then per column k one pivot launch (one block per
// window) and one rank-1 update launch spread over the GPU, then a
// per-window solve. Column k pivots on the first maximum |a|; a zero column
// is skipped and leaves a zero on U's diagonal, which fails the solve
// (lambda then grows). Success clears factor_failed.
__global__ void k_wb_failed_list(const WinState *ws, int W, int *list, int *count) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= W) return;
    if (ws[w].active && ws[w].factor_failed && !ws[w].solve_failed) list[atomicAdd(count, 1)] = w;
}

__global__ void k_wb_lu_copy(const double *Sall, double *Lall, const long long *s_off, const int *n_w,
                             const int *list) {
    const int w = list[blockIdx.y];
    const long long nn = (long long)n_w[w] * n_w[w];
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nn; i += (long long)gridDim.x * blockDim.x)
        Lall[s_off[w] + i] = Sall[s_off[w] + i];
}

__global__ void __launch_bounds__(256) k_wb_lu_pivot(double *Lall, const long long *s_off, const int *n_w,
                                                     const int *slot_base, int *perm_all, const int *list, int k) {
    __shared__ double bv[256];
    __shared__ int bi[256];
    const int w = list[blockIdx.x];
    const int n = n_w[w];
    if (k >= n) return;
    double *A = Lall + s_off[w];
    int *perm = perm_all + slot_base[w];
    const int tid = threadIdx.x;
    double best = -1.0;
    int besti = k;
    for (int r = k + tid; r < n; r += blockDim.x) {
        const double v = fabs(A[(size_t)r * n + k]);
        if (v > best) { best = v; besti = r; }
    }
    bv[tid] = best;
    bi[tid] = besti;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if (tid < h) {
            const double o = bv[tid + h];
            const int oi = bi[tid + h];
            if (o > bv[tid] || (o == bv[tid] && oi < bi[tid])) { bv[tid] = o; bi[tid] = oi; }
        }
        __syncthreads();
    }
    const int piv = bi[0];
    const double diag = A[(size_t)piv * n + k];
    if (diag == 0.0) {
        if (tid == 0) perm[k] = -1;
        return;
    }
    if (piv != k)
        for (int c = tid; c < n; c += blockDim.x) {
            const double t = A[(size_t)k * n + c];
            A[(size_t)k * n + c] = A[(size_t)piv * n + c];
            A[(size_t)piv * n + c] = t;
        }
    if (tid == 0) perm[k] = piv;
    __syncthreads();
    for (int r = k + 1 + tid; r < n; r += blockDim.x) A[(size_t)r * n + k] /= diag;
}

// Rows k+1.. of the trailing matrix: grid (column blocks, rows, windows).
__global__ void k_wb_lu_update(double *Lall, const long long *s_off, const int *n_w, const int *slot_base,
                               const int *perm_all, const int *list, int k) {
    const int w = list[blockIdx.z];
    const int n = n_w[w];
    const int r = k + 1 + blockIdx.y;
    const int c = k + 1 + blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n || c >= n) return;
    if (perm_all[slot_base[w] + k] < 0) return;
    double *A = Lall + s_off[w];
    A[(size_t)r * n + c] -= A[(size_t)r * n + k] * A[(size_t)k * n + c];
}

// The column loop of the two kernels above in one cooperative launch: per
// column k, the failed windows' pivots (a block per window, grid-stride),
// a grid barrier, the rank-1 updates of all their trailing rows (a block per
// (window, row), grid-stride), a grid barrier: 2 barriers per column
// instead of 2 launches. Same arithmetic in the same order.
__global__ void __launch_bounds__(256) k_wb_lu_coop(double *Lall, const long long *s_off, const int *n_w,
                                                     const int *slot_base, int *perm_all, const int *list, int nf,
                                                     int max_n) {
    namespace cg = cooperative_groups;
    cg::grid_group grid = cg::this_grid();
    __shared__ double bv[256];
    __shared__ int bi[256];
    const int tid = threadIdx.x;
    for (int k = 0; k < max_n; ++k) {
        for (int f = blockIdx.x; f < nf; f += gridDim.x) {
            const int w = list[f];
            const int n = n_w[w];
            if (k >= n) continue;
            double *A = Lall + s_off[w];
            int *perm = perm_all + slot_base[w];
            double best = -1.0;
            int besti = k;
            for (int r = k + tid; r < n; r += blockDim.x) {
                const double v = fabs(A[(size_t)r * n + k]);
                if (v > best) { best = v; besti = r; }
            }
            bv[tid] = best;
            bi[tid] = besti;
            __syncthreads();
            for (int h = blockDim.x / 2; h > 0; h >>= 1) {
                if (tid < h) {
                    const double o = bv[tid + h];
                    const int oi = bi[tid + h];
                    if (o > bv[tid] || (o == bv[tid] && oi < bi[tid])) { bv[tid] = o; bi[tid] = oi; }
                }
                __syncthreads();
            }
            const int piv = bi[0];
            const double diag = A[(size_t)piv * n + k];
            if (diag != 0.0) {
                if (piv != k)
                    for (int c = tid; c < n; c += blockDim.x) {
                        const double t = A[(size_t)k * n + c];
                        A[(size_t)k * n + c] = A[(size_t)piv * n + c];
                        A[(size_t)piv * n + c] = t;
                    }
                __syncthreads();
                for (int r = k + 1 + tid; r < n; r += blockDim.x) A[(size_t)r * n + k] /= diag;
            }
            if (tid == 0) perm[k] = diag != 0.0 ? piv : -1;
            __syncthreads();  // bv / bi are reused by the next window
        }
        grid.sync();
        const int m = max_n - k - 1;
        if (m <= 0) break;
        for (long long q = blockIdx.x; q < (long long)nf * m; q += gridDim.x) {
            const int f = (int)(q / m), r = k + 1 + (int)(q - (long long)f * m);
            const int w = list[f];
            const int n = n_w[w];
            if (r >= n || perm_all[slot_base[w] + k] < 0) continue;
            double *A = Lall + s_off[w];
            const double lrk = A[(size_t)r * n + k];
            for (int c = k + 1 + tid; c < n; c += blockDim.x) A[(size_t)r * n + c] -= lrk * A[(size_t)k * n + c];
        }
        grid.sync();
    }
}

__global__ void __launch_bounds__(1024) k_wb_lu_solve(const double *Lall, const long long *s_off, const int *n_w,
                                                       const int *slot_base, const int *perm_all, const int *list,
                                                       const double *rhs, double *x, WinState *ws) {
    __shared__ double red[32];
    __shared__ int bad;
    const int w = list[blockIdx.x];
    WinState &st = ws[w];
    const int n = n_w[w];
    const double *A = Lall + s_off[w];
    const int *perm = perm_all + slot_base[w];
    const double *b = rhs + slot_base[w];
    double *xo = x + slot_base[w];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int a = tid; a < n; a += blockDim.x) xo[a] = b[a];
    if (tid == 0) bad = 0;
    __syncthreads();
    if (tid == 0)
        for (int k = 0; k < n; ++k)
            if (perm[k] >= 0 && perm[k] != k) {
                const double t = xo[k];
                xo[k] = xo[perm[k]];
                xo[perm[k]] = t;
            }
    __syncthreads();
    // forward (unit lower), then backward (upper); block reductions per row
    for (int pass = 0; pass < 2; ++pass) {
        for (int q = 0; q < n; ++q) {
            const int i = pass == 0 ? q : n - 1 - q;
            const int lo = pass == 0 ? 0 : i + 1, hi = pass == 0 ? i : n;
            double sum = 0.0;
            for (int k = lo + tid; k < hi; k += blockDim.x) sum += A[(size_t)i * n + k] * xo[k];
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, off);
            if (lane == 0) red[warp] = sum;
            __syncthreads();
            if (tid == 0) {
                double t = 0.0;
                for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
                if (pass == 0) {
                    xo[i] -= t;
                } else {
                    const double d = A[(size_t)i * n + i];
                    if (d == 0.0) bad = 1;
                    else xo[i] = (xo[i] - t) / d;
                }
            }
            __syncthreads();
            if (bad) break;
        }
    }
    if (tid == 0) {
        if (bad) st.solve_failed = 1;
        else st.factor_failed = 0;
    }
}

template <typename F>
void dispatch_D(int D, F &&f) {
    switch (D) {
    case 6: f(std::integral_constant<int, 6>()); break;
    case 9: f(std::integral_constant<int, 9>()); break;
    case 10: f(std::integral_constant<int, 10>()); break;
    case 11: f(std::integral_constant<int, 11>()); break;
    case 14: f(std::integral_constant<int, 14>()); break;
    default: throw Error(SFMBA_ERR_INTERNAL, "unsupported image block width");
    }
}

const size_t kSmemTwoTiles = 2 * NB * LD * sizeof(double);
const size_t kSmemPanel = (NB + PANEL_ROWS) * LD * sizeof(double);

void set_smem_limits() {
    static bool done = false;
    if (done) return;
    SFMBA_CUDA(cudaFuncSetAttribute(k_wb_chol_diag, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemTwoTiles));
    SFMBA_CUDA(cudaFuncSetAttribute(k_wb_chol_update, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemTwoTiles));
    SFMBA_CUDA(cudaFuncSetAttribute(k_wb_chol_panel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemPanel));
    SFMBA_CUDA(cudaFuncSetAttribute(k_wb_oz_update, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kOzSmem));
    done = true;
}

int grid1(int n) { return div_up(n > 0 ? n : 1, 128); }

}  // namespace

void launch_wb_window_of_points(const int *win_of_input_point, const int *perm, int nP, int *pt_win,
                                cudaStream_t s) {
    if (nP == 0) return;
    k_wb_window_of_points<<<div_up(nP, 256), 256, 0, s>>>(win_of_input_point, perm, nP, pt_win);
    SFMBA_LAUNCH_CHECK();
}

void launch_wb_live(const Bufs &b, const WinBufs &w, bool retry, cudaStream_t s) {
    const long long m = b.nP > b.nI ? b.nP : b.nI;
    if (m == 0) return;
    k_wb_live<<<div_up(m, 256), 256, 0, s>>>(w.ws, w.img_win, w.pt_win, b.nI, b.nP, retry ? 1 : 0, b.img_live,
                                             b.pt_live);
    SFMBA_LAUNCH_CHECK();
}

void launch_wb_init(const WinBufs &w, double initial_lambda, cudaStream_t s) {
    k_wb_init<<<grid1(w.W), 128, 0, s>>>(w.ws, w.n_w, w.W, initial_lambda);
    SFMBA_LAUNCH_CHECK();
}

void launch_wb_begin_outer(const WinBufs &w, int max_iterations, cudaStream_t s) {
    k_wb_begin_outer<<<grid1(w.W), 128, 0, s>>>(w.ws, w.W, max_iterations);
    SFMBA_LAUNCH_CHECK();
}

void launch_wb_begin_retry(const WinBufs &w, cudaStream_t s) {
    k_wb_begin_retry<<<grid1(w.W), 128, 0, s>>>(w.ws, w.W);
    SFMBA_LAUNCH_CHECK();
}

void launch_wb_point_inverse(const Bufs &b, const WinBufs &w, cudaStream_t s) {
    if (b.nP == 0) return;
    if (b.mixed)
        k_wb_point_inverse<float><<<div_up(b.nP, kPointInvBlock), kPointInvBlock, 0, s>>>((const float *)b.pt_C, (const float *)b.pt_g,
                                                                    b.pt_nfree, w.pt_win, w.ws, b.nP,
                                                                    (float *)b.pt_Cinv, (float *)b.pt_h, b.pt_ok,
                                                                    b.pt_live);
    else
        k_wb_point_inverse<double><<<div_up(b.nP, kPointInvBlock), kPointInvBlock, 0, s>>>((const double *)b.pt_C, (const double *)b.pt_g,
                                                                     b.pt_nfree, w.pt_win, w.ws, b.nP,
                                                                     (double *)b.pt_Cinv, (double *)b.pt_h, b.pt_ok,
                                                                     b.pt_live);
    SFMBA_LAUNCH_CHECK();
}

template <typename T, int V>
void wb_schur_v(const Bufs &b, const WinBufs &w, cudaStream_t s) {
    constexpr int W = WbSchurShape<T, V>::kW;
    dispatch_D(b.D, [&](auto dc) {
        constexpr int D = decltype(dc)::value;
        k_wb_schur_pairs<T, D, V><<<div_up(b.ngroups, W), 32 * W, 0, s>>>(
            (const T *)b.rec, b.pairs, b.group_start, b.group_ij, b.group_order, b.ngroups, b.ob_pt,
            (const T *)b.pt_Cinv, b.pt_ok, b.img_H, w.img_win, w.img_base, w.nid_w, w.simg_off, w.ws, b.S_img);
    });
}

template <typename T>
void wb_schur_t(const Bufs &b, const WinBufs &w, cudaStream_t s, int variant) {
    switch (variant) {
    case 0: wb_schur_v<T, 0>(b, w, s); break;
    case 1: wb_schur_v<T, 1>(b, w, s); break;
    default: wb_schur_v<T, 2>(b, w, s); break;
    }
}

void launch_wb_schur(const Bufs &b, const WinBufs &w, cudaStream_t s, int variant) {
    if (b.ngroups == 0) return;
    if (b.mixed) wb_schur_t<float>(b, w, s, variant);
    else wb_schur_t<double>(b, w, s, variant);
    SFMBA_LAUNCH_CHECK();
}

void launch_wb_fold(const Bufs &b, const WinBufs &w, cudaStream_t s) {
    if (w.max_n == 0 || b.n == 0) return;
    k_wb_envelope_init<<<div_up(b.n, 256), 256, 0, s>>>(w.slot_win, w.slot_base, b.n, w.ws, w.row_first);
    SFMBA_LAUNCH_CHECK();
    k_wb_gather_rhs<<<div_up(b.n, 256), 256, 0, s>>>(w.slot_perm, w.slot_win, b.n, b.rhs, w.rhs_p, w.ws);
    SFMBA_LAUNCH_CHECK();
    if (w.n_fold_blk == 0) return;
    k_wb_fold<<<w.n_fold_blk, 128, 0, s>>>(w.fold_blk, b.S_img, w.simg_off, w.nid_w, w.n_w, w.slot_base, w.s_off,
                                           w.img_base, b.D, w.slot_perm, b.slot_pre_start, b.slot_pre,
                                           b.slot_masked, b.diagB, w.ws, b.S, b.L, w.row_first);
    SFMBA_LAUNCH_CHECK();
}

void launch_wb_cholesky(const Bufs &b, const WinBufs &w, cudaStream_t s) {
    set_smem_limits();
    for (int k0 = 0; k0 < w.max_n; k0 += NB) {
        k_wb_chol_diag<<<w.W, 256, kSmemTwoTiles, s>>>(b.L, w.s_off, w.n_w, b.Linv, w.linv_off, k0, w.ws);
        SFMBA_LAUNCH_CHECK();
        const int rem = w.max_n - k0 - NB;
        if (rem <= 0) break;
        dim3 gp(div_up(rem, PANEL_ROWS), w.W);
        k_wb_chol_panel<<<gp, 256, kSmemPanel, s>>>(b.L, w.s_off, w.n_w, b.Linv, w.linv_off, k0, w.ws, w.row_first,
                                                    w.slot_base);
        SFMBA_LAUNCH_CHECK();
        const long long tiles = div_up(rem, NB);
        dim3 gu((unsigned)(tiles * (tiles + 1) / 2), w.W);
        if (b.oz_slices) {  // tensor-core update (ozaki.cuh)
            k_wb_oz_split<<<dim3(div_up(rem, 8), w.W), 256, 0, s>>>(b.L, w.s_off, w.n_w, k0, w.ws, w.slot_base, b.n,
                                                                    (__nv_bfloat16 *)b.oz_slices, b.oz_exp);
            SFMBA_LAUNCH_CHECK();
            k_wb_oz_update<<<gu, 128, kOzSmem, s>>>(b.L, w.s_off, w.n_w, k0, w.ws, w.row_first, w.slot_base, b.n,
                                                    (const __nv_bfloat16 *)b.oz_slices, b.oz_exp);
        } else {
            k_wb_chol_update<<<gu, 256, kSmemTwoTiles, s>>>(b.L, w.s_off, w.n_w, k0, w.ws, w.row_first, w.slot_base);
        }
        SFMBA_LAUNCH_CHECK();
    }
}

// Solves of the permuted window systems: rhs_p -> x_p = b.work2 (b.work is
// the solve's scratch).
void launch_wb_solve(const Bufs &b, const WinBufs &w, const double *rhs, double *x, cudaStream_t s) {
    k_wb_chol_solve<<<w.W, 256, 0, s>>>(b.L, w.s_off, w.n_w, b.Linv, w.linv_off, w.slot_base, rhs, b.work, x, w.ws,
                                        w.row_first);
    SFMBA_LAUNCH_CHECK();
}

void launch_wb_refine(const Bufs &b, const WinBufs &w, cudaStream_t s) {
    k_wb_residual<<<w.W, 256, 0, s>>>(b.S, w.s_off, w.n_w, w.slot_base, b.work2, w.rhs_p, b.ref_res, w.ws);
    SFMBA_LAUNCH_CHECK();
    launch_wb_solve(b, w, b.ref_res, b.ref_corr, s);
    if (b.n > 0) {
        k_wb_axpy<<<div_up(b.n, 256), 256, 0, s>>>(w.slot_win, b.n, b.ref_corr, b.work2, w.ws);
        SFMBA_LAUNCH_CHECK();
    }
}

void launch_wb_scatter(const Bufs &b, const WinBufs &w, cudaStream_t s) {
    if (b.n == 0) return;
    k_wb_scatter_delta<<<div_up(b.n, 256), 256, 0, s>>>(w.slot_perm, w.slot_win, b.n, b.work2, b.delta, w.ws);
    SFMBA_LAUNCH_CHECK();
}

void launch_wb_cost(const Bufs &b, const WinBufs &w, bool trial, cudaStream_t s) {
    if (w.ncblk > 0 && b.mixed && b.df_cost) {
        launch_pose_rt64(trial ? b.poses_trial : b.poses, b.nI, b.img_rt64, s);
        launch_split_df(b, trial, s);
        k_wb_cost_partials_df<<<w.ncblk, 256, 0, s>>>(
            b.rt_df, b.cams_df, b.pts_df, b.cam_of_img, b.cam_model, b.ob_img, b.ob_pt, b.ob_xy_df, w.cblk_win,
            w.cblk_lo, b.loss, b.loss_scale, trial ? 1 : 0, w.ws, w.cpart, w.cpart_n,
            b.ob_rs ? (trial ? b.ob_rs_trial : b.ob_rs) : nullptr);
        SFMBA_LAUNCH_CHECK();
    } else if (w.ncblk > 0) {
        launch_pose_rt64(trial ? b.poses_trial : b.poses, b.nI, b.img_rt64, s);
        k_wb_cost_partials<<<w.ncblk, 256, 0, s>>>(
            b.img_rt64, trial ? b.cams_trial : b.cams, trial ? b.points_trial : b.points,
            b.cam_of_img, b.cam_model, b.ob_img, b.ob_pt, b.ob_xy, w.cblk_win, w.cblk_lo, b.loss, b.loss_scale,
            trial ? 1 : 0, w.ws, w.cpart, w.cpart_n,
            (b.mixed && b.ob_rs) ? (trial ? b.ob_rs_trial : b.ob_rs) : nullptr);
        SFMBA_LAUNCH_CHECK();
    }
    k_wb_cost_finalize<<<grid1(w.W), 128, 0, s>>>(w.wblk_start, w.cpart, w.cpart_n, w.W, trial ? 1 : 0, w.ws);
    SFMBA_LAUNCH_CHECK();
}

void launch_wb_accept_commit(const Bufs &b, const WinBufs &w, cudaStream_t s) {
    k_wb_accept<<<grid1(w.W), 128, 0, s>>>(w.ws, w.W);
    SFMBA_LAUNCH_CHECK();
    const bool rs = b.mixed && b.ob_rs;
    long long m = b.nP;
    if (7LL * b.nI > m) m = 7LL * b.nI;
    if (8LL * b.nC > m) m = 8LL * b.nC;
    if (rs && b.nO > m) m = b.nO;
    if (m == 0) return;
    k_wb_commit<<<div_up(m, 256), 256, 0, s>>>(w.ws, w.pt_win, w.img_win, w.cam_win, b.nI, b.nC, b.nP, b.poses_trial,
                                               b.cams_trial, b.points_trial, b.poses, b.cams, b.points,
                                               b.mixed ? b.points32 : nullptr, b.nO, b.ob_pt,
                                               rs ? b.ob_rs_trial : nullptr, rs ? b.ob_rs : nullptr);
    SFMBA_LAUNCH_CHECK();
}

void launch_wb_reject_failed(const WinBufs &w, cudaStream_t s) {
    k_wb_reject_failed<<<grid1(w.W), 128, 0, s>>>(w.ws, w.W);
    SFMBA_LAUNCH_CHECK();
}

void launch_wb_end_outer(const WinBufs &w, int max_iterations, bool polish_allowed, double target_cost,
                         cudaStream_t s) {
    k_wb_end_outer<<<grid1(w.W), 128, 0, s>>>(w.ws, w.W, max_iterations, polish_allowed ? 1 : 0, target_cost);
    SFMBA_LAUNCH_CHECK();
}

void launch_wb_start_polish(const WinBufs &w, cudaStream_t s) {
    k_wb_start_polish<<<grid1(w.W), 128, 0, s>>>(w.ws, w.W);
    SFMBA_LAUNCH_CHECK();
}

void launch_wb_summary(const WinBufs &w, cudaStream_t s) {
    k_wb_summary<<<1, 256, 0, s>>>(w.ws, w.W, w.counts);
    SFMBA_LAUNCH_CHECK();
}

void launch_wb_lu(const Bufs &b, const WinBufs &w, int n_failed, cudaStream_t s) {
    if (n_failed <= 0 || w.max_n == 0) return;
    SFMBA_CUDA(cudaMemsetAsync(w.lu_count, 0, sizeof(int), s));
    k_wb_failed_list<<<grid1(w.W), 128, 0, s>>>(w.ws, w.W, w.lu_list, w.lu_count);
    SFMBA_LAUNCH_CHECK();
    const int nf = n_failed;
    k_wb_lu_copy<<<dim3(64, nf), 256, 0, s>>>(b.S, b.L, w.s_off, w.n_w, w.lu_list);
    SFMBA_LAUNCH_CHECK();
    static int cap_dev = -1, cap = 0;  // co-resident blocks of the cooperative column loop
    int dev = 0;
    SFMBA_CUDA(cudaGetDevice(&dev));
    if (cap_dev != dev) {
        int per_sm = 0, sms = 0;
        SFMBA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_wb_lu_coop, 256, 0));
        SFMBA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        cap = per_sm * sms;
        cap_dev = dev;
    }
    if (cap > 0) {
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3((unsigned)cap);
        cfg.blockDim = dim3(256);
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        SFMBA_CUDA(cudaLaunchKernelEx(&cfg, k_wb_lu_coop, b.L, (const long long *)w.s_off, (const int *)w.n_w,
                                      (const int *)w.slot_base, b.lu_perm, (const int *)w.lu_list, nf, w.max_n));
        SFMBA_LAUNCH_CHECK();
    }
    for (int k = 0; cap == 0 && k < w.max_n; ++k) {
        k_wb_lu_pivot<<<nf, 256, 0, s>>>(b.L, w.s_off, w.n_w, w.slot_base, b.lu_perm, w.lu_list, k);
        SFMBA_LAUNCH_CHECK();
        const int m = w.max_n - k - 1;
        if (m <= 0) break;
        k_wb_lu_update<<<dim3(div_up(m, 128), m, nf), 128, 0, s>>>(b.L, w.s_off, w.n_w, w.slot_base, b.lu_perm,
                                                                   w.lu_list, k);
        SFMBA_LAUNCH_CHECK();
    }
    k_wb_lu_solve<<<nf, 1024, 0, s>>>(b.L, w.s_off, w.n_w, w.slot_base, b.lu_perm, w.lu_list, w.rhs_p, b.work2,
                                      w.ws);
    SFMBA_LAUNCH_CHECK();
}

}  // namespace sfmba
