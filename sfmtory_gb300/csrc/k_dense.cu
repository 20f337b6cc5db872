// Dense reduced camera system:
//   * Schur reduction S_ij = [i==j] H_i - sum_p E_ip C_p^-1 E_jp^T, one warp
//     per image pair, walking the pair list grouped by image pair (the
//     visibility-sorted order), so every block is written exactly once and
//     no global atomics are used (reference: lib.rs:114-211, :981-1043);
//   * fold of the image-level system onto the reference's slot order with
//     damping, per-parameter masks and symmetrisation (lib.rs:918-956,
//     :1051-1074);
//   * blocked right-looking FP64 Cholesky (64-wide panels) with triangular
//     solves and one FP64 refinement step, and a partial-pivoting LU
//     fallback (lib.rs:1081-1094). On the mixed path the trailing updates
//     run on the BF16 tensor cores by error-free splitting (ozaki.cuh), to
//     FP64 accuracy; the plain FP64 path keeps FP64 fused multiply-adds.
#include <cooperative_groups.h>

#include <algorithm>
#include <type_traits>

#include "chol_block.cuh"
#include "kernels.cuh"
#include "ozaki.cuh"
#include "schur.cuh"

namespace sfmba {

namespace {

template <typename T>
constexpr int schur_warps() { return sizeof(T) == 4 ? 4 : 2; }

template <typename T, int D>
__global__ void __launch_bounds__(32 * schur_warps<T>())
    k_schur_pairs(const T *__restrict__ rec, const int2 *__restrict__ pairs,
                  const int *__restrict__ group_start, const int2 *__restrict__ group_ij,
                  const int *__restrict__ group_order, int ngroups,
                  const int *__restrict__ ob_pt, const T *__restrict__ pt_Cinv,
                  const unsigned char *__restrict__ pt_ok, const double *__restrict__ img_H, int nID,
                  double *__restrict__ S_img) {
    constexpr int W = schur_warps<T>();
    using Tile = SchurTile<T, D>;
    __shared__ T sA[W][32][Tile::LDS];
    __shared__ T sP[W][32][Tile::LDS];
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (blockIdx.x * W + wl >= ngroups) return;
    const int g = group_order[blockIdx.x * W + wl];
    const int2 ij = group_ij[g];
    double out[Tile::RH][Tile::CQ];
    schur_group<T, D>(rec, pairs, group_start[g], group_start[g + 1], ob_pt, pt_Cinv, pt_ok, sA[wl], sP[wl], lane,
                      out);
    if (lane >= Tile::LS) return;
    const int i = ij.x, j = ij.y;
    const int r0 = (lane >> 2) * Tile::RH, c0 = (lane & 3) * Tile::CQ;
#pragma unroll
    for (int a = 0; a < Tile::RH; ++a)
#pragma unroll
        for (int b = 0; b < Tile::CQ; ++b) {
            const int r = r0 + a, c = c0 + b;
            if (r >= D || c >= D) continue;
            const double v = out[a][b];
            if (i == j) {
                S_img[(size_t)(i * D + r) * nID + i * D + c] = img_H[(size_t)i * D * D + r * D + c] + v;
            } else {
                S_img[(size_t)(i * D + r) * nID + j * D + c] = v;
                S_img[(size_t)(j * D + c) * nID + i * D + r] = v;
            }
        }
}

// S[a][b] = sym( sum_{u in pre(a), w in pre(b)} S_img[u][w] ) + [a==b] lambda diag(B)[a];
// masked parameters become identity rows/columns (lib.rs:1051-1070).
__global__ void k_fold(const double *__restrict__ S_img, int nID, const int *__restrict__ pre_start,
                       const int *__restrict__ pre, const unsigned char *__restrict__ masked,
                       const double *__restrict__ diagB, const LMState *__restrict__ st, int n,
                       double *__restrict__ S, double *__restrict__ L) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    const int a = blockIdx.y;
    if (b >= n || a >= n) return;
    double v;
    if (masked[a] || masked[b]) {
        v = a == b ? 1.0 : 0.0;
    } else {
        double vab = 0.0, vba = 0.0;
        const int as = pre_start[a], ae = pre_start[a + 1], bs = pre_start[b], be = pre_start[b + 1];
        for (int x = as; x < ae; ++x)
            for (int y = bs; y < be; ++y) {
                vab += S_img[(size_t)pre[x] * nID + pre[y]];
                vba += S_img[(size_t)pre[y] * nID + pre[x]];
            }
        v = 0.5 * (vab + vba);
        if (a == b) v += diagB[a] * st->lambda;
    }
    S[(size_t)a * n + b] = v;
    L[(size_t)a * n + b] = v;
}

__global__ void k_fold_rhs(const double *img_rhs, const int *pre_start, const int *pre,
                           const unsigned char *masked, int n, double *rhs) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    double v = 0.0;
    if (!masked[a])
        for (int x = pre_start[a]; x < pre_start[a + 1]; ++x) v += img_rhs[pre[x]];
    rhs[a] = v;
}

// ---------------------------------------------------------------- Cholesky

constexpr int NB = kCholNB;
constexpr int LD = NB + 1;

// Factor the diagonal block k0 (in place, lower) and write the inverse of
// its factor to Linv (sm: two NB x LD tiles, buf: NB + 3). Sets
// state->factor_failed when a pivot is not > 0 (nalgebra Cholesky::new
// semantics: 0, negative and NaN all fail).
__device__ __forceinline__ void chol_diag_body(double *L, int n, int k0, double *Linv, LMState *st, double *sm,
                                               double *buf) {
    double *A = sm;            // NB x LD
    double *X = sm + NB * LD;  // NB x LD
    static_assert(LD == kBlkLD, "tile stride of chol_block_factor_invert");
    if (st->factor_failed) return;
    const int nb = min(NB, n - k0);
    const int tid = threadIdx.x;
    for (int idx = tid; idx < nb * nb; idx += blockDim.x) {
        const int r = idx / nb, c = idx - r * nb;
        A[r * LD + c] = c <= r ? L[(size_t)(k0 + r) * n + k0 + c] : 0.0;
    }
    __syncthreads();
    if (!chol_block_factor_invert(A, X, nb, buf)) {
        if (tid == 0) st->factor_failed = 1;
        return;
    }
    for (int idx = tid; idx < nb * nb; idx += blockDim.x) {
        const int r = idx / nb, c = idx - r * nb;
        if (c <= r) L[(size_t)(k0 + r) * n + k0 + c] = A[r * LD + c];
    }
    double *out = Linv + (size_t)(k0 / NB) * NB * NB;
    for (int idx = tid; idx < NB * NB; idx += blockDim.x) {
        const int r = idx / NB, c = idx - r * NB;
        out[idx] = (r < nb && c < nb) ? X[r * LD + c] : 0.0;
    }
}

__global__ void __launch_bounds__(256) k_chol_diag(double *L, int n, int k0, double *Linv, LMState *st) {
    extern __shared__ double sm[];
    __shared__ double buf[NB + 3];
    chol_diag_body(L, n, k0, Linv, st, sm, buf);
}

// Panel below the diagonal block: A[r, k-block] <- A[r, k-block] Lkk^-T,
// rows k0 + nb + blk PANEL_ROWS onwards (sm: NB + PANEL_ROWS rows of LD).
constexpr int PANEL_ROWS = 32;
__device__ __forceinline__ void chol_panel_body(double *L, int n, int k0, const double *Linv, const LMState *st,
                                                int blk, double *sm) {
    double *Li = sm;             // NB x LD
    double *R = sm + NB * LD;    // PANEL_ROWS x LD
    if (st->factor_failed) return;
    const int nb = min(NB, n - k0);
    const int r0 = k0 + nb + blk * PANEL_ROWS;
    const int rows = min(PANEL_ROWS, n - r0);
    if (rows <= 0) return;
    const double *inv = Linv + (size_t)(k0 / NB) * NB * NB;
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

__global__ void __launch_bounds__(256) k_chol_panel(double *L, int n, int k0, const double *Linv,
                                                     const LMState *st) {
    extern __shared__ double sm[];
    chol_panel_body(L, n, k0, Linv, st, blockIdx.x, sm);
}

// Tile (ti, tj), tj <= ti, of block q of a trailing update launch. part 0:
// every lower tile; 1: the first tile column (tj = 0, the next diagonal
// block's column, updated first for the look-ahead); 2: the others.
__device__ __forceinline__ void trailing_tile(long long q, int part, int &ti, int &tj) {
    if (part == 1) {
        ti = (int)q;
        tj = 0;
        return;
    }
    int a = (int)((sqrt(8.0 * (double)q + 1.0) - 1.0) * 0.5);
    while ((long long)(a + 1) * (a + 2) / 2 <= q) ++a;
    while ((long long)a * (a + 1) / 2 > q) --a;
    ti = a;
    tj = (int)(q - (long long)a * (a + 1) / 2);
    if (part == 2) {
        ++ti;
        ++tj;
    }
}

// Trailing update of the lower triangle: A[I,J] -= P_I P_J^T for the 64x64
// tiles (I >= J) right of the panel. Each thread owns a 4x4 register tile.
__device__ __forceinline__ void chol_update_body(double *L, int n, int k0, int ti, int tj, const LMState *st,
                                                 double *sm) {
    double *Pi = sm;            // NB x LD
    double *Pj = sm + NB * LD;  // NB x LD
    if (st->factor_failed) return;
    const int nb = min(NB, n - k0);
    const int t0 = k0 + nb;
    const int ri = t0 + ti * NB, rj = t0 + tj * NB;
    if (ri >= n || rj >= n) return;
    const int mi = min(NB, n - ri), mj = min(NB, n - rj);
    for (int idx = threadIdx.x; idx < NB * nb; idx += blockDim.x) {
        const int r = idx / nb, c = idx - r * nb;
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
    for (int t = 0; t < nb; ++t) {
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

__global__ void __launch_bounds__(256) k_chol_update(double *L, int n, int k0, int part, const LMState *st) {
    extern __shared__ double sm[];
    int ti, tj;
    trailing_tile(blockIdx.x, part, ti, tj);
    chol_update_body(L, n, k0, ti, tj, st, sm);
}

// The column loop of k_lu_pivot / k_lu_update (below) in one cooperative
// launch: block 0 pivots, swaps and scales column k, then every block
// updates its rows of the trailing matrix; two grid barriers per column
// instead of two launches, the same operations in the same order (the same
// factors).
__global__ void __launch_bounds__(256) k_lu_coop(double *A, int n, int *perm, const LMState *st) {
    namespace cg = cooperative_groups;
    cg::grid_group grid = cg::this_grid();
    __shared__ double bv[256];
    __shared__ int bi[256];
    if (!st->factor_failed || st->solve_failed) return;
    const int tid = threadIdx.x;
    for (int k = 0; k < n; ++k) {
        if (blockIdx.x == 0) {
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
            if (tid == 0) perm[k] = diag != 0.0 ? piv : -1;  // a zero column is skipped
            __syncthreads();
        }
        grid.sync();
        if (k + 1 >= n) break;
        if (((volatile const int *)perm)[k] >= 0)
            for (int r = k + 1 + blockIdx.x; r < n; r += gridDim.x) {
                const double lrk = A[(size_t)r * n + k];
                for (int c = k + 1 + tid; c < n; c += blockDim.x) A[(size_t)r * n + c] -= lrk * A[(size_t)k * n + c];
            }
        grid.sync();
    }
}

// ------------------------------------------------ tensor-core trailing update
// Slices and exponents of the panel rows below the diagonal block k0 (one
// warp per row; ozaki.cuh). slices: [kOzSlices][n][64] BF16.
__global__ void __launch_bounds__(256) k_oz_split(const double *L, int n, int k0, __nv_bfloat16 *slices, int *exps,
                                                   const LMState *st) {
    if (st->factor_failed) return;
    const int nb = min(NB, n - k0);
    const int r = k0 + nb + (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (r >= n) return;
    oz_split_row(L + (size_t)r * n + k0, nb, threadIdx.x & 31, slices + (size_t)r * kOzK, (size_t)n * kOzK,
                 exps + r);
}

// A[I, J] -= P_I P_J^T for the 64 x 64 lower tiles (I >= J) right of the
// panel, from the slices of k_oz_split (ozaki.cuh). One 4-warp block per
// tile; a diagonal tile writes its lower triangle.
__global__ void __launch_bounds__(128, 1) k_oz_update(double *L, int n, int k0, int part,
                                                      const __nv_bfloat16 *slices, const int *exps,
                                                      const LMState *st) {
    extern __shared__ __align__(16) unsigned char oz_sm[];
    __shared__ double fR[kOzTile], fC[kOzTile];
    if (st->factor_failed) return;
    const int t0 = k0 + NB;
    int ti, tj;
    trailing_tile(blockIdx.x, part, ti, tj);
    const int ri = t0 + ti * kOzTile, rj = t0 + tj * kOzTile;
    if (ri >= n || rj >= n) return;
    oz_tile_update(L + (size_t)ri * n + rj, (size_t)n, min(kOzTile, n - ri), min(kOzTile, n - rj), ti == tj,
                   slices + (size_t)ri * kOzK, slices + (size_t)rj * kOzK, (size_t)n * kOzK, exps + ri, exps + rj,
                   oz_sm, fR, fC);
}

// Forward step k of L y = b: y_k = Lkk^-1 b_k, then b_r -= L[r, k-block] y_k
// for the rows below (one warp per row).
__global__ void __launch_bounds__(256) k_trsv_fwd(const double *L, int n, int k0, const double *Linv,
                                                   double *b, double *y, const LMState *st) {
    __shared__ double yk[NB];
    __shared__ double bk[NB];
    if (st->factor_failed) return;
    const int nb = min(NB, n - k0);
    const double *inv = Linv + (size_t)(k0 / NB) * NB * NB;
    if (threadIdx.x < nb) bk[threadIdx.x] = b[k0 + threadIdx.x];
    __syncthreads();
    if (threadIdx.x < nb) {  // four interleaved partial sums (FP64 latency)
        const int r = threadIdx.x;
        double s[4] = {0.0, 0.0, 0.0, 0.0};
        for (int t = 0; t <= r; ++t) s[t & 3] += inv[r * NB + t] * bk[t];
        const double v = (s[0] + s[1]) + (s[2] + s[3]);
        yk[r] = v;
        if (blockIdx.x == 0) y[k0 + r] = v;
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int rows_per_block = blockDim.x >> 5;
    const int r = k0 + nb + blockIdx.x * rows_per_block + warp;
    if (r >= n) return;
    double s = 0.0;
    for (int t = lane; t < nb; t += 32) s += L[(size_t)r * n + k0 + t] * yk[t];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (lane == 0) b[r] -= s;
}

// Backward step k of L^T x = y: x_k = Lkk^-T y_k, then y_r -= L[k-block, r]^T x_k
// for the rows above (one thread per row, coalesced over r).
__global__ void __launch_bounds__(256) k_trsv_bwd(const double *L, int n, int k0, const double *Linv,
                                                   double *y, double *x, const LMState *st) {
    __shared__ double xk[NB];
    __shared__ double yk[NB];
    if (st->factor_failed) return;
    const int nb = min(NB, n - k0);
    const double *inv = Linv + (size_t)(k0 / NB) * NB * NB;
    if (threadIdx.x < nb) yk[threadIdx.x] = y[k0 + threadIdx.x];
    __syncthreads();
    if (threadIdx.x < nb) {  // four interleaved partial sums: FP64 latency, not a 64-long chain
        const int c = threadIdx.x;
        double s[4] = {0.0, 0.0, 0.0, 0.0};
        for (int r = c; r < nb; ++r) s[(r - c) & 3] += inv[r * NB + c] * yk[r];
        const double v = (s[0] + s[1]) + (s[2] + s[3]);
        xk[c] = v;
        if (blockIdx.x == 0) x[k0 + c] = v;
    }
    __syncthreads();
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= k0) return;
    double s[4] = {0.0, 0.0, 0.0, 0.0};
    for (int t = 0; t < nb; t += 4)
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (t + u < nb) s[u] += L[(size_t)(k0 + t + u) * n + r] * xk[t + u];
    y[r] -= (s[0] + s[1]) + (s[2] + s[3]);
}

// Both triangular solves of L L^T x = rhs in one cooperative launch: the
// forward sweep (L y = rhs, rhs copied to `work` and updated in place) then
// the backward sweep (L^T x = y, y updated in place), one grid barrier per
// 64-wide block step instead of a launch. Every block forms the step's
// diagonal product with Lkk^-1 itself from the same data (so no barrier is
// spent on publishing it), then updates its share of the remaining rows: one
// warp per row below in the forward sweep, one thread per row above (reading
// L down its columns, coalesced) in the backward sweep.
__global__ void __launch_bounds__(256) k_trsv_coop(const double *L, int n, const double *Linv, double *work,
                                                    double *y, double *x, const LMState *st) {
    namespace cg = cooperative_groups;
    cg::grid_group grid = cg::this_grid();
    __shared__ double vk[NB], bk[NB];
    if (st->factor_failed) return;  // read-only here: every block takes the same branch
    const int nblk = (n + NB - 1) / NB;
    const int tid = threadIdx.x, lane = tid & 31;
    const int gw = (int)((blockIdx.x * blockDim.x + tid) >> 5), nw = (int)((gridDim.x * blockDim.x) >> 5);
    for (int k = 0; k < nblk; ++k) {
        const int k0 = k * NB, nb = min(NB, n - k0);
        const double *inv = Linv + (size_t)k * NB * NB;
        if (tid < nb) bk[tid] = work[k0 + tid];
        __syncthreads();
        if (tid < nb) {  // y_k = Lkk^-1 b_k, four interleaved partial sums
            double s[4] = {0.0, 0.0, 0.0, 0.0};
            for (int t = 0; t <= tid; ++t) s[t & 3] += inv[tid * NB + t] * bk[t];
            const double v = (s[0] + s[1]) + (s[2] + s[3]);
            vk[tid] = v;
            if (blockIdx.x == 0) y[k0 + tid] = v;
        }
        __syncthreads();
        for (int r = k0 + nb + gw; r < n; r += nw) {
            double s = 0.0;
            for (int t = lane; t < nb; t += 32) s += L[(size_t)r * n + k0 + t] * vk[t];
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
            if (lane == 0) work[r] -= s;
        }
        grid.sync();
    }
    for (int k = nblk - 1; k >= 0; --k) {
        const int k0 = k * NB, nb = min(NB, n - k0);
        const double *inv = Linv + (size_t)k * NB * NB;
        if (tid < nb) bk[tid] = y[k0 + tid];
        __syncthreads();
        if (tid < nb) {  // x_k = Lkk^-T y_k
            double s[4] = {0.0, 0.0, 0.0, 0.0};
            for (int r = tid; r < nb; ++r) s[(r - tid) & 3] += inv[r * NB + tid] * bk[r];
            const double v = (s[0] + s[1]) + (s[2] + s[3]);
            vk[tid] = v;
            if (blockIdx.x == 0) x[k0 + tid] = v;
        }
        __syncthreads();
        for (int r = blockIdx.x * blockDim.x + tid; r < k0; r += gridDim.x * blockDim.x) {
            double s[4] = {0.0, 0.0, 0.0, 0.0};
            for (int t = 0; t < nb; t += 4)
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (t + u < nb) s[u] += L[(size_t)(k0 + t + u) * n + r] * vk[t + u];
            y[r] -= (s[0] + s[1]) + (s[2] + s[3]);
        }
        grid.sync();
    }
}

// res = rhs - S x (one warp per row).
__global__ void k_residual(const double *S, int n, const double *x, const double *rhs, double *res,
                           const LMState *st) {
    if (st->factor_failed) return;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= n) return;
    double s = 0.0;
    for (int c = lane; c < n; c += 32) s += S[(size_t)warp * n + c] * x[c];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (lane == 0) res[warp] = rhs[warp] - s;
}

__global__ void k_axpy_inplace(int n, const double *c, double *x, const LMState *st) {
    if (st->factor_failed) return;
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a < n) x[a] += c[a];
}

// ---------------------------------------------------------------- LU fallback

// Column k: pivot on max |a| (first maximum), swap rows, scale the
// multipliers. A zero column is skipped (no swap, no elimination).
__global__ void __launch_bounds__(1024) k_lu_pivot(double *A, int n, int k, int *perm, const LMState *st) {
    __shared__ double bv[1024];
    __shared__ int bi[1024];
    if (!st->factor_failed || st->solve_failed) return;
    double best = -1.0;
    int besti = k;
    for (int r = k + threadIdx.x; r < n; r += blockDim.x) {
        const double v = fabs(A[(size_t)r * n + k]);
        if (v > best) { best = v; besti = r; }
    }
    bv[threadIdx.x] = best;
    bi[threadIdx.x] = besti;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            const double o = bv[threadIdx.x + w];
            const int oi = bi[threadIdx.x + w];
            if (o > bv[threadIdx.x] || (o == bv[threadIdx.x] && oi < bi[threadIdx.x])) {
                bv[threadIdx.x] = o;
                bi[threadIdx.x] = oi;
            }
        }
        __syncthreads();
    }
    const int piv = bi[0];
    const double diag = A[(size_t)piv * n + k];
    if (diag == 0.0) {
        if (threadIdx.x == 0) perm[k] = -1;  // zero column: skipped
        return;
    }
    if (piv != k)
        for (int c = threadIdx.x; c < n; c += blockDim.x) {
            const double t = A[(size_t)k * n + c];
            A[(size_t)k * n + c] = A[(size_t)piv * n + c];
            A[(size_t)piv * n + c] = t;
        }
    if (threadIdx.x == 0) perm[k] = piv;
    __syncthreads();
    for (int r = k + 1 + threadIdx.x; r < n; r += blockDim.x) A[(size_t)r * n + k] /= diag;
}

__global__ void k_lu_update(double *A, int n, int k, const int *perm, const LMState *st) {
    if (!st->factor_failed || st->solve_failed) return;
    if (perm[k] < 0) return;
    const int c = k + 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int r = k + 1 + blockIdx.y;
    if (c >= n || r >= n) return;
    A[(size_t)r * n + c] -= A[(size_t)r * n + k] * A[(size_t)k * n + c];
}

// Apply the row swaps to rhs, solve unit-lower then upper. A zero diagonal
// of U fails the solve (lambda then grows); success clears factor_failed so
// the back-substitution and trial kernels run.
// Sum of v over the 1024-thread block (warp sums, then the 32 warps' sums
// by warp 0), valid in every thread; two barriers.
__device__ __forceinline__ double block_sum_1024(double v, double *red) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = (threadIdx.x & 31) < (blockDim.x >> 5) ? red[threadIdx.x & 31] : 0.0;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
    __syncthreads();  // red is reused by the next call
    return t;
}

__global__ void __launch_bounds__(1024) k_lu_solve(const double *A, int n, const int *perm,
                                                    const double *rhs, double *x, LMState *st) {
    __shared__ double red[32];
    __shared__ int bad;
    if (!st->factor_failed || st->solve_failed) return;
    if (threadIdx.x == 0) bad = 0;
    for (int a = threadIdx.x; a < n; a += blockDim.x) x[a] = rhs[a];
    __syncthreads();
    if (threadIdx.x == 0)
        for (int k = 0; k < n; ++k)
            if (perm[k] >= 0 && perm[k] != k) {
                const double t = x[k];
                x[k] = x[perm[k]];
                x[perm[k]] = t;
            }
    __syncthreads();
    for (int i = 0; i < n; ++i) {
        double s = 0.0;
        for (int k = threadIdx.x; k < i; k += blockDim.x) s += A[(size_t)i * n + k] * x[k];
        s = block_sum_1024(s, red);
        if (threadIdx.x == 0) x[i] -= s;
        __syncthreads();
    }
    for (int i = n - 1; i >= 0; --i) {
        double s = 0.0;
        for (int k = i + 1 + threadIdx.x; k < n; k += blockDim.x) s += A[(size_t)i * n + k] * x[k];
        s = block_sum_1024(s, red);
        if (threadIdx.x == 0) {
            const double d = A[(size_t)i * n + i];
            if (d == 0.0) bad = 1;
            else x[i] = (x[i] - s) / d;
        }
        __syncthreads();
        if (bad) break;
    }
    if (threadIdx.x == 0) {
        if (bad) st->solve_failed = 1;
        else st->factor_failed = 0;
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
    SFMBA_CUDA(cudaFuncSetAttribute(k_chol_diag, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemTwoTiles));
    SFMBA_CUDA(cudaFuncSetAttribute(k_chol_update, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemTwoTiles));
    SFMBA_CUDA(cudaFuncSetAttribute(k_chol_panel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemPanel));
    SFMBA_CUDA(cudaFuncSetAttribute(k_oz_update, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kOzSmem));
    done = true;
}

}  // namespace

void launch_schur_pairs(const Bufs &b, cudaStream_t s) {
    if (b.ngroups == 0) return;
    dispatch_D(b.D, [&](auto dc) {
        constexpr int D = decltype(dc)::value;
        if (b.mixed)
            k_schur_pairs<float, D><<<div_up(b.ngroups, schur_warps<float>()), 32 * schur_warps<float>(), 0, s>>>(
                (const float *)b.rec, b.pairs, b.group_start, b.group_ij, b.group_order, b.ngroups, b.ob_pt,
                (const float *)b.pt_Cinv, b.pt_ok, b.img_H, b.nID, b.S_img);
        else
            k_schur_pairs<double, D><<<div_up(b.ngroups, schur_warps<double>()), 32 * schur_warps<double>(), 0, s>>>(
                (const double *)b.rec, b.pairs, b.group_start, b.group_ij, b.group_order, b.ngroups, b.ob_pt,
                (const double *)b.pt_Cinv, b.pt_ok, b.img_H, b.nID, b.S_img);
    });
    SFMBA_LAUNCH_CHECK();
}

void launch_fold_system(const Bufs &b, cudaStream_t s) {
    if (b.n == 0) return;
    dim3 grid(div_up(b.n, 128), b.n);
    k_fold<<<grid, 128, 0, s>>>(b.S_img, b.nID, b.slot_pre_start, b.slot_pre, b.slot_masked, b.diagB,
                                b.state, b.n, b.S, b.L);
    SFMBA_LAUNCH_CHECK();
    k_fold_rhs<<<div_up(b.n, 256), 256, 0, s>>>(b.img_rhs, b.slot_pre_start, b.slot_pre, b.slot_masked,
                                                b.n, b.rhs);
    SFMBA_LAUNCH_CHECK();
}

void launch_fold_rhs(const Bufs &b, cudaStream_t s) {
    if (b.n == 0) return;
    k_fold_rhs<<<div_up(b.n, 256), 256, 0, s>>>(b.img_rhs, b.slot_pre_start, b.slot_pre, b.slot_masked, b.n,
                                                b.rhs);
    SFMBA_LAUNCH_CHECK();
}

namespace {

// Second stream and two events of the look-ahead, per host thread and device.
struct LookAhead {
    int device = -1;
    cudaStream_t s2 = nullptr;
    cudaEvent_t col_done = nullptr, next_ready = nullptr;
    ~LookAhead() {
        if (col_done) cudaEventDestroy(col_done);
        if (next_ready) cudaEventDestroy(next_ready);
        if (s2) cudaStreamDestroy(s2);
    }
};

LookAhead &look_ahead() {
    thread_local LookAhead la;
    int dev = 0;
    SFMBA_CUDA(cudaGetDevice(&dev));
    if (la.device != dev) {
        if (la.s2) {
            cudaEventDestroy(la.col_done);
            cudaEventDestroy(la.next_ready);
            cudaStreamDestroy(la.s2);
        }
        la.device = dev;
        // The highest priority: the next panel's blocks are dispatched as soon
        // as the trailing update's blocks free an SM, not after all of them.
        int least = 0, greatest = 0;
        SFMBA_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        SFMBA_CUDA(cudaStreamCreateWithPriority(&la.s2, cudaStreamNonBlocking, greatest));
        SFMBA_CUDA(cudaEventCreateWithFlags(&la.col_done, cudaEventDisableTiming));
        SFMBA_CUDA(cudaEventCreateWithFlags(&la.next_ready, cudaEventDisableTiming));
    }
    return la;
}

}  // namespace

// Blocked right-looking Cholesky with a look-ahead of one panel: after the
// panel of block k, the tile column of block k + 1 is updated first; then
// the diagonal factor, panel (and slices) of block k + 1 run on a second
// stream while the rest of block k's trailing update runs on s. The
// diagonal factor is the serial part (one block, FP64-pipe bound), so it
// hides behind the bulk update. Tensor-core updates read the panel slices of
// their own step: two slice buffers alternate by step.
// Cooperative launch of kernel k with `want` blocks of 256 threads at most
// what the GPU holds at once (cap: co-resident blocks, queried once per
// device by the caller); false when none can be resident.
template <typename... Args>
bool launch_coop(void (*k)(Args...), int cap, int want, size_t smem, cudaStream_t s, Args... args) {
    if (cap < 1) return false;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)std::max(1, std::min(cap, want)));
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    SFMBA_CUDA(cudaLaunchKernelEx(&cfg, k, args...));
    SFMBA_LAUNCH_CHECK();
    return true;
}

// Co-resident blocks of a 256-thread kernel with `smem` dynamic shared memory.
template <typename K>
int coop_capacity(K k, size_t smem) {
    int dev = 0, per_sm = 0, sms = 0;
    SFMBA_CUDA(cudaGetDevice(&dev));
    SFMBA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 256, smem));
    SFMBA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    return per_sm * sms;
}

void launch_cholesky(const Bufs &b, cudaStream_t s) {
    set_smem_limits();
    const int n = b.n;
    if (n == 0) return;
    const bool oz = b.oz_slices != nullptr;
    const size_t slice_elems = (size_t)kOzSlices * n * kOzK;
    auto slices = [&](int k0) { return (__nv_bfloat16 *)b.oz_slices + ((k0 / NB) & 1) * slice_elems; };
    auto exps = [&](int k0) { return b.oz_exp + ((k0 / NB) & 1) * (size_t)n; };
    // diagonal factor, panel and (tensor path) slices of block k0, on stream st
    auto head = [&](int k0, cudaStream_t st) {
        k_chol_diag<<<1, 256, kSmemTwoTiles, st>>>(b.L, n, k0, b.Linv, b.state);
        SFMBA_LAUNCH_CHECK();
        const int rem = n - k0 - NB;
        if (rem <= 0) return;
        k_chol_panel<<<div_up(rem, PANEL_ROWS), 256, kSmemPanel, st>>>(b.L, n, k0, b.Linv, b.state);
        SFMBA_LAUNCH_CHECK();
        if (oz) {
            k_oz_split<<<div_up(rem, 8), 256, 0, st>>>(b.L, n, k0, slices(k0), exps(k0), b.state);
            SFMBA_LAUNCH_CHECK();
        }
    };
    auto update = [&](int k0, int part, long long blocks, cudaStream_t st) {
        if (blocks <= 0) return;
        if (oz)
            k_oz_update<<<(unsigned)blocks, 128, kOzSmem, st>>>(b.L, n, k0, part, slices(k0), exps(k0), b.state);
        else
            k_chol_update<<<(unsigned)blocks, 256, kSmemTwoTiles, st>>>(b.L, n, k0, part, b.state);
        SFMBA_LAUNCH_CHECK();
    };
    head(0, s);
    for (int k0 = 0; k0 + NB < n; k0 += NB) {
        const long long tiles = div_up(n - k0 - NB, NB);
        const int k1 = k0 + NB;
        update(k0, 1, tiles, s);  // tile column of block k1
        if (tiles == 1) {
            head(k1, s);
            continue;
        }
        LookAhead &la = look_ahead();
        SFMBA_CUDA(cudaEventRecord(la.col_done, s));
        SFMBA_CUDA(cudaStreamWaitEvent(la.s2, la.col_done, 0));
        head(k1, la.s2);
        SFMBA_CUDA(cudaEventRecord(la.next_ready, la.s2));
        update(k0, 2, (tiles - 1) * tiles / 2, s);
        SFMBA_CUDA(cudaStreamWaitEvent(s, la.next_ready, 0));
    }
}

void launch_cholesky_solve(const Bufs &b, const double *rhs, double *x, cudaStream_t s) {
    const int n = b.n;
    if (n == 0) return;
    // forward: work <- rhs (updated in place), y -> work2
    SFMBA_CUDA(cudaMemcpyAsync(b.work, rhs, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    static int cap_dev = -1, cap = 0;  // one block per SM: the diagonal products are formed per block
    int dev = 0;
    SFMBA_CUDA(cudaGetDevice(&dev));
    if (cap_dev != dev) {
        int per_sm = 0, sms = 0;
        SFMBA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trsv_coop, 256, 0));
        SFMBA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        cap = per_sm > 0 ? sms : 0;
        cap_dev = dev;
    }
    if (cap > 0) {
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3((unsigned)std::min(cap, div_up(n, 8)));
        cfg.blockDim = dim3(256);
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        SFMBA_CUDA(cudaLaunchKernelEx(&cfg, k_trsv_coop, (const double *)b.L, n, (const double *)b.Linv, b.work,
                                      b.work2, x, (const LMState *)b.state));
        SFMBA_LAUNCH_CHECK();
        return;
    }
    for (int k0 = 0; k0 < n; k0 += NB) {
        const int rem = n - k0 - NB;
        const int grid = rem > 0 ? div_up(rem, 8) : 1;
        k_trsv_fwd<<<grid, 256, 0, s>>>(b.L, n, k0, b.Linv, b.work, b.work2, b.state);
        SFMBA_LAUNCH_CHECK();
    }
    const int last = ((n - 1) / NB) * NB;
    for (int k0 = last; k0 >= 0; k0 -= NB) {
        const int grid = k0 > 0 ? div_up(k0, 256) : 1;
        k_trsv_bwd<<<grid, 256, 0, s>>>(b.L, n, k0, b.Linv, b.work2, x, b.state);
        SFMBA_LAUNCH_CHECK();
    }
}

void launch_refine(const Bufs &b, cudaStream_t s) {
    // One FP64 iterative-refinement step: res = rhs - S delta, solve, delta += c.
    k_residual<<<div_up((long long)b.n * 32, 256), 256, 0, s>>>(b.S, b.n, b.delta, b.rhs, b.ref_res, b.state);
    SFMBA_LAUNCH_CHECK();
    launch_cholesky_solve(b, b.ref_res, b.ref_corr, s);
    k_axpy_inplace<<<div_up(b.n, 256), 256, 0, s>>>(b.n, b.ref_corr, b.delta, b.state);
    SFMBA_LAUNCH_CHECK();
}

void launch_lu_factor(const Bufs &b, cudaStream_t s) {
    const int n = b.n;
    SFMBA_CUDA(cudaMemcpyAsync(b.L, b.S, sizeof(double) * (size_t)n * n, cudaMemcpyDeviceToDevice, s));
    // One block per SM at most: every column costs two grid barriers, whose
    // cost grows with the blocks taking part, while its update is small.
    static int cap_dev = -1, cap = 0, sms = 0;
    int dev = 0;
    SFMBA_CUDA(cudaGetDevice(&dev));
    if (cap_dev != dev) {
        cap = coop_capacity(k_lu_coop, 0);
        SFMBA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        cap_dev = dev;
    }
    if (n > 0 && launch_coop(k_lu_coop, cap, std::min(n, sms), 0, s, b.L, n, b.lu_perm, (const LMState *)b.state))
        return;
    for (int k = 0; k < n; ++k) {
        k_lu_pivot<<<1, 1024, 0, s>>>(b.L, n, k, b.lu_perm, b.state);
        SFMBA_LAUNCH_CHECK();
        if (k + 1 < n) {
            dim3 grid(div_up(n - k - 1, 128), n - k - 1);
            k_lu_update<<<grid, 128, 0, s>>>(b.L, n, k, b.lu_perm, b.state);
            SFMBA_LAUNCH_CHECK();
        }
    }
}

void launch_lu_solve(const Bufs &b, cudaStream_t s) {
    k_lu_solve<<<1, 1024, 0, s>>>(b.L, b.n, b.lu_perm, b.rhs, b.delta, b.state);
    SFMBA_LAUNCH_CHECK();
}

}  // namespace sfmba
