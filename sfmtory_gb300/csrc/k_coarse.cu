// Two-level preconditioner of the matrix-free Schur PCG: block-Jacobi on
// the image blocks plus an additive coarse correction Z A_c^-1 Z^T, where Z
// is piecewise constant over clusters of consecutive images (one coarse
// unknown per cluster and image-block column) and A_c = Z^T S Z is the exact
// Galerkin projection of the damped Schur complement
//   S = (B + lambda diag B) - E C^-1 E^T.
// Block-Jacobi leaves the smooth, long-range modes of a long camera sequence
// (drift along the trajectory) to the Krylov iteration; the coarse space
// removes them. Z^T B Z is the sum of a cluster's image blocks; Z^T E C^-1
// E^T Z sums, for every point, Y_c^T C_p^-1 Y_c' over the clusters c, c' its
// observations fall in, with Y_c = sum over its observations in cluster c of
// Jx~^T Jc~ (the Jacobians recomputed or read as in the PCG passes).
//
// The point-cluster pairs are grouped by cluster pair once per solve
// (sorted, so each group's points are in point order) and cut into chunks
// of at most kCoarseChunk points; one warp per chunk forms the chunk's
// D x D contribution with the register-tiled product of the Schur
// reduction (inner dimension 3 per point), and one block per group sums its
// chunks in order — no atomics, so A_c is bit-reproducible. A_c is small
// (clusters x D <= 1792) and is inverted in FP32 by a block sweep in one
// cooperative launch (k_coarse_sweep below); the inverse is applied as a
// dense product each iteration.
#include <cooperative_groups.h>

#include <algorithm>

#include <cub/cub.cuh>

#include "mf_passes.cuh"

namespace sfmba {

namespace {

// Distinct clusters among a point's observations, in increasing order.
__device__ int point_clusters(const int *ob_img, const int *img_cluster, int s, int e, int *out) {
    int k = 0;
    for (int o = s; o < e; ++o) {
        const int c = img_cluster[ob_img[o]];
        bool seen = false;
        for (int j = 0; j < k && !seen; ++j) seen = out[j] == c;
        if (seen) continue;
        int j = k++;
        while (j > 0 && out[j - 1] > c) {  // insertion keeps them sorted
            out[j] = out[j - 1];
            --j;
        }
        out[j] = c;
    }
    return k;
}

__global__ void k_coarse_count(const int *pt_start, const int *ob_img, const int *img_cluster, int nP,
                               long long *count, long long *kcount) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nP) return;
    int cl[kMaxCoarseClusters];
    const int k = point_clusters(ob_img, img_cluster, pt_start[p], pt_start[p + 1], cl);
    count[p] = (long long)k * (k + 1) / 2;
    kcount[p] = k;
}

__global__ void k_coarse_emit(const int *pt_start, const int *ob_img, const int *img_cluster, int nP, int nc,
                              const long long *off, const long long *inc_off, int *key, int *val, int *inc_cl,
                              int *inc_pt) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nP) return;
    int cl[kMaxCoarseClusters];
    const int k = point_clusters(ob_img, img_cluster, pt_start[p], pt_start[p + 1], cl);
    long long w = off[p];
    for (int a = 0; a < k; ++a) {
        inc_cl[inc_off[p] + a] = cl[a];
        inc_pt[inc_off[p] + a] = p;
        for (int b = a; b < k; ++b) {
            key[w] = cl[a] * nc + cl[b];
            val[w] = p;
            ++w;
        }
    }
}

// Sort keys of the incidences: their point's track length (capped at 2^16 - 1).
__global__ void k_inc_keys(const int *pt_start, const long long *inc_off, int nP, int *key, int *val) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nP) return;
    const int len = min(pt_start[p + 1] - pt_start[p], 65535);
    for (long long a = inc_off[p]; a < inc_off[p + 1]; ++a) {
        key[a] = len;
        val[a] = (int)a;
    }
}

// Size of every group from the sorted keys: the first element of a run adds
// -start and the last adds end + 1, so only two integer atomics per group
// land on a counter (no contention on long runs) and the sum is exact.
__global__ void k_key_counts(const int *key, long long n, int *counts) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int k = key[t];
    const bool first = t == 0 || key[t - 1] != k;
    const bool last = t == n - 1 || key[t + 1] != k;
    if (first && last) atomicAdd(&counts[k], 1);
    else if (first) atomicAdd(&counts[k], -(int)t);
    else if (last) atomicAdd(&counts[k], (int)(t + 1));
}

// A_c = 0, then block (c, c) = sum over the cluster's images of
// (H_i + lambda diag H_i) on the image's own unknown columns (pmask: a
// shared camera's columns are not in the coarse space).
__global__ void k_coarse_diag(const double *img_H, const int *img_active, const int *clu_start, int nc, int D,
                              const LMState *st, double *A) {
    const int c = blockIdx.x;
    if (c >= nc) return;
    const int Nc = nc * D;
    const double lam = st->lambda;
    for (int e = threadIdx.x; e < D * D; e += blockDim.x) {
        const int a = e / D, b = e - a * D;
        double s = 0.0;
        for (int i = clu_start[c]; i < clu_start[c + 1]; ++i) {
            const int act = img_active[i];
            if (!((act >> a) & 1) || !((act >> b) & 1)) continue;
            const double h = img_H[(size_t)i * D * D + a * D + b];
            s += h + (a == b ? lam * h : 0.0);
        }
        A[(size_t)(c * D + a) * Nc + c * D + b] = s;
    }
}

// Y_c = sum over the point's observations in cluster c of Jx~^T Jc~ (3 x D,
// row-major), one thread per point-cluster incidence, the observations
// taken in the point's order; every point-cluster pair of the assembly then
// reads its two Y instead of recomputing the Jacobians per pair.
template <typename T, int D, bool RC, int M>
__global__ void __launch_bounds__(128) k_coarse_y(JacSrc<T> J, const int *__restrict__ pt_start,
                                                  const int *__restrict__ img_cluster,
                                                  const int *__restrict__ img_pmask,
                                                  const int *__restrict__ inc_pt, const int *__restrict__ inc_cl,
                                                  const int *__restrict__ inc_order, long long ninc,
                                                  const unsigned char *__restrict__ pt_ok, T *__restrict__ Y) {
    // Threads take the incidences in track-length order, so a warp's
    // threads walk tracks of similar length.
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= ninc) return;
    const long long j = inc_order[t];
    const int p = inc_pt[j], c = inc_cl[j];
    T y[3][D];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int d = 0; d < D; ++d) y[r][d] = T(0);
    if (pt_ok[p]) {
        for (int o = pt_start[p]; o < pt_start[p + 1]; ++o) {
            const int4 rc = __ldg(J.obrec + o);
            if (img_cluster[rc.x] != c) continue;
            ObsOp<T, D, RC, M> op;
            make_op_point_major<T, D, RC>(J, o, rc, op);
            T jx[6], jc[2 * D];
            op.jx_rows(jx);
            op.jc_rows(jc);
            const int pm = img_pmask[rc.x];  // a shared camera's columns are not in the coarse space
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int d = 0; d < D; ++d)
                    if ((pm >> d) & 1) y[r][d] += jx[r] * jc[d] + jx[3 + r] * jc[D + d];
        }
    }
    T *dst = Y + (size_t)j * 3 * D;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int d = 0; d < D; ++d) dst[r * D + d] = y[r][d];
}

// Chunk q of the pair groups: minus sum over its points of Y_c^T C^-1 Y_c'.
// One warp per chunk; per round of 32 points lane t stages A_t = Y_c (3 x D)
// and P_t = C^-1 Y_c' (3 x D); the D x D product over 3 x 32 inner terms is
// register-tiled as in the Schur reduction, rounds added with Kahan
// compensation (FP32), output in FP64.
template <typename T>
constexpr int coarse_warps() { return sizeof(T) == 4 ? 4 : 2; }  // static shared memory under 48 KB

template <typename T, int D>
__global__ void __launch_bounds__(32 * coarse_warps<T>()) k_coarse_pairs(const T *__restrict__ Y,
                                                      const long long *__restrict__ inc_off,
                                                      const int *__restrict__ inc_cl,
                                                      const int4 *__restrict__ chunks, int nchunks,
                                                      const int *__restrict__ pair_pt,
                                                      const int2 *__restrict__ group_cc, const T *__restrict__ pt_Cinv,
                                                      const unsigned char *__restrict__ pt_ok,
                                                      double *__restrict__ part) {
    constexpr int RH = (D + 1) / 2, CQ = (D + 3) / 4;
    constexpr int LD = 3 * D + 1;
    constexpr int WPB = coarse_warps<T>();
    __shared__ T sA[WPB][32][LD];
    __shared__ T sP[WPB][32][LD];
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (q >= nchunks) return;
    const int4 ch = chunks[q];  // {group, first, end}
    const int2 cc = group_cc[ch.x];
    const int sg = lane >> 3, l8 = lane & 7;
    const int r0 = (l8 >> 2) * RH, c0 = (l8 & 3) * CQ;
    T acc[RH][CQ], comp[RH][CQ];
#pragma unroll
    for (int a = 0; a < RH; ++a)
#pragma unroll
        for (int b = 0; b < CQ; ++b) acc[a][b] = comp[a][b] = T(0);
    for (int base = ch.y; base < ch.z; base += 32) {
        const int k = base + lane;
        bool staged = false;
        if (k < ch.z) {
            const int p = pair_pt[k];
            long long ia = inc_off[p], ib = ia;  // the point's incidences of clusters c and c'
            const long long iend = inc_off[p + 1];
            while (ia < iend && inc_cl[ia] != cc.x) ++ia;
            ib = ia;
            while (ib < iend && inc_cl[ib] != cc.y) ++ib;
            if (pt_ok[p] && ib < iend) {
                const T *ya = Y + (size_t)ia * 3 * D, *yb = Y + (size_t)ib * 3 * D;
                const T *Ci = pt_Cinv + 6 * (size_t)p;
                const T m00 = Ci[0], m01 = Ci[1], m02 = Ci[2], m11 = Ci[3], m12 = Ci[4], m22 = Ci[5];
#pragma unroll
                for (int c = 0; c < D; ++c) {
                    const T b0 = yb[c], b1 = yb[D + c], b2 = yb[2 * D + c];
                    sA[wl][lane][c] = ya[c];
                    sA[wl][lane][D + c] = ya[D + c];
                    sA[wl][lane][2 * D + c] = ya[2 * D + c];
                    sP[wl][lane][c] = m00 * b0 + m01 * b1 + m02 * b2;
                    sP[wl][lane][D + c] = m01 * b0 + m11 * b1 + m12 * b2;
                    sP[wl][lane][2 * D + c] = m02 * b0 + m12 * b1 + m22 * b2;
                }
                staged = true;
            }
        }
        if (!staged) {
#pragma unroll
            for (int f = 0; f < 3 * D; ++f) sA[wl][lane][f] = sP[wl][lane][f] = T(0);
        }
    __syncwarp();
        T pt[RH][CQ];
#pragma unroll
        for (int a = 0; a < RH; ++a)
#pragma unroll
            for (int b = 0; b < CQ; ++b) pt[a][b] = T(0);
#pragma unroll 2
        for (int kk = 0; kk < 8; ++kk) {
            const int t = sg + 4 * kk;
#pragma unroll
            for (int rho = 0; rho < 3; ++rho) {
                T av[RH], pv[CQ];
#pragma unroll
                for (int a = 0; a < RH; ++a) av[a] = (r0 + a < D) ? sA[wl][t][rho * D + r0 + a] : T(0);
#pragma unroll
                for (int b = 0; b < CQ; ++b) pv[b] = (c0 + b < D) ? sP[wl][t][rho * D + c0 + b] : T(0);
#pragma unroll
                for (int a = 0; a < RH; ++a)
#pragma unroll
                    for (int b = 0; b < CQ; ++b) pt[a][b] += av[a] * pv[b];
            }
        }
#pragma unroll
        for (int a = 0; a < RH; ++a)
#pragma unroll
            for (int b = 0; b < CQ; ++b) {
                if constexpr (std::is_same<T, float>::value) {
                    const T y = pt[a][b] - comp[a][b];
                    const T t = acc[a][b] + y;
                    comp[a][b] = (t - acc[a][b]) - y;
                    acc[a][b] = t;
                } else {
                    acc[a][b] += pt[a][b];
                }
            }
        __syncwarp();
    }
    double *dst = part + (size_t)q * D * D;
#pragma unroll
    for (int a = 0; a < RH; ++a)
#pragma unroll
        for (int b = 0; b < CQ; ++b) {
            double v = (double)acc[a][b] - (double)comp[a][b];
            v += __shfl_xor_sync(0xffffffffu, v, 8);
            v += __shfl_xor_sync(0xffffffffu, v, 16);
            const int row = r0 + a, col = c0 + b;
            if (lane < 8 && row < D && col < D) dst[row * D + col] = -v;
        }
}

// Group g's chunks summed in order into block (c, c') of A_c, and its
// transpose into (c', c) for c != c'. Columns that are not unknowns of any
// image are left at zero (k_coarse_sweep puts 1 on their diagonal).
__global__ void k_coarse_finish(const double *part, const int *group_chunk_off, const int2 *group_cc, int ngroups,
                                int nc, int D, double *A) {
    const int g = blockIdx.x;
    if (g >= ngroups) return;
    const int Nc = nc * D;
    const int2 cc = group_cc[g];
    for (int e = threadIdx.x; e < D * D; e += blockDim.x) {
        const int a = e / D, b = e - a * D;
        double s = 0.0;
        for (int q = group_chunk_off[g]; q < group_chunk_off[g + 1]; ++q) s += part[(size_t)q * D * D + e];
        A[(size_t)(cc.x * D + a) * Nc + cc.y * D + b] += s;
        if (cc.x != cc.y) A[(size_t)(cc.y * D + b) * Nc + cc.x * D + a] += s;
    }
}

// ------------------------------------------------------------ coarse inverse
// A_c^-1 by the block sweep (Gauss-Jordan elimination in place, symmetric
// positive definite, pivot blocks of kSwPiv in order, no pivoting). Sweeping
// the pivot block K of the current matrix M with P = M_KK^-1 gives
//   M_KK <- -P,  M_RK <- M_RK P,  M_KR <- P M_KR,  M_RR <- M_RR - M_RK P M_KR
// (R: every other index); after every block is swept M = -A^-1. The pivot
// block of an unswept K is a Schur complement of A, so it stays positive
// definite. Every step is a rank-32 update of the whole matrix, written to
// the other of two buffers (ping-pong), so one grid barrier per step
// suffices. The matrix is padded to a multiple of kSwTile with an identity
// block (its inverse is the identity, and it does not couple to A). The
// whole sweep is FP32: n^3 FP64 operations would take ~0.3 ms at the GPU's
// FP64 rate, and the inverse is a preconditioner applied in FP32. The
// diagonal is lifted by kCoarseLift relative first.
//
// Each block computes the step's P itself (one warp, rows in registers,
// the scalar sweep with shuffles), from the same data in the same order, so
// every block gets the same P and takes the same branches. In exact
// arithmetic every pivot of the lifted, scaled matrix (unit diagonal) is
// at least the lift, kCoarseLift (a Schur complement of A + D is at least
// D);
// an FP32 pivot below that (rounding in a nearly singular direction) is
// raised to it, which sweeps A + E with E >= 0 diagonal: still a symmetric
// positive-definite preconditioner. A non-finite pivot stops every block at
// the same step, before the next barrier. Then the block writes its
// 64 x 64 output tiles.
constexpr int kSwPiv = 32;
constexpr int kSwTile = 64;
// Relative diagonal lift of A_c. It bounds how much the coarse correction
// amplifies the nearly singular direction (the reconstruction's free
// scale), where the FP32 PCG vectors carry rounding of ~1e-7 of their
// norm: with a 1e-6 lift the FP32 path's last LM steps lost up to 10x of
// their decrease to that noise on the 2000-camera problem, with 1e-5 they
// follow the FP64 path's steps (the FP64 path is unchanged either way).
constexpr double kCoarseLift = 1e-5;

// Lane r of the calling warp holds row r of the 32 x 32 block and floor,
// the smallest admissible value of pivot r; on return it holds row r of
// -A^-1 (the block swept on every index, pivots below their floor raised to
// it, counted in *raised). False if a pivot is not finite (the same answer
// in every lane).
__device__ __forceinline__ bool sweep32(float (&a)[kSwPiv], float floor, int lane, int *raised) {
#pragma unroll
    for (int j = 0; j < kSwPiv; ++j) {
        float piv = __shfl_sync(0xffffffffu, a[j], j);
        const float fl = __shfl_sync(0xffffffffu, floor, j);
        if (!isfinite(piv)) return false;
        if (!(piv > fl)) {
            piv = fl;
            ++*raised;
        }
        const float ip = 1.0f / piv;
        if (!isfinite(ip)) return false;
        const float f = a[j];
#pragma unroll
        for (int c = 0; c < kSwPiv; ++c) {
            if (c == j) continue;
            const float ajc = __shfl_sync(0xffffffffu, a[c], j) * ip;
            a[c] = lane == j ? ajc : fmaf(-f, ajc, a[c]);
        }
        a[j] = lane == j ? -ip : f * ip;
    }
    return true;
}

// Diagonal entry of the swept matrix: lifted by kCoarseLift relative; an
// empty row/column gets 1, and a negative entry (FP32 assembly noise on a
// nearly singular column) its magnitude, which keeps the preconditioner
// positive definite.
__device__ __forceinline__ double lifted_diagonal(double d) {
    return d == 0.0 ? 1.0 : fabs(d) * (1.0 + kCoarseLift);
}

struct SweepArgs {
    const double *A;  // [Nc x Nc] coarse matrix (FP64)
    int Nc, Np;       // size, padded size (multiple of kSwTile)
    float *X0, *X1;   // [Np x Np] ping-pong buffers
    float *Ainv;      // [Nc x Nc] result
    double *scl;      // [Np] symmetric scaling 1 / sqrt(lifted diagonal)
    int *stats;       // [0]: set on a non-finite pivot; [1]: pivots raised to their floor
};

__global__ void __launch_bounds__(256) k_coarse_sweep(SweepArgs g) {
    namespace cg = cooperative_groups;
    cg::grid_group grid = cg::this_grid();
    __shared__ float sP[kSwPiv][kSwPiv + 1];
    __shared__ float sC[kSwTile][kSwPiv + 1];   // M[I rows, K]
    __shared__ float sB[kSwPiv][kSwTile + 1];   // M[K, J cols]
    __shared__ float sW[kSwPiv][kSwTile + 1];   // P M[K, J cols]
    __shared__ float sV[kSwTile][kSwPiv + 1];   // M[I rows, K] P
    __shared__ int sfail;
    const int Nc = g.Nc, Np = g.Np;
    const int nt = Np / kSwTile, tiles = nt * nt;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int tx = tid & 15, ty = tid >> 4;
    // Start: the diagonal lifted by kCoarseLift relative (keeps a nearly
    // singular coarse matrix away from breakdown; it is a preconditioner; an
    // empty row/column gets a unit diagonal), then scaled symmetrically to a
    // unit diagonal, D^-1/2 A D^-1/2: the columns mix units (rotations,
    // translations, focal lengths, distortion) over many orders of
    // magnitude, which an unscaled FP32 elimination does not resolve. The
    // padded FP32 copy of the scaled matrix is swept; its inverse is scaled
    // back at the end.
    for (long long r = blockIdx.x * (long long)blockDim.x + tid; r < Np; r += (long long)gridDim.x * blockDim.x) {
        g.scl[r] = 1.0 / sqrt(lifted_diagonal(r < Nc ? g.A[(size_t)r * Nc + r] : 1.0));
    }
    grid.sync();
    for (int t = blockIdx.x; t < tiles; t += gridDim.x) {
        const int R0 = (t / nt) * kSwTile, C0 = (t % nt) * kSwTile;
        for (int e = tid; e < kSwTile * kSwTile; e += blockDim.x) {
            const int r = R0 + e / kSwTile, c = C0 + e % kSwTile;
            double v = r == c ? 1.0 : 0.0;
            if (r < Nc && c < Nc) {
                v = g.A[(size_t)r * Nc + c];
                if (r == c) v = lifted_diagonal(v);
                v *= g.scl[r] * g.scl[c];
            }
            g.X0[(size_t)r * Np + c] = (float)v;
        }
    }
    grid.sync();
    const int steps = Np / kSwPiv;
    for (int k = 0; k < steps; ++k) {
        const float *src = (k & 1) ? g.X1 : g.X0;
        float *dst = (k & 1) ? g.X0 : g.X1;
        const int k0 = k * kSwPiv;
        if (warp == 0) {
            float a[kSwPiv];
            const float4 *row = reinterpret_cast<const float4 *>(src + (size_t)(k0 + lane) * Np + k0);
#pragma unroll
            for (int q = 0; q < kSwPiv / 4; ++q) {
                const float4 v = row[q];
                a[4 * q] = v.x;
                a[4 * q + 1] = v.y;
                a[4 * q + 2] = v.z;
                a[4 * q + 3] = v.w;
            }
            int raised = 0;
            const bool ok = sweep32(a, (float)kCoarseLift, lane, &raised);  // the scaled, lifted diagonal is 1
            if (lane == 0) {
                sfail = ok ? 0 : 1;
                if (blockIdx.x == 0 && raised) g.stats[1] += raised;
            }
#pragma unroll
            for (int c = 0; c < kSwPiv; ++c) sP[lane][c] = -a[c];
        }
        __syncthreads();
        if (sfail) {  // every block stops at this step; the result is all zeros
            if (blockIdx.x == 0 && tid == 0) g.stats[0] = 1;
            for (long long e = blockIdx.x * (long long)blockDim.x + tid; e < (long long)Nc * Nc;
                 e += (long long)gridDim.x * blockDim.x)
                g.Ainv[e] = 0.0f;
            return;
        }
        for (int t = blockIdx.x; t < tiles; t += gridDim.x) {
            const int R0 = (t / nt) * kSwTile, C0 = (t % nt) * kSwTile;
            const int rK = (k0 >= R0 && k0 < R0 + kSwTile) ? k0 - R0 : -1;  // tile rows in K
            const int cK = (k0 >= C0 && k0 < C0 + kSwTile) ? k0 - C0 : -1;  // tile columns in K
            for (int e = tid; e < kSwTile * kSwPiv; e += blockDim.x) {
                const int r = e / kSwPiv, q = e % kSwPiv;
                sC[r][q] = src[(size_t)(R0 + r) * Np + k0 + q];
                const int u = e / kSwTile, c = e % kSwTile;
                sB[u][c] = src[(size_t)(k0 + u) * Np + C0 + c];
            }
            __syncthreads();
            for (int e = tid; e < kSwPiv * kSwTile; e += blockDim.x) {  // W = P B
                const int u = e / kSwTile, c = e % kSwTile;
                float w = 0.0f;
#pragma unroll 8
                for (int q = 0; q < kSwPiv; ++q) w = fmaf(sP[u][q], sB[q][c], w);
                sW[u][c] = w;
            }
            if (cK >= 0)
                for (int e = tid; e < kSwTile * kSwPiv; e += blockDim.x) {  // V = C P
                    const int r = e / kSwPiv, c = e % kSwPiv;
                    float v = 0.0f;
#pragma unroll 8
                    for (int q = 0; q < kSwPiv; ++q) v = fmaf(sC[r][q], sP[q][c], v);
                    sV[r][c] = v;
                }
            __syncthreads();
            float acc[4][4] = {};
#pragma unroll 4
            for (int q = 0; q < kSwPiv; ++q) {
                float x[4], y[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) x[i] = sC[ty * 4 + i][q];
#pragma unroll
                for (int j = 0; j < 4; ++j) y[j] = sW[q][tx + 16 * j];
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(x[i], y[j], acc[i][j]);
            }
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int r = ty * 4 + i;
                const bool inK_r = rK >= 0 && r >= rK && r < rK + kSwPiv;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int c = tx + 16 * j;
                    const bool inK_c = cK >= 0 && c >= cK && c < cK + kSwPiv;
                    float v;
                    if (inK_r && inK_c) v = -sP[r - rK][c - cK];
                    else if (inK_r) v = sW[r - rK][c];
                    else if (inK_c) v = sV[r][c - cK];
                    else v = src[(size_t)(R0 + r) * Np + C0 + c] - acc[i][j];
                    dst[(size_t)(R0 + r) * Np + C0 + c] = v;
                }
            }
            __syncthreads();  // the shared tiles are reused by the next tile
        }
        grid.sync();
    }
    // The swept matrix is -(D^-1/2 A D^-1/2)^-1: Ainv = -D^-1/2 (X + X^T) / 2
    // D^-1/2 (symmetric to the last bit).
    const float *X = (steps & 1) ? g.X1 : g.X0;
    for (long long e = blockIdx.x * (long long)blockDim.x + tid; e < (long long)Nc * Nc;
         e += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(e / Nc), c = (int)(e - (long long)r * Nc);
        const float s = (float)g.scl[r] * (float)g.scl[c];
        g.Ainv[e] = -0.5f * (X[(size_t)r * Np + c] + X[(size_t)c * Np + r]) * s;
    }
}

// zc = Z^T r: per cluster and column, the sum over the cluster's images in
// image order. One warp per cluster.
template <typename T, int D>
__global__ void __launch_bounds__(256) k_coarse_restrict(const T *__restrict__ r, const int *__restrict__ clu_start,
                                                         const int *__restrict__ img_pmask, int nc,
                                                         const LMState *__restrict__ st, int check_done,
                                                         double *__restrict__ zc) {
    if (check_done && st->pcg_done) return;
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (c >= nc || lane >= D) return;
    double s = 0.0;
    const int i1 = clu_start[c + 1];
    int i = clu_start[c];
    for (; i + 8 <= i1; i += 8) {  // loads eight at a time, added in image order
        T w[8];
#pragma unroll
        for (int u = 0; u < 8; ++u)
            w[u] = ((img_pmask[i + u] >> lane) & 1) ? r[(size_t)(i + u) * D + lane] : T(0);
#pragma unroll
        for (int u = 0; u < 8; ++u) s += (double)w[u];
    }
    for (; i < i1; ++i)
        if ((img_pmask[i] >> lane) & 1) s += (double)r[(size_t)i * D + lane];
    zc[c * D + lane] = s;
}

// cc = A_c^-1 zc, one warp per row (the 16-byte loads of the FP32 inverse
// are the traffic: Nc^2 x 4 bytes, L2-resident between iterations).
template <typename T>
__global__ void __launch_bounds__(256) k_coarse_gemv(const float *__restrict__ Ainv, const double *__restrict__ zc,
                                                     int Nc, const LMState *__restrict__ st, int check_done,
                                                     T *__restrict__ cc) {
    if (check_done && st->pcg_done) return;
    const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= Nc) return;
    const float *a = Ainv + (size_t)row * Nc;
    double s = 0.0;
    int j = lane;
    for (; j + 7 * 32 < Nc; j += 8 * 32) {  // loads eight at a time, accumulated in column order
        float w[8];
        double y[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            w[u] = __ldg(a + j + 32 * u);
            y[u] = zc[j + 32 * u];
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) s += (double)w[u] * y[u];
    }
    for (; j < Nc; j += 32) s += (double)__ldg(a + j) * zc[j];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (lane == 0) cc[row] = (T)s;
}

// z_i += cc[cluster(i)] on the image's unknown columns; partials of r.z and
// r.r. init: the start of a solve — p = z (and its padded FP32 copy), and the
// solve's done flag (set by the previous solve) is not consulted.
template <typename T, int D>
__global__ void __launch_bounds__(256) k_coarse_z(const T *__restrict__ r, const T *__restrict__ cc,
                                                  const int *__restrict__ img_cluster,
                                                  const int *__restrict__ img_pmask,
                                                  const int *__restrict__ img_dmask, const LMState *__restrict__ st,
                                                  int nI, int init, T *__restrict__ z, T *__restrict__ p,
                                                  float *__restrict__ p4, double *__restrict__ part) {
    if (!init && st->pcg_done) return;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= nI) return;
    const size_t base = (size_t)i * D;
    double rz = 0.0, rr = 0.0;
    if (lane < D) {
        const double rc = (double)r[base + lane];
        double zc = (double)z[base + lane];
        const bool own = (img_pmask[i] >> lane) & 1;  // a shared camera's columns keep their entries
        if (own) zc += (double)cc[(size_t)img_cluster[i] * D + lane];
        const T zt = (T)zc;
        z[base + lane] = zt;
        if (init && own) {
            p[base + lane] = zt;
            if (p4) store_dir(p4, nI, i, lane, (float)zt);
        }
        if ((img_dmask[i] >> lane) & 1) {
            rz = rc * (double)zt;
            rr = rc * rc;
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        rz += __shfl_xor_sync(0xffffffffu, rz, off);
        rr += __shfl_xor_sync(0xffffffffu, rr, off);
    }
    if (lane == 0) {
        part[i] = rz;
        part[nI + i] = rr;
    }
}

}  // namespace

size_t coarse_setup_temp_bytes(int nP, long long npairs_max) {
    size_t a = 0, bsz = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, a, (long long *)nullptr, (long long *)nullptr, nP > 0 ? nP : 1);
    const int n = (int)std::max<long long>(1, std::min<long long>(npairs_max, (1LL << 31) - 1));
    cub::DeviceRadixSort::SortPairs(nullptr, bsz, (int *)nullptr, (int *)nullptr, (int *)nullptr, (int *)nullptr, n);
    return std::max(a, bsz);
}

long long launch_coarse_count(const Bufs &b, long long *count, long long *off, long long *kcount,
                              long long *inc_off, long long *ninc, void *temp, size_t temp_bytes, cudaStream_t s) {
    *ninc = 0;
    if (b.nP == 0) return 0;
    k_coarse_count<<<div_up(b.nP, 128), 128, 0, s>>>(b.pt_start, b.ob_img, b.co.img_cluster, b.nP, count, kcount);
    SFMBA_LAUNCH_CHECK();
    size_t tb = temp_bytes;
    SFMBA_CUDA(cub::DeviceScan::ExclusiveSum(temp, tb, count, off, b.nP, s));
    tb = temp_bytes;
    SFMBA_CUDA(cub::DeviceScan::ExclusiveSum(temp, tb, kcount, inc_off, b.nP + 1, s));  // kcount[nP] = 0
    long long last_off = 0, last_cnt = 0;
    SFMBA_CUDA(cudaMemcpyAsync(&last_off, off + b.nP - 1, sizeof(long long), cudaMemcpyDeviceToHost, s));
    SFMBA_CUDA(cudaMemcpyAsync(&last_cnt, count + b.nP - 1, sizeof(long long), cudaMemcpyDeviceToHost, s));
    SFMBA_CUDA(cudaMemcpyAsync(ninc, inc_off + b.nP, sizeof(long long), cudaMemcpyDeviceToHost, s));
    SFMBA_CUDA(cudaStreamSynchronize(s));
    return last_off + last_cnt;
}

void launch_coarse_group(const Bufs &b, const long long *off, long long npairs, int *key, int *val, int *key2,
                         int *val_sorted, int *key_counts, void *temp, size_t temp_bytes, cudaStream_t s) {
    const int nc = b.co.nc;
    k_coarse_emit<<<div_up(b.nP, 128), 128, 0, s>>>(b.pt_start, b.ob_img, b.co.img_cluster, b.nP, nc, off,
                                                    b.co.inc_off, key, val, b.co.inc_cl, b.co.inc_pt);
    SFMBA_LAUNCH_CHECK();
    size_t tb = temp_bytes;
    int bits = 1;
    while ((1LL << bits) < (long long)nc * nc) ++bits;
    SFMBA_CUDA(cub::DeviceRadixSort::SortPairs(temp, tb, key, key2, val, val_sorted, (int)npairs, 0, bits, s));
    SFMBA_CUDA(cudaMemsetAsync(key_counts, 0, sizeof(int) * (size_t)nc * nc, s));
    k_key_counts<<<div_up(npairs, 256), 256, 0, s>>>(key2, npairs, key_counts);
    SFMBA_LAUNCH_CHECK();
}

void launch_coarse_inc_order(const Bufs &b, int *key, int *val, int *key2, void *temp, size_t temp_bytes,
                             cudaStream_t s) {
    const CoarseBufs &co = b.co;
    if (co.ninc <= 0) return;
    k_inc_keys<<<div_up(b.nP, 128), 128, 0, s>>>(b.pt_start, co.inc_off, b.nP, key, val);
    SFMBA_LAUNCH_CHECK();
    size_t tb = temp_bytes;
    SFMBA_CUDA(cub::DeviceRadixSort::SortPairs(temp, tb, key, key2, val, co.inc_order, (int)co.ninc, 0, 16, s));
}

void launch_coarse_assemble(const Bufs &b, cudaStream_t s) {
    const CoarseBufs &co = b.co;
    const int D = b.D, Nc = co.nc * D;
    SFMBA_CUDA(cudaMemsetAsync(co.A, 0, sizeof(double) * (size_t)Nc * Nc, s));
    k_coarse_diag<<<co.nc, 128, 0, s>>>(b.img_H, b.img_pmask, co.clu_start, co.nc, D, b.state, co.A);
    SFMBA_LAUNCH_CHECK();
    if (co.nchunks > 0) {
        const unsigned yb = (unsigned)div_up(co.ninc, 128);
        dispatch_TDR(b, [&](auto t, auto dc, auto rc, auto mc) {  // Y with the camera model compiled in
            using T = decltype(t);
            k_coarse_y<T, decltype(dc)::value, decltype(rc)::value, decltype(mc)::value><<<yb, 128, 0, s>>>(
                jac_src<T>(b), b.pt_start, co.img_cluster, b.img_pmask, co.inc_pt, co.inc_cl, co.inc_order, co.ninc,
                b.pt_ok, (T *)co.ybuf);
        });
        SFMBA_LAUNCH_CHECK();
        dispatch_D(D, [&](auto dc) {
            constexpr int DD = decltype(dc)::value;
            if (b.mixed) {
                k_coarse_pairs<float, DD><<<div_up(co.nchunks, 4), 128, 0, s>>>(
                    (const float *)co.ybuf, co.inc_off, co.inc_cl, co.chunk, co.nchunks, co.pair_pt, co.group_cc,
                    (const float *)b.pt_Cinv, b.pt_ok, co.chunk_part);
            } else {
                k_coarse_pairs<double, DD><<<div_up(co.nchunks, 2), 64, 0, s>>>(
                    (const double *)co.ybuf, co.inc_off, co.inc_cl, co.chunk, co.nchunks, co.pair_pt, co.group_cc,
                    (const double *)b.pt_Cinv, b.pt_ok, co.chunk_part);
            }
        });
        SFMBA_LAUNCH_CHECK();
        k_coarse_finish<<<co.ngroups, 128, 0, s>>>(co.chunk_part, co.group_chunk_off, co.group_cc, co.ngroups, co.nc,
                                                   D, co.A);
        SFMBA_LAUNCH_CHECK();
    }
}

int coarse_padded_size(int Nc) { return div_up(Nc, kSwTile) * kSwTile; }

void launch_coarse_invert(const Bufs &b, cudaStream_t s) {
    const CoarseBufs &co = b.co;
    const int Nc = co.nc * b.D, Np = coarse_padded_size(Nc);
    SFMBA_CUDA(cudaMemsetAsync(co.fail, 0, 2 * sizeof(int), s));
    static int cap_dev = -1, cap = 0;  // co-resident blocks, queried once per device
    int dev = 0;
    SFMBA_CUDA(cudaGetDevice(&dev));
    if (cap_dev != dev) {
        int per_sm = 0, sms = 0;
        SFMBA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_coarse_sweep, 256, 0));
        SFMBA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        cap = per_sm * sms;
        cap_dev = dev;
    }
    if (cap < 1) throw Error(SFMBA_ERR_INTERNAL, "the coarse inverse kernel cannot be resident");
    const int nt = Np / kSwTile;
    SweepArgs g{co.A, Nc, Np, co.X32, co.X32 + (size_t)Np * Np, co.Ainv,
                reinterpret_cast<double *>(co.X32 + (size_t)2 * Np * Np), co.fail};
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)std::min(nt * nt, cap));
    cfg.blockDim = dim3(256);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    SFMBA_CUDA(cudaLaunchKernelEx(&cfg, k_coarse_sweep, g));
    SFMBA_LAUNCH_CHECK();
}

void launch_coarse_correct(const Bufs &b, bool init, cudaStream_t s) {
    const CoarseBufs &co = b.co;
    const int Nc = co.nc * b.D;
    dispatch_D(b.D, [&](auto dc) {
        constexpr int D = decltype(dc)::value;
        auto run = [&](auto t) {
            using T = decltype(t);
            k_coarse_restrict<T, D><<<div_up(co.nc, 8), 256, 0, s>>>((const T *)b.pcg_r, co.clu_start, b.img_pmask,
                                                                     co.nc, b.state, init ? 0 : 1, co.zc);
            SFMBA_LAUNCH_CHECK();
            k_coarse_gemv<T><<<div_up(Nc, 8), 256, 0, s>>>(co.Ainv, co.zc, Nc, b.state, init ? 0 : 1, (T *)co.cc);
            SFMBA_LAUNCH_CHECK();
            k_coarse_z<T, D><<<div_up(b.nI, 8), 256, 0, s>>>(
                (const T *)b.pcg_r, (const T *)co.cc, co.img_cluster, b.img_pmask, b.img_dmask, b.state, b.nI,
                init ? 1 : 0,
                (T *)b.pcg_z, (T *)b.pcg_p, std::is_same<T, float>::value ? b.pcg_p4 : nullptr, b.pcg_part);
            SFMBA_LAUNCH_CHECK();
        };
        if (b.mixed) run(0.0f);
        else run(0.0);
    });
}

}  // namespace sfmba
