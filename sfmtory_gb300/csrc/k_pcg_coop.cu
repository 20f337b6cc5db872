// The vector side of one PCG iteration as a single cooperative launch.
//
// After the two observation passes, an iteration needs a chain of small
// steps with a grid-wide dependency between each: q = S p from the image
// pass's partials (and the sum over a shared camera's images), the p.q
// reduction and alpha, x/r updates with z = M^-1 r, the coarse correction
// (restriction over image clusters, the dense product with A_c^-1,
// prolongation), the r.z reduction, beta and the new direction. As separate
// launches each step costs a launch and a drain of the GPU; here one grid of
// co-resident blocks runs them all with grid-wide barriers between them
// (cooperative launch: every block is resident, so the barriers cannot
// wait on a block that never runs). The dot products are summed per warp
// over its images, then per block, and after the barrier every block adds
// the blocks' partials in block order: each reduction that decides whether
// to stop is computed by every block in the same order, so all blocks take
// the same branch and reach the same barriers.
#include <cooperative_groups.h>

#include <algorithm>
#include <type_traits>

#include "kernels.cuh"

namespace cg = cooperative_groups;

namespace sfmba {

namespace {

// Sums of the blocks' partials X[0, G) and Y[0, G) (Y may be null), added
// by the block's first warp in a fixed order (lane l: X[l], X[l + 32], ...,
// then a butterfly) and handed to every thread: every block that reads the
// same partials gets the same bits. One warp adds, so the block's other
// warps do not contend for the FP64 pipe.
__device__ __forceinline__ double2 grid_sums(const double *X, const double *Y, int G, double *sh) {
    __syncthreads();  // sh is free: its previous readers are done
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        double sx = 0.0, sy = 0.0;
        for (int base = 0; base < G; base += 8 * 32) {
            double wx[8], wy[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int j = base + lane + 32 * u;
                wx[u] = j < G ? X[j] : 0.0;
                wy[u] = (Y && j < G) ? Y[j] : 0.0;
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                sx += wx[u];
                sy += wy[u];
            }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            sx += __shfl_xor_sync(0xffffffffu, sx, off);
            sy += __shfl_xor_sync(0xffffffffu, sy, off);
        }
        if (lane == 0) {
            sh[0] = sx;
            sh[1] = sy;
        }
    }
    __syncthreads();
    return make_double2(sh[0], sh[1]);
}

template <typename T>
struct VecArgs {
    const T *ipart;
    const int *ipart_off;
    const double *img_H;  // FP64 path: H_i (damped here)
    const float *img_Hf;  // FP32 path: H_i + lambda diag H_i
    const int *img_active, *img_pmask, *img_dmask;
    const T *Minv;
    T *p, *q, *x, *r, *z;
    float *p4;
    double *blk;  // per-block partial sums [4][gridDim.x]: p.q, p.q of shared cameras, r.z, r.r
    LMState *st;
    int nI, nID, parity;
    // shared cameras (nsh = 0: none)
    int nsh;
    const int *sh_img_start, *sh_imgs, *img_owner;
    // coarse correction (nc = 0: none)
    int nc, Nc;
    const int *clu_start, *img_cluster;
    const float *Ainv;
    double *zc;
    T *cc;
    // fused coarse phase: every warp holds one image and block b images
    // [8b, 8b + 8), so a block restricts its own images (zpart: [blocks][3][D]
    // per-block sums over the <= 3 clusters they touch) and, after one
    // barrier, applies the coarse correction to them (zc rebuilt per block).
    int fused;
    double *zpart;
};

// Writes this block's sum of its warps' values (warp order) to out[blockIdx.x].
__device__ __forceinline__ void block_partial(double warp_value, double *sh, double *out) {
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = warp_value;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r += sh[w];
        out[blockIdx.x] = r;
    }
}

template <typename T, int D>
__global__ void __launch_bounds__(256) k_pcg_vec_coop(VecArgs<T> a) {
    cg::grid_group grid = cg::this_grid();
    __shared__ double sh[32];
    LMState *st = a.st;
    // Read before any block of this launch writes the state (block 0 writes
    // it only after the first grid barrier), so every block sees one value.
    if (st->pcg_done) return;
    const int nI = a.nI;
    const int G = gridDim.x;
    const int lane = threadIdx.x & 31;
    const int gw = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int nw = (int)((gridDim.x * blockDim.x) >> 5);
    const double lam = st->lambda;
    double *PQ = a.blk, *PQS = a.blk + G, *RZ = a.blk + 2 * G, *RR = a.blk + 3 * G;
    T *zpart = reinterpret_cast<T *>(a.zpart);  // the fused restriction's per-block sums, kernel precision
    // q_i = (H_i + lambda diag H_i) p_i - sum of the image's partials; p.q over
    // pmask, summed per warp over its images, then per block.
    {
        double pq_w = 0.0;
        for (int i = gw; i < nI; i += nw) {
            const int act = a.img_active[i], pm = a.img_pmask[i];
            const T *pv = a.p + (size_t)i * D;
            T pq = T(0);
            if (lane < D) {
                const int c = lane;
                T sch = T(0);
                const int k1 = a.ipart_off[i + 1];
                int k = a.ipart_off[i];
                for (; k + 8 <= k1; k += 8) {
                    T w[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) w[u] = a.ipart[(size_t)(k + u) * D + c];
#pragma unroll
                    for (int u = 0; u < 8; ++u) sch += w[u];
                }
                for (; k < k1; ++k) sch += a.ipart[(size_t)k * D + c];
                T hp = T(0);
                if constexpr (std::is_same<T, float>::value) {
                    const float *H = a.img_Hf + (size_t)i * D * D;
#pragma unroll
                    for (int d = 0; d < D; ++d) hp += H[c * D + d] * pv[d];
                } else {
                    const double *H = a.img_H + (size_t)i * D * D;
#pragma unroll
                    for (int d = 0; d < D; ++d) hp += H[c * D + d] * pv[d];
                    hp += lam * H[c * D + c] * pv[c];
                }
                const T qc = ((act >> c) & 1) ? hp - sch : T(0);
                a.q[(size_t)i * D + c] = qc;
                if ((pm >> c) & 1) pq = pv[c] * qc;
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) pq += __shfl_xor_sync(0xffffffffu, pq, off);
            pq_w += (double)pq;
        }
        block_partial(pq_w, sh, PQ);
    }
    const bool shared_cams = D > 6 && a.nsh > 0;
    grid.sync();
    if constexpr (D > 6) {
        if (shared_cams) {  // shared cameras: q summed over each camera's images, the owner's p.q
            constexpr int KC = D - 6;
            double pq_w = 0.0;
            for (int c = gw; c < a.nsh; c += nw) {
                const int i0 = a.sh_img_start[c], i1 = a.sh_img_start[c + 1];
                const int owner = a.sh_imgs[i0];
                double pq = 0.0;
                if (lane < KC) {
                    double s = 0.0;
                    for (int k = i0; k < i1; ++k) s += (double)a.q[(size_t)a.sh_imgs[k] * D + 6 + lane];
                    const T qt = (T)s;
                    for (int k = i0; k < i1; ++k) a.q[(size_t)a.sh_imgs[k] * D + 6 + lane] = qt;
                    pq = (double)a.p[(size_t)owner * D + 6 + lane] * (double)qt;
                }
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) pq += __shfl_xor_sync(0xffffffffu, pq, off);
                pq_w += pq;
            }
            block_partial(pq_w, sh, PQS);
            grid.sync();
        }
    }
    // alpha = (r.z) / (p.q); x += alpha p; r -= alpha q; z = M^-1 r; r.z, r.r partials.
    {
        const double2 pqs = grid_sums(PQ, shared_cams ? PQS : nullptr, G, sh);
        const double pq = shared_cams ? pqs.x + pqs.y : pqs.x;
        if (!(pq > 0.0) || !isfinite(pq)) {  // breakdown (every block sees it): keep the iterate
            if (blockIdx.x == 0 && threadIdx.x == 0) {
                st->pcg_done = 1;
                st->pcg_breakdowns += 1;
                st->pcg_alpha = 0.0;
            }
            return;
        }
        const double alpha = st->pcg_rzbuf[a.parity] / pq;
        if (blockIdx.x == 0 && threadIdx.x == 0) st->pcg_alpha = alpha;
        __shared__ T rs[8][16];  // fused coarse: this block's images' restricted residuals
        const T al = (T)alpha;
        double rz_w = 0.0, rr_w = 0.0;
        for (int i = gw; i < nI; i += nw) {
            const size_t base = (size_t)i * D;
            T rc = T(0);
            if (lane < D) {
                a.x[base + lane] = a.x[base + lane] + al * a.p[base + lane];
                rc = a.r[base + lane] - al * a.q[base + lane];
                a.r[base + lane] = rc;
            }
            T zc = T(0);
            const T *M = a.Minv + (size_t)i * D * D;
#pragma unroll
            for (int d = 0; d < D; ++d) {
                const T rd = __shfl_sync(0xffffffffu, rc, d);
                if (lane < D) zc += M[lane * D + d] * rd;
            }
            T rz = T(0), rr = T(0);
            if (lane < D) {
                a.z[base + lane] = zc;
                if ((a.img_dmask[i] >> lane) & 1) {
                    rz = rc * zc;
                    rr = rc * rc;
                }
                if (a.fused) rs[threadIdx.x >> 5][lane] = ((a.img_pmask[i] >> lane) & 1) ? rc : T(0);
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                rz += __shfl_xor_sync(0xffffffffu, rz, off);
                rr += __shfl_xor_sync(0xffffffffu, rr, off);
            }
            rz_w += (double)rz;
            rr_w += (double)rr;
        }
        if (a.fused) {  // per-block sums of the restriction over the clusters of images [8b, 8b + 8)
            __syncthreads();
            const int i0 = blockIdx.x * 8, i1 = min(i0 + 8, nI);
            if (i0 < nI && (int)threadIdx.x < 3 * D) {
                const int s = threadIdx.x / D, d = threadIdx.x - s * D;
                const int c = a.img_cluster[i0] + s;
                T v = T(0);
                for (int i = i0; i < i1; ++i)
                    if (a.img_cluster[i] == c) v += rs[i - i0][d];
                zpart[((size_t)blockIdx.x * 3 + s) * D + d] = v;
            }
        } else if (a.nc == 0) {  // no coarse correction: these are the iteration's r.z, r.r
            block_partial(rz_w, sh, RZ);
            block_partial(rr_w, sh, RR);
        }
    }
    grid.sync();
    if (a.nc > 0 && a.fused) {
        // zc = Z^T r from the per-block sums (every block rebuilds all of it),
        // cc rows of this block's clusters, z_i += cc[cluster(i)] for its
        // images, r.z / r.r partials.
        __shared__ T zcs[kMaxCoarseClusters * 14];
        __shared__ T ccs[3 * 16];
        __shared__ int cls[kMaxCoarseClusters + 1];  // clu_start
        __shared__ int cl0[kMaxCoarseClusters];      // cluster of the first image of a cluster's first block
        for (int c = threadIdx.x; c <= a.nc; c += blockDim.x) {
            const int st0 = a.clu_start[c];
            cls[c] = st0;
            if (c < a.nc) cl0[c] = a.clu_start[c + 1] > st0 ? a.img_cluster[(st0 >> 3) * 8] : 0;  // empty: unused
        }
        __syncthreads();
        // Cluster c spans blocks b0..b1; every block after b0 starts inside c
        // (its slot 0), block b0 holds c in slot c - cluster(8 b0). Sums in
        // block order; the loads of a chunk are issued before its adds.
        for (int e = threadIdx.x; e < a.Nc; e += blockDim.x) {
            const int c = e / D, d = e - c * D;
            const int b0 = cls[c] >> 3, b1 = (cls[c + 1] - 1) >> 3;
            T v = T(0);
            if (b1 >= b0) {
                v = zpart[((size_t)b0 * 3 + (c - cl0[c])) * D + d];
                for (int b = b0 + 1; b <= b1; b += 8) {
                    T w[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) w[u] = b + u <= b1 ? zpart[(size_t)(b + u) * 3 * D + d] : T(0);
#pragma unroll
                    for (int u = 0; u < 8; ++u)
                        if (b + u <= b1) v += w[u];
                }
            }
            zcs[e] = v;
        }
        __syncthreads();
        const int i0 = blockIdx.x * 8, i1 = min(i0 + 8, nI);
        double rz = 0.0, rr = 0.0;
        if (i0 < nI) {
            const int c0 = a.img_cluster[i0], nrow = (a.img_cluster[i1 - 1] - c0 + 1) * D;
            const int wl = threadIdx.x >> 5;
            // Rows rl, rl + 8, rl + 16 of A_c^-1 per warp at a time, eight
            // column loads per row in flight; each lane adds its columns in
            // column order, then the butterfly.
            constexpr int RW = 3;
            for (int rl = wl; rl < nrow; rl += 8 * RW) {
                const float *ar[RW];
                T s[RW];
#pragma unroll
                for (int k = 0; k < RW; ++k) {
                    const int row = min(rl + 8 * k, nrow - 1);
                    ar[k] = a.Ainv + (size_t)(c0 * D + row) * a.Nc;
                    s[k] = T(0);
                }
                for (int base = 0; base < a.Nc; base += 8 * 32) {
                    float w[RW][8];
#pragma unroll
                    for (int k = 0; k < RW; ++k)
#pragma unroll
                        for (int u = 0; u < 8; ++u) {
                            const int j = base + lane + 32 * u;
                            w[k][u] = j < a.Nc ? __ldg(ar[k] + j) : 0.0f;
                        }
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const int j = base + lane + 32 * u;
                        if (j < a.Nc) {
                            const T zj = zcs[j];
#pragma unroll
                            for (int k = 0; k < RW; ++k) s[k] += (T)w[k][u] * zj;
                        }
                    }
                }
#pragma unroll
                for (int k = 0; k < RW; ++k) {
#pragma unroll
                    for (int off = 16; off > 0; off >>= 1) s[k] += __shfl_xor_sync(0xffffffffu, s[k], off);
                    if (lane == 0 && rl + 8 * k < nrow) ccs[rl + 8 * k] = s[k];
                }
            }
            __syncthreads();
            const int i = gw;
            if (i < i1) {
                const size_t base = (size_t)i * D;
                T rzl = T(0), rrl = T(0);
                if (lane < D) {
                    const T rc = a.r[base + lane];
                    T zc = a.z[base + lane];
                    if ((a.img_pmask[i] >> lane) & 1) zc += ccs[(a.img_cluster[i] - c0) * D + lane];
                    a.z[base + lane] = zc;
                    if ((a.img_dmask[i] >> lane) & 1) {
                        rzl = rc * zc;
                        rrl = rc * rc;
                    }
                }
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) {
                    rzl += __shfl_xor_sync(0xffffffffu, rzl, off);
                    rrl += __shfl_xor_sync(0xffffffffu, rrl, off);
                }
                rz = (double)rzl;
                rr = (double)rrl;
            }
        }
        block_partial(rz, sh, RZ);
        block_partial(rr, sh, RR);
        grid.sync();
    } else if (a.nc > 0) {
        // zc = Z^T r (per cluster and column, image order, own columns only)
        for (int c = gw; c < a.nc; c += nw) {
            if (lane < D) {
                double s = 0.0;
                const int i1 = a.clu_start[c + 1];
                int i = a.clu_start[c];
                for (; i + 8 <= i1; i += 8) {
                    T w[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u)
                        w[u] = ((a.img_pmask[i + u] >> lane) & 1) ? a.r[(size_t)(i + u) * D + lane] : T(0);
#pragma unroll
                    for (int u = 0; u < 8; ++u) s += (double)w[u];
                }
                for (; i < i1; ++i)
                    if ((a.img_pmask[i] >> lane) & 1) s += (double)a.r[(size_t)i * D + lane];
                a.zc[c * D + lane] = s;
            }
        }
        grid.sync();
        // cc = A_c^-1 zc, one warp per row
        for (int row = gw; row < a.Nc; row += nw) {
            const float *ar = a.Ainv + (size_t)row * a.Nc;
            double s = 0.0;
            int j = lane;
            for (; j + 7 * 32 < a.Nc; j += 8 * 32) {
                float w[8];
                double y[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    w[u] = __ldg(ar + j + 32 * u);
                    y[u] = a.zc[j + 32 * u];
                }
#pragma unroll
                for (int u = 0; u < 8; ++u) s += (double)w[u] * y[u];
            }
            for (; j < a.Nc; j += 32) s += (double)__ldg(ar + j) * a.zc[j];
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
            if (lane == 0) a.cc[row] = (T)s;
        }
        grid.sync();
        // z_i += cc[cluster(i)] on the image's own columns; r.z, r.r partials
        double rz_w = 0.0, rr_w = 0.0;
        for (int i = gw; i < nI; i += nw) {
            const size_t base = (size_t)i * D;
            double rz = 0.0, rr = 0.0;
            if (lane < D) {
                const double rc = (double)a.r[base + lane];
                double zc = (double)a.z[base + lane];
                if ((a.img_pmask[i] >> lane) & 1) zc += (double)a.cc[(size_t)a.img_cluster[i] * D + lane];
                const T zt = (T)zc;
                a.z[base + lane] = zt;
                if ((a.img_dmask[i] >> lane) & 1) {
                    rz = rc * (double)zt;
                    rr = rc * rc;
                }
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                rz += __shfl_xor_sync(0xffffffffu, rz, off);
                rr += __shfl_xor_sync(0xffffffffu, rr, off);
            }
            rz_w += rz;
            rr_w += rr;
        }
        block_partial(rz_w, sh, RZ);
        block_partial(rr_w, sh, RR);
        grid.sync();
    }
    // convergence test, beta, p = z + beta p
    const double2 rzr = grid_sums(RZ, RR, G, sh);
    const double rz = rzr.x, rr = rzr.y;
    const bool stop = rr <= st->pcg_tol2 * st->pcg_bb || !(rz > 0.0) || !isfinite(rz);
    const double beta = stop ? 0.0 : rz / st->pcg_rzbuf[a.parity];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        st->pcg_iterations += 1;
        st->pcg_total += 1;
        st->pcg_rr = rr;
        if (stop) {
            st->pcg_done = 1;
            if (!(rr <= st->pcg_tol2 * st->pcg_bb)) st->pcg_breakdowns += 1;
        } else {
            st->pcg_beta = beta;
            st->pcg_rzbuf[a.parity ^ 1] = rz;
        }
    }
    if (stop) return;
    const int nthreads = gridDim.x * blockDim.x;
    const T bt = (T)beta;
    for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < a.nID; u += nthreads) {
        const int i = u / D, c = u - i * D;
        const int zu = (a.img_owner && c >= 6) ? a.img_owner[i] * D + c : u;
        const T pn = a.z[zu] + bt * a.p[u];
        a.p[u] = pn;
        if (a.p4) store_dir(a.p4, nI, i, c, (float)pn);
    }
}

template <typename F>
void dispatch_D_coop(int D, F &&f) {
    switch (D) {
    case 6: f(std::integral_constant<int, 6>()); break;
    case 9: f(std::integral_constant<int, 9>()); break;
    case 10: f(std::integral_constant<int, 10>()); break;
    case 11: f(std::integral_constant<int, 11>()); break;
    case 14: f(std::integral_constant<int, 14>()); break;
    default: throw Error(SFMBA_ERR_INTERNAL, "unsupported image block width");
    }
}

template <typename T, int D>
void run_coop(const Bufs &b, cudaStream_t s, int parity, bool coarse) {
    VecArgs<T> a{};
    a.ipart = (const T *)b.ipart;
    a.ipart_off = b.ipart_off;
    a.img_H = b.img_H;
    a.img_Hf = b.img_Hf;
    a.img_active = b.img_active;
    a.img_pmask = b.img_pmask;
    a.img_dmask = b.img_dmask;
    a.Minv = (const T *)b.pcg_Minv;
    a.p = (T *)b.pcg_p;
    a.q = (T *)b.pcg_q;
    a.x = (T *)b.pcg_x;
    a.r = (T *)b.pcg_r;
    a.z = (T *)b.pcg_z;
    a.p4 = std::is_same<T, float>::value ? b.pcg_p4 : nullptr;
    a.blk = b.pcg_blk;
    a.st = b.state;
    a.nI = b.nI;
    a.nID = b.nID;
    a.parity = parity;
    a.nsh = b.sh.nsh;
    a.sh_img_start = b.sh.sh_img_start;
    a.sh_imgs = b.sh.sh_imgs;
    a.img_owner = b.sh.nsh > 0 ? b.sh.img_owner : nullptr;
    if (coarse) {
        a.nc = b.co.nc;
        a.Nc = b.co.nc * D;
        a.clu_start = b.co.clu_start;
        a.img_cluster = b.co.img_cluster;
        a.Ainv = b.co.Ainv;
        a.zc = b.co.zc;
        a.cc = (T *)b.co.cc;
    }
    // Co-resident grid: as many blocks as the widest phase needs, at most
    // what the GPU holds at once (queried once per instance and device).
    static int cap_dev = -1, cap = 0;
    int dev = 0;
    SFMBA_CUDA(cudaGetDevice(&dev));
    if (cap_dev != dev) {
        int per_sm = 0, sms = 0;
        SFMBA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg_vec_coop<T, D>, 256, 0));
        SFMBA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        cap = per_sm * sms;
        cap_dev = dev;
    }
    if (cap < 1) throw Error(SFMBA_ERR_INTERNAL, "the PCG vector kernel cannot be resident");
    const int want = std::max(std::max(std::max(div_up(b.nI, 8), div_up(a.Nc, 8)), div_up(a.nsh, 8)), 1);
    const int grid = std::min(std::min(want, cap), kPcgMaxCoopBlocks);
    // The fused coarse phase needs image i on warp i (block b: images 8b..8b+7).
    a.fused = (coarse && (long long)grid * 8 >= b.nI && D <= 16 && b.co.zpart) ? 1 : 0;
    a.zpart = b.co.zpart;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    SFMBA_CUDA(cudaLaunchKernelEx(&cfg, k_pcg_vec_coop<T, D>, a));
    SFMBA_LAUNCH_CHECK();
}

}  // namespace

void launch_pcg_iteration_vector(const Bufs &b, cudaStream_t s, int parity, bool coarse) {
    dispatch_D_coop(b.D, [&](auto dc) {
        constexpr int D = decltype(dc)::value;
        if (b.mixed) run_coop<float, D>(b, s, parity, coarse);
        else run_coop<double, D>(b, s, parity, coarse);
    });
}

}  // namespace sfmba
