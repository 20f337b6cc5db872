// Matrix-free Schur-complement PCG for the reduced camera system, at image
// level (each free camera belongs to one image, so image blocks and the
// reference's slot blocks coincide up to order).
//
//   S p = (H + lambda diag H) p - sum_p E_p^T C_p^-1 E_p p
//
// is applied in two passes without forming S: a point pass that gathers
// u_p = C_p^-1 sum_o Jx~_o^T (Jc~_o p_img(o)) (observations are point-major)
// and an image pass that reduces q_i = (H_i + lambda diag H_i) p_i -
// sum_{o in i} Jc~_o^T (Jx~_o u_p) over the image-major permutation, one
// warp per image, with no atomics. The preconditioner is block Jacobi on the
// exact image diagonal blocks of S (Cholesky-inverted per image). Scalars of
// the iteration live in the device state so the host only polls for
// convergence every few iterations. Vectors are in the kernel precision
// (FP32 on the mixed path); every dot product accumulates in FP64.
#include <type_traits>

#include "kernels.cuh"

namespace sfmba {

namespace {

template <typename T>
__device__ __forceinline__ void kahan_add(T &s, T &c, T x) {
    if constexpr (std::is_same<T, float>::value) {
        const T y = x - c;
        const T t = s + y;
        c = (t - s) - y;
        s = t;
    } else {
        s += x;
    }
}

__device__ __forceinline__ double block_sum(double v, double *sh) {
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}

// Block-Jacobi preconditioner of image i and the start vectors.
template <typename T, int D>
__global__ void __launch_bounds__(128) k_pcg_precond(const T *rec, const int *img_start, const int *img_obs,
                                                     const int *ob_pt, const T *pt_Cinv,
                                                     const unsigned char *pt_ok, const double *img_H,
                                                     const int *img_active, const double *img_rhs,
                                                     const LMState *st, int nI, T *Minv_out, T *x, T *r,
                                                     T *z, T *p, double *part) {
    constexpr int RS = RecLayout<D>::kStride;
    constexpr int F = 2 * D + 3;
    constexpr int CH = 32;
    constexpr int NH = D * (D + 1) / 2;
    __shared__ T sh[CH][F + 1];
    __shared__ double blk[D][D + 1];
    __shared__ double Mi[D][D + 1];
    __shared__ double rv[D];
    __shared__ double dg[D];
    __shared__ int fallback;
    const int i = blockIdx.x;
    if (i >= nI) return;
    const int tid = threadIdx.x;
    int ea = 0, eb = 0;
    if (tid < NH) {
        int t = tid, a = 0;
        while (t >= D - a) { t -= D - a; ++a; }
        ea = a; eb = a + t;
    }
    T acc = 0, comp = 0;
    const int s = img_start[i], e = img_start[i + 1];
    for (int base = s; base < e; base += CH) {
        const int cnt = min(CH, e - base);
        for (int idx = tid; idx < cnt * 2 * D; idx += blockDim.x) {
            const int k = idx / (2 * D), f = idx - k * 2 * D;
            sh[k][f] = rec[(size_t)img_obs[base + k] * RS + 8 + f];
        }
        if (tid < cnt) {
            const int o = img_obs[base + tid];
            const int pt = ob_pt[o];
            T m00 = 0, m01 = 0, m11 = 0;
            if (pt_ok[pt]) {
                const T *ra = rec + (size_t)o * RS;
                const T *Ci = pt_Cinv + 6 * (size_t)pt;
                T U[2][3];
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    const T a0 = ra[2 + 3 * q], a1 = ra[3 + 3 * q], a2 = ra[4 + 3 * q];
                    U[q][0] = a0 * Ci[0] + a1 * Ci[1] + a2 * Ci[2];
                    U[q][1] = a0 * Ci[1] + a1 * Ci[3] + a2 * Ci[4];
                    U[q][2] = a0 * Ci[2] + a1 * Ci[4] + a2 * Ci[5];
                }
                m00 = U[0][0] * ra[2] + U[0][1] * ra[3] + U[0][2] * ra[4];
                m01 = U[0][0] * ra[5] + U[0][1] * ra[6] + U[0][2] * ra[7];
                m11 = U[1][0] * ra[5] + U[1][1] * ra[6] + U[1][2] * ra[7];
            }
            sh[tid][2 * D] = m00;
            sh[tid][2 * D + 1] = m01;
            sh[tid][2 * D + 2] = m11;
        }
        __syncthreads();
        if (tid < NH)
            for (int k = 0; k < cnt; ++k) {
                const T m00 = sh[k][2 * D], m01 = sh[k][2 * D + 1], m11 = sh[k][2 * D + 2];
                const T a0 = sh[k][ea], a1 = sh[k][D + ea], b0 = sh[k][eb], b1 = sh[k][D + eb];
                kahan_add(acc, comp, a0 * (m00 * b0 + m01 * b1) + a1 * (m01 * b0 + m11 * b1));
            }
        __syncthreads();
    }
    const double lam = st->lambda;
    const int act = img_active[i];
    const double *H = img_H + (size_t)i * D * D;
    if (tid < NH) {
        double v = H[ea * D + eb] - ((double)acc - (double)comp);
        if (ea == eb) v += H[ea * D + ea] * lam;
        const bool on = ((act >> ea) & 1) && ((act >> eb) & 1);
        if (!on) v = ea == eb ? 1.0 : 0.0;
        blk[ea][eb] = v;
        blk[eb][ea] = v;
        if (ea == eb) dg[ea] = v;
    }
    if (tid < D) rv[tid] = ((act >> tid) & 1) ? img_rhs[(size_t)i * D + tid] : 0.0;
    __syncthreads();
    if (tid == 0) {
        // Cholesky of the D x D block in place (lower), then its inverse.
        fallback = 0;
        for (int j = 0; j < D && !fallback; ++j) {
            double d = blk[j][j];
            for (int k = 0; k < j; ++k) d -= blk[j][k] * blk[j][k];
            if (!(d > 0.0)) { fallback = 1; break; }
            d = sqrt(d);
            blk[j][j] = d;
            for (int q = j + 1; q < D; ++q) {
                double v = blk[q][j];
                for (int k = 0; k < j; ++k) v -= blk[q][k] * blk[j][k];
                blk[q][j] = v / d;
            }
        }
        if (!fallback) {
            for (int c = 0; c < D; ++c) {
                double y[D];
                for (int q = 0; q < D; ++q) {
                    double v = q == c ? 1.0 : 0.0;
                    for (int k = 0; k < q; ++k) v -= blk[q][k] * y[k];
                    y[q] = v / blk[q][q];
                }
                for (int q = D - 1; q >= 0; --q) {
                    double v = y[q];
                    for (int k = q + 1; k < D; ++k) v -= blk[k][q] * Mi[k][c];
                    Mi[q][c] = v / blk[q][q];
                }
            }
        }
    }
    __syncthreads();
    if (fallback) {
        // Jacobi on the block's diagonal (the block was not SPD in the
        // kernel precision).
        for (int idx = tid; idx < D * D; idx += blockDim.x) {
            const int a = idx / D, c = idx - a * D;
            Mi[a][c] = (a == c && dg[a] > 0.0) ? 1.0 / dg[a] : 0.0;
        }
        __syncthreads();
    }
    for (int idx = tid; idx < D * D; idx += blockDim.x) {
        const int a = idx / D, c = idx - a * D;
        const bool on = ((act >> a) & 1) && ((act >> c) & 1);
        const double v = on ? Mi[a][c] : 0.0;
        Minv_out[(size_t)i * D * D + idx] = (T)v;
        if (!on) Mi[a][c] = 0.0;
    }
    __syncthreads();
    __shared__ double rz_part[D], rr_part[D];
    if (tid < D) {
        double zc = 0.0;
        for (int d = 0; d < D; ++d) zc += Mi[tid][d] * rv[d];
        const size_t u = (size_t)i * D + tid;
        x[u] = T(0);
        r[u] = (T)rv[tid];
        z[u] = (T)zc;
        p[u] = (T)zc;
        rz_part[tid] = (double)(T)rv[tid] * (double)(T)zc;
        rr_part[tid] = (double)(T)rv[tid] * (double)(T)rv[tid];
    }
    __syncthreads();
    if (tid == 0) {
        double a = 0.0, b = 0.0;
        for (int d = 0; d < D; ++d) { a += rz_part[d]; b += rr_part[d]; }
        part[i] = a;
        part[nI + i] = b;
    }
}

__global__ void k_pcg_scalar_init(const double *part, int nI, double tol2, LMState *st) {
    __shared__ double sh[256];
    double a = 0.0, b = 0.0;
    for (int k = threadIdx.x; k < nI; k += blockDim.x) { a += part[k]; b += part[nI + k]; }
    a = block_sum(a, sh);
    b = block_sum(b, sh);
    if (threadIdx.x == 0) {
        st->pcg_rz = a;
        st->pcg_bb = b;
        st->pcg_rr = b;
        st->pcg_tol2 = tol2;
        st->pcg_iterations = 0;
        st->pcg_done = (b > 0.0 && a > 0.0 && isfinite(a)) ? 0 : 1;
        st->pcg_alpha = 0.0;
        st->pcg_beta = 0.0;
    }
}

// Jx~ (2x3) and Jc~ (2xD) of observation o, read with 16-byte vector loads.
template <typename T, int D>
__device__ __forceinline__ void load_jac(const T *__restrict__ rec, long long o, T jx[6], T jc[2 * D]) {
    constexpr int RS = RecLayout<D>::kStride;
    constexpr int NV = 8 + 2 * D;  // elements [0, NV) cover r~, Jx~, Jc~
    T v[(NV + 3) / 4 * 4];
    if constexpr (std::is_same<T, float>::value) {
        const float4 *q = reinterpret_cast<const float4 *>(rec + (size_t)o * RS);
#pragma unroll
        for (int k = 0; k < (NV + 3) / 4; ++k) {
            const float4 t = __ldg(q + k);
            v[4 * k] = t.x; v[4 * k + 1] = t.y; v[4 * k + 2] = t.z; v[4 * k + 3] = t.w;
        }
    } else {
        const double2 *q = reinterpret_cast<const double2 *>(rec + (size_t)o * RS);
#pragma unroll
        for (int k = 0; k < (NV + 1) / 2; ++k) {
            const double2 t = __ldg(q + k);
            v[2 * k] = t.x; v[2 * k + 1] = t.y;
        }
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) jx[k] = v[2 + k];
#pragma unroll
    for (int k = 0; k < 2 * D; ++k) jc[k] = v[8 + k];
}

// Point pass over point-aligned chunks of kChunkObs observations, one warp
// per chunk: each lane takes one observation, contributions
// Jx~^T (Jc~ p_img) are summed per point by a segmented warp scan (a point's
// observations are contiguous and never straddle chunks; the running sum is
// carried across the chunk's 32-observation rounds), and the lane ending a
// point writes u_p = C_p^-1 t_p. No atomics; a track of 200 observations
// costs its own lanes, not a whole warp's.
template <typename T, int D>
__global__ void __launch_bounds__(256) k_pcg_points(const T *__restrict__ rec, const int *__restrict__ ob_pt,
                                                    const int *__restrict__ ob_img, const int *__restrict__ pchunk,
                                                    int nchunks, const T *__restrict__ pt_Cinv,
                                                    const unsigned char *__restrict__ pt_ok, const T *__restrict__ p,
                                                    const LMState *__restrict__ st, T *__restrict__ u) {
    if (st->pcg_done) return;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= nchunks) return;
    const int cs = pchunk[warp], ce = pchunk[warp + 1];
    T carry0 = 0, carry1 = 0, carry2 = 0;
    int carry_pt = -1;
    for (int base = cs; base < ce; base += 32) {
        const int o = base + lane;
        const bool valid = o < ce;
        const int pt = valid ? ob_pt[o] : -1;
        T c0 = 0, c1 = 0, c2 = 0;
        if (valid) {
            T jx[6], jc[2 * D];
            load_jac<T, D>(rec, o, jx, jc);
            const T *pv = p + (size_t)ob_img[o] * D;
            T s0 = 0, s1 = 0;
#pragma unroll
            for (int c = 0; c < D; ++c) {
                const T v = pv[c];
                s0 += jc[c] * v;
                s1 += jc[D + c] * v;
            }
            c0 = jx[0] * s0 + jx[3] * s1;
            c1 = jx[1] * s0 + jx[4] * s1;
            c2 = jx[2] * s0 + jx[5] * s1;
            if (lane == 0 && pt == carry_pt) { c0 += carry0; c1 += carry1; c2 += carry2; }
        }
        const int prev = __shfl_up_sync(0xffffffffu, pt, 1);
        bool head = lane == 0 || pt != prev;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const T a0 = __shfl_up_sync(0xffffffffu, c0, off);
            const T a1 = __shfl_up_sync(0xffffffffu, c1, off);
            const T a2 = __shfl_up_sync(0xffffffffu, c2, off);
            const bool hf = __shfl_up_sync(0xffffffffu, head, off);
            if (lane >= off) {
                if (!head) { c0 += a0; c1 += a1; c2 += a2; }
                head = head || hf;
            }
        }
        int next = __shfl_down_sync(0xffffffffu, pt, 1);
        if (lane == 31) next = (o + 1 < ce) ? ob_pt[o + 1] : -1;
        const bool tail = valid && next != pt;
        if (tail) {
            T u0 = 0, u1 = 0, u2 = 0;
            if (pt_ok[pt]) {
                const T *Ci = pt_Cinv + 6 * (size_t)pt;
                u0 = Ci[0] * c0 + Ci[1] * c1 + Ci[2] * c2;
                u1 = Ci[1] * c0 + Ci[3] * c1 + Ci[4] * c2;
                u2 = Ci[2] * c0 + Ci[4] * c1 + Ci[5] * c2;
            }
            T *uo = u + 4 * (size_t)pt;
            uo[0] = u0; uo[1] = u1; uo[2] = u2;
        }
        const bool cont = valid && !tail;  // segment continues into the next round (lane 31 only matters)
        carry0 = __shfl_sync(0xffffffffu, c0, 31);
        carry1 = __shfl_sync(0xffffffffu, c1, 31);
        carry2 = __shfl_sync(0xffffffffu, c2, 31);
        carry_pt = __shfl_sync(0xffffffffu, cont ? pt : -1, 31);
    }
}

// Image pass over fixed chunks of kChunkObs image-major observations, one
// warp per chunk: lanes accumulate Jc~^T (Jx~ u_p) for the chunk's current
// image; at an image change the warp reduces and writes one partial sum for
// (chunk, image). A second kernel adds an image's partials (deterministic,
// no atomics).
template <typename T, int D>
__global__ void __launch_bounds__(256) k_pcg_images(const T *__restrict__ rec, const int *__restrict__ img_obs,
                                                    const int *__restrict__ isort_img,
                                                    const int *__restrict__ isort_pt, long long nO,
                                                    const int *__restrict__ img_start,
                                                    const int *__restrict__ ipart_off, const T *__restrict__ u,
                                                    const LMState *__restrict__ st, T *__restrict__ ipart) {
    if (st->pcg_done) return;
    const long long chunk = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const long long cs = chunk * kChunkObs;
    if (cs >= nO) return;
    const long long ce = cs + kChunkObs < nO ? cs + kChunkObs : nO;
    T acc[D];
#pragma unroll
    for (int c = 0; c < D; ++c) acc[c] = T(0);
    int cur = isort_img[cs];
    auto flush = [&](int img) {
#pragma unroll
        for (int c = 0; c < D; ++c) {
            T v = acc[c];
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
            acc[c] = v;
        }
        if (lane == 0) {
            const int slot = ipart_off[img] + (int)(chunk - img_start[img] / kChunkObs);
            T *dst = ipart + (size_t)slot * D;
#pragma unroll
            for (int c = 0; c < D; ++c) dst[c] = acc[c];
        }
#pragma unroll
        for (int c = 0; c < D; ++c) acc[c] = T(0);
    };
    for (long long base = cs; base < ce; base += 32) {
        const long long k = base + lane;
        const bool valid = k < ce;
        const int img = valid ? isort_img[k] : 0x7fffffff;
        T cv[D];
#pragma unroll
        for (int c = 0; c < D; ++c) cv[c] = T(0);
        if (valid) {
            const int o = img_obs[k];
            const float4 *up4 = nullptr;
            T u0, u1, u2;
            if constexpr (std::is_same<T, float>::value) {
                up4 = reinterpret_cast<const float4 *>(u) + isort_pt[k];
                const float4 t = __ldg(up4);
                u0 = t.x; u1 = t.y; u2 = t.z;
            } else {
                const T *up = u + 4 * (size_t)isort_pt[k];
                u0 = up[0]; u1 = up[1]; u2 = up[2];
            }
            T jx[6], jc[2 * D];
            load_jac<T, D>(rec, o, jx, jc);
            const T z0 = jx[0] * u0 + jx[1] * u1 + jx[2] * u2;
            const T z1 = jx[3] * u0 + jx[4] * u1 + jx[5] * u2;
#pragma unroll
            for (int c = 0; c < D; ++c) cv[c] = jc[c] * z0 + jc[D + c] * z1;
        }
        while (true) {
            if (valid && img == cur) {
#pragma unroll
                for (int c = 0; c < D; ++c) acc[c] += cv[c];
            }
            const unsigned rest = __ballot_sync(0xffffffffu, valid && img > cur);
            if (!rest) break;
            flush(cur);
            cur = __shfl_sync(0xffffffffu, img, __ffs(rest) - 1);
        }
    }
    flush(cur);
}

// q_i = (H_i + lambda diag H_i) p_i - sum of the image's partials; part[i] = p_i . q_i.
template <typename T, int D>
__global__ void __launch_bounds__(128) k_pcg_images_finish(const T *__restrict__ ipart,
                                                           const int *__restrict__ ipart_off,
                                                           const double *__restrict__ img_H,
                                                           const int *__restrict__ img_active,
                                                           const T *__restrict__ p, const LMState *__restrict__ st,
                                                           int nI, T *__restrict__ q, double *__restrict__ part) {
    if (st->pcg_done) return;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= nI) return;
    const double lam = st->lambda;
    const int act = img_active[i];
    const double *H = img_H + (size_t)i * D * D;
    const T *pv = p + (size_t)i * D;
    double pq = 0.0;
    if (lane < D) {
        const int c = lane;
        double sch = 0.0;
        for (int k = ipart_off[i]; k < ipart_off[i + 1]; ++k) sch += (double)ipart[(size_t)k * D + c];
        double hp = 0.0;
#pragma unroll
        for (int d = 0; d < D; ++d) hp += H[c * D + d] * (double)pv[d];
        hp += lam * H[c * D + c] * (double)pv[c];
        const double qc = ((act >> c) & 1) ? hp - sch : 0.0;
        q[(size_t)i * D + c] = (T)qc;
        pq = (double)pv[c] * (double)(T)qc;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) pq += __shfl_xor_sync(0xffffffffu, pq, off);
    if (lane == 0) part[i] = pq;
}

__global__ void k_point_chunks(const int *pt_start, int nP, long long nO, int nchunks, int *pchunk) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k > nchunks) return;
    long long t = (long long)k * kChunkObs;
    if (t > nO) t = nO;
    int lo = 0, hi = nP;  // first point whose start is >= t (pt_start[nP] == nO)
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (pt_start[mid] < t) lo = mid + 1;
        else hi = mid;
    }
    pchunk[k] = k == nchunks ? (int)nO : pt_start[lo];
}

__global__ void k_isort_pt(const int *img_obs, const int *ob_pt, long long nO, int *isort_pt) {
    const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k < nO) isort_pt[k] = ob_pt[img_obs[k]];
}

__global__ void k_pcg_scalar_alpha(const double *part, int nI, LMState *st) {
    __shared__ double sh[256];
    if (st->pcg_done) return;
    double a = 0.0;
    for (int k = threadIdx.x; k < nI; k += blockDim.x) a += part[k];
    a = block_sum(a, sh);
    if (threadIdx.x == 0) {
        if (!(a > 0.0) || !isfinite(a)) {
            st->pcg_done = 1;  // breakdown: keep the current iterate
            st->pcg_alpha = 0.0;
        } else {
            st->pcg_alpha = st->pcg_rz / a;
        }
    }
}

// x += alpha p; r -= alpha q; z = M^-1 r; part = (r.z, r.r) per image. One warp per image.
template <typename T, int D>
__global__ void __launch_bounds__(128) k_pcg_update(const T *Minv, const T *p, const T *q, const LMState *st,
                                                    int nI, T *x, T *r, T *z, double *part) {
    if (st->pcg_done) return;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= nI) return;
    const double alpha = st->pcg_alpha;
    const size_t base = (size_t)i * D;
    T rc = T(0);
    if (lane < D) {
        x[base + lane] = (T)((double)x[base + lane] + alpha * (double)p[base + lane]);
        rc = (T)((double)r[base + lane] - alpha * (double)q[base + lane]);
        r[base + lane] = rc;
    }
    double zc = 0.0;
    const T *M = Minv + (size_t)i * D * D;
#pragma unroll
    for (int d = 0; d < D; ++d) {
        const T rd = __shfl_sync(0xffffffffu, rc, d);
        if (lane < D) zc += (double)M[lane * D + d] * (double)rd;
    }
    double rz = 0.0, rr = 0.0;
    if (lane < D) {
        z[base + lane] = (T)zc;
        rz = (double)rc * (double)(T)zc;
        rr = (double)rc * (double)rc;
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

__global__ void k_pcg_scalar_beta(const double *part, int nI, LMState *st) {
    __shared__ double sh[256];
    if (st->pcg_done) return;
    double a = 0.0, b = 0.0;
    for (int k = threadIdx.x; k < nI; k += blockDim.x) { a += part[k]; b += part[nI + k]; }
    a = block_sum(a, sh);
    b = block_sum(b, sh);
    if (threadIdx.x == 0) {
        st->pcg_iterations += 1;
        st->pcg_total += 1;
        st->pcg_rr = b;
        if (b <= st->pcg_tol2 * st->pcg_bb || !(a > 0.0) || !isfinite(a)) {
            st->pcg_done = 1;
        } else {
            st->pcg_beta = a / st->pcg_rz;
            st->pcg_rz = a;
        }
    }
}

template <typename T>
__global__ void k_pcg_dir(const T *z, const LMState *st, int nID, T *p) {
    if (st->pcg_done) return;
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= nID) return;
    p[u] = (T)((double)z[u] + st->pcg_beta * (double)p[u]);
}

template <typename T>
__global__ void k_pcg_scatter(const T *x, const int *pre_start, const int *pre, const unsigned char *masked,
                              int n, double *delta) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    double v = 0.0;
    if (!masked[a] && pre_start[a] < pre_start[a + 1]) v = (double)x[pre[pre_start[a]]];
    delta[a] = v;
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

template <typename T, int D>
void setup_t(const Bufs &b, cudaStream_t s) {
    k_pcg_precond<T, D><<<b.nI, 128, 0, s>>>(
        (const T *)b.rec, b.img_start, b.img_obs, b.ob_pt, (const T *)b.pt_Cinv, b.pt_ok, b.img_H,
        b.img_active, b.img_rhs, b.state, b.nI, (T *)b.pcg_Minv, (T *)b.pcg_x, (T *)b.pcg_r,
        (T *)b.pcg_z, (T *)b.pcg_p, b.pcg_part);
    SFMBA_LAUNCH_CHECK();
    k_pcg_scalar_init<<<1, 256, 0, s>>>(b.pcg_part, b.nI, b.pcg_tol * b.pcg_tol, b.state);
    SFMBA_LAUNCH_CHECK();
}

template <typename T, int D>
void points_t(const Bufs &b, cudaStream_t s) {
    if (b.nP == 0 || b.npchunks == 0) return;
    k_pcg_points<T, D><<<div_up((long long)b.npchunks * 32, 256), 256, 0, s>>>(
        (const T *)b.rec, b.ob_pt, b.ob_img, b.pchunk, b.npchunks, (const T *)b.pt_Cinv, b.pt_ok,
        (const T *)b.pcg_p, b.state, (T *)b.pcg_u);
    SFMBA_LAUNCH_CHECK();
}

template <typename T, int D>
void images_t(const Bufs &b, cudaStream_t s) {
    if (b.nO > 0) {
        const long long chunks = (b.nO + kChunkObs - 1) / kChunkObs;
        k_pcg_images<T, D><<<div_up(chunks * 32, 256), 256, 0, s>>>(
            (const T *)b.rec, b.img_obs, b.isort_img, b.isort_pt, b.nO, b.img_start, b.ipart_off,
            (const T *)b.pcg_u, b.state, (T *)b.ipart);
        SFMBA_LAUNCH_CHECK();
    }
    k_pcg_images_finish<T, D><<<div_up(b.nI, 4), 128, 0, s>>>((const T *)b.ipart, b.ipart_off, b.img_H,
                                                              b.img_active, (const T *)b.pcg_p, b.state, b.nI,
                                                              (T *)b.pcg_q, b.pcg_part);
    SFMBA_LAUNCH_CHECK();
}

template <typename T, int D>
void vector_t(const Bufs &b, cudaStream_t s) {
    k_pcg_scalar_alpha<<<1, 256, 0, s>>>(b.pcg_part, b.nI, b.state);
    SFMBA_LAUNCH_CHECK();
    k_pcg_update<T, D><<<div_up(b.nI, 4), 128, 0, s>>>((const T *)b.pcg_Minv, (const T *)b.pcg_p,
                                                       (const T *)b.pcg_q, b.state, b.nI, (T *)b.pcg_x,
                                                       (T *)b.pcg_r, (T *)b.pcg_z, b.pcg_part);
    SFMBA_LAUNCH_CHECK();
    k_pcg_scalar_beta<<<1, 256, 0, s>>>(b.pcg_part, b.nI, b.state);
    SFMBA_LAUNCH_CHECK();
    k_pcg_dir<T><<<div_up(b.nID, 256), 256, 0, s>>>((const T *)b.pcg_z, b.state, b.nID, (T *)b.pcg_p);
    SFMBA_LAUNCH_CHECK();
}

}  // namespace

void launch_pcg_setup(const Bufs &b, cudaStream_t s) {
    dispatch_D(b.D, [&](auto dc) {
        constexpr int D = decltype(dc)::value;
        if (b.mixed) setup_t<float, D>(b, s);
        else setup_t<double, D>(b, s);
    });
}

#define SFMBA_PCG_LAUNCHER(name, impl)                           \
    void name(const Bufs &b, cudaStream_t s) {                   \
        dispatch_D(b.D, [&](auto dc) {                           \
            constexpr int D = decltype(dc)::value;               \
            if (b.mixed) impl<float, D>(b, s);                   \
            else impl<double, D>(b, s);                          \
        });                                                      \
    }
SFMBA_PCG_LAUNCHER(launch_pcg_points, points_t)
SFMBA_PCG_LAUNCHER(launch_pcg_images, images_t)
SFMBA_PCG_LAUNCHER(launch_pcg_vector, vector_t)
#undef SFMBA_PCG_LAUNCHER

void launch_pcg_partition(Bufs &b, const int *img_keys_sorted, cudaStream_t s) {
    b.npchunks = (int)((b.nO + kChunkObs - 1) / kChunkObs);
    k_point_chunks<<<div_up(b.npchunks + 1, 256), 256, 0, s>>>(b.pt_start, b.nP, b.nO, b.npchunks, b.pchunk);
    SFMBA_LAUNCH_CHECK();
    if (b.nO > 0) {
        SFMBA_CUDA(cudaMemcpyAsync(b.isort_img, img_keys_sorted, sizeof(int) * (size_t)b.nO,
                                   cudaMemcpyDeviceToDevice, s));
        k_isort_pt<<<div_up(b.nO, 256), 256, 0, s>>>(b.img_obs, b.ob_pt, b.nO, b.isort_pt);
        SFMBA_LAUNCH_CHECK();
    }
}

void launch_pcg_finish(const Bufs &b, double *delta_slot, cudaStream_t s) {
    if (b.n == 0) return;
    if (b.mixed)
        k_pcg_scatter<float><<<div_up(b.n, 256), 256, 0, s>>>((const float *)b.pcg_x, b.slot_pre_start,
                                                              b.slot_pre, b.slot_masked, b.n, delta_slot);
    else
        k_pcg_scatter<double><<<div_up(b.n, 256), 256, 0, s>>>((const double *)b.pcg_x, b.slot_pre_start,
                                                               b.slot_pre, b.slot_masked, b.n, delta_slot);
    SFMBA_LAUNCH_CHECK();
}

}  // namespace sfmba
