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

// Point pass: u_p = C_p^-1 sum_o Jx~_o^T (Jc~_o p_img(o)).
template <typename T, int D>
__global__ void __launch_bounds__(128) k_pcg_points(const T *rec, const int *pt_start, const int *ob_img,
                                                    const T *pt_Cinv, const unsigned char *pt_ok,
                                                    const T *p, const LMState *st, int nP, T *u) {
    constexpr int RS = RecLayout<D>::kStride;
    if (st->pcg_done) return;
    const int pt = blockIdx.x * blockDim.x + threadIdx.x;
    if (pt >= nP) return;
    T t0 = 0, t1 = 0, t2 = 0;
    if (pt_ok[pt]) {
        for (int o = pt_start[pt]; o < pt_start[pt + 1]; ++o) {
            const T *r = rec + (size_t)o * RS;
            const T *pv = p + (size_t)ob_img[o] * D;
            T s0 = 0, s1 = 0;
#pragma unroll
            for (int c = 0; c < D; ++c) {
                const T v = pv[c];
                s0 += r[8 + c] * v;
                s1 += r[8 + D + c] * v;
            }
            t0 += r[2] * s0 + r[5] * s1;
            t1 += r[3] * s0 + r[6] * s1;
            t2 += r[4] * s0 + r[7] * s1;
        }
        const T *Ci = pt_Cinv + 6 * (size_t)pt;
        const T u0 = Ci[0] * t0 + Ci[1] * t1 + Ci[2] * t2;
        const T u1 = Ci[1] * t0 + Ci[3] * t1 + Ci[4] * t2;
        const T u2 = Ci[2] * t0 + Ci[4] * t1 + Ci[5] * t2;
        t0 = u0; t1 = u1; t2 = u2;
    }
    T *uo = u + 4 * (size_t)pt;
    uo[0] = t0; uo[1] = t1; uo[2] = t2; uo[3] = T(0);
}

// Image pass: q_i = (H_i + lambda diag H_i) p_i - sum_o Jc~^T (Jx~ u_p); part[i] = p_i . q_i.
template <typename T, int D>
__global__ void __launch_bounds__(128) k_pcg_images(const T *rec, const int *img_start, const int *img_obs,
                                                    const int *ob_pt, const T *u, const double *img_H,
                                                    const int *img_active, const T *p, const LMState *st,
                                                    int nI, T *q, double *part) {
    constexpr int RS = RecLayout<D>::kStride;
    if (st->pcg_done) return;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= nI) return;
    T acc[D], comp[D];
#pragma unroll
    for (int c = 0; c < D; ++c) acc[c] = comp[c] = T(0);
    const int s = img_start[i], e = img_start[i + 1];
    for (int k = s + lane; k < e; k += 32) {
        const int o = img_obs[k];
        const T *r = rec + (size_t)o * RS;
        const T *up = u + 4 * (size_t)ob_pt[o];
        const T u0 = up[0], u1 = up[1], u2 = up[2];
        const T z0 = r[2] * u0 + r[3] * u1 + r[4] * u2;
        const T z1 = r[5] * u0 + r[6] * u1 + r[7] * u2;
#pragma unroll
        for (int c = 0; c < D; ++c) kahan_add(acc[c], comp[c], r[8 + c] * z0 + r[8 + D + c] * z1);
    }
    const double lam = st->lambda;
    const int act = img_active[i];
    const double *H = img_H + (size_t)i * D * D;
    const T *pv = p + (size_t)i * D;
    double pq = 0.0;
#pragma unroll
    for (int c = 0; c < D; ++c) {
        double v = (double)acc[c] - (double)comp[c];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
        if (lane == c) {
            double hp = 0.0;
            for (int d = 0; d < D; ++d) hp += H[c * D + d] * (double)pv[d];
            hp += lam * H[c * D + c] * (double)pv[c];
            const double qc = ((act >> c) & 1) ? hp - v : 0.0;
            q[(size_t)i * D + c] = (T)qc;
            pq = (double)pv[c] * (double)(T)qc;
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) pq += __shfl_xor_sync(0xffffffffu, pq, off);
    if (lane == 0) part[i] = pq;
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
    if (b.nP == 0) return;
    k_pcg_points<T, D><<<div_up(b.nP, 128), 128, 0, s>>>((const T *)b.rec, b.pt_start, b.ob_img,
                                                         (const T *)b.pt_Cinv, b.pt_ok, (const T *)b.pcg_p,
                                                         b.state, b.nP, (T *)b.pcg_u);
    SFMBA_LAUNCH_CHECK();
}

template <typename T, int D>
void images_t(const Bufs &b, cudaStream_t s) {
    k_pcg_images<T, D><<<div_up(b.nI, 4), 128, 0, s>>>((const T *)b.rec, b.img_start, b.img_obs, b.ob_pt,
                                                       (const T *)b.pcg_u, b.img_H, b.img_active,
                                                       (const T *)b.pcg_p, b.state, b.nI, (T *)b.pcg_q,
                                                       b.pcg_part);
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
