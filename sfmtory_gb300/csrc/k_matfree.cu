// Observation passes of the matrix-free (PCG) path; see matfree.cuh for the
// chunked work partition. Reference arithmetic: crates/sfm-ba/src/lib.rs
// :859-909 (point/image blocks), :958-965 and :114-211 (Schur terms, here
// applied as operators), :1100-1120 (point back-substitution).
#include "matfree.cuh"

namespace sfmba {

namespace {

template <typename T, int N>
__device__ __forceinline__ void seg_scan(T (&v)[N], bool head, int lane) {
    bool h = head;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        T a[N];
#pragma unroll
        for (int n = 0; n < N; ++n) a[n] = shfl_up(v[n], off);
        const bool hf = __shfl_up_sync(0xffffffffu, h, off);
        if (lane >= off) {
            if (!h) {
#pragma unroll
                for (int n = 0; n < N; ++n) v[n] += a[n];
            }
            h = h || hf;
        }
    }
}

// Walks one point-aligned chunk: contrib(o, img, pt, v) fills the lane's N
// values; consume(pt, v) runs on the lane holding a point's complete sum.
template <typename T, int N, typename Contrib, typename Consume>
__device__ __forceinline__ void point_chunk(const int *__restrict__ ob_pt, const int *__restrict__ ob_img, int cs,
                                            int ce, int lane, Contrib contrib, Consume consume) {
    T carry[N];
#pragma unroll
    for (int n = 0; n < N; ++n) carry[n] = T(0);
    int carry_pt = -1;
    for (int base = cs; base < ce; base += 32) {
        const int o = base + lane;
        const bool valid = o < ce;
        const int pt = valid ? ob_pt[o] : -1;
        T v[N];
#pragma unroll
        for (int n = 0; n < N; ++n) v[n] = T(0);
        if (valid) {
            contrib(o, ob_img[o], pt, v);
            if (lane == 0 && pt == carry_pt) {
#pragma unroll
                for (int n = 0; n < N; ++n) v[n] += carry[n];
            }
        }
        const int prev = __shfl_up_sync(0xffffffffu, pt, 1);
        seg_scan<T, N>(v, lane == 0 || pt != prev, lane);
        int next = __shfl_down_sync(0xffffffffu, pt, 1);
        if (lane == 31) next = (o + 1 < ce) ? ob_pt[o + 1] : -1;
        const bool tail = valid && next != pt;
        if (tail) consume(pt, v);
#pragma unroll
        for (int n = 0; n < N; ++n) carry[n] = __shfl_sync(0xffffffffu, v[n], 31);
        carry_pt = __shfl_sync(0xffffffffu, (valid && !tail) ? pt : -1, 31);
    }
}

// C_p = sum Jx~^T Jx~, g_p = sum Jx~^T r~, free-block count (lib.rs:863-864, :870-879).
template <typename T, int D, bool RC>
__global__ void __launch_bounds__(256) k_mf_point_reduce(JacSrc<T> J, const unsigned char *__restrict__ ob_valid,
                                                         const int *__restrict__ img_free,
                                                         const int *__restrict__ pchunk, int nchunks,
                                                         T *__restrict__ pt_C, T *__restrict__ pt_g,
                                                         int *__restrict__ pt_nfree) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= nchunks) return;
    point_chunk<T, 10>(
        J.ob_pt, J.ob_img, pchunk[warp], pchunk[warp + 1], lane,
        [&](int o, int img, int pt, T (&v)[10]) {
            T rr[2], jx[6], jc[2 * D];
            bool ok = jac_point_major<T, D, RC>(J, o, img, pt, rr, jx, jc);
            if constexpr (!RC) ok = ob_valid[o] != 0;
            const T a0 = jx[0], a1 = jx[1], a2 = jx[2], b0 = jx[3], b1 = jx[4], b2 = jx[5];
            v[0] = a0 * a0 + b0 * b0; v[1] = a0 * a1 + b0 * b1; v[2] = a0 * a2 + b0 * b2;
            v[3] = a1 * a1 + b1 * b1; v[4] = a1 * a2 + b1 * b2; v[5] = a2 * a2 + b2 * b2;
            v[6] = a0 * rr[0] + b0 * rr[1]; v[7] = a1 * rr[0] + b1 * rr[1]; v[8] = a2 * rr[0] + b2 * rr[1];
            v[9] = (ok && img_free[img]) ? T(1) : T(0);
        },
        [&](int pt, const T (&v)[10]) {
            T *C = pt_C + 6 * (size_t)pt;
#pragma unroll
            for (int n = 0; n < 6; ++n) C[n] = v[n];
            T *g = pt_g + 3 * (size_t)pt;
            g[0] = v[6]; g[1] = v[7]; g[2] = v[8];
            pt_nfree[pt] = (int)(v[9] + T(0.5));
        });
}

// Image-major accumulation of sum_o Jc~^T W_o Jc~ (upper triangle) and
// sum_o Jc~^T v_o into one partial per (chunk, image). Each lane owns a few
// entries; the round's observations are staged in shared memory.
//   MODE 0: W = I, v = r~                 -> H_i, b_i
//   MODE 1: W = Jx~ C^-1 Jx~^T, v = Jx~ h -> Schur diagonal block, rhs term
template <typename T, int D, bool RC, int MODE>
__global__ void __launch_bounds__(128) k_mf_image_accum(JacSrc<T> J, const int *__restrict__ isort_img,
                                                        const int *__restrict__ isort_pt, long long nO,
                                                        const int *__restrict__ img_start,
                                                        const int *__restrict__ ipart_off,
                                                        const T *__restrict__ pt_Cinv, const T *__restrict__ pt_h,
                                                        const unsigned char *__restrict__ pt_ok,
                                                        T *__restrict__ part) {
    constexpr int NH = D * (D + 1) / 2;
    constexpr int NV = NH + D;
    constexpr int NE = (NV + 31) / 32;
    constexpr int WPB = 4;
    __shared__ T sJ[WPB][32][2 * D + 1];
    __shared__ T sW[WPB][32][5];
    __shared__ int sImg[WPB][32];
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long chunk = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long cs = chunk * kChunkObs;
    if (cs >= nO) return;
    const long long ce = cs + kChunkObs < nO ? cs + kChunkObs : nO;
    int ea[NE], eb[NE];
#pragma unroll
    for (int j = 0; j < NE; ++j) {
        const int e = lane + 32 * j;
        ea[j] = -1;
        eb[j] = -1;
        if (e < NH) {
            int t = e, a = 0;
            while (t >= D - a) { t -= D - a; ++a; }
            ea[j] = a;
            eb[j] = a + t;
        } else if (e < NV) {
            ea[j] = e - NH;
        }
    }
    T acc[NE];
#pragma unroll
    for (int j = 0; j < NE; ++j) acc[j] = T(0);
    int cur = isort_img[cs];
    auto flush = [&](int img) {
        T *dst = part + (size_t)partial_slot(ipart_off, img_start, img, chunk) * NV;
#pragma unroll
        for (int j = 0; j < NE; ++j) {
            const int e = lane + 32 * j;
            if (e < NV) dst[e] = acc[j];
            acc[j] = T(0);
        }
    };
    for (long long base = cs; base < ce; base += 32) {
        const long long k = base + lane;
        const bool valid = k < ce;
        T rr[2] = {0, 0}, jx[6] = {0, 0, 0, 0, 0, 0}, jc[2 * D];
#pragma unroll
        for (int c = 0; c < 2 * D; ++c) jc[c] = T(0);
        T w00 = 0, w01 = 0, w11 = 0, v0 = 0, v1 = 0;
        int img = 0x7fffffff;
        if (valid) {
            img = isort_img[k];
            const int pt = isort_pt[k];
            jac_image_major<T, D, RC>(J, k, img, pt, rr, jx, jc);
            if constexpr (MODE == 0) {
                w00 = T(1); w11 = T(1);
                v0 = rr[0]; v1 = rr[1];
            } else if (pt_ok[pt]) {
                const T *Ci = pt_Cinv + 6 * (size_t)pt;
                T U[2][3];
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    const T a0 = jx[3 * q], a1 = jx[3 * q + 1], a2 = jx[3 * q + 2];
                    U[q][0] = a0 * Ci[0] + a1 * Ci[1] + a2 * Ci[2];
                    U[q][1] = a0 * Ci[1] + a1 * Ci[3] + a2 * Ci[4];
                    U[q][2] = a0 * Ci[2] + a1 * Ci[4] + a2 * Ci[5];
                }
                w00 = U[0][0] * jx[0] + U[0][1] * jx[1] + U[0][2] * jx[2];
                w01 = U[0][0] * jx[3] + U[0][1] * jx[4] + U[0][2] * jx[5];
                w11 = U[1][0] * jx[3] + U[1][1] * jx[4] + U[1][2] * jx[5];
                const T *h = pt_h + 3 * (size_t)pt;
                v0 = jx[0] * h[0] + jx[1] * h[1] + jx[2] * h[2];
                v1 = jx[3] * h[0] + jx[4] * h[1] + jx[5] * h[2];
            }
        }
#pragma unroll
        for (int c = 0; c < 2 * D; ++c) sJ[wl][lane][c] = jc[c];
        sW[wl][lane][0] = w00; sW[wl][lane][1] = w01; sW[wl][lane][2] = w11;
        sW[wl][lane][3] = v0; sW[wl][lane][4] = v1;
        sImg[wl][lane] = img;
        __syncwarp();
        const int cnt = (int)(ce - base < 32 ? ce - base : 32);
        for (int t = 0; t < cnt; ++t) {
            const int it = sImg[wl][t];
            if (it != cur) {
                flush(cur);
                cur = it;
            }
            const T m00 = sW[wl][t][0], m01 = sW[wl][t][1], m11 = sW[wl][t][2];
            const T q0 = sW[wl][t][3], q1 = sW[wl][t][4];
#pragma unroll
            for (int j = 0; j < NE; ++j) {
                const int a = ea[j], b = eb[j];
                if (a < 0) continue;
                const T xa = sJ[wl][t][a], ya = sJ[wl][t][D + a];
                if (b >= 0) {
                    const T xb = sJ[wl][t][b], yb = sJ[wl][t][D + b];
                    acc[j] += xa * (m00 * xb + m01 * yb) + ya * (m01 * xb + m11 * yb);
                } else {
                    acc[j] += xa * q0 + ya * q1;
                }
            }
        }
        __syncwarp();
    }
    flush(cur);
}

// H_i (full symmetric, FP64) and b_i from the image's MODE-0 partials.
template <typename T, int D>
__global__ void __launch_bounds__(128) k_mf_image_finish0(const T *__restrict__ part,
                                                          const int *__restrict__ ipart_off, int nI,
                                                          double *__restrict__ img_H, double *__restrict__ img_b) {
    constexpr int NH = D * (D + 1) / 2;
    constexpr int NV = NH + D;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= nI) return;
    for (int e = lane; e < NV; e += 32) {
        double s = 0.0;
        for (int k = ipart_off[i]; k < ipart_off[i + 1]; ++k) s += (double)part[(size_t)k * NV + e];
        if (e < NH) {
            int t = e, a = 0;
            while (t >= D - a) { t -= D - a; ++a; }
            const int b = a + t;
            img_H[(size_t)i * D * D + a * D + b] = s;
            img_H[(size_t)i * D * D + b * D + a] = s;
        } else {
            img_b[(size_t)i * D + (e - NH)] = s;
        }
    }
}

// Block-Jacobi preconditioner (exact image diagonal block of the Schur
// complement, Cholesky-inverted), reduced rhs and the PCG start vectors
// (x = 0, r = rhs, p = z = M^-1 r) of image i, from its MODE-1 partials.
template <typename T, int D>
__global__ void __launch_bounds__(128) k_mf_precond_finish(const T *__restrict__ part,
                                                           const int *__restrict__ ipart_off,
                                                           const double *__restrict__ img_H,
                                                           const double *__restrict__ img_b,
                                                           const int *__restrict__ img_active,
                                                           const LMState *__restrict__ st, int nI,
                                                           double *__restrict__ img_rhs, T *__restrict__ Minv_out,
                                                           T *__restrict__ x, T *__restrict__ r, T *__restrict__ z,
                                                           T *__restrict__ p, double *__restrict__ dots) {
    constexpr int NH = D * (D + 1) / 2;
    constexpr int NV = NH + D;
    __shared__ double sum[NV];
    __shared__ double blk[D][D + 1];
    __shared__ double Mi[D][D + 1];
    __shared__ double rv[D];
    __shared__ double dg[D];
    __shared__ int fallback;
    const int i = blockIdx.x;
    if (i >= nI) return;
    const int tid = threadIdx.x;
    for (int e = tid; e < NV; e += blockDim.x) {
        double s = 0.0;
        for (int k = ipart_off[i]; k < ipart_off[i + 1]; ++k) s += (double)part[(size_t)k * NV + e];
        sum[e] = s;
    }
    __syncthreads();
    const double lam = st->lambda;
    const int act = img_active[i];
    const double *H = img_H + (size_t)i * D * D;
    for (int e = tid; e < NH; e += blockDim.x) {
        int t = e, a = 0;
        while (t >= D - a) { t -= D - a; ++a; }
        const int b = a + t;
        double v = H[a * D + b] - sum[e];
        if (a == b) v += H[a * D + a] * lam;
        const bool on = ((act >> a) & 1) && ((act >> b) & 1);
        if (!on) v = a == b ? 1.0 : 0.0;
        blk[a][b] = v;
        blk[b][a] = v;
        if (a == b) dg[a] = v;
    }
    if (tid < D) {
        const double rhs = ((act >> tid) & 1) ? -img_b[(size_t)i * D + tid] + sum[NH + tid] : 0.0;
        rv[tid] = rhs;
        img_rhs[(size_t)i * D + tid] = rhs;
    }
    __syncthreads();
    if (tid == 0) {
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
        // Not SPD in the kernel precision: Jacobi on the block's diagonal.
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
    }
    __syncthreads();
    if (tid < 32) {
        double rz = 0.0, rr = 0.0;
        if (tid < D) {
            const bool on_r = (act >> tid) & 1;
            double zc = 0.0;
            for (int d = 0; d < D; ++d)
                if (on_r && ((act >> d) & 1)) zc += Mi[tid][d] * rv[d];
            const size_t u = (size_t)i * D + tid;
            const T rt = (T)rv[tid], zt = (T)zc;
            x[u] = T(0);
            r[u] = rt;
            z[u] = zt;
            p[u] = zt;
            rz = (double)rt * (double)zt;
            rr = (double)rt * (double)rt;
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            rz += __shfl_xor_sync(0xffffffffu, rz, off);
            rr += __shfl_xor_sync(0xffffffffu, rr, off);
        }
        if (tid == 0) {
            dots[i] = rz;
            dots[nI + i] = rr;
        }
    }
}

// PCG point pass: u_p = C_p^-1 sum_o Jx~^T (Jc~_o p_img(o)).
template <typename T, int D, bool RC>
__global__ void __launch_bounds__(256) k_mf_points(JacSrc<T> J, const int *__restrict__ pchunk, int nchunks,
                                                   const T *__restrict__ pt_Cinv,
                                                   const unsigned char *__restrict__ pt_ok, const T *__restrict__ p,
                                                   const LMState *__restrict__ st, T *__restrict__ u) {
    if (st->pcg_done) return;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= nchunks) return;
    point_chunk<T, 3>(
        J.ob_pt, J.ob_img, pchunk[warp], pchunk[warp + 1], lane,
        [&](int o, int img, int pt, T (&v)[3]) {
            T rr[2], jx[6], jc[2 * D];
            jac_point_major<T, D, RC>(J, o, img, pt, rr, jx, jc);
            const T *pv = p + (size_t)img * D;
            T s0 = 0, s1 = 0;
#pragma unroll
            for (int c = 0; c < D; ++c) {
                const T w = pv[c];
                s0 += jc[c] * w;
                s1 += jc[D + c] * w;
            }
            v[0] = jx[0] * s0 + jx[3] * s1;
            v[1] = jx[1] * s0 + jx[4] * s1;
            v[2] = jx[2] * s0 + jx[5] * s1;
        },
        [&](int pt, const T (&v)[3]) {
            T u0 = 0, u1 = 0, u2 = 0;
            if (pt_ok[pt]) {
                const T *Ci = pt_Cinv + 6 * (size_t)pt;
                u0 = Ci[0] * v[0] + Ci[1] * v[1] + Ci[2] * v[2];
                u1 = Ci[1] * v[0] + Ci[3] * v[1] + Ci[4] * v[2];
                u2 = Ci[2] * v[0] + Ci[4] * v[1] + Ci[5] * v[2];
            }
            T *uo = u + 4 * (size_t)pt;
            uo[0] = u0; uo[1] = u1; uo[2] = u2;
        });
}

// PCG image pass: partial sums of Jc~^T (Jx~ u_p) per (chunk, image).
template <typename T, int D, bool RC>
__global__ void __launch_bounds__(256) k_mf_images(JacSrc<T> J, const int *__restrict__ isort_img,
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
            T *dst = ipart + (size_t)partial_slot(ipart_off, img_start, img, chunk) * D;
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
            const int pt = isort_pt[k];
            T u0, u1, u2;
            if constexpr (std::is_same<T, float>::value) {
                const float4 t = __ldg(reinterpret_cast<const float4 *>(u) + pt);
                u0 = t.x; u1 = t.y; u2 = t.z;
            } else {
                const T *up = u + 4 * (size_t)pt;
                u0 = up[0]; u1 = up[1]; u2 = up[2];
            }
            T rr[2], jx[6], jc[2 * D];
            jac_image_major<T, D, RC>(J, k, img, pt, rr, jx, jc);
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

// Point back-substitution: delta_p = -C_p^-1 (g_p + sum_o Jx~^T (Jc~ delta_img)),
// trial point = p + delta_p (lib.rs:1100-1120, :1138-1141). Points without
// a usable inverse keep their value (points_trial is a copy beforehand).
template <typename T, int D, bool RC>
__global__ void __launch_bounds__(256) k_mf_backsub(JacSrc<T> J, const int *__restrict__ pchunk, int nchunks,
                                                    const T *__restrict__ img_delta, const T *__restrict__ pt_Cinv,
                                                    const T *__restrict__ pt_g, const unsigned char *__restrict__ pt_ok,
                                                    const double *__restrict__ points,
                                                    double *__restrict__ points_trial) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= nchunks) return;
    point_chunk<T, 3>(
        J.ob_pt, J.ob_img, pchunk[warp], pchunk[warp + 1], lane,
        [&](int o, int img, int pt, T (&v)[3]) {
            T rr[2], jx[6], jc[2 * D];
            jac_point_major<T, D, RC>(J, o, img, pt, rr, jx, jc);
            const T *d = img_delta + (size_t)img * D;
            T t0 = 0, t1 = 0;
#pragma unroll
            for (int c = 0; c < D; ++c) {
                t0 += jc[c] * d[c];
                t1 += jc[D + c] * d[c];
            }
            v[0] = jx[0] * t0 + jx[3] * t1;
            v[1] = jx[1] * t0 + jx[4] * t1;
            v[2] = jx[2] * t0 + jx[5] * t1;
        },
        [&](int pt, const T (&v)[3]) {
            if (!pt_ok[pt]) return;
            const T *g = pt_g + 3 * (size_t)pt;
            const T a0 = g[0] + v[0], a1 = g[1] + v[1], a2 = g[2] + v[2];
            const T *Ci = pt_Cinv + 6 * (size_t)pt;
            const T d0 = Ci[0] * a0 + Ci[1] * a1 + Ci[2] * a2;
            const T d1 = Ci[1] * a0 + Ci[3] * a1 + Ci[4] * a2;
            const T d2 = Ci[2] * a0 + Ci[4] * a1 + Ci[5] * a2;
            const double *X = points + 3 * (size_t)pt;
            double *Y = points_trial + 3 * (size_t)pt;
            Y[0] = X[0] + (double)(-d0);
            Y[1] = X[1] + (double)(-d1);
            Y[2] = X[2] + (double)(-d2);
        });
}

__global__ void k_isort_xy32(const int *img_obs, const double2 *ob_xy, long long nO, float2 *ob_xy32,
                             float2 *isort_xy32) {
    const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k >= nO) return;
    const double2 a = ob_xy[k];
    ob_xy32[k] = make_float2((float)a.x, (float)a.y);
    const double2 b = ob_xy[img_obs[k]];
    isort_xy32[k] = make_float2((float)b.x, (float)b.y);
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

// FP32 recomputes the Jacobian in every pass; FP64 reads stored records.
template <typename F>
void dispatch_TDR(const Bufs &b, F &&f) {
    dispatch_D(b.D, [&](auto dc) {
        constexpr int D = decltype(dc)::value;
        if (b.mixed) f((float)0, dc, std::true_type());
        else f((double)0, dc, std::false_type());
    });
}

template <typename T>
JacSrc<T> jac_src(const Bufs &b) {
    JacSrc<T> J;
    J.rec = (const T *)b.rec;
    J.img_lin = (const ImageLin<T> *)b.img_lin;
    J.points32 = b.points32;
    J.points64 = b.points;
    J.ob_xy32 = b.ob_xy32;
    J.ob_xy64 = b.ob_xy;
    J.isort_xy32 = b.isort_xy32;
    J.ob_img = b.ob_img;
    J.ob_pt = b.ob_pt;
    J.img_obs = b.img_obs;
    J.loss = b.loss;
    J.scale = (T)b.loss_scale;
    return J;
}

int warps_grid(long long warps, int threads) { return div_up(warps * 32, threads); }

}  // namespace

void launch_mf_prepare(const Bufs &b, cudaStream_t s) {
    if (b.mixed && b.nO > 0) {
        k_isort_xy32<<<div_up(b.nO, 256), 256, 0, s>>>(b.img_obs, b.ob_xy, b.nO, b.ob_xy32, b.isort_xy32);
        SFMBA_LAUNCH_CHECK();
    }
}

void launch_mf_point_reduce(const Bufs &b, cudaStream_t s) {
    if (b.npchunks == 0) return;
    dispatch_TDR(b, [&](auto t, auto dc, auto rc) {
        using T = decltype(t);
        constexpr int D = decltype(dc)::value;
        k_mf_point_reduce<T, D, decltype(rc)::value><<<warps_grid(b.npchunks, 256), 256, 0, s>>>(
            jac_src<T>(b), b.ob_valid, b.img_free, b.pchunk, b.npchunks, (T *)b.pt_C, (T *)b.pt_g, b.pt_nfree);
    });
    SFMBA_LAUNCH_CHECK();
}

void launch_mf_image_blocks(const Bufs &b, cudaStream_t s) {
    dispatch_TDR(b, [&](auto t, auto dc, auto rc) {
        using T = decltype(t);
        constexpr int D = decltype(dc)::value;
        if (b.nO > 0) {
            const long long chunks = (b.nO + kChunkObs - 1) / kChunkObs;
            k_mf_image_accum<T, D, decltype(rc)::value, 0><<<warps_grid(chunks, 128), 128, 0, s>>>(
                jac_src<T>(b), b.isort_img, b.isort_pt, b.nO, b.img_start, b.ipart_off, (const T *)b.pt_Cinv,
                (const T *)b.pt_h, b.pt_ok, (T *)b.ipart2);
            SFMBA_LAUNCH_CHECK();
        }
        k_mf_image_finish0<T, D><<<div_up(b.nI, 4), 128, 0, s>>>((const T *)b.ipart2, b.ipart_off, b.nI, b.img_H,
                                                                b.img_b);
        SFMBA_LAUNCH_CHECK();
    });
}

void launch_mf_precond(const Bufs &b, cudaStream_t s) {
    dispatch_TDR(b, [&](auto t, auto dc, auto rc) {
        using T = decltype(t);
        constexpr int D = decltype(dc)::value;
        if (b.nO > 0) {
            const long long chunks = (b.nO + kChunkObs - 1) / kChunkObs;
            k_mf_image_accum<T, D, decltype(rc)::value, 1><<<warps_grid(chunks, 128), 128, 0, s>>>(
                jac_src<T>(b), b.isort_img, b.isort_pt, b.nO, b.img_start, b.ipart_off, (const T *)b.pt_Cinv,
                (const T *)b.pt_h, b.pt_ok, (T *)b.ipart2);
            SFMBA_LAUNCH_CHECK();
        }
        k_mf_precond_finish<T, D><<<b.nI, 128, 0, s>>>((const T *)b.ipart2, b.ipart_off, b.img_H, b.img_b,
                                                       b.img_active, b.state, b.nI, b.img_rhs, (T *)b.pcg_Minv,
                                                       (T *)b.pcg_x, (T *)b.pcg_r, (T *)b.pcg_z, (T *)b.pcg_p,
                                                       b.pcg_part);
        SFMBA_LAUNCH_CHECK();
    });
}

void launch_mf_points(const Bufs &b, cudaStream_t s) {
    if (b.npchunks == 0) return;
    dispatch_TDR(b, [&](auto t, auto dc, auto rc) {
        using T = decltype(t);
        constexpr int D = decltype(dc)::value;
        k_mf_points<T, D, decltype(rc)::value><<<warps_grid(b.npchunks, 256), 256, 0, s>>>(
            jac_src<T>(b), b.pchunk, b.npchunks, (const T *)b.pt_Cinv, b.pt_ok, (const T *)b.pcg_p, b.state,
            (T *)b.pcg_u);
    });
    SFMBA_LAUNCH_CHECK();
}

void launch_mf_images(const Bufs &b, cudaStream_t s) {
    if (b.nO == 0) return;
    dispatch_TDR(b, [&](auto t, auto dc, auto rc) {
        using T = decltype(t);
        constexpr int D = decltype(dc)::value;
        const long long chunks = (b.nO + kChunkObs - 1) / kChunkObs;
        k_mf_images<T, D, decltype(rc)::value><<<warps_grid(chunks, 256), 256, 0, s>>>(
            jac_src<T>(b), b.isort_img, b.isort_pt, b.nO, b.img_start, b.ipart_off, (const T *)b.pcg_u, b.state,
            (T *)b.ipart);
    });
    SFMBA_LAUNCH_CHECK();
}

void launch_mf_backsub(const Bufs &b, const double *delta_slot, cudaStream_t s) {
    launch_gather_delta(b, delta_slot, s);
    if (b.nP > 0)
        SFMBA_CUDA(cudaMemcpyAsync(b.points_trial, b.points, sizeof(double) * 3 * (size_t)b.nP,
                                   cudaMemcpyDeviceToDevice, s));
    if (b.npchunks > 0) {
        dispatch_TDR(b, [&](auto t, auto dc, auto rc) {
            using T = decltype(t);
            constexpr int D = decltype(dc)::value;
            k_mf_backsub<T, D, decltype(rc)::value><<<warps_grid(b.npchunks, 256), 256, 0, s>>>(
                jac_src<T>(b), b.pchunk, b.npchunks, (const T *)b.img_delta, (const T *)b.pt_Cinv,
                (const T *)b.pt_g, b.pt_ok, b.points, b.points_trial);
        });
        SFMBA_LAUNCH_CHECK();
    }
    launch_update_images(b, delta_slot, s);
}

}  // namespace sfmba
