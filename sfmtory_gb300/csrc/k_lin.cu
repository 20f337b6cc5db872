// Linearisation and Levenberg-Marquardt bookkeeping kernels:
//   per-image constants, observation-parallel residual + adjoint Jacobian,
//   point blocks (C_p, g_p), image blocks (H_i, b_i), damped point inverses,
//   reduced right-hand side, point back-substitution, trial update, FP64 cost,
//   accept / reject.
// Reference: crates/sfm-ba/src/lib.rs:816-1221 (bundle_adjust loop).
#include <type_traits>

#include "camera.cuh"
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

__device__ __forceinline__ void quat_to_R(const double *q, double R[9]) {
    const double w = q[0], x = q[1], y = q[2], z = q[3];
    const double ww = w * w, xx = x * x, yy = y * y, zz = z * z;
    R[0] = ww + xx - yy - zz; R[1] = 2 * (x * y - w * z); R[2] = 2 * (w * y + x * z);
    R[3] = 2 * (w * z + x * y); R[4] = ww - xx + yy - zz; R[5] = 2 * (y * z - w * x);
    R[6] = 2 * (x * z - w * y); R[7] = 2 * (w * x + y * z); R[8] = ww - xx - yy + zz;
}

template <typename T>
__global__ void k_prepare_images(const double *poses, const double *cams, const int *cam_of_img,
                                 const int *cam_model, const int *img_active, int nI,
                                 ImageLin<T> *out, float4 *mv) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nI) return;
    const double *q = poses + 7 * (size_t)i;
    double R[9];
    quat_to_R(q, R);
    ImageLin<T> im;
#pragma unroll
    for (int k = 0; k < 9; ++k) im.R[k] = (T)R[k];
    im.t[0] = (T)q[4]; im.t[1] = (T)q[5]; im.t[2] = (T)q[6];
    const int c = cam_of_img[i];
#pragma unroll
    for (int k = 0; k < 8; ++k) im.c[k] = (T)cams[8 * (size_t)c + k];
    im.model = cam_model[c];
    im.active = img_active[i];
    im.pad[0] = im.pad[1] = 0;
    out[i] = im;
    if (mv) {  // the same FP32 values in planes (MvOp): R, t, then the model's scalars {f, fy, k1, k2} and {cx, cy}
        const float4 m0 = make_float4((float)im.R[0], (float)im.R[1], (float)im.R[2], (float)im.R[3]);
        const float4 m1 = make_float4((float)im.R[4], (float)im.R[5], (float)im.R[6], (float)im.R[7]);
        const float4 m2 = make_float4((float)im.R[8], (float)im.t[0], (float)im.t[1], (float)im.t[2]);
        mv[i] = m0;
        mv[nI + i] = m1;
        mv[2 * (size_t)nI + i] = m2;
        // PINHOLE: fx, fy, cx, cy; SIMPLE_PINHOLE / SIMPLE_RADIAL / RADIAL: f, cx, cy, k1, k2
        // (the operator serves only these four models)
        const bool pin = im.model == SFMBA_PINHOLE;
        const float f = (float)im.c[0], fy = (float)(pin ? im.c[1] : im.c[0]);
        const float cx = (float)(pin ? im.c[2] : im.c[1]), cy = (float)(pin ? im.c[3] : im.c[2]);
        const float k1 = (im.model == SFMBA_SIMPLE_RADIAL || im.model == SFMBA_RADIAL) ? (float)im.c[3] : 0.f;
        const float k2 = im.model == SFMBA_RADIAL ? (float)im.c[4] : 0.f;
        mv[3 * (size_t)nI + i] = make_float4(f, fy, k1, k2);
        mv[4 * (size_t)nI + i] = make_float4(cx, cy, 0.f, 0.f);
    }
}

template <typename T>
__device__ __forceinline__ void load_point(const double *points, const float4 *points32, int p,
                                           T &X0, T &X1, T &X2) {
    if constexpr (std::is_same<T, float>::value) {
        const float4 v = points32[p];
        X0 = v.x; X1 = v.y; X2 = v.z;
    } else {
        X0 = points[3 * (size_t)p]; X1 = points[3 * (size_t)p + 1]; X2 = points[3 * (size_t)p + 2];
    }
}

template <typename T, int D>
__global__ void __launch_bounds__(256) k_linearize(const ImageLin<T> *img_lin, const double *points,
                                                   const float4 *points32, const int *ob_img,
                                                   const int *ob_pt, const double2 *ob_xy,
                                                   long long nO, int loss, T scale, T *rec,
                                                   unsigned char *ob_valid, const float4 *rs,
                                                   const unsigned char *img_live) {
    constexpr int RS = RecLayout<D>::kStride;
    long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (o >= nO) return;
    const int i = ob_img[o], p = ob_pt[o];
    if (img_live && !img_live[i]) return;
    const ImageLin<T> im = img_lin[i];
    T X0, X1, X2;
    load_point<T>(points, points32, p, X0, X1, X2);
    const double2 xy = ob_xy[o];
    Res64 rin;
    if (rs) {  // FP32 records: FP64 residual and weight stored by the cost kernel
        const float4 v = rs[o];
        rin.use = true;
        rin.r0 = v.x; rin.r1 = v.y; rin.s = v.z; rin.ok = v.w != 0.f;
    }
    T buf[RS];
    T rr[2], jx[6], jc[2 * D];
    const bool ok = linearize<T, D>(im, X0, X1, X2, (T)xy.x, (T)xy.y, loss, scale, rr, jx, jc, nullptr, rin);
    buf[0] = rr[0]; buf[1] = rr[1];
#pragma unroll
    for (int k = 0; k < 6; ++k) buf[2 + k] = jx[k];
#pragma unroll
    for (int k = 0; k < 2 * D; ++k) buf[8 + k] = jc[k];
#pragma unroll
    for (int k = 8 + 2 * D; k < RS; ++k) buf[k] = T(0);
    T *dst = rec + (size_t)o * RS;
    if constexpr (std::is_same<T, float>::value) {
#pragma unroll
        for (int k = 0; k < RS; k += 4)
            *reinterpret_cast<float4 *>(dst + k) = make_float4(buf[k], buf[k + 1], buf[k + 2], buf[k + 3]);
    } else {
#pragma unroll
        for (int k = 0; k < RS; k += 2) *reinterpret_cast<double2 *>(dst + k) = make_double2(buf[k], buf[k + 1]);
    }
    ob_valid[o] = ok ? 1 : 0;
}

// C_p = sum Jx~^T Jx~, g_p = sum Jx~^T r~ over the point's observations
// (lib.rs:863-864), and whether the point has any free pose/camera block.
template <typename T, int D>
__global__ void k_point_reduce(const T *rec, const int *pt_start, const int *ob_img,
                               const unsigned char *ob_valid, const int *img_free, int nP, T *pt_C,
                               T *pt_g, int *pt_nfree, const unsigned char *pt_live) {
    constexpr int RS = RecLayout<D>::kStride;
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nP) return;
    if (pt_live && !pt_live[p]) return;
    const int s = pt_start[p], e = pt_start[p + 1];
    T c00 = 0, c01 = 0, c02 = 0, c11 = 0, c12 = 0, c22 = 0, g0 = 0, g1 = 0, g2 = 0;
    int nfree = 0;
    for (int o = s; o < e; ++o) {
        const T *r = rec + (size_t)o * RS;
        const T r0 = r[0], r1 = r[1];
        const T a0 = r[2], a1 = r[3], a2 = r[4], b0 = r[5], b1 = r[6], b2 = r[7];
        c00 += a0 * a0 + b0 * b0; c01 += a0 * a1 + b0 * b1; c02 += a0 * a2 + b0 * b2;
        c11 += a1 * a1 + b1 * b1; c12 += a1 * a2 + b1 * b2; c22 += a2 * a2 + b2 * b2;
        g0 += a0 * r0 + b0 * r1; g1 += a1 * r0 + b1 * r1; g2 += a2 * r0 + b2 * r1;
        nfree += (ob_valid[o] && img_free[ob_img[o]]) ? 1 : 0;
    }
    T *C = pt_C + 6 * (size_t)p;
    C[0] = c00; C[1] = c01; C[2] = c02; C[3] = c11; C[4] = c12; C[5] = c22;
    T *g = pt_g + 3 * (size_t)p;
    g[0] = g0; g[1] = g1; g[2] = g2;
    pt_nfree[p] = nfree;
}

// diag(B) at slot level: sum of the image-level diagonal entries mapped
// onto each slot (a camera shared by several images sums them).
__global__ void k_diag_fold(const double *img_H, const int *slot_pre_start, const int *slot_pre,
                            int n, int D, double *diagB) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    double s = 0.0;
    for (int k = slot_pre_start[a]; k < slot_pre_start[a + 1]; ++k) {
        const int u = slot_pre[k];
        const int i = u / D, r = u - i * D;
        s += img_H[(size_t)i * D * D + r * D + r];
    }
    diagB[a] = s;
}

// (C_p + lambda diag C_p)^-1 for points with a free block (lib.rs:958-965),
// adjugate over determinant (None iff det == 0), and h_p = C^-1 g_p
// (point_inverse_block: FP64, or FP32 for well-conditioned blocks on the
// FP32 path).
template <typename T>
__global__ void __launch_bounds__(kPointInvBlock) k_point_inverse(const T *pt_C, const T *pt_g, const int *pt_nfree,
                                                                  const LMState *state, int nP, T *pt_Cinv, T *pt_h,
                                                                  unsigned char *pt_ok) {
    const double lam = state->lambda;
    point_inverse_block<T>(pt_C, pt_g, pt_nfree, nP, [&](int) { return lam; }, [](int) { return true; }, pt_Cinv,
                           pt_h, pt_ok);
}

// rhs_i = -b_i + sum_o Jc~_o^T (Jx~_o h_p): the reduced right-hand side
// (lib.rs:919-944 and :199-210). One warp per image.
template <typename T, int D>
__global__ void k_image_rhs(const T *rec, const int *img_start, const int *img_obs,
                            const int *ob_pt, const T *pt_h, const unsigned char *pt_ok,
                            const double *img_b, int nI, double *img_rhs, const unsigned char *img_live) {
    constexpr int RS = RecLayout<D>::kStride;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= nI) return;
    const int i = warp;
    if (img_live && !img_live[i]) return;
    T acc[D], comp[D];
#pragma unroll
    for (int c = 0; c < D; ++c) acc[c] = comp[c] = T(0);
    const int s = img_start[i], e = img_start[i + 1];
    for (int k = s + lane; k < e; k += 32) {
        const int o = img_obs[k];
        const int p = ob_pt[o];
        if (!pt_ok[p]) continue;
        const T *r = rec + (size_t)o * RS;
        const T *h = pt_h + 3 * (size_t)p;
        const T z0 = r[2] * h[0] + r[3] * h[1] + r[4] * h[2];
        const T z1 = r[5] * h[0] + r[6] * h[1] + r[7] * h[2];
#pragma unroll
        for (int c = 0; c < D; ++c) kahan_add(acc[c], comp[c], r[8 + c] * z0 + r[8 + D + c] * z1);
    }
#pragma unroll
    for (int c = 0; c < D; ++c) {
        double v = (double)acc[c] - (double)comp[c];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
        if (lane == 0) img_rhs[(size_t)i * D + c] = -img_b[(size_t)i * D + c] + v;
    }
}

template <typename T>
__global__ void k_gather_delta(const double *delta_slot, const int *img_slot, int nID, T *img_delta) {
    int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= nID) return;
    const int s = img_slot[u];
    img_delta[u] = s >= 0 ? (T)delta_slot[s] : T(0);
}

// delta_p = -C^-1 (g_p + sum_o Jx~^T (Jc~ delta_img)), trial point = p + delta_p
// (lib.rs:1100-1120, :1138-1141).
template <typename T, int D>
__global__ void k_backsub(const T *rec, const int *pt_start, const int *ob_img, const T *img_delta,
                          const T *pt_Cinv, const T *pt_g, const unsigned char *pt_ok,
                          const double *points, const LMState *state, int nP, double *points_trial,
                          const unsigned char *pt_live) {
    constexpr int RS = RecLayout<D>::kStride;
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nP) return;
    if (state->factor_failed) return;
    if (pt_live && !pt_live[p]) return;
    const double *X = points + 3 * (size_t)p;
    double *Y = points_trial + 3 * (size_t)p;
    if (!pt_ok[p]) {
        Y[0] = X[0]; Y[1] = X[1]; Y[2] = X[2];
        return;
    }
    const T *g = pt_g + 3 * (size_t)p;
    T a0 = g[0], a1 = g[1], a2 = g[2];
    for (int o = pt_start[p]; o < pt_start[p + 1]; ++o) {
        const T *r = rec + (size_t)o * RS;
        const T *d = img_delta + (size_t)ob_img[o] * D;
        T t0 = 0, t1 = 0;
#pragma unroll
        for (int c = 0; c < D; ++c) {
            t0 += r[8 + c] * d[c];
            t1 += r[8 + D + c] * d[c];
        }
        a0 += r[2] * t0 + r[5] * t1;
        a1 += r[3] * t0 + r[6] * t1;
        a2 += r[4] * t0 + r[7] * t1;
    }
    const T *Ci = pt_Cinv + 6 * (size_t)p;
    const T d0 = Ci[0] * a0 + Ci[1] * a1 + Ci[2] * a2;
    const T d1 = Ci[1] * a0 + Ci[3] * a1 + Ci[4] * a2;
    const T d2 = Ci[2] * a0 + Ci[4] * a1 + Ci[5] * a2;
    Y[0] = X[0] + (double)(-d0);
    Y[1] = X[1] + (double)(-d1);
    Y[2] = X[2] + (double)(-d2);
}

// Trial poses R <- exp(w) R, t <- t + dt (lib.rs:263-269, :1122-1136) and
// trial camera parameters params + delta (lib.rs:1143-1160).
__global__ void k_update_images(const double *poses, const double *cams, const int *pose_slot,
                                const int *cam_slot, const int *cam_model, const double *delta,
                                int nI, int nC, double *poses_trial, double *cams_trial) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nI) {
        const double *q = poses + 7 * (size_t)t;
        double *o = poses_trial + 7 * (size_t)t;
        const int s = pose_slot[t];
        if (s < 0) {
            for (int k = 0; k < 7; ++k) o[k] = q[k];
        } else {
            const double w0 = delta[s], w1 = delta[s + 1], w2 = delta[s + 2];
            const double th = sqrt(w0 * w0 + w1 * w1 + w2 * w2);
            double dw = 1.0, dx = 0.0, dy = 0.0, dz = 0.0;
            if (th > 0.0) {
                const double sc = sin(0.5 * th) / th;
                dw = cos(0.5 * th); dx = w0 * sc; dy = w1 * sc; dz = w2 * sc;
            }
            o[0] = dw * q[0] - dx * q[1] - dy * q[2] - dz * q[3];
            o[1] = dw * q[1] + dx * q[0] + dy * q[3] - dz * q[2];
            o[2] = dw * q[2] - dx * q[3] + dy * q[0] + dz * q[1];
            o[3] = dw * q[3] + dx * q[2] - dy * q[1] + dz * q[0];
            o[4] = q[4] + delta[s + 3];
            o[5] = q[5] + delta[s + 4];
            o[6] = q[6] + delta[s + 5];
        }
    }
    if (t < nC) {
        const double *c = cams + 8 * (size_t)t;
        double *o = cams_trial + 8 * (size_t)t;
        const int s = cam_slot[t];
        const int k = model_dof(cam_model[t]);
        for (int j = 0; j < 8; ++j) o[j] = (s >= 0 && j < k) ? c[j] + delta[s + j] : c[j];
    }
}

// FP64 cost over all observations with a fixed grid so the summation order
// is the same on every call. mode 0: sum w |r|^2 (lib.rs:727-745);
// mode 1: sum |r| (lib.rs:708-725); mode 2: sum |r|^2.
// Per-image FP64 rotation matrix and translation of the poses the cost
// evaluates ([nI][12]).
__global__ void k_pose_rt64(const double *poses, int nI, double *rt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nI) return;
    const double *q = poses + 7 * (size_t)i;
    double R[9];
    quat_to_R(q, R);
    double *o = rt + 12 * (size_t)i;
#pragma unroll
    for (int k = 0; k < 9; ++k) o[k] = R[k];
    o[9] = q[4];
    o[10] = q[5];
    o[11] = q[6];
}

// Robust cost / mean error of all observations in FP64 (lib.rs:708-745),
// block partial sums in a fixed order. M: the camera model when every camera
// has it (-1: the runtime switch).
template <int M>
__global__ void __launch_bounds__(256) k_cost(const double *rt, const double *cams,
                                              const double *points, const int *cam_of_img,
                                              const int *cam_model, const int *ob_img,
                                              const int *ob_pt, const double2 *ob_xy, long long nO,
                                              int loss, double scale, int mode, double *partials,
                                              long long *count_partials, float4 *rs_out) {
    double sum = 0.0;
    long long cnt = 0;
    for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < nO;
         o += (long long)gridDim.x * blockDim.x) {
        const int i = ob_img[o], p = ob_pt[o];
        const int c = cam_of_img[i];
        const double *X = points + 3 * (size_t)p;
        const double2 xy = ob_xy[o];
        double rx, ry;
        const bool ok = residual64_rt<M>(rt + 12 * (size_t)i, M >= 0 ? M : cam_model[c], cams + 8 * (size_t)c, X[0],
                                         X[1], X[2], xy.x, xy.y, rx, ry);
        if (rs_out) {  // FP64 residual and sqrt(weight) for the next linearisation's gradient terms
            double sw = 1.0;
            if (ok && loss != SFMBA_LOSS_NONE) sw = sqrt(robust_weight<double>(sqrt(rx * rx + ry * ry), loss, scale));
            rs_out[o] = ok ? make_float4((float)rx, (float)ry, (float)sw, 1.f) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        if (ok) {
            const double n2 = rx * rx + ry * ry;
            if (mode == 0) {
                if (loss == SFMBA_LOSS_NONE) sum += n2;
                else {
                    const double n = sqrt(n2);
                    sum += robust_weight<double>(n, loss, scale) * n * n;
                }
            } else if (mode == 1) {
                sum += sqrt(n2);
            } else {
                sum += n2;
            }
            ++cnt;
        }
    }
    __shared__ double ssum[256];
    __shared__ long long scnt[256];
    ssum[threadIdx.x] = sum;
    scnt[threadIdx.x] = cnt;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            ssum[threadIdx.x] += ssum[threadIdx.x + w];
            scnt[threadIdx.x] += scnt[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = ssum[0];
        count_partials[blockIdx.x] = scnt[0];
    }
}

// The FP32 path's cost (mode 0): k_cost with the projection chain in
// double-float arithmetic on the FP32 pipe; robust weights, the depth test
// near its threshold and the block sums stay FP64. The per-thread sum of
// squared norms is carried as a pair and added to FP64 once per thread.
template <int M>
__global__ void __launch_bounds__(256) k_cost_df(const float *rt_df, const float *cams_df, const float4 *pts_df,
                                                 const int *cam_of_img, const int *cam_model, const int *ob_img,
                                                 const int *ob_pt, const float4 *xy_df, long long nO, int loss,
                                                 double scale, double *partials, long long *count_partials,
                                                 float4 *rs_out) {
    dfl sum2 = df_make(0.f);
    double wsum = 0.0;
    long long cnt = 0;
    for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < nO;
         o += (long long)gridDim.x * blockDim.x) {
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
        const bool ok = residual_df<M>(rt, M >= 0 ? M : cam_model[c], cp, {pa.x, pa.y}, {pa.z, pa.w}, {pb.x, pb.y},
                                       {xy.x, xy.y}, {xy.z, xy.w}, rx, ry);
        const dfl n2 = ok ? rx * rx + ry * ry : df_make(0.f);
        float sw = 1.f;
        if (ok && loss != SFMBA_LOSS_NONE) {
            const double n2d = df_to_double(n2), n = sqrt(n2d), w = robust_weight<double>(n, loss, scale);
            sw = (float)sqrt(w);
            wsum += w * n * n;
        }
        if (rs_out)  // residual and sqrt(weight) for the next linearisation's gradient terms
            rs_out[o] = ok ? make_float4(rx.hi, ry.hi, sw, 1.f) : make_float4(0.f, 0.f, 0.f, 0.f);
        if (ok) {
            if (loss == SFMBA_LOSS_NONE) sum2 = sum2 + n2;
            ++cnt;
        }
    }
    __shared__ double ssum[256];
    __shared__ long long scnt[256];
    ssum[threadIdx.x] = df_to_double(sum2) + wsum;
    scnt[threadIdx.x] = cnt;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            ssum[threadIdx.x] += ssum[threadIdx.x + w];
            scnt[threadIdx.x] += scnt[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = ssum[0];
        count_partials[blockIdx.x] = scnt[0];
    }
}

// Pairs of the points, pose matrices and camera parameters the cost
// evaluates: threads [0, nP) points, then nI * 12 pose entries, then nC * 8
// camera parameters.
__global__ void k_split_df(const double *points, int nP, const double *rt64, int nI, const double *cams, int nC,
                           float4 *pts_df, float *rt_df, float *cams_df) {
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < nP) {
        const double *X = points + 3 * (size_t)t;
        const dfl x = df_from(X[0]), y = df_from(X[1]), z = df_from(X[2]);
        pts_df[2 * t] = make_float4(x.hi, x.lo, y.hi, y.lo);
        pts_df[2 * t + 1] = make_float4(z.hi, z.lo, 0.f, 0.f);
        return;
    }
    t -= nP;
    if (t < 12LL * nI) {
        const dfl v = df_from(rt64[t]);
        rt_df[2 * t] = v.hi;
        rt_df[2 * t + 1] = v.lo;
        return;
    }
    t -= 12LL * nI;
    if (t < 8LL * nC) {
        const dfl v = df_from(cams[t]);
        cams_df[2 * t] = v.hi;
        cams_df[2 * t + 1] = v.lo;
    }
}

__global__ void k_split_xy_df(const double2 *xy, long long nO, float4 *xy_df) {
    const long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (o >= nO) return;
    const double2 v = xy[o];
    const dfl x = df_from(v.x), y = df_from(v.y);
    xy_df[o] = make_float4(x.hi, x.lo, y.hi, y.lo);
}

__global__ void k_cost_finalize(const double *partials, const long long *count_partials, int nb,
                                double *out, long long *out_count) {
    __shared__ double ssum[256];
    __shared__ long long scnt[256];
    double s = 0.0;
    long long c = 0;
    for (int k = threadIdx.x; k < nb; k += blockDim.x) {
        s += partials[k];
        c += count_partials[k];
    }
    ssum[threadIdx.x] = s;
    scnt[threadIdx.x] = c;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            ssum[threadIdx.x] += ssum[threadIdx.x + w];
            scnt[threadIdx.x] += scnt[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        *out = ssum[0];
        if (out_count) *out_count = scnt[0];
    }
}

// Accept iff the trial cost is finite and lower (lib.rs:1188-1212):
// lambda = max(lambda/3, 1e-12), nu = 2; otherwise lambda *= nu, nu *= 2.
__global__ void k_accept(LMState *st) {
    if (st->factor_failed) return;
    const double t = st->trial_cost;
    if (isfinite(t) && t < st->cost) {
        st->accepted = 1;
        st->cost = t;
        st->valid_obs = st->trial_valid_obs;
        st->lambda = fmax(st->lambda / 3.0, 1e-12);
        st->nu = 2.0;
    } else {
        st->accepted = 0;
        st->lambda *= st->nu;
        st->nu *= 2.0;
    }
}

// Both Cholesky and LU failed: grow the damping (lib.rs:1089-1091).
__global__ void k_reject(LMState *st) {
    if (!st->solve_failed) return;
    st->accepted = 0;
    st->lambda *= st->nu;
    st->nu *= 2.0;
}

__global__ void k_begin_outer(LMState *st) {
    st->cost_before = st->cost;
    st->accepted = 0;
    st->factor_failed = 0;
    st->solve_failed = 0;
}

__global__ void k_begin_retry(LMState *st) {
    st->accepted = 0;
    st->factor_failed = 0;
    st->solve_failed = 0;
}

__global__ void k_commit(const LMState *st, int nI, int nC, int nP, const double *poses_trial,
                         const double *cams_trial, const double *points_trial, double *poses,
                         double *cams, double *points, float4 *points32, long long nO,
                         const float4 *rs_trial, float4 *rs) {
    if (!st->accepted) return;
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (rs && t < nO) rs[t] = rs_trial[t];
    if (t < nP) {
        const double x = points_trial[3 * t], y = points_trial[3 * t + 1], z = points_trial[3 * t + 2];
        points[3 * t] = x; points[3 * t + 1] = y; points[3 * t + 2] = z;
        if (points32) points32[t] = make_float4((float)x, (float)y, (float)z, 0.f);
    }
    if (t < 7LL * nI) poses[t] = poses_trial[t];
    if (t < 8LL * nC) cams[t] = cams_trial[t];
}

__global__ void k_refresh_points32(const double *points, int nP, float4 *points32) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nP) return;
    points32[p] = make_float4((float)points[3 * (size_t)p], (float)points[3 * (size_t)p + 1],
                              (float)points[3 * (size_t)p + 2], 0.f);
}

// Unweighted residual and Jacobians of each observation in input order,
// every column an unknown (the solver's device code, for parity checks).
template <typename T>
__global__ void k_jacobian_probe(JacProbe q) {
    long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (o >= q.nO) return;
    const int i = q.obs_img[o], p = q.obs_pt[o], c = q.cam_of_img[i];
    double R[9];
    quat_to_R(q.poses + 7 * (size_t)i, R);
    ImageLin<T> im;
    for (int k = 0; k < 9; ++k) im.R[k] = (T)R[k];
    for (int k = 0; k < 3; ++k) im.t[k] = (T)q.poses[7 * (size_t)i + 4 + k];
    for (int k = 0; k < 8; ++k) im.c[k] = (T)q.cams[8 * (size_t)c + k];
    im.model = q.cam_model[c];
    im.active = 0x3FFF;
    T rr[2], jx[6], jc[28];
    const bool ok = linearize<T, 14>(im, (T)q.points[3 * (size_t)p], (T)q.points[3 * (size_t)p + 1],
                                     (T)q.points[3 * (size_t)p + 2], (T)q.obs_xy[2 * o],
                                     (T)q.obs_xy[2 * o + 1], SFMBA_LOSS_NONE, T(1), rr, jx, jc);
    q.r[2 * o] = rr[0];
    q.r[2 * o + 1] = rr[1];
    for (int k = 0; k < 6; ++k) q.jx[6 * o + k] = jx[k];
    for (int row = 0; row < 2; ++row) {
        for (int k = 0; k < 6; ++k) q.jp[12 * o + 6 * row + k] = jc[14 * row + k];
        for (int k = 0; k < 8; ++k) q.jc[16 * o + 8 * row + k] = jc[14 * row + 6 + k];
    }
    q.valid[o] = ok ? 1 : 0;
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

}  // namespace

void launch_prepare_images(const Bufs &b, cudaStream_t s) {
    if (b.nI == 0) return;
    if (b.mixed)
        k_prepare_images<float><<<div_up(b.nI, 128), 128, 0, s>>>(
            b.poses, b.cams, b.cam_of_img, b.cam_model, b.img_active, b.nI, (ImageLin<float> *)b.img_lin, b.img_mv);
    else
        k_prepare_images<double><<<div_up(b.nI, 128), 128, 0, s>>>(
            b.poses, b.cams, b.cam_of_img, b.cam_model, b.img_active, b.nI, (ImageLin<double> *)b.img_lin,
            nullptr);
    SFMBA_LAUNCH_CHECK();
}

void launch_linearize(const Bufs &b, cudaStream_t s) {
    if (b.nO == 0) return;
    dispatch_D(b.D, [&](auto dc) {
        constexpr int D = decltype(dc)::value;
        if (b.mixed)
            k_linearize<float, D><<<div_up(b.nO, 256), 256, 0, s>>>(
                (const ImageLin<float> *)b.img_lin, b.points, b.points32, b.ob_img, b.ob_pt, b.ob_xy,
                b.nO, b.loss, (float)b.loss_scale, (float *)b.rec, b.ob_valid, b.ob_rs, b.img_live);
        else
            k_linearize<double, D><<<div_up(b.nO, 256), 256, 0, s>>>(
                (const ImageLin<double> *)b.img_lin, b.points, b.points32, b.ob_img, b.ob_pt, b.ob_xy,
                b.nO, b.loss, b.loss_scale, (double *)b.rec, b.ob_valid, nullptr, b.img_live);
    });
    SFMBA_LAUNCH_CHECK();
}

void launch_point_reduce(const Bufs &b, cudaStream_t s) {
    if (b.nP == 0) return;
    dispatch_D(b.D, [&](auto dc) {
        constexpr int D = decltype(dc)::value;
        if (b.mixed)
            k_point_reduce<float, D><<<div_up(b.nP, 128), 128, 0, s>>>(
                (const float *)b.rec, b.pt_start, b.ob_img, b.ob_valid, b.img_free, b.nP,
                (float *)b.pt_C, (float *)b.pt_g, b.pt_nfree, b.pt_live);
        else
            k_point_reduce<double, D><<<div_up(b.nP, 128), 128, 0, s>>>(
                (const double *)b.rec, b.pt_start, b.ob_img, b.ob_valid, b.img_free, b.nP,
                (double *)b.pt_C, (double *)b.pt_g, b.pt_nfree, b.pt_live);
    });
    SFMBA_LAUNCH_CHECK();
}

void launch_diag_fold(const Bufs &b, cudaStream_t s) {
    if (b.n == 0) return;
    k_diag_fold<<<div_up(b.n, 256), 256, 0, s>>>(b.img_H, b.slot_pre_start, b.slot_pre, b.n, b.D,
                                                 b.diagB);
    SFMBA_LAUNCH_CHECK();
}

void launch_point_inverse(const Bufs &b, cudaStream_t s) {
    if (b.nP == 0) return;
    if (b.mixed)
        k_point_inverse<float><<<div_up(b.nP, kPointInvBlock), kPointInvBlock, 0, s>>>(
            (const float *)b.pt_C, (const float *)b.pt_g, b.pt_nfree, b.state, b.nP,
            (float *)b.pt_Cinv, (float *)b.pt_h, b.pt_ok);
    else
        k_point_inverse<double><<<div_up(b.nP, kPointInvBlock), kPointInvBlock, 0, s>>>(
            (const double *)b.pt_C, (const double *)b.pt_g, b.pt_nfree, b.state, b.nP,
            (double *)b.pt_Cinv, (double *)b.pt_h, b.pt_ok);
    SFMBA_LAUNCH_CHECK();
}

void launch_image_rhs(const Bufs &b, cudaStream_t s) {
    if (b.nI == 0) return;
    dispatch_D(b.D, [&](auto dc) {
        constexpr int D = decltype(dc)::value;
        const int warps_per_block = 4;
        if (b.mixed)
            k_image_rhs<float, D><<<div_up(b.nI, warps_per_block), 32 * warps_per_block, 0, s>>>(
                (const float *)b.rec, b.img_start, b.img_obs, b.ob_pt, (const float *)b.pt_h, b.pt_ok,
                b.img_b, b.nI, b.img_rhs, b.img_live);
        else
            k_image_rhs<double, D><<<div_up(b.nI, warps_per_block), 32 * warps_per_block, 0, s>>>(
                (const double *)b.rec, b.img_start, b.img_obs, b.ob_pt, (const double *)b.pt_h,
                b.pt_ok, b.img_b, b.nI, b.img_rhs, b.img_live);
    });
    SFMBA_LAUNCH_CHECK();
}

void launch_gather_delta(const Bufs &b, const double *delta_slot, cudaStream_t s) {
    if (b.nID == 0) return;
    if (b.mixed)
        k_gather_delta<float><<<div_up(b.nID, 256), 256, 0, s>>>(delta_slot, b.img_slot, b.nID,
                                                                 (float *)b.img_delta);
    else
        k_gather_delta<double><<<div_up(b.nID, 256), 256, 0, s>>>(delta_slot, b.img_slot, b.nID,
                                                                  (double *)b.img_delta);
    SFMBA_LAUNCH_CHECK();
}

void launch_backsub_update(const Bufs &b, const double *delta_slot, cudaStream_t s) {
    launch_gather_delta(b, delta_slot, s);
    if (b.nP > 0) {
        dispatch_D(b.D, [&](auto dc) {
            constexpr int D = decltype(dc)::value;
            if (b.mixed)
                k_backsub<float, D><<<div_up(b.nP, 128), 128, 0, s>>>(
                    (const float *)b.rec, b.pt_start, b.ob_img, (const float *)b.img_delta,
                    (const float *)b.pt_Cinv, (const float *)b.pt_g, b.pt_ok, b.points, b.state, b.nP,
                    b.points_trial, b.pt_live);
            else
                k_backsub<double, D><<<div_up(b.nP, 128), 128, 0, s>>>(
                    (const double *)b.rec, b.pt_start, b.ob_img, (const double *)b.img_delta,
                    (const double *)b.pt_Cinv, (const double *)b.pt_g, b.pt_ok, b.points, b.state,
                    b.nP, b.points_trial, b.pt_live);
        });
        SFMBA_LAUNCH_CHECK();
    }
    launch_update_images(b, delta_slot, s);
}

void launch_update_images(const Bufs &b, const double *delta_slot, cudaStream_t s) {
    const int m = b.nI > b.nC ? b.nI : b.nC;
    if (m > 0) {
        k_update_images<<<div_up(m, 128), 128, 0, s>>>(b.poses, b.cams, b.pose_slot, b.cam_slot,
                                                       b.cam_model, delta_slot, b.nI, b.nC,
                                                       b.poses_trial, b.cams_trial);
        SFMBA_LAUNCH_CHECK();
    }
}

void launch_split_df(const Bufs &b, bool trial, cudaStream_t s) {
    const long long nsplit = (long long)b.nP + 12LL * b.nI + 8LL * b.nC;
    if (nsplit == 0) return;
    k_split_df<<<div_up(nsplit, 256), 256, 0, s>>>(trial ? b.points_trial : b.points, b.nP, b.img_rt64, b.nI,
                                                   trial ? b.cams_trial : b.cams, b.nC, b.pts_df, b.rt_df,
                                                   b.cams_df);
    SFMBA_LAUNCH_CHECK();
}

void launch_split_xy_df(const Bufs &b, cudaStream_t s) {
    if (!b.df_cost || b.nO == 0) return;
    k_split_xy_df<<<div_up(b.nO, 256), 256, 0, s>>>(b.ob_xy, b.nO, b.ob_xy_df);
    SFMBA_LAUNCH_CHECK();
}

void launch_pose_rt64(const double *poses, int nI, double *rt, cudaStream_t s) {
    if (nI == 0) return;
    k_pose_rt64<<<div_up(nI, 128), 128, 0, s>>>(poses, nI, rt);
    SFMBA_LAUNCH_CHECK();
}

static void cost_impl(const Bufs &b, bool trial, int mode, double *out, long long *out_count,
                      cudaStream_t s, float4 *rs_out = nullptr) {
    launch_pose_rt64(trial ? b.poses_trial : b.poses, b.nI, b.img_rt64, s);
    const double *cams = trial ? b.cams_trial : b.cams, *points = trial ? b.points_trial : b.points;
    if (mode == 0 && b.mixed && b.df_cost) {
        launch_split_df(b, trial, s);
        auto run_df = [&](auto mc) {
            k_cost_df<decltype(mc)::value><<<kCostBlocks, 256, 0, s>>>(
                b.rt_df, b.cams_df, b.pts_df, b.cam_of_img, b.cam_model, b.ob_img, b.ob_pt, b.ob_xy_df, b.nO, b.loss,
                b.loss_scale, b.partials, b.count_partials, rs_out);
        };
        switch (b.uniform_model) {
        case SFMBA_SIMPLE_PINHOLE: run_df(std::integral_constant<int, SFMBA_SIMPLE_PINHOLE>()); break;
        case SFMBA_PINHOLE: run_df(std::integral_constant<int, SFMBA_PINHOLE>()); break;
        case SFMBA_SIMPLE_RADIAL: run_df(std::integral_constant<int, SFMBA_SIMPLE_RADIAL>()); break;
        case SFMBA_RADIAL: run_df(std::integral_constant<int, SFMBA_RADIAL>()); break;
        case SFMBA_OPENCV: run_df(std::integral_constant<int, SFMBA_OPENCV>()); break;
        default: run_df(std::integral_constant<int, -1>()); break;
        }
        SFMBA_LAUNCH_CHECK();
        k_cost_finalize<<<1, 256, 0, s>>>(b.partials, b.count_partials, kCostBlocks, out, out_count);
        SFMBA_LAUNCH_CHECK();
        return;
    }
    auto run = [&](auto mc) {
        k_cost<decltype(mc)::value><<<kCostBlocks, 256, 0, s>>>(
            b.img_rt64, cams, points, b.cam_of_img, b.cam_model,
            b.ob_img, b.ob_pt, b.ob_xy, b.nO, b.loss, b.loss_scale, mode, b.partials, b.count_partials, rs_out);
    };
    switch (b.uniform_model) {
    case SFMBA_SIMPLE_PINHOLE: run(std::integral_constant<int, SFMBA_SIMPLE_PINHOLE>()); break;
    case SFMBA_PINHOLE: run(std::integral_constant<int, SFMBA_PINHOLE>()); break;
    case SFMBA_SIMPLE_RADIAL: run(std::integral_constant<int, SFMBA_SIMPLE_RADIAL>()); break;
    case SFMBA_RADIAL: run(std::integral_constant<int, SFMBA_RADIAL>()); break;
    case SFMBA_OPENCV: run(std::integral_constant<int, SFMBA_OPENCV>()); break;
    case SFMBA_OPENCV_FISHEYE: run(std::integral_constant<int, SFMBA_OPENCV_FISHEYE>()); break;
    default: run(std::integral_constant<int, -1>()); break;
    }
    SFMBA_LAUNCH_CHECK();
    k_cost_finalize<<<1, 256, 0, s>>>(b.partials, b.count_partials, kCostBlocks, out, out_count);
    SFMBA_LAUNCH_CHECK();
}

void launch_cost(const Bufs &b, bool trial, bool into_trial, cudaStream_t s) {
    // FP32 PCG path: the cost's FP64 residuals are kept for the point and
    // image passes' gradient terms (ob_rs: current parameters; ob_rs_trial:
    // the trial, made current by the commit when accepted).
    float4 *rs = nullptr;
    if (b.mixed && b.ob_rs) rs = into_trial ? b.ob_rs_trial : b.ob_rs;
    if (into_trial)
        cost_impl(b, trial, 0, &b.state->trial_cost, &b.state->trial_valid_obs, s, rs);
    else
        cost_impl(b, trial, 0, &b.state->cost, &b.state->valid_obs, s, rs);
}

void launch_mean_error(const Bufs &b, cudaStream_t s) {
    // sum |r| into state->trial_cost, count into state->trial_valid_obs
    cost_impl(b, false, 1, &b.state->trial_cost, &b.state->trial_valid_obs, s);
}

void launch_accept(const Bufs &b, cudaStream_t s) {
    k_accept<<<1, 1, 0, s>>>(b.state);
    SFMBA_LAUNCH_CHECK();
}

void launch_reject(const Bufs &b, cudaStream_t s) {
    k_reject<<<1, 1, 0, s>>>(b.state);
    SFMBA_LAUNCH_CHECK();
}

void launch_begin_outer(const Bufs &b, cudaStream_t s) {
    k_begin_outer<<<1, 1, 0, s>>>(b.state);
    SFMBA_LAUNCH_CHECK();
}

void launch_begin_retry(const Bufs &b, cudaStream_t s) {
    k_begin_retry<<<1, 1, 0, s>>>(b.state);
    SFMBA_LAUNCH_CHECK();
}

void launch_commit(const Bufs &b, cudaStream_t s) {
    const bool rs = b.mixed && b.ob_rs;
    long long m = b.nP;
    if (7LL * b.nI > m) m = 7LL * b.nI;
    if (8LL * b.nC > m) m = 8LL * b.nC;
    if (rs && b.nO > m) m = b.nO;
    if (m == 0) return;
    k_commit<<<div_up(m, 256), 256, 0, s>>>(b.state, b.nI, b.nC, b.nP, b.poses_trial, b.cams_trial,
                                            b.points_trial, b.poses, b.cams, b.points,
                                            b.mixed ? b.points32 : nullptr, b.nO, rs ? b.ob_rs_trial : nullptr,
                                            rs ? b.ob_rs : nullptr);
    SFMBA_LAUNCH_CHECK();
}

void launch_refresh_points32(const Bufs &b, cudaStream_t s) {
    if (!b.mixed || b.nP == 0) return;
    k_refresh_points32<<<div_up(b.nP, 256), 256, 0, s>>>(b.points, b.nP, b.points32);
    SFMBA_LAUNCH_CHECK();
}

void launch_count_valid(const Bufs &b, cudaStream_t s) { launch_cost(b, false, false, s); }

void launch_jacobian_probe(const JacProbe &q, bool fp32, cudaStream_t s) {
    if (q.nO == 0) return;
    if (fp32) k_jacobian_probe<float><<<div_up(q.nO, 128), 128, 0, s>>>(q);
    else k_jacobian_probe<double><<<div_up(q.nO, 128), 128, 0, s>>>(q);
    SFMBA_LAUNCH_CHECK();
}

}  // namespace sfmba
