// Camera models (COLMAP names and parameter order) and the per-observation
// residual with its hand-written adjoint Jacobian, for FP32 and FP64.
//
// Reference semantics: crates/sfm-core/src/camera.rs:204-244 (project),
// crates/sfm-core/src/pose.rs:46-48 (transform_point),
// crates/sfm-ba/src/lib.rs:249-261 (reprojection_residual),
// crates/sfm-ba/src/lib.rs:282-590 (pose_point_jacobians, analytic_jacobians),
// crates/sfm-ba/src/lib.rs:677-694 (robust_weight).
#pragma once

#include "common.cuh"
#include "dfloat.cuh"

namespace sfmba {

template <typename T>
__device__ __forceinline__ T dev_sqrt(T x);
template <>
__device__ __forceinline__ float dev_sqrt<float>(float x) { return sqrtf(x); }
template <>
__device__ __forceinline__ double dev_sqrt<double>(double x) { return sqrt(x); }

template <typename T>
__device__ __forceinline__ T dev_atan(T x);
template <>
__device__ __forceinline__ float dev_atan<float>(float x) { return atanf(x); }
template <>
__device__ __forceinline__ double dev_atan<double>(double x) { return atan(x); }

// Per-image constants of one linearisation pass, in the kernel's precision:
// rotation matrix and translation of the pose, the camera's parameters and
// which columns of the image block are unknowns.
template <typename T>
struct __align__(16) ImageLin {
    T R[9];
    T t[3];
    T c[8];
    int model;
    int active;  // bit r set: column r of the image block is an unknown
    int pad[2];
};

// Forward projection of normalised coordinates plus the local derivatives
// the adjoint pass needs: A = d(u,v)/d(xp,yp) (2x2) and the parameter
// columns G = d(u,v)/d(params) (2x8, zero past the model's count).
template <typename T, int M = -1>
__device__ __forceinline__ void distort(int model, const T *c, T xp, T yp, T &u, T &v, T A[2][2],
                                        T G[2][8]) {
    if constexpr (M >= 0) model = M;
#pragma unroll
    for (int i = 0; i < 8; ++i) { G[0][i] = T(0); G[1][i] = T(0); }
    A[0][1] = T(0);
    A[1][0] = T(0);
    switch (model) {
    case SFMBA_SIMPLE_PINHOLE: {
        const T f = c[0];
        u = f * xp + c[1];
        v = f * yp + c[2];
        A[0][0] = f; A[1][1] = f;
        G[0][0] = xp; G[0][1] = T(1);
        G[1][0] = yp; G[1][2] = T(1);
        break;
    }
    case SFMBA_PINHOLE: {
        u = c[0] * xp + c[2];
        v = c[1] * yp + c[3];
        A[0][0] = c[0]; A[1][1] = c[1];
        G[0][0] = xp; G[0][2] = T(1);
        G[1][1] = yp; G[1][3] = T(1);
        break;
    }
    case SFMBA_SIMPLE_RADIAL:
    case SFMBA_RADIAL: {
        const bool two = model == SFMBA_RADIAL;
        const T f = c[0], k1 = c[3], k2 = two ? c[4] : T(0);
        const T r2 = xp * xp + yp * yp;
        const T d = two ? T(1) + k1 * r2 + k2 * r2 * r2 : T(1) + k1 * r2;
        const T dd = two ? k1 + T(2) * k2 * r2 : k1;  // d(d)/d(r2)
        u = f * xp * d + c[1];
        v = f * yp * d + c[2];
        A[0][0] = f * (d + T(2) * dd * xp * xp);
        A[0][1] = T(2) * f * dd * xp * yp;
        A[1][0] = A[0][1];
        A[1][1] = f * (d + T(2) * dd * yp * yp);
        G[0][0] = xp * d; G[0][1] = T(1); G[0][3] = f * xp * r2;
        G[1][0] = yp * d; G[1][2] = T(1); G[1][3] = f * yp * r2;
        if (two) {
            G[0][4] = f * xp * r2 * r2;
            G[1][4] = f * yp * r2 * r2;
        }
        break;
    }
    case SFMBA_OPENCV: {
        const T fx = c[0], fy = c[1], k1 = c[4], k2 = c[5], p1 = c[6], p2 = c[7];
        const T r2 = xp * xp + yp * yp;
        const T rad = T(1) + k1 * r2 + k2 * r2 * r2;
        const T xd = xp * rad + T(2) * p1 * xp * yp + p2 * (r2 + T(2) * xp * xp);
        const T yd = yp * rad + p1 * (r2 + T(2) * yp * yp) + T(2) * p2 * xp * yp;
        u = fx * xd + c[2];
        v = fy * yd + c[3];
        const T kr = k1 + T(2) * k2 * r2;
        const T dxx = rad + T(2) * kr * xp * xp + T(2) * p1 * yp + T(6) * p2 * xp;
        const T dxy = T(2) * kr * xp * yp + T(2) * p1 * xp + T(2) * p2 * yp;
        const T dyy = rad + T(2) * kr * yp * yp + T(6) * p1 * yp + T(2) * p2 * xp;
        A[0][0] = fx * dxx; A[0][1] = fx * dxy;
        A[1][0] = fy * dxy; A[1][1] = fy * dyy;
        G[0][0] = xd; G[0][2] = T(1);
        G[0][4] = fx * xp * r2; G[0][5] = fx * xp * r2 * r2;
        G[0][6] = fx * T(2) * xp * yp; G[0][7] = fx * (r2 + T(2) * xp * xp);
        G[1][1] = yd; G[1][3] = T(1);
        G[1][4] = fy * yp * r2; G[1][5] = fy * yp * r2 * r2;
        G[1][6] = fy * (r2 + T(2) * yp * yp); G[1][7] = fy * T(2) * xp * yp;
        break;
    }
    default: {  // SFMBA_OPENCV_FISHEYE (equidistant)
        const T fx = c[0], fy = c[1], k1 = c[4], k2 = c[5], k3 = c[6], k4 = c[7];
        T r = dev_sqrt<T>(xp * xp + yp * yp);
        r = r > T(1e-12) ? r : T(1e-12);
        const T th = dev_atan<T>(r), t2 = th * th, t4 = t2 * t2, t6 = t4 * t2, t8 = t4 * t4;
        const T poly = T(1) + k1 * t2 + k2 * t4 + k3 * t6 + k4 * t8;
        const T thd = th * poly, s = thd / r;
        u = fx * (xp * s) + c[2];
        v = fy * (yp * s) + c[3];
        const T dpoly = k1 + T(2) * k2 * t2 + T(3) * k3 * t4 + T(4) * k4 * t6;
        const T dthd = poly + T(2) * t2 * dpoly;
        const T ds_dr = (dthd / (T(1) + r * r) * r - thd) / (r * r);
        const T dsx = ds_dr * (xp / r), dsy = ds_dr * (yp / r);
        A[0][0] = fx * (s + xp * dsx); A[0][1] = fx * xp * dsy;
        A[1][0] = fy * yp * dsx;       A[1][1] = fy * (s + yp * dsy);
        G[0][0] = xp * s; G[0][2] = T(1);
        G[1][1] = yp * s; G[1][3] = T(1);
        const T tk[4] = {th * t2, th * t4, th * t6, th * t8};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            G[0][4 + i] = fx * xp * tk[i] / r;
            G[1][4 + i] = fy * yp * tk[i] / r;
        }
        break;
    }
    }
}

template <typename T>
__device__ __forceinline__ T robust_weight(T n, int loss, T scale) {
    const T s = scale > T(1e-9) ? scale : T(1e-9);
    if (loss == SFMBA_LOSS_HUBER) return n <= s ? T(1) : s / n;
    if (loss == SFMBA_LOSS_CAUCHY) {
        const T q = n / s;
        return T(1) / (T(1) + q * q);
    }
    return T(1);
}

// Optional FP64 residual of an observation. The FP32 path computes the
// pixel residual u - obs from ~1e3 px quantities, which leaves ~1e-4 px of
// rounding: far above what the gradient near the minimum can tolerate. The
// kernels that form gradient terms pass the residual and sqrt of the robust
// weight that the FP64 cost kernel computed for these parameters, stored
// rounded to FP32 (relative error 6e-8 of a value that is already small,
// against the ~1e-4 px absolute error of an FP32 projection); they are
// combined in FP32, which keeps GB300's narrow FP64 pipe out of the passes.
struct Res64 {
    bool use = false;
    bool ok = false;
    float r0 = 0.f, r1 = 0.f;  // unweighted residual
    float s = 1.f;             // sqrt of the robust weight
};

// Residual and Jacobian of one observation, weighted by sqrt(w).
//
// Forward pass: pc = R X + t, (xp, yp) = (pc.x, pc.y) / pc.z, pixel = distort.
// Adjoint pass, once per pixel row (u, then v): the row's sensitivity to the
// normalised coordinates (row of A) is pulled back through the perspective
// divide to the camera-frame point (pbar), then to the world point
// (R^T pbar) and to the left rotation increment ((pc - t) x pbar) and the
// translation (pbar). Camera-parameter columns come straight from G.
// Returns false (and zeros) when pc.z <= 1e-9.
template <typename T, int D>
__device__ __forceinline__ bool linearize(const ImageLin<T> &im, T X0, T X1, T X2, T ox, T oy,
                                          int loss, T scale, T rr[2], T jx[6], T jc[2 * D],
                                          T *weight = nullptr, const Res64 &rin = Res64()) {
    const T q0 = im.R[0] * X0 + im.R[1] * X1 + im.R[2] * X2;
    const T q1 = im.R[3] * X0 + im.R[4] * X1 + im.R[5] * X2;
    const T q2 = im.R[6] * X0 + im.R[7] * X1 + im.R[8] * X2;
    const T pc0 = q0 + im.t[0], pc1 = q1 + im.t[1], pc2 = q2 + im.t[2];
    if (!(pc2 > T(kMinDepth)) || (rin.use && !rin.ok)) {
        rr[0] = rr[1] = T(0);
#pragma unroll
        for (int i = 0; i < 6; ++i) jx[i] = T(0);
#pragma unroll
        for (int i = 0; i < 2 * D; ++i) jc[i] = T(0);
        if (weight) *weight = T(0);
        return false;
    }
    const T iz = T(1) / pc2;
    const T xp = pc0 * iz, yp = pc1 * iz;
    T u, v, A[2][2], G[2][8];
    distort<T>(im.model, im.c, xp, yp, u, v, A, G);
    T s;
    if (rin.use) {
        s = (T)rin.s;
        rr[0] = (T)rin.r0 * s;
        rr[1] = (T)rin.r1 * s;
        if (weight) *weight = s * s;
    } else {
        rr[0] = u - ox;
        rr[1] = v - oy;
        const T n = dev_sqrt<T>(rr[0] * rr[0] + rr[1] * rr[1]);
        const T w = robust_weight<T>(n, loss, scale);
        s = dev_sqrt<T>(w);
        if (weight) *weight = w;
        rr[0] *= s;
        rr[1] *= s;
    }
#pragma unroll
    for (int row = 0; row < 2; ++row) {
        // pbar = d(pixel_row)/d(pc)
        const T a0 = A[row][0] * s, a1 = A[row][1] * s;
        const T pb0 = a0 * iz, pb1 = a1 * iz, pb2 = -(a0 * xp + a1 * yp) * iz;
        jx[row * 3 + 0] = im.R[0] * pb0 + im.R[3] * pb1 + im.R[6] * pb2;
        jx[row * 3 + 1] = im.R[1] * pb0 + im.R[4] * pb1 + im.R[7] * pb2;
        jx[row * 3 + 2] = im.R[2] * pb0 + im.R[5] * pb1 + im.R[8] * pb2;
        T *o = jc + row * D;
        const bool pose_on = im.active & 1;
        o[0] = pose_on ? q1 * pb2 - q2 * pb1 : T(0);
        o[1] = pose_on ? q2 * pb0 - q0 * pb2 : T(0);
        o[2] = pose_on ? q0 * pb1 - q1 * pb0 : T(0);
        o[3] = pose_on ? pb0 : T(0);
        o[4] = pose_on ? pb1 : T(0);
        o[5] = pose_on ? pb2 : T(0);
#pragma unroll
        for (int k = 0; k < D - 6; ++k) o[6 + k] = ((im.active >> (6 + k)) & 1) ? G[row][k] * s : T(0);
    }
    return true;
}

// Compact linearisation of one observation: everything needed to apply its
// Jacobian and transpose without forming them. With q = R X, the pixel-row
// sensitivities d_row = d(pixel_row)/d(pc) and the camera-parameter rows
// g_row (all weighted by sqrt(w)):
//   pose rotation columns of row  = q x d_row, translation columns = d_row,
//   point columns of row          = R^T d_row, camera columns = g_row.
template <typename T, int D>
struct LinCompact {
    static constexpr int K = D > 6 ? D - 6 : 1;
    T q[3];
    T d[2][3];
    T g[2][K];
    T r[2];
    bool pose_on;
};

template <typename T, int D, int M = -1>
__device__ __forceinline__ bool linearize_compact(const ImageLin<T> &im, T X0, T X1, T X2, T ox, T oy, int loss,
                                                  T scale, LinCompact<T, D> &L, const Res64 &rin = Res64()) {
    L.q[0] = im.R[0] * X0 + im.R[1] * X1 + im.R[2] * X2;
    L.q[1] = im.R[3] * X0 + im.R[4] * X1 + im.R[5] * X2;
    L.q[2] = im.R[6] * X0 + im.R[7] * X1 + im.R[8] * X2;
    L.pose_on = im.active & 1;
    const T pc0 = L.q[0] + im.t[0], pc1 = L.q[1] + im.t[1], pc2 = L.q[2] + im.t[2];
    if (!(pc2 > T(kMinDepth)) || (rin.use && !rin.ok)) {
#pragma unroll
        for (int row = 0; row < 2; ++row) {
            L.r[row] = T(0);
#pragma unroll
            for (int c = 0; c < 3; ++c) L.d[row][c] = T(0);
#pragma unroll
            for (int k = 0; k < LinCompact<T, D>::K; ++k) L.g[row][k] = T(0);
        }
        return false;
    }
    const T iz = T(1) / pc2;
    const T xp = pc0 * iz, yp = pc1 * iz;
    T u, v, A[2][2], G[2][8];
    distort<T, M>(im.model, im.c, xp, yp, u, v, A, G);
    T s;
    if (rin.use) {
        s = (T)rin.s;
        L.r[0] = (T)rin.r0 * s;
        L.r[1] = (T)rin.r1 * s;
    } else {
        const T r0 = u - ox, r1 = v - oy;
        s = loss == SFMBA_LOSS_NONE ? T(1) : dev_sqrt<T>(robust_weight<T>(dev_sqrt<T>(r0 * r0 + r1 * r1), loss, scale));
        L.r[0] = r0 * s;
        L.r[1] = r1 * s;
    }
#pragma unroll
    for (int row = 0; row < 2; ++row) {
        const T a0 = A[row][0] * s, a1 = A[row][1] * s;
        L.d[row][0] = a0 * iz;
        L.d[row][1] = a1 * iz;
        L.d[row][2] = -(a0 * xp + a1 * yp) * iz;
#pragma unroll
        for (int k = 0; k < LinCompact<T, D>::K; ++k)
            L.g[row][k] = (D > 6 && ((im.active >> (6 + k)) & 1)) ? G[row][k] * s : T(0);
    }
    return true;
}

// Pixel of normalised coordinates (xn, yn) under `model` in FP64
// (crates/sfm-core/src/camera.rs:204-244).
template <int M = -1>
__device__ __forceinline__ void project64(int model, const double *c, double xn, double yn, double &u, double &v) {
    if constexpr (M >= 0) model = M;
    switch (model) {
    case SFMBA_SIMPLE_PINHOLE: u = c[0] * xn + c[1]; v = c[0] * yn + c[2]; break;
    case SFMBA_PINHOLE: u = c[0] * xn + c[2]; v = c[1] * yn + c[3]; break;
    case SFMBA_SIMPLE_RADIAL: {
        const double r2 = xn * xn + yn * yn, d = 1.0 + c[3] * r2;
        u = c[0] * (xn * d) + c[1]; v = c[0] * (yn * d) + c[2];
        break;
    }
    case SFMBA_RADIAL: {
        const double r2 = xn * xn + yn * yn, d = 1.0 + c[3] * r2 + c[4] * r2 * r2;
        u = c[0] * (xn * d) + c[1]; v = c[0] * (yn * d) + c[2];
        break;
    }
    case SFMBA_OPENCV: {
        const double r2 = xn * xn + yn * yn, rad = 1.0 + c[4] * r2 + c[5] * r2 * r2;
        const double xd = xn * rad + 2.0 * c[6] * xn * yn + c[7] * (r2 + 2.0 * xn * xn);
        const double yd = yn * rad + c[6] * (r2 + 2.0 * yn * yn) + 2.0 * c[7] * xn * yn;
        u = c[0] * xd + c[2]; v = c[1] * yd + c[3];
        break;
    }
    default: {
        double r = sqrt(xn * xn + yn * yn);
        r = r > 1e-12 ? r : 1e-12;
        const double th = atan(r), t2 = th * th;
        const double thd = th * (1.0 + c[4] * t2 + c[5] * t2 * t2 + c[6] * t2 * t2 * t2 + c[7] * t2 * t2 * t2 * t2);
        const double s = thd / r;
        u = c[0] * (xn * s) + c[2]; v = c[1] * (yn * s) + c[3];
        break;
    }
    }
}

// FP64 residual as the reference's cost evaluates it: quaternion rotation
// (pose.rs:46-48) and project() (the perspective divide as one reciprocal).
__device__ __forceinline__ bool residual64(const double *pose7, int model, const double *c,
                                           double X0, double X1, double X2, double ox, double oy,
                                           double &rx, double &ry) {
    const double w = pose7[0], x = pose7[1], y = pose7[2], z = pose7[3];
    const double tx = 2.0 * (y * X2 - z * X1);
    const double ty = 2.0 * (z * X0 - x * X2);
    const double tz = 2.0 * (x * X1 - y * X0);
    const double pc0 = X0 + w * tx + (y * tz - z * ty) + pose7[4];
    const double pc1 = X1 + w * ty + (z * tx - x * tz) + pose7[5];
    const double pc2 = X2 + w * tz + (x * ty - y * tx) + pose7[6];
    if (!(pc2 > kMinDepth)) return false;
    const double iz = 1.0 / pc2;
    double u, v;
    project64(model, c, pc0 * iz, pc1 * iz, u, v);
    rx = u - ox;
    ry = v - oy;
    return true;
}

// The same residual from the pose's FP64 rotation matrix and translation
// (rt = R row-major, then t): R X + t in 9 multiply-adds instead of the
// quaternion form's ~30 operations on GB300's narrow FP64 pipe. R is the
// quaternion's exact rotation up to rounding, so the two forms agree to
// ~1e-16 relative per coordinate.
template <int M = -1>
__device__ __forceinline__ bool residual64_rt(const double *rt, int model, const double *c, double X0, double X1,
                                              double X2, double ox, double oy, double &rx, double &ry) {
    const double pc0 = rt[0] * X0 + rt[1] * X1 + rt[2] * X2 + rt[9];
    const double pc1 = rt[3] * X0 + rt[4] * X1 + rt[5] * X2 + rt[10];
    const double pc2 = rt[6] * X0 + rt[7] * X1 + rt[8] * X2 + rt[11];
    if (!(pc2 > kMinDepth)) return false;
    const double iz = 1.0 / pc2;
    double u, v;
    project64<M>(model, c, pc0 * iz, pc1 * iz, u, v);
    rx = u - ox;
    ry = v - oy;
    return true;
}

// project64 in double-float arithmetic, operation for operation, for the
// five models without a transcendental (OPENCV_FISHEYE stays in FP64).
// c: the camera's parameters as pairs.
template <int M = -1>
__device__ __forceinline__ void project_df(int model, const dfl *c, dfl xn, dfl yn, dfl &u, dfl &v) {
    if constexpr (M >= 0) model = M;
    const dfl one = df_make(1.f);
    switch (model) {
    case SFMBA_SIMPLE_PINHOLE: u = c[0] * xn + c[1]; v = c[0] * yn + c[2]; break;
    case SFMBA_PINHOLE: u = c[0] * xn + c[2]; v = c[1] * yn + c[3]; break;
    case SFMBA_SIMPLE_RADIAL: {
        const dfl r2 = xn * xn + yn * yn, d = one + c[3] * r2;
        u = c[0] * (xn * d) + c[1]; v = c[0] * (yn * d) + c[2];
        break;
    }
    case SFMBA_RADIAL: {
        const dfl r2 = xn * xn + yn * yn, d = one + c[3] * r2 + c[4] * r2 * r2;
        u = c[0] * (xn * d) + c[1]; v = c[0] * (yn * d) + c[2];
        break;
    }
    default: {  // SFMBA_OPENCV
        const dfl r2 = xn * xn + yn * yn, rad = one + c[4] * r2 + c[5] * r2 * r2;
        const dfl xy = xn * yn;
        const dfl xd = xn * rad + df_scale2(c[6], 2.f) * xy + c[7] * (r2 + df_scale2(xn * xn, 2.f));
        const dfl yd = yn * rad + c[6] * (r2 + df_scale2(yn * yn, 2.f)) + df_scale2(c[7], 2.f) * xy;
        u = c[0] * xd + c[2]; v = c[1] * yd + c[3];
        break;
    }
    }
}

// residual64_rt in double-float arithmetic: rt as 12 pairs (R row-major,
// then t), the point and the observation as pairs.
template <int M = -1>
__device__ __forceinline__ bool residual_df(const dfl *rt, int model, const dfl *c, dfl X0, dfl X1, dfl X2, dfl ox,
                                            dfl oy, dfl &rx, dfl &ry) {
    const dfl pc0 = rt[0] * X0 + rt[1] * X1 + rt[2] * X2 + rt[9];
    const dfl pc1 = rt[3] * X0 + rt[4] * X1 + rt[5] * X2 + rt[10];
    const dfl pc2 = rt[6] * X0 + rt[7] * X1 + rt[8] * X2 + rt[11];
    // pc2 > kMinDepth, decided in FP64 only near the threshold
    const bool front = pc2.hi > 2e-9f ? true : pc2.hi < 5e-10f ? false : df_to_double(pc2) > kMinDepth;
    if (!front) return false;
    const dfl iz = df_recip(pc2);
    dfl u, v;
    project_df<M>(model, c, pc0 * iz, pc1 * iz, u, v);
    rx = u - ox;
    ry = v - oy;
    return true;
}

}  // namespace sfmba
