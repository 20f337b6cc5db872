// Observation-pass building blocks of the matrix-free (PCG) path.
//
// Every pass walks the observations in fixed chunks of kChunkObs, one warp
// per chunk, one observation per lane per 32-observation round:
//   * point-major passes use chunks aligned to point starts, so a point's
//     observations never straddle chunks and per-point sums are a segmented
//     warp scan with a carry between rounds;
//   * image-major passes use plain chunks; a warp accumulates the chunk's
//     current image and writes one partial per (chunk, image), summed per
//     image by a finishing kernel.
// The Jacobian of an observation comes either from the stored record
// (RC = false) or is recomputed from the per-image constants, the point and
// the pixel (RC = true): a 16-byte packed observation record instead of a
// 128-256 byte Jacobian record, for ~150 flops. The recomputed form applies
// the Jacobian and its transpose in structured form (rotation columns
// q x d, translation d, point R^T d) without materialising it.
#pragma once

#include <type_traits>

#include "camera.cuh"
#include "kernels.cuh"

namespace sfmba {

template <typename T>
struct JacSrc {
    const T *rec = nullptr;                  // stored records (RC = false)
    const ImageLin<T> *img_lin = nullptr;    // per-image constants (RC = true)
    const float4 *points32 = nullptr;        // T = float
    const double *points64 = nullptr;        // T = double
    const int4 *obrec = nullptr;             // point-major {image, point, x, y}
    const int4 *isrec = nullptr;             // image-major {image, point, x, y}
    const int *img_obs = nullptr;            // image-major -> point-major index
    int loss = 0;
    T scale = T(1);
    // FP64 residuals of gradient terms (FP32 operators only): the point-major
    // store of residual, sqrt(weight) and validity that the cost kernel wrote
    // for the current parameters.
    const float4 *rs = nullptr;
    const unsigned char *img_live = nullptr;  // batched windows: images taking part (NULL: all)
    const float4 *mv = nullptr;  // FP32 PCG: MvOp's per-image constants in planes (Bufs::img_mv)
    int nI = 0;
};

// Jr~, Jx~ (2x3), Jc~ (2xD) of a stored record, 16-byte vector loads.
template <typename T, int D>
__device__ __forceinline__ void load_record(const T *__restrict__ rec, long long o, T rr[2], T jx[6],
                                            T jc[2 * D]) {
    constexpr int RS = RecLayout<D>::kStride;
    constexpr int NV = 8 + 2 * D;
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
    rr[0] = v[0]; rr[1] = v[1];
#pragma unroll
    for (int k = 0; k < 6; ++k) jx[k] = v[2 + k];
#pragma unroll
    for (int k = 0; k < 2 * D; ++k) jc[k] = v[8 + k];
}

// The Jacobian of one observation as an operator. Two forms with one
// interface: recomputed from the pixel, point and image constants (RC), or
// read from a stored record. Image blocks are D wide: 3 rotation, 3
// translation, then the camera's parameters.
template <typename T, int D, bool RC, int M = -1>
struct ObsOp;

template <typename T, int D, int M>
struct ObsOp<T, D, true, M> {
    static constexpr int K = LinCompact<T, D>::K;
    LinCompact<T, D> L;
    T R[9];
    bool valid;

    // Gradient terms of the FP32 path replace the FP32 residual and weight of
    // point-major observation o64 (>= 0) by the FP64 ones the cost kernel
    // stored for the current parameters (J.rs).
    __device__ __forceinline__ void build(const JacSrc<T> &J, int img, int pt, int4 rc, long long o64 = -1) {
        const ImageLin<T> im = J.img_lin[img];
        T X0, X1, X2;
        if constexpr (std::is_same<T, float>::value) {
            const float4 v = __ldg(J.points32 + pt);
            X0 = v.x; X1 = v.y; X2 = v.z;
        } else {
            X0 = J.points64[3 * (size_t)pt]; X1 = J.points64[3 * (size_t)pt + 1]; X2 = J.points64[3 * (size_t)pt + 2];
        }
        Res64 rin;
        if (o64 >= 0 && J.rs) {
            const float4 v = J.rs[o64];
            rin.use = true;
            rin.r0 = v.x; rin.r1 = v.y; rin.s = v.z; rin.ok = v.w != 0.f;
        }
        valid = linearize_compact<T, D, M>(im, X0, X1, X2, (T)__int_as_float(rc.z), (T)__int_as_float(rc.w), J.loss,
                                        J.scale, L, rin);
#pragma unroll
        for (int k = 0; k < 9; ++k) R[k] = im.R[k];
    }
    __device__ __forceinline__ T r(int row) const { return L.r[row]; }
    // (s0, s1) = Jc~ v for an image-block vector v.
    __device__ __forceinline__ void jc_dot(const T *v, T &s0, T &s1) const {
        T w0 = T(0), w1 = T(0), w2 = T(0);
        if (L.pose_on) {  // omega x q + dt
            w0 = v[1] * L.q[2] - v[2] * L.q[1] + v[3];
            w1 = v[2] * L.q[0] - v[0] * L.q[2] + v[4];
            w2 = v[0] * L.q[1] - v[1] * L.q[0] + v[5];
        }
        s0 = L.d[0][0] * w0 + L.d[0][1] * w1 + L.d[0][2] * w2;
        s1 = L.d[1][0] * w0 + L.d[1][1] * w1 + L.d[1][2] * w2;
        if constexpr (D > 6) {
#pragma unroll
            for (int k = 0; k < K; ++k) {
                s0 += L.g[0][k] * v[6 + k];
                s1 += L.g[1][k] * v[6 + k];
            }
        }
    }
    // out = Jx~^T (a0, a1) = R^T (a0 d0 + a1 d1)
    __device__ __forceinline__ void jx_t(T a0, T a1, T out[3]) const {
        const T e0 = a0 * L.d[0][0] + a1 * L.d[1][0];
        const T e1 = a0 * L.d[0][1] + a1 * L.d[1][1];
        const T e2 = a0 * L.d[0][2] + a1 * L.d[1][2];
        out[0] = R[0] * e0 + R[3] * e1 + R[6] * e2;
        out[1] = R[1] * e0 + R[4] * e1 + R[7] * e2;
        out[2] = R[2] * e0 + R[5] * e1 + R[8] * e2;
    }
    // (z0, z1) = Jx~ u = d_row . (R u)
    __device__ __forceinline__ void jx(T u0, T u1, T u2, T &z0, T &z1) const {
        const T a = R[0] * u0 + R[1] * u1 + R[2] * u2;
        const T b = R[3] * u0 + R[4] * u1 + R[5] * u2;
        const T c = R[6] * u0 + R[7] * u1 + R[8] * u2;
        z0 = L.d[0][0] * a + L.d[0][1] * b + L.d[0][2] * c;
        z1 = L.d[1][0] * a + L.d[1][1] * b + L.d[1][2] * c;
    }
    // out = Jc~^T (z0, z1) = [q x e, e, z0 g0 + z1 g1], e = z0 d0 + z1 d1
    __device__ __forceinline__ void jc_t(T z0, T z1, T out[D]) const {
        const T e0 = z0 * L.d[0][0] + z1 * L.d[1][0];
        const T e1 = z0 * L.d[0][1] + z1 * L.d[1][1];
        const T e2 = z0 * L.d[0][2] + z1 * L.d[1][2];
        const T on = L.pose_on ? T(1) : T(0);
        out[0] = on * (L.q[1] * e2 - L.q[2] * e1);
        out[1] = on * (L.q[2] * e0 - L.q[0] * e2);
        out[2] = on * (L.q[0] * e1 - L.q[1] * e0);
        out[3] = on * e0;
        out[4] = on * e1;
        out[5] = on * e2;
#pragma unroll
        for (int k = 0; k < D - 6; ++k) out[6 + k] = z0 * L.g[0][k] + z1 * L.g[1][k];
    }
    __device__ __forceinline__ void jx_rows(T jx[6]) const {
        jx_t(T(1), T(0), jx);
        jx_t(T(0), T(1), jx + 3);
    }
    __device__ __forceinline__ void jc_rows(T jc[2 * D]) const {
        jc_t(T(1), T(0), jc);
        jc_t(T(0), T(1), jc + D);
    }
};

template <typename T, int D, int M>
struct ObsOp<T, D, false, M> {
    T rr[2], jxm[6], jcm[2 * D];
    bool valid;

    __device__ __forceinline__ void build_record(const T *rec, long long o) {
        load_record<T, D>(rec, o, rr, jxm, jcm);
        valid = true;
    }
    __device__ __forceinline__ T r(int row) const { return rr[row]; }
    __device__ __forceinline__ void jc_dot(const T *v, T &s0, T &s1) const {
        s0 = T(0);
        s1 = T(0);
#pragma unroll
        for (int c = 0; c < D; ++c) {
            s0 += jcm[c] * v[c];
            s1 += jcm[D + c] * v[c];
        }
    }
    __device__ __forceinline__ void jx_t(T a0, T a1, T out[3]) const {
#pragma unroll
        for (int c = 0; c < 3; ++c) out[c] = a0 * jxm[c] + a1 * jxm[3 + c];
    }
    __device__ __forceinline__ void jx(T u0, T u1, T u2, T &z0, T &z1) const {
        z0 = jxm[0] * u0 + jxm[1] * u1 + jxm[2] * u2;
        z1 = jxm[3] * u0 + jxm[4] * u1 + jxm[5] * u2;
    }
    __device__ __forceinline__ void jc_t(T z0, T z1, T out[D]) const {
#pragma unroll
        for (int c = 0; c < D; ++c) out[c] = z0 * jcm[c] + z1 * jcm[D + c];
    }
    __device__ __forceinline__ void jx_rows(T jx[6]) const {
#pragma unroll
        for (int c = 0; c < 6; ++c) jx[c] = jxm[c];
    }
    __device__ __forceinline__ void jc_rows(T jc[2 * D]) const {
#pragma unroll
        for (int c = 0; c < 2 * D; ++c) jc[c] = jcm[c];
    }
};

// The Jacobian of one observation as the PCG passes apply it, recomputed in
// FP32 for a camera model known at compile time (SIMPLE_PINHOLE, PINHOLE,
// SIMPLE_RADIAL, RADIAL): instead of forming the 2 x 2 pixel derivative A,
// the 2 x k parameter columns G and the compact rows d = s A Pn, it keeps
// the normalised point (xp, yp), 1/z, q = R X and the model's scalars and
// applies each factor in closed form. With Pn = [[1, 0, -xp], [0, 1, -yp]]/z:
//   pose and point:  J v = s A Pn (omega x q + dt + R dX),
//   transposes:      e = Pn^T A^T (s a); pose = [q x e, e], point = R^T e,
//   camera:          J p_cam = s G p_cam, J^T a = s G^T a.
// For the radial models A = f (d I + 2 d' x x^T) with x = (xp, yp) is
// symmetric, so A and A^T are one formula. The same values as ObsOp in
// exact arithmetic (about half the FP32 instructions); columns that are not
// unknowns need no mask here because the PCG vectors are zero on them and
// the image pass's sums for them are discarded by k_pcg_images_finish. The
// per-image constants come from planes of float4 (Bufs::img_mv: R and t in
// three, the model's scalars {f, fy, k1, k2} in the fourth, {cx, cy} in a
// fifth read only for a robust loss), so neighbouring images share cache
// lines.
template <int M>
__host__ __device__ constexpr bool mv_model() {
    return M == SFMBA_SIMPLE_PINHOLE || M == SFMBA_PINHOLE || M == SFMBA_SIMPLE_RADIAL || M == SFMBA_RADIAL;
}

template <int D, int M>
struct MvOp {
    static_assert(model_fits_width(M, D), "MvOp covers exactly the model's columns");
    float R[9];
    float q0, q1, q2;
    float xp, yp, iz, s;
    float f, fy, d, dd2, r2;  // model scalars: fx (f), fy, radial factor d, 2 d(d)/d(r2), r^2

    __device__ __forceinline__ void build(const JacSrc<float> &J, int img, int pt, int4 rc) {
        const float4 *mv = J.mv + img;
        const size_t nI = (size_t)J.nI;
        const float4 m0 = __ldg(mv), m1 = __ldg(mv + nI), m2 = __ldg(mv + 2 * nI), ms = __ldg(mv + 3 * nI);
        const float4 X = __ldg(J.points32 + pt);
        build_from(J, img, m0, m1, m2, ms, X, rc);
    }
    // From the image's constants (R, t, {f, fy, k1, k2}) and the point, wherever they were loaded.
    __device__ __forceinline__ void build_from(const JacSrc<float> &J, int img, float4 m0, float4 m1, float4 m2,
                                               float4 ms, float4 X, int4 rc) {
        R[0] = m0.x; R[1] = m0.y; R[2] = m0.z; R[3] = m0.w;
        R[4] = m1.x; R[5] = m1.y; R[6] = m1.z; R[7] = m1.w;
        R[8] = m2.x;
        q0 = R[0] * X.x + R[1] * X.y + R[2] * X.z;
        q1 = R[3] * X.x + R[4] * X.y + R[5] * X.z;
        q2 = R[6] * X.x + R[7] * X.y + R[8] * X.z;
        const float pc0 = q0 + m2.y, pc1 = q1 + m2.z, pc2 = q2 + m2.w;
        const bool ok = pc2 > float(kMinDepth);
        iz = ok ? __fdividef(1.0f, pc2) : 0.0f;  // approximate reciprocal (FP32 Jacobian operator)
        xp = pc0 * iz;
        yp = pc1 * iz;
        f = ms.x;
        fy = ms.y;
        d = 1.0f;
        dd2 = 0.0f;
        r2 = xp * xp + yp * yp;
        if constexpr (M == SFMBA_SIMPLE_RADIAL) {
            d = 1.0f + ms.z * r2;
            dd2 = 2.0f * ms.z;
        } else if constexpr (M == SFMBA_RADIAL) {
            d = 1.0f + r2 * (ms.z + ms.w * r2);
            dd2 = 2.0f * (ms.z + 2.0f * ms.w * r2);
        }
        s = ok ? 1.0f : 0.0f;
        if (ok && J.loss != SFMBA_LOSS_NONE) {  // sqrt of the robust weight of the FP32 residual
            const float4 cc = __ldg(J.mv + 4 * (size_t)J.nI + img);  // cx, cy
            const float r0 = f * xp * d + cc.x - __int_as_float(rc.z);
            const float r1 = fy * yp * d + cc.y - __int_as_float(rc.w);
            s = sqrtf(robust_weight<float>(sqrtf(r0 * r0 + r1 * r1), J.loss, J.scale));
        }
    }
    // (a0, a1) = A (x, y)
    __device__ __forceinline__ void apply_A(float x, float y, float &a0, float &a1) const {
        if constexpr (M == SFMBA_SIMPLE_RADIAL || M == SFMBA_RADIAL) {
            const float t = dd2 * (xp * x + yp * y);
            a0 = f * (d * x + xp * t);
            a1 = f * (d * y + yp * t);
        } else {
            a0 = f * x;
            a1 = fy * y;
        }
    }
    // (s0, s1) = J~ v for an image-block vector v (pose, then camera columns).
    __device__ __forceinline__ void jc_dot(const float *v, float &s0, float &s1) const {
        const float w0 = v[1] * q2 - v[2] * q1 + v[3];
        const float w1 = v[2] * q0 - v[0] * q2 + v[4];
        const float w2 = v[0] * q1 - v[1] * q0 + v[5];
        float a0, a1;
        apply_A((w0 - xp * w2) * iz, (w1 - yp * w2) * iz, a0, a1);
        if constexpr (M == SFMBA_SIMPLE_PINHOLE) {
            a0 += xp * v[6] + v[7];
            a1 += yp * v[6] + v[8];
        } else if constexpr (M == SFMBA_PINHOLE) {
            a0 += xp * v[6] + v[8];
            a1 += yp * v[7] + v[9];
        } else {
            float k = d * v[6] + f * r2 * v[9];
            if constexpr (M == SFMBA_RADIAL) k += f * r2 * r2 * v[10];
            a0 += xp * k + v[7];
            a1 += yp * k + v[8];
        }
        s0 = s * a0;
        s1 = s * a1;
    }
    // e = Pn^T A^T (s a)
    __device__ __forceinline__ void pull(float a0, float a1, float &e0, float &e1, float &e2) const {
        float b0, b1;
        apply_A(s * a0, s * a1, b0, b1);  // A symmetric (radial) or diagonal (pinhole)
        e0 = b0 * iz;
        e1 = b1 * iz;
        e2 = -(xp * b0 + yp * b1) * iz;
    }
    // out = Jx~^T (a0, a1) = R^T e
    __device__ __forceinline__ void jx_t(float a0, float a1, float out[3]) const {
        float e0, e1, e2;
        pull(a0, a1, e0, e1, e2);
        out[0] = R[0] * e0 + R[3] * e1 + R[6] * e2;
        out[1] = R[1] * e0 + R[4] * e1 + R[7] * e2;
        out[2] = R[2] * e0 + R[5] * e1 + R[8] * e2;
    }
    // (z0, z1) = Jx~ u = s A Pn R u
    __device__ __forceinline__ void jx(float u0, float u1, float u2, float &z0, float &z1) const {
        const float a = R[0] * u0 + R[1] * u1 + R[2] * u2;
        const float b = R[3] * u0 + R[4] * u1 + R[5] * u2;
        const float c = R[6] * u0 + R[7] * u1 + R[8] * u2;
        float a0, a1;
        apply_A((a - xp * c) * iz, (b - yp * c) * iz, a0, a1);
        z0 = s * a0;
        z1 = s * a1;
    }
    // out = Jc~^T (z0, z1) = [q x e, e, s G^T z]
    __device__ __forceinline__ void jc_t(float z0, float z1, float out[D]) const {
        float e0, e1, e2;
        pull(z0, z1, e0, e1, e2);
        out[0] = q1 * e2 - q2 * e1;
        out[1] = q2 * e0 - q0 * e2;
        out[2] = q0 * e1 - q1 * e0;
        out[3] = e0;
        out[4] = e1;
        out[5] = e2;
        const float g0 = s * z0, g1 = s * z1;
        if constexpr (M == SFMBA_SIMPLE_PINHOLE) {
            out[6] = xp * g0 + yp * g1;
            out[7] = g0;
            out[8] = g1;
        } else if constexpr (M == SFMBA_PINHOLE) {
            out[6] = xp * g0;
            out[7] = yp * g1;
            out[8] = g0;
            out[9] = g1;
        } else {
            const float t = xp * g0 + yp * g1;
            out[6] = d * t;
            out[7] = g0;
            out[8] = g1;
            out[9] = f * r2 * t;
            if constexpr (M == SFMBA_RADIAL) out[10] = f * r2 * r2 * t;
        }
    }
};

// Operator of point-major observation o with packed record rc. With
// `gradient` the recomputed form takes its residual and weight from the
// FP64 parameters (see Res64).
template <typename T, int D, bool RC, int M>
__device__ __forceinline__ void make_op_point_major(const JacSrc<T> &J, int o, int4 rc, ObsOp<T, D, RC, M> &op,
                                                    bool gradient = false) {
    if constexpr (RC) op.build(J, rc.x, rc.y, rc, gradient ? (long long)o : -1LL);
    else op.build_record(J.rec, o);
}

// Operator of image-major observation k with packed record rc.
template <typename T, int D, bool RC, int M>
__device__ __forceinline__ void make_op_image_major(const JacSrc<T> &J, long long k, int4 rc, ObsOp<T, D, RC, M> &op,
                                                    bool gradient = false) {
    if constexpr (RC) op.build(J, rc.x, rc.y, rc, gradient ? (long long)J.img_obs[k] : -1LL);
    else op.build_record(J.rec, J.img_obs[k]);
}

template <typename T>
__device__ __forceinline__ T shfl_up(T v, int off) {
    return __shfl_up_sync(0xffffffffu, v, off);
}

// Slot of the partial of (chunk, image) in the image-major passes.
__device__ __forceinline__ int partial_slot(const int *ipart_off, const int *img_start, int img,
                                            long long chunk) {
    return ipart_off[img] + (int)(chunk - img_start[img] / kChunkObs);
}

}  // namespace sfmba
