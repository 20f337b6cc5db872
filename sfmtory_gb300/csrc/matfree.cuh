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
