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
// the pixel (RC = true): 16-32 bytes of input instead of a 128-256 byte
// record, for the cost of ~200 flops.
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
    const float2 *ob_xy32 = nullptr;         // point-major pixels, T = float
    const double2 *ob_xy64 = nullptr;        // point-major pixels, T = double
    const float2 *isort_xy32 = nullptr;      // image-major pixels, T = float
    const int *ob_img = nullptr;
    const int *ob_pt = nullptr;
    const int *img_obs = nullptr;
    int loss = 0;
    T scale = T(1);
};

// Jx~ (2x3), Jc~ (2xD) and r~ of a stored record, 16-byte vector loads.
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

template <typename T>
__device__ __forceinline__ void load_point_T(const JacSrc<T> &J, int p, T &X0, T &X1, T &X2) {
    if constexpr (std::is_same<T, float>::value) {
        const float4 v = __ldg(J.points32 + p);
        X0 = v.x; X1 = v.y; X2 = v.z;
    } else {
        X0 = J.points64[3 * (size_t)p]; X1 = J.points64[3 * (size_t)p + 1]; X2 = J.points64[3 * (size_t)p + 2];
    }
}

// Point-major observation o (image i, point p). Returns whether it is in
// front of its camera (stored path: the record of a culled observation is 0).
template <typename T, int D, bool RC>
__device__ __forceinline__ bool jac_point_major(const JacSrc<T> &J, int o, int i, int p, T rr[2], T jx[6],
                                                T jc[2 * D]) {
    if constexpr (RC) {
        const ImageLin<T> im = J.img_lin[i];
        T X0, X1, X2;
        load_point_T<T>(J, p, X0, X1, X2);
        T ox, oy;
        if constexpr (std::is_same<T, float>::value) {
            const float2 xy = __ldg(J.ob_xy32 + o);
            ox = xy.x; oy = xy.y;
        } else {
            const double2 xy = J.ob_xy64[o];
            ox = xy.x; oy = xy.y;
        }
        return linearize<T, D>(im, X0, X1, X2, ox, oy, J.loss, J.scale, rr, jx, jc);
    } else {
        load_record<T, D>(J.rec, o, rr, jx, jc);
        return true;
    }
}

// Image-major observation k (image i, point p).
template <typename T, int D, bool RC>
__device__ __forceinline__ bool jac_image_major(const JacSrc<T> &J, long long k, int i, int p, T rr[2], T jx[6],
                                                T jc[2 * D]) {
    if constexpr (RC) {
        const ImageLin<T> im = J.img_lin[i];
        T X0, X1, X2;
        load_point_T<T>(J, p, X0, X1, X2);
        T ox, oy;
        if constexpr (std::is_same<T, float>::value) {
            const float2 xy = __ldg(J.isort_xy32 + k);
            ox = xy.x; oy = xy.y;
        } else {
            const double2 xy = J.ob_xy64[J.img_obs[k]];
            ox = xy.x; oy = xy.y;
        }
        return linearize<T, D>(im, X0, X1, X2, ox, oy, J.loss, J.scale, rr, jx, jc);
    } else {
        load_record<T, D>(J.rec, J.img_obs[k], rr, jx, jc);
        return true;
    }
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
