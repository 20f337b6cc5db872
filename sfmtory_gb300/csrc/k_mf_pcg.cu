// Launchers of the two observation passes of every PCG iteration (point
// pass u = C^-1 E^T p, image pass E u), in the launch-shape variants the
// autotuner picks from; the point pass's last variant streams its records
// by bulk copies (mf_tma.cuh).
#include "mf_tma.cuh"

namespace sfmba {

namespace {

// The record-streaming point pass where it applies (FP32 recomputed operator
// of a camera model MvOp serves); false otherwise.
bool mf_points_tma(const Bufs &b, cudaStream_t s) {
    if (!b.mixed || !b.pcg_p4 || !b.points32 || !b.img_mv) return false;
    bool ran = false;
    dispatch_TDR(b, [&](auto t, auto dc, auto rc, auto mc) {
        using T = decltype(t);
        constexpr int D = decltype(dc)::value;
        constexpr int M = decltype(mc)::value;
        if constexpr (std::is_same<T, float>::value && decltype(rc)::value && mv_model<M>() && pad4(D) <= 12) {
            k_mf_points_tma<D, M><<<div_up(b.npchunks, kTmaWarps), 32 * kTmaWarps, 0, s>>>(
                jac_src<float>(b), b.pchunk, b.npchunks, (const float *)b.pt_Cinv, b.pt_ok, b.pcg_p4, b.state,
                (float *)b.pcg_u);
            SFMBA_LAUNCH_CHECK();
            ran = true;
        }
    });
    return ran;
}

}  // namespace

template <int V>
void mf_points_v(const Bufs &b, cudaStream_t s) {
    dispatch_TDR(b, [&](auto t, auto dc, auto rc, auto mc) {
        using T = decltype(t);
        constexpr int D = decltype(dc)::value;
        constexpr int VV = std::is_same<T, float>::value ? V : 0;  // FP64: one variant
        k_mf_points<T, D, decltype(rc)::value, VV, decltype(mc)::value><<<warps_grid(b.npchunks, 256), 256, 0, s>>>(
            jac_src<T>(b), b.pchunk, b.npchunks, (const T *)b.pt_Cinv, b.pt_ok, (const T *)b.pcg_p,
            std::is_same<T, float>::value ? (const T *)(const void *)b.pcg_p4 : nullptr, b.state, (T *)b.pcg_u);
    });
    SFMBA_LAUNCH_CHECK();
}

template <int V>
void mf_images_v(const Bufs &b, cudaStream_t s) {
    dispatch_TDR(b, [&](auto t, auto dc, auto rc, auto mc) {
        using T = decltype(t);
        constexpr int D = decltype(dc)::value;
        constexpr int VV = std::is_same<T, float>::value ? V : 0;
        const long long chunks = (b.nO + kChunkObs - 1) / kChunkObs;
        k_mf_images<T, D, decltype(rc)::value, VV, decltype(mc)::value><<<warps_grid(chunks, 256), 256, 0, s>>>(
            jac_src<T>(b), b.nO, b.img_start, b.ipart_off, (const T *)b.pcg_u, b.state, (T *)b.ipart);
    });
    SFMBA_LAUNCH_CHECK();
}

void launch_mf_points(const Bufs &b, cudaStream_t s, int variant) {
    if (b.npchunks == 0) return;
    switch (variant) {
    case 0: mf_points_v<0>(b, s); break;
    case 1: mf_points_v<1>(b, s); break;
    case 2: mf_points_v<2>(b, s); break;
    case 3: mf_points_v<3>(b, s); break;
    case 4: mf_points_v<4>(b, s); break;
    case 5: mf_points_v<5>(b, s); break;
    case 6: mf_points_v<6>(b, s); break;
    case 7: mf_points_v<7>(b, s); break;
    case 8: mf_points_v<8>(b, s); break;
    case 9: mf_points_v<9>(b, s); break;
    default:  // records by bulk copy, where it applies; else the same sums by variant 8
        if (!mf_points_tma(b, s)) mf_points_v<8>(b, s);
        break;
    }
}

void launch_mf_images(const Bufs &b, cudaStream_t s, int variant) {
    if (b.nO == 0) return;
    switch (variant) {
    case 0: mf_images_v<0>(b, s); break;
    case 1: mf_images_v<1>(b, s); break;
    case 2: mf_images_v<2>(b, s); break;
    case 3: mf_images_v<3>(b, s); break;
    case 4: mf_images_v<4>(b, s); break;
    case 5: mf_images_v<5>(b, s); break;
    case 6: mf_images_v<6>(b, s); break;
    case 7: mf_images_v<7>(b, s); break;
    case 8: mf_images_v<8>(b, s); break;
    default: mf_images_v<9>(b, s); break;
    }
}

}  // namespace sfmba
