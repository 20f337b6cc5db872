// Schur reduction of one image pair (i, j) by one warp:
//   S_ij = [i == j] H_i - sum_{points p seen by i and j} Jc~_a^T M_ab Jc~_b,
//   M_ab = Jx~_a C_p^-1 Jx~_b^T (2x2),
// over the pair list grouped by image pair (visibility-sorted order), so
// each block is produced by one warp and no global atomics are used
// (reference: crates/sfm-ba/src/lib.rs:114-211, :981-1043).
//
// Per round of 32 pairs, lane t stages pair t: A_t = Jc~_a (2xD) and
// P_t = M_ab Jc~_b (2xD). S_ij -= sum_t sum_rho A_t[rho]^T P_t[rho] is then a
// D x D product with inner dimension 2 x 32, register-tiled: the warp is SG
// subgroups of 32/SG lanes, subgroup g takes pairs t = g (mod SG), and its
// lanes form a (8/SG) x 4 grid over the output, each owning a
// ceil(D SG/8) x ceil(D/4) tile. Each round's partial sums are added into
// the running sums with Kahan compensation (for FP32), and the subgroups'
// sums are combined in FP64 at the end. Fewer subgroups mean smaller tiles
// (fewer registers per lane, more warps resident) for more shared-memory
// reads per multiply-add.
#pragma once

#include <type_traits>

#include "common.cuh"

namespace sfmba {

template <typename T, int D, int SG = 4>
struct SchurTile {
    static_assert(SG == 1 || SG == 2 || SG == 4, "subgroups of 32, 16 or 8 lanes");
    static constexpr int LS = 32 / SG;                   // lanes per subgroup
    static constexpr int GR = LS / 4;                    // rows of the subgroup's lane grid
    static constexpr int RH = (D + GR - 1) / GR;         // output rows per lane
    static constexpr int CQ = (D + 3) / 4;               // output columns per lane
    static constexpr int LDS = 2 * D + 1;                // staged row length (odd: fewer bank conflicts)
};

template <typename T>
__device__ __forceinline__ void kahan_add_t(T &s, T &c, T x) {
    if constexpr (std::is_same<T, float>::value) {
        const T y = x - c;
        const T t = s + y;
        c = (t - s) - y;
        s = t;
    } else {
        s += x;
    }
}

// Jc~ part (2D values from offset 8) of stored record r, vector loads.
template <typename T, int D>
__device__ __forceinline__ void load_jc_part(const T *__restrict__ r, T jc[2 * D]) {
    constexpr int NJ = 2 * D;
    if constexpr (std::is_same<T, float>::value) {
        constexpr int NV = (NJ + 3) / 4;
        const float4 *q = reinterpret_cast<const float4 *>(r + 8);
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            const float4 v = __ldg(q + k);
            if (4 * k + 0 < NJ) jc[4 * k + 0] = v.x;
            if (4 * k + 1 < NJ) jc[4 * k + 1] = v.y;
            if (4 * k + 2 < NJ) jc[4 * k + 2] = v.z;
            if (4 * k + 3 < NJ) jc[4 * k + 3] = v.w;
        }
    } else {
        constexpr int NV = (NJ + 1) / 2;
        const double2 *q = reinterpret_cast<const double2 *>(r + 8);
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            const double2 v = __ldg(q + k);
            if (2 * k + 0 < NJ) jc[2 * k + 0] = v.x;
            if (2 * k + 1 < NJ) jc[2 * k + 1] = v.y;
        }
    }
}

// Accumulates the Schur term of pairs [gs, ge) and returns, in lanes
// 0..LS-1, the lane's output tile in FP64: out[a][b] = -sum (rows r0+a,
// cols c0+b) with r0 = (lane >> 2) * RH, c0 = (lane & 3) * CQ. sA, sP: this
// warp's staging rows [32][LDS].
template <typename T, int D, int SG = 4>
__device__ __forceinline__ void schur_group(const T *__restrict__ rec, const int2 *__restrict__ pairs, int gs,
                                            int ge, const int *__restrict__ ob_pt, const T *__restrict__ pt_Cinv,
                                            const unsigned char *__restrict__ pt_ok,
                                            T (*sA)[SchurTile<T, D, SG>::LDS], T (*sP)[SchurTile<T, D, SG>::LDS],
                                            int lane,
                                            double out[SchurTile<T, D, SG>::RH][SchurTile<T, D, SG>::CQ]) {
    constexpr int RS = RecLayout<D>::kStride;
    using Tile = SchurTile<T, D, SG>;
    constexpr int RH = Tile::RH, CQ = Tile::CQ, LS = Tile::LS;
    const int sg = lane / LS, ll = lane % LS;
    const int r0 = (ll >> 2) * RH, c0 = (ll & 3) * CQ;
    T acc[RH][CQ], comp[RH][CQ];
#pragma unroll
    for (int a = 0; a < RH; ++a)
#pragma unroll
        for (int b = 0; b < CQ; ++b) acc[a][b] = comp[a][b] = T(0);
    for (int base = gs; base < ge; base += 32) {
        const int e = base + lane;
        bool staged = false;
        if (e < ge) {
            const int2 ab = pairs[e];
            const int p = ob_pt[ab.x];
            if (pt_ok[p]) {
                const T *ra = rec + (size_t)ab.x * RS;
                const T *rb = rec + (size_t)ab.y * RS;
                const T *Ci = pt_Cinv + 6 * (size_t)p;
                const T c00 = Ci[0], c01 = Ci[1], c02 = Ci[2], c11 = Ci[3], c12 = Ci[4], c22 = Ci[5];
                T U[2][3];
#pragma unroll
                for (int r = 0; r < 2; ++r) {
                    const T x0 = ra[2 + 3 * r], x1 = ra[3 + 3 * r], x2 = ra[4 + 3 * r];
                    U[r][0] = x0 * c00 + x1 * c01 + x2 * c02;
                    U[r][1] = x0 * c01 + x1 * c11 + x2 * c12;
                    U[r][2] = x0 * c02 + x1 * c12 + x2 * c22;
                }
                T M[2][2];
#pragma unroll
                for (int r = 0; r < 2; ++r)
#pragma unroll
                    for (int q = 0; q < 2; ++q)
                        M[r][q] = U[r][0] * rb[2 + 3 * q] + U[r][1] * rb[3 + 3 * q] + U[r][2] * rb[4 + 3 * q];
                T jc[2 * D];
                load_jc_part<T, D>(rb, jc);
#pragma unroll
                for (int c = 0; c < D; ++c) {
                    sP[lane][c] = M[0][0] * jc[c] + M[0][1] * jc[D + c];
                    sP[lane][D + c] = M[1][0] * jc[c] + M[1][1] * jc[D + c];
                }
                load_jc_part<T, D>(ra, jc);
#pragma unroll
                for (int f = 0; f < 2 * D; ++f) sA[lane][f] = jc[f];
                staged = true;
            }
        }
        if (!staged) {
#pragma unroll
            for (int f = 0; f < 2 * D; ++f) sA[lane][f] = sP[lane][f] = T(0);
        }
        __syncwarp();
        T part[RH][CQ];
#pragma unroll
        for (int a = 0; a < RH; ++a)
#pragma unroll
            for (int b = 0; b < CQ; ++b) part[a][b] = T(0);
#pragma unroll 2
        for (int k = 0; k < 32 / SG; ++k) {
            const int t = sg + SG * k;
#pragma unroll
            for (int rho = 0; rho < 2; ++rho) {
                T av[RH], pv[CQ];
#pragma unroll
                for (int a = 0; a < RH; ++a) av[a] = (r0 + a < D) ? sA[t][rho * D + r0 + a] : T(0);
#pragma unroll
                for (int b = 0; b < CQ; ++b) pv[b] = (c0 + b < D) ? sP[t][rho * D + c0 + b] : T(0);
#pragma unroll
                for (int a = 0; a < RH; ++a)
#pragma unroll
                    for (int b = 0; b < CQ; ++b) part[a][b] += av[a] * pv[b];
            }
        }
#pragma unroll
        for (int a = 0; a < RH; ++a)
#pragma unroll
            for (int b = 0; b < CQ; ++b) kahan_add_t(acc[a][b], comp[a][b], part[a][b]);
        __syncwarp();
    }
#pragma unroll
    for (int a = 0; a < RH; ++a)
#pragma unroll
        for (int b = 0; b < CQ; ++b) {
            double v = (double)acc[a][b] - (double)comp[a][b];
#pragma unroll
            for (int off = LS; off < 32; off <<= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
            out[a][b] = -v;
        }
}

}  // namespace sfmba
