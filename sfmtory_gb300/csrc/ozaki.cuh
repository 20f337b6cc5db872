// FP64 trailing update of the blocked Cholesky on the BF16 tensor cores, by
// error-free splitting (Ozaki, Ogita, Oishi & Rump, "Error-free
// transformations of matrix multiplication by using fast routines of matrix
// multiplication and its applications", Numer. Algorithms 59, 2012).
//
// The update is A[I, J] -= P_I P_J^T with P the 64-column panel below the
// diagonal block. Each panel row r is scaled by 2^-e_r (e_r: the binary
// exponent of its largest entry, so |x| < 1) and cut into kOzSlices slices
// of 8 bits:
//   P[r, t] = 2^e_r sum_{i=1..7} s_i[r, t] 2^-8i,  s_i integer, |s_i| <= 255
// (exact to 56 bits >= 53). An integer of at most 8 significant bits is a
// BF16 value and a product of two is below 2^16, so a 64-term dot product
// of slices is an integer below 2^22 that the tensor cores' FP32
// accumulation holds exactly. The update is
//   (P P^T)[r, c] = 2^(e_r + e_c) sum_{i,j} 2^-8(i+j) G_ij[r, c],
//   G_ij = S_i[R] S_j[C]^T,
// of which the 28 terms with i + j <= 8 are kept (the others lie below
// 2^-64 of the scale). Products of one weight d = i + j share an FP32
// accumulator G_d (exact for d <= 5: at most four products, < 2^24; the
// five of d = 6 may round by a unit, 2^-52 of the scale). The groups
// d <= 6 are combined exactly in 64-bit integers,
//   L = 2^32 G_2 + 2^24 G_3 + 2^16 G_4 + 2^8 G_5 + G_6   (< 2^55),
// the last two in FP32, T = G_7 + G_8 / 2^8 (rounding below 2^-80 of the
// scale), and
//   (P P^T)[r, c] = 2^(e_r + e_c - 48) (L + T / 2^8)
// is formed in FP64 (L rounds to 53 bits: the FP64 rounding of the product
// itself) and subtracted: five FP64 operations per entry and panel instead
// of 64 fused multiply-adds.
//
// The products run as warp-level mma.sync m16n8k16 (BF16 in, FP32
// accumulate) from shared memory through ldmatrix; a 4-warp block owns a
// 64 x 64 output tile, each warp 32 x 32.
#pragma once

#include <cuda_bf16.h>

#include "common.cuh"

namespace sfmba {

constexpr int kOzSlices = 7;
constexpr int kOzK = 64;     // panel width (the Cholesky block)
constexpr int kOzLds = 72;   // shared row stride in BF16 (144 bytes: the 8 rows of an ldmatrix on distinct banks)
constexpr int kOzTile = 64;  // output tile
constexpr size_t kOzSmem = (size_t)2 * kOzSlices * kOzTile * kOzLds * sizeof(__nv_bfloat16);

// Slices and exponent of one panel row of nb <= 64 entries (one warp; lane
// owns columns lane and lane + 32; missing columns are zero).
// out + i * slice_stride: slice i of the row, 64 BF16 values.
__device__ __forceinline__ void oz_split_row(const double *__restrict__ row, int nb, int lane,
                                             __nv_bfloat16 *__restrict__ out, size_t slice_stride, int *e_out) {
    const double v0 = lane < nb ? row[lane] : 0.0;
    const double v1 = lane + 32 < nb ? row[lane + 32] : 0.0;
    double m = fmax(fabs(v0), fabs(v1));
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, off));
    int e = 0;
    if (m > 0.0) frexp(m, &e);  // m = f 2^e, f in [0.5, 1): |v| 2^-e < 1
    double x0 = ldexp(v0, -e), x1 = ldexp(v1, -e);
#pragma unroll
    for (int i = 0; i < kOzSlices; ++i) {
        const double y0 = x0 * 256.0, y1 = x1 * 256.0;  // exact (power of two)
        const double s0 = trunc(y0), s1 = trunc(y1);    // |s| <= 255
        x0 = y0 - s0;                                   // exact (the fraction)
        x1 = y1 - s1;
        out[(size_t)i * slice_stride + lane] = __float2bfloat16_rn((float)s0);
        out[(size_t)i * slice_stride + lane + 32] = __float2bfloat16_rn((float)s1);
    }
    if (lane == 0) *e_out = e;
}

__device__ __forceinline__ void oz_ldmatrix_x4(const __nv_bfloat16 *p, unsigned (&r)[4]) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}

__device__ __forceinline__ void oz_mma(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
        "{%0, %1, %2, %3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// acc += S_i[warp rows] S_j[warp cols]^T over the 64 panel columns.
// sR, sC: [kOzSlices][64][kOzLds] slices of the tile's rows and columns.
// The warp (wr, wc) covers rows 32 wr.. and columns 32 wc..: two m16 blocks
// times four n8 blocks; acc[m][nn][e] holds row 16 m + lane/4 + 8 (e/2),
// column 8 nn + 2 (lane%4) + e%2 of it (the mma accumulator layout).
__device__ __forceinline__ void oz_product(const __nv_bfloat16 *sR, const __nv_bfloat16 *sC, int i, int j, int wr,
                                           int wc, int lane, float (&acc)[2][4][4]) {
    const __nv_bfloat16 *A = sR + ((size_t)i * kOzTile + wr * 32) * kOzLds;
    const __nv_bfloat16 *B = sC + ((size_t)j * kOzTile + wc * 32) * kOzLds;
#pragma unroll
    for (int kk = 0; kk < kOzK; kk += 16) {
        unsigned a[2][4], b[2][4];
        // A fragments: lanes 0-15 give rows 0-15 at k, lanes 16-31 the same rows at k + 8.
#pragma unroll
        for (int m = 0; m < 2; ++m)
            oz_ldmatrix_x4(A + (size_t)(m * 16 + (lane & 15)) * kOzLds + kk + 8 * (lane >> 4), a[m]);
        // B fragments of two n8 blocks: matrices (n 0-7, k), (n 0-7, k+8), (n 8-15, k), (n 8-15, k+8).
#pragma unroll
        for (int h = 0; h < 2; ++h)
            oz_ldmatrix_x4(B + (size_t)(h * 16 + (lane & 7) + 8 * (lane >> 4)) * kOzLds + kk + 8 * ((lane >> 3) & 1),
                           b[h]);
#pragma unroll
        for (int m = 0; m < 2; ++m)
#pragma unroll
            for (int nn = 0; nn < 4; ++nn)
                oz_mma(acc[m][nn], a[m], b[nn >> 1][2 * (nn & 1)], b[nn >> 1][2 * (nn & 1) + 1]);
    }
}

// One 64 x 64 tile of the update, A[r, c] -= (P P^T)[r, c] for r < mi,
// c < mj (c <= r on a diagonal tile), by a 128-thread block. A: the tile's
// first entry, row stride lda. slR / slC: slice 0 of the tile's first row /
// column (64 BF16 per row, slice i at + i * slice_stride). eR / eC: the
// exponents of those rows. smem: kOzSmem bytes of dynamic shared memory;
// fR, fC: [64] shared.
__device__ __forceinline__ void oz_tile_update(double *A, size_t lda, int mi, int mj, bool diag,
                                               const __nv_bfloat16 *slR, const __nv_bfloat16 *slC,
                                               size_t slice_stride, const int *eR, const int *eC,
                                               unsigned char *smem, double *fR, double *fC) {
    __nv_bfloat16 *sR = reinterpret_cast<__nv_bfloat16 *>(smem);
    __nv_bfloat16 *sC = sR + (size_t)kOzSlices * kOzTile * kOzLds;
    auto load = [&](__nv_bfloat16 *dst, const __nv_bfloat16 *src, int rows) {  // 16-byte pieces, missing rows zero
        for (int e = threadIdx.x; e < kOzSlices * kOzTile * 8; e += blockDim.x) {
            const int i = e / (kOzTile * 8), rr = (e / 8) % kOzTile, ch = e % 8;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (rr < rows) v = *reinterpret_cast<const uint4 *>(src + (size_t)i * slice_stride + (size_t)rr * kOzK + ch * 8);
            *reinterpret_cast<uint4 *>(dst + ((size_t)i * kOzTile + rr) * kOzLds + ch * 8) = v;
        }
    };
    load(sR, slR, mi);
    if (!diag) load(sC, slC, mj);
    const __nv_bfloat16 *cs = diag ? sR : sC;
    if (threadIdx.x < kOzTile) {
        fR[threadIdx.x] = (int)threadIdx.x < mi ? ldexp(1.0, eR[threadIdx.x] - 48) : 0.0;
    } else if (threadIdx.x < 2 * kOzTile) {
        const int c = threadIdx.x - kOzTile;
        fC[c] = c < mj ? ldexp(1.0, eC[c]) : 0.0;
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wr = warp >> 1, wc = warp & 1;
    float T[2][4][4], acc[2][4][4];
    long long I[2][4][4];
    for (int d = 2; d <= 8; ++d) {  // weight 2^-8d; the largest first
#pragma unroll
        for (int m = 0; m < 2; ++m)
#pragma unroll
            for (int nn = 0; nn < 4; ++nn)
#pragma unroll
                for (int e = 0; e < 4; ++e) acc[m][nn][e] = 0.0f;
        for (int i = max(1, d - kOzSlices); i <= min(kOzSlices, d - 1); ++i)
            oz_product(sR, cs, i - 1, d - i - 1, wr, wc, lane, acc);
#pragma unroll
        for (int m = 0; m < 2; ++m)
#pragma unroll
            for (int nn = 0; nn < 4; ++nn)
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const float g = acc[m][nn][e];
                    if (d == 2) I[m][nn][e] = (long long)__float2int_rn(g);
                    else if (d <= 6) I[m][nn][e] = I[m][nn][e] * 256 + (long long)__float2int_rn(g);
                    else if (d == 7) T[m][nn][e] = g;
                    else T[m][nn][e] = fmaf(g, 0.00390625f, T[m][nn][e]);
                }
    }
    const int g = lane >> 2, tg = lane & 3;
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
        for (int nn = 0; nn < 4; ++nn)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int r = wr * 32 + m * 16 + g + 8 * (e >> 1), c = wc * 32 + nn * 8 + 2 * tg + (e & 1);
                if (r >= mi || c >= mj || (diag && c > r)) continue;
                const double v = fma((double)T[m][nn][e], 0.00390625, (double)I[m][nn][e]);
                double *a = A + (size_t)r * lda + c;
                *a = fma(-v * fR[r], fC[c], *a);
            }
}

}  // namespace sfmba
