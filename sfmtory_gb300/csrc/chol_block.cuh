// Cholesky factor and factor inverse of one diagonal block (at most 64 x 64)
// by a 256-thread block, the sequential core of the blocked factorisations
// (k_dense.cu, k_batched.cu).
//
// Thread (ty, tx) = (tid / 16, tid % 16) keeps the 4 x 4 entries (ty + 16a,
// tx + 16b) of the block in registers for the whole factorisation (strided,
// so the lower-triangle work is spread evenly). Step j of the right-looking
// factorisation: the owner of (j, j) publishes it, every thread reads the
// pivot (so all threads see a failed pivot together), the owners of column j
// scale it and publish it, and every thread updates its entries right of
// and below the pivot. The factor's inverse is formed the same way on the
// identity (step k: row k scaled by 1/L_kk and published, the rows below
// updated). Two barriers per step, no integer division in the loops.
#pragma once

#include "common.cuh"

namespace sfmba {

constexpr int kBlkLD = 65;  // row stride of the 64 x 64 shared tiles

// A: [64][kBlkLD] shared, lower triangle of the nb x nb block on entry, the
// factor on exit. X: [64][kBlkLD] shared, L^-1 on exit (zeros above the
// diagonal and outside nb). buf: [65] shared scratch. Returns false (and
// leaves A, X unspecified) if a pivot is not > 0 (0, negative and NaN all
// fail, as nalgebra's Cholesky::new). Every thread of the block must call it.
__device__ __forceinline__ bool chol_block_factor_invert(double *A, double *X, int nb, double *buf) {
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    double a[4][4];
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int i = ty + 16 * p, l = tx + 16 * q;
            a[p][q] = (i < nb && l <= i) ? A[i * kBlkLD + l] : 0.0;
        }
    __syncthreads();
    bool ok = true;
    for (int j = 0; j < nb; ++j) {
        const int pj = j >> 4, rj = j & 15;
        if (ty == rj && tx == rj) {  // owner of (j, j)
#pragma unroll
            for (int p = 0; p < 4; ++p)
                if (p == pj) buf[64] = a[p][p];
        }
        __syncthreads();
        const double d = buf[64];
        if (!(d > 0.0)) {
            ok = false;
            break;  // every thread read the same pivot
        }
        const double sd = sqrt(d), inv = 1.0 / sd;
        if (tx == rj) {  // owners of column j: scale it below the pivot, publish it
#pragma unroll
            for (int p = 0; p < 4; ++p) {
                const int i = ty + 16 * p;
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if (q == pj) {
                        if (i == j) a[p][q] = sd;
                        else if (i > j) a[p][q] *= inv;
                        if (i >= j && i < nb) buf[i] = a[p][q];
                    }
            }
        }
        __syncthreads();
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            const int i = ty + 16 * p;
            if (i <= j || i >= nb) continue;
            const double li = buf[i];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int l = tx + 16 * q;
                if (l > j && l <= i) a[p][q] -= li * buf[l];
            }
        }
    }
    if (!ok) return false;
    // The factor back to A (lower triangle), X = I.
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int i = ty + 16 * p, l = tx + 16 * q;
            if (i < nb && l <= i) A[i * kBlkLD + l] = a[p][q];
            a[p][q] = (i == l && i < nb) ? 1.0 : 0.0;
        }
    __syncthreads();
    // L X = I, right-looking over the rows of X.
    for (int k = 0; k < nb; ++k) {
        const int pk = k >> 4, rk = k & 15;
        const double inv = 1.0 / A[k * kBlkLD + k];
        if (ty == rk) {  // owners of row k: scale and publish it
#pragma unroll
            for (int p = 0; p < 4; ++p)
                if (p == pk)
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        a[p][q] *= inv;
                        buf[tx + 16 * q] = a[p][q];
                    }
        }
        __syncthreads();
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            const int i = ty + 16 * p;
            if (i <= k || i >= nb) continue;
            const double lik = A[i * kBlkLD + k];
#pragma unroll
            for (int q = 0; q < 4; ++q) a[p][q] -= lik * buf[tx + 16 * q];
        }
        __syncthreads();
    }
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int i = ty + 16 * p, l = tx + 16 * q;
            X[i * kBlkLD + l] = (i < nb && l < nb && l <= i) ? a[p][q] : 0.0;
        }
    __syncthreads();
    return true;
}

}  // namespace sfmba
