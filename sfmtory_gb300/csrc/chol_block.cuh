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
// updated). Two barriers per step, no integer division in the loops. A
// step only visits the 16-row / 16-column register blocks that can hold
// live entries (rows below the pivot, columns in the lower triangle), so
// the FP64 pipe, the bound here (GB300 issues ~2 FP64 FMAs per clock per
// SM), is not spent on predicated-off entries.
#pragma once

#include "common.cuh"

namespace sfmba {

constexpr int kBlkLD = 65;  // row stride of the 64 x 64 shared tiles

// Step j of the factorisation on the register blocks p >= P0, P0 <= q <= p
// (P0 = j / 16): a[i][l] -= L[i][j] L[l][j] for j < l <= i < nb.
template <int P0>
__device__ __forceinline__ void chol_step_update(double (&a)[4][4], const double *buf, int j, int nb, int tx,
                                                 int ty) {
#pragma unroll
    for (int p = P0; p < 4; ++p) {
        const int i = ty + 16 * p;
        const bool row = i > j && i < nb;
        const double li = row ? buf[i] : 0.0;
#pragma unroll
        for (int q = P0; q <= p; ++q) {
            const int l = tx + 16 * q;
            if (row && l > j && l <= i) a[p][q] -= li * buf[l];
        }
    }
}

// Step k of L X = I on the rows in blocks p >= P0 and the columns in blocks
// q <= P0 (P0 = k / 16; row k of X is zero right of column k).
template <int P0>
__device__ __forceinline__ void inv_step_update(double (&a)[4][4], const double *A, const double *buf, int k,
                                                int nb, int tx, int ty) {
#pragma unroll
    for (int p = P0; p < 4; ++p) {
        const int i = ty + 16 * p;
        if (i <= k || i >= nb) continue;
        const double lik = A[i * kBlkLD + k];
#pragma unroll
        for (int q = 0; q <= P0; ++q) a[p][q] -= lik * buf[tx + 16 * q];
    }
}

// A: [64][kBlkLD] shared, lower triangle of the nb x nb block on entry, the
// factor on exit. X: [64][kBlkLD] shared, L^-1 on exit (zeros above the
// diagonal and outside nb). buf: [67] shared scratch. Returns false (and
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
        if (ty == rj && tx == rj) {  // owner of (j, j): the pivot, its square root and reciprocal
            double d = 0.0;
#pragma unroll
            for (int p = 0; p < 4; ++p)
                if (p == pj) d = a[p][p];
            buf[64] = d;
            if (d > 0.0) {  // once per step (FP64 square roots and divisions are slow on this GPU)
                const double sd = sqrt(d);
                buf[65] = sd;
                buf[66] = 1.0 / sd;
                X[j] = buf[66];  // kept for the inverse (X is written only at its end)
            }
        }
        __syncthreads();
        const double d = buf[64];
        if (!(d > 0.0)) {
            ok = false;
            break;  // every thread read the same pivot
        }
        if (tx == rj) {  // owners of column j: scale it below the pivot, publish it
            const double sd = buf[65], inv = buf[66];
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
        switch (j >> 4) {  // blocks p, q >= j / 16 with q <= p
        case 0: chol_step_update<0>(a, buf, j, nb, tx, ty); break;
        case 1: chol_step_update<1>(a, buf, j, nb, tx, ty); break;
        case 2: chol_step_update<2>(a, buf, j, nb, tx, ty); break;
        default: chol_step_update<3>(a, buf, j, nb, tx, ty); break;
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
        if (ty == rk) {  // owners of row k: scale by 1 / L_kk (from the factorisation) and publish it
            const double inv = X[k];
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
        switch (k >> 4) {  // rows in blocks p >= k / 16, columns in blocks q <= k / 16
        case 0: inv_step_update<0>(a, A, buf, k, nb, tx, ty); break;
        case 1: inv_step_update<1>(a, A, buf, k, nb, tx, ty); break;
        case 2: inv_step_update<2>(a, A, buf, k, nb, tx, ty); break;
        default: inv_step_update<3>(a, A, buf, k, nb, tx, ty); break;
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
