// Observation-pass kernels of the matrix-free (PCG) path and the image-block
// accumulation shared with the dense paths; see matfree.cuh for the chunked
// work partition. Reference arithmetic: crates/sfm-ba/src/lib.rs :859-909
// (point/image blocks), :958-965 and :114-211 (Schur terms, here applied as
// operators), :1100-1120 (point back-substitution). Included by the
// translation units that launch them (k_matfree.cu, k_mf_pcg.cu).
#pragma once

#include "matfree.cuh"

namespace sfmba {

namespace {

// Inclusive segmented warp scan (segments start at head lanes). The lane
// `off` places back is added while it lies in the lane's segment, found once
// from the ballot of heads (the same additions in the same order as carrying
// a head flag through the levels). All five levels run unrolled: skipping
// the levels no segment needs (a warp-wide maximum and a loop) was measured
// slower on the 2000-camera problem's point pass (86.8 against 82.7 us).
template <typename T, int N>
__device__ __forceinline__ void seg_scan(T (&v)[N], bool head, int lane) {
    const unsigned heads = __ballot_sync(0xffffffffu, head) | 1u;
    const int seg_start = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        T a[N];
#pragma unroll
        for (int n = 0; n < N; ++n) a[n] = shfl_up(v[n], off);
        if (lane - off >= seg_start) {
#pragma unroll
            for (int n = 0; n < N; ++n) v[n] += a[n];
        }
    }
}

// Walks one point-aligned chunk: contrib(o, rc, v) fills the lane's N
// values from observation o with packed record rc = {image, point, x, y};
// consume(pt, v) runs on the lane holding a point's complete sum. With
// ILP = 2 two rounds of 32 observations are taken per step and both rounds'
// contributions are computed before either round's segmented scan, so their
// independent loads and arithmetic overlap. With PF the records of the next
// step are loaded while the current step computes (their DRAM latency leaves
// the dependent chain record -> gathers -> arithmetic). Whether lane 31's
// point continues past its round is read from the first record of the next
// round, which is already in registers except for a step's last round
// without PF. The scans (and so the sums) are the same in every form.
template <typename T, int N, int ILP = 2, bool PF = false, typename Contrib, typename Consume>
__device__ __forceinline__ void point_chunk(const int4 *__restrict__ obrec, int cs, int ce, int lane,
                                            Contrib contrib, Consume consume) {
    T carry[N];
#pragma unroll
    for (int n = 0; n < N; ++n) carry[n] = T(0);
    int carry_pt = -1;
    // next31: on lane 31, the point of the observation after this round (-1 past the chunk)
    auto scan_round = [&](T (&v)[N], bool valid, int pt, int next31) {
        if (valid && lane == 0 && pt == carry_pt) {
#pragma unroll
            for (int n = 0; n < N; ++n) v[n] += carry[n];
        }
        const int prev = __shfl_up_sync(0xffffffffu, pt, 1);
        seg_scan<T, N>(v, lane == 0 || pt != prev, lane);
        int next = __shfl_down_sync(0xffffffffu, pt, 1);
        if (lane == 31) next = next31;
        const bool tail = valid && next != pt;
        if (tail) consume(pt, v);
#pragma unroll
        for (int n = 0; n < N; ++n) carry[n] = __shfl_sync(0xffffffffu, v[n], 31);
        carry_pt = __shfl_sync(0xffffffffu, (valid && !tail) ? pt : -1, 31);
    };
    // invalid lanes hold point -1, so "next" past the chunk reads as -1
    auto load = [&](int base, int4 (&rc)[ILP]) {
#pragma unroll
        for (int r = 0; r < ILP; ++r) {
            const int o = base + 32 * r + lane;
            rc[r] = make_int4(0, -1, 0, 0);
            if (o < ce) rc[r] = __ldg(obrec + o);
        }
    };
    int4 nx[ILP];
    if constexpr (PF) load(cs, nx);
    for (int base = cs; base < ce; base += 32 * ILP) {
        int4 rc[ILP];
        if constexpr (PF) {
#pragma unroll
            for (int r = 0; r < ILP; ++r) rc[r] = nx[r];
            load(base + 32 * ILP, nx);
        } else {
            load(base, rc);
        }
        T v[ILP][N];
#pragma unroll
        for (int r = 0; r < ILP; ++r) {
#pragma unroll
            for (int n = 0; n < N; ++n) v[r][n] = T(0);
            if (base + 32 * r + lane < ce) contrib(base + 32 * r + lane, rc[r], v[r]);
        }
#pragma unroll
        for (int r = 0; r < ILP; ++r) {
            if (base + 32 * r >= ce) break;
            int n31;
            if (r + 1 < ILP) {
                n31 = __shfl_sync(0xffffffffu, rc[r + 1 < ILP ? r + 1 : r].y, 0);
            } else if constexpr (PF) {
                n31 = __shfl_sync(0xffffffffu, nx[0].y, 0);
            } else {
                const int o = base + 32 * r + 31;
                n31 = (lane == 31 && o + 1 < ce) ? __ldg(obrec + o + 1).y : -1;
            }
            const bool valid = base + 32 * r + lane < ce;
            scan_round(v[r], valid, rc[r].y, n31);
        }
    }
}

// Step shape of the once-per-retry point-major passes (point reduction,
// back-substitution): in FP32 one round per step with the next step's
// records loaded ahead, the shape the PCG point pass measured fastest; in
// FP64 two rounds per step. The sums are the same either way.
template <typename T>
constexpr int kPtPassILP = sizeof(T) == 4 ? 1 : 2;
template <typename T>
constexpr bool kPtPassPF = sizeof(T) == 4;

// C_p = sum Jx~^T Jx~, g_p = sum Jx~^T r~, free-block count (lib.rs:863-864, :870-879).
template <typename T, int D, bool RC, int M>
__global__ void __launch_bounds__(256) k_mf_point_reduce(JacSrc<T> J, const unsigned char *__restrict__ ob_valid,
                                                         const int *__restrict__ img_free,
                                                         const int *__restrict__ pchunk, int nchunks,
                                                         T *__restrict__ pt_C, T *__restrict__ pt_g,
                                                         int *__restrict__ pt_nfree) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= nchunks) return;
    point_chunk<T, 10, kPtPassILP<T>, kPtPassPF<T>>(
        J.obrec, pchunk[warp], pchunk[warp + 1], lane,
        [&](int o, int4 rc, T (&v)[10]) {
            ObsOp<T, D, RC, M> op;
            make_op_point_major<T, D, RC>(J, o, rc, op, true);
            bool ok = op.valid;
            if constexpr (!RC) ok = ob_valid[o] != 0;
            T jx[6];
            op.jx_rows(jx);
            const T r0 = op.r(0), r1 = op.r(1);
            const T a0 = jx[0], a1 = jx[1], a2 = jx[2], b0 = jx[3], b1 = jx[4], b2 = jx[5];
            v[0] = a0 * a0 + b0 * b0; v[1] = a0 * a1 + b0 * b1; v[2] = a0 * a2 + b0 * b2;
            v[3] = a1 * a1 + b1 * b1; v[4] = a1 * a2 + b1 * b2; v[5] = a2 * a2 + b2 * b2;
            v[6] = a0 * r0 + b0 * r1; v[7] = a1 * r0 + b1 * r1; v[8] = a2 * r0 + b2 * r1;
            v[9] = (ok && img_free[rc.x]) ? T(1) : T(0);
        },
        [&](int pt, const T (&v)[10]) {
            T *C = pt_C + 6 * (size_t)pt;
#pragma unroll
            for (int n = 0; n < 6; ++n) C[n] = v[n];
            T *g = pt_g + 3 * (size_t)pt;
            g[0] = v[6]; g[1] = v[7]; g[2] = v[8];
            pt_nfree[pt] = (int)(v[9] + T(0.5));
        });
}

// Image-major accumulation of H_i = sum_o Jc~^T W_o Jc~ (upper triangle) and
// sum_o Jc~^T v_o over image-aligned chunks (at most kChunkObs observations
// of one image, one warp each), one partial per chunk:
//   MODE 0: W = I, v = r~                 -> H_i, b_i
//   MODE 1: W = Jx~ C^-1 Jx~^T, v = Jx~ h -> Schur diagonal block, rhs term
//   MODE 2: both in one pass, P_t = [A_t | r~ | W A_t | v] (2 x 2(D+1)); the
//           chunk's partial holds the MODE-0 sums, then the MODE-1 sums
// Per round of 32 observations lane t stages A_t = Jc~ (2 x D) and
// P_t = [W A_t | v_t] (2 x (D+1)); the chunk's sum of A_t^T P_t is then a
// product with inner dimension 2 x 32 per round, register-tiled like the
// Schur reduction: four 8-lane subgroups take observations t = g (mod 4) and
// each lane owns a ceil(D/2) x ceil((D+1)/4) tile of [H | b].
template <typename T>
constexpr int accum_warps() { return sizeof(T) == 4 ? 4 : 2; }

template <typename T, int D, bool RC, int MODE, int M = -1>
__global__ void __launch_bounds__(32 * accum_warps<T>())
    k_mf_image_accum(JacSrc<T> J, const int4 *__restrict__ chunks, int nchunks, const T *__restrict__ pt_Cinv,
                     const T *__restrict__ pt_h, const unsigned char *__restrict__ pt_ok, T *__restrict__ part) {
    constexpr int NH = D * (D + 1) / 2;
    constexpr int NV = NH + D;
    constexpr int E = D + 1;                       // columns of one block of P: W A, then v
    constexpr int EP = MODE == 2 ? 2 * E : E;      // columns of P
    constexpr int NVP = MODE == 2 ? 2 * NV : NV;   // partial entries per chunk
    constexpr int RH = (D + 1) / 2, CQ = (EP + 3) / 4;
    constexpr int LA = 2 * D + 1, LP = 2 * EP + 1;
    constexpr int WPB = accum_warps<T>();
    __shared__ T sA[WPB][32][LA];
    __shared__ T sP[WPB][32][LP];
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (c >= nchunks) return;
    const int4 ch = chunks[c];  // {image, first, end}
    if (J.img_live && !J.img_live[ch.x]) return;  // batched windows not taking part
    const int sg = lane >> 3, l8 = lane & 7;
    const int r0 = (l8 >> 2) * RH, c0 = (l8 & 3) * CQ;
    T acc[RH][CQ];
#pragma unroll
    for (int a = 0; a < RH; ++a)
#pragma unroll
        for (int b = 0; b < CQ; ++b) acc[a][b] = T(0);
    for (int base = ch.y; base < ch.z; base += 32) {
        const int k = base + lane;
        bool staged = false;
        if (k < ch.z) {
            const int4 rc = __ldg(J.isrec + k);
            ObsOp<T, D, RC, M> op;
            make_op_image_major<T, D, RC>(J, k, rc, op, MODE != 1);
            T jc[2 * D];
            op.jc_rows(jc);
#pragma unroll
            for (int f = 0; f < 2 * D; ++f) sA[wl][lane][f] = jc[f];
            if constexpr (MODE == 2) {
#pragma unroll
                for (int q = 0; q < D; ++q) {
                    sP[wl][lane][q] = jc[q];
                    sP[wl][lane][EP + q] = jc[D + q];
                }
                sP[wl][lane][D] = op.r(0);
                sP[wl][lane][EP + D] = op.r(1);
                const int pt = rc.y;
                T w00 = T(0), w01 = T(0), w11 = T(0), v0 = T(0), v1 = T(0);
                if (pt_ok[pt]) {  // otherwise the observation adds to H_i, b_i only
                    T jx[6];
                    op.jx_rows(jx);
                    const T *Ci = pt_Cinv + 6 * (size_t)pt;
                    T U[2][3];
#pragma unroll
                    for (int q = 0; q < 2; ++q) {
                        const T a0 = jx[3 * q], a1 = jx[3 * q + 1], a2 = jx[3 * q + 2];
                        U[q][0] = a0 * Ci[0] + a1 * Ci[1] + a2 * Ci[2];
                        U[q][1] = a0 * Ci[1] + a1 * Ci[3] + a2 * Ci[4];
                        U[q][2] = a0 * Ci[2] + a1 * Ci[4] + a2 * Ci[5];
                    }
                    w00 = U[0][0] * jx[0] + U[0][1] * jx[1] + U[0][2] * jx[2];
                    w01 = U[0][0] * jx[3] + U[0][1] * jx[4] + U[0][2] * jx[5];
                    w11 = U[1][0] * jx[3] + U[1][1] * jx[4] + U[1][2] * jx[5];
                    const T *h = pt_h + 3 * (size_t)pt;
                    v0 = jx[0] * h[0] + jx[1] * h[1] + jx[2] * h[2];
                    v1 = jx[3] * h[0] + jx[4] * h[1] + jx[5] * h[2];
                }
#pragma unroll
                for (int q = 0; q < D; ++q) {
                    sP[wl][lane][E + q] = w00 * jc[q] + w01 * jc[D + q];
                    sP[wl][lane][EP + E + q] = w01 * jc[q] + w11 * jc[D + q];
                }
                sP[wl][lane][E + D] = v0;
                sP[wl][lane][EP + E + D] = v1;
                staged = true;
            } else if constexpr (MODE == 0) {
#pragma unroll
                for (int q = 0; q < D; ++q) {
                    sP[wl][lane][q] = jc[q];
                    sP[wl][lane][E + q] = jc[D + q];
                }
                sP[wl][lane][D] = op.r(0);
                sP[wl][lane][E + D] = op.r(1);
                staged = true;
            } else {
                const int pt = rc.y;
                if (pt_ok[pt]) {
                    T jx[6];
                    op.jx_rows(jx);
                    const T *Ci = pt_Cinv + 6 * (size_t)pt;
                    T U[2][3];
#pragma unroll
                    for (int q = 0; q < 2; ++q) {
                        const T a0 = jx[3 * q], a1 = jx[3 * q + 1], a2 = jx[3 * q + 2];
                        U[q][0] = a0 * Ci[0] + a1 * Ci[1] + a2 * Ci[2];
                        U[q][1] = a0 * Ci[1] + a1 * Ci[3] + a2 * Ci[4];
                        U[q][2] = a0 * Ci[2] + a1 * Ci[4] + a2 * Ci[5];
                    }
                    const T w00 = U[0][0] * jx[0] + U[0][1] * jx[1] + U[0][2] * jx[2];
                    const T w01 = U[0][0] * jx[3] + U[0][1] * jx[4] + U[0][2] * jx[5];
                    const T w11 = U[1][0] * jx[3] + U[1][1] * jx[4] + U[1][2] * jx[5];
                    const T *h = pt_h + 3 * (size_t)pt;
#pragma unroll
                    for (int q = 0; q < D; ++q) {
                        sP[wl][lane][q] = w00 * jc[q] + w01 * jc[D + q];
                        sP[wl][lane][E + q] = w01 * jc[q] + w11 * jc[D + q];
                    }
                    sP[wl][lane][D] = jx[0] * h[0] + jx[1] * h[1] + jx[2] * h[2];
                    sP[wl][lane][E + D] = jx[3] * h[0] + jx[4] * h[1] + jx[5] * h[2];
                    staged = true;
                }
            }
        }
        if (!staged) {
#pragma unroll
            for (int f = 0; f < 2 * D; ++f) sA[wl][lane][f] = T(0);
#pragma unroll
            for (int f = 0; f < 2 * EP; ++f) sP[wl][lane][f] = T(0);
        }
        __syncwarp();
        const int rounds = (min(32, ch.z - base) + 3 - sg) / 4;  // observations of this subgroup
        for (int kk = 0; kk < rounds; ++kk) {
            const int t = sg + 4 * kk;
#pragma unroll
            for (int rho = 0; rho < 2; ++rho) {
                T av[RH], pv[CQ];
#pragma unroll
                for (int a = 0; a < RH; ++a) av[a] = (r0 + a < D) ? sA[wl][t][rho * D + r0 + a] : T(0);
#pragma unroll
                for (int b = 0; b < CQ; ++b) pv[b] = (c0 + b < EP) ? sP[wl][t][rho * EP + c0 + b] : T(0);
#pragma unroll
                for (int a = 0; a < RH; ++a)
#pragma unroll
                    for (int b = 0; b < CQ; ++b) acc[a][b] += av[a] * pv[b];
            }
        }
        __syncwarp();
    }
    T *dst = part + (size_t)c * NVP;
#pragma unroll
    for (int a = 0; a < RH; ++a)
#pragma unroll
        for (int b = 0; b < CQ; ++b) {
            T v = acc[a][b];
            v += __shfl_xor_sync(0xffffffffu, v, 8);
            v += __shfl_xor_sync(0xffffffffu, v, 16);
            const int row = r0 + a, col = c0 + b;
            const int blk = col >= E ? 1 : 0, cl = col - blk * E;  // block of P, column within it
            if (lane < 8 && row < D && col < EP) {
                T *d = dst + blk * NV;
                if (cl < D && row <= cl) d[row * D - row * (row - 1) / 2 + (cl - row)] = v;
                else if (cl == D) d[NH + row] = v;
            }
        }
}

// H_i (full symmetric, FP64) and b_i from the image's MODE-0 partials.
template <typename T, int D>
__global__ void __launch_bounds__(128) k_mf_image_finish0(const T *__restrict__ part,
                                                          const int *__restrict__ ipart_off, int nI,
                                                          const unsigned char *__restrict__ img_live,
                                                          double *__restrict__ img_H, double *__restrict__ img_b,
                                                          int stride) {
    constexpr int NH = D * (D + 1) / 2;
    constexpr int NV = NH + D;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= nI) return;
    if (img_live && !img_live[i]) return;
    for (int e = lane; e < NV; e += 32) {
        double s = 0.0;
        const int k1 = ipart_off[i + 1];
        int k = ipart_off[i];
        for (; k + 8 <= k1; k += 8) {  // eight loads in flight, added in partial order
            T w[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) w[u] = part[(size_t)(k + u) * stride + e];
#pragma unroll
            for (int u = 0; u < 8; ++u) s += (double)w[u];
        }
        for (; k < k1; ++k) s += (double)part[(size_t)k * stride + e];
        if (e < NH) {
            int t = e, a = 0;
            while (t >= D - a) { t -= D - a; ++a; }
            const int b = a + t;
            img_H[(size_t)i * D * D + a * D + b] = s;
            img_H[(size_t)i * D * D + b * D + a] = s;
        } else {
            img_b[(size_t)i * D + (e - NH)] = s;
        }
    }
}

// Minimum pivot of the FP32 factorisation of a unit-diagonal block: below
// it the block is factorised in FP64 instead.
constexpr float kMinScaledPivot = 1e-3f;

// FP32 inverse of the damped image block L (FP64, symmetric) into Mi: the
// block scaled to a unit diagonal (s_a = 1/sqrt(L_aa)), factorised by a
// right-looking Cholesky in FP32, its inverse one column per lane, and
// Mi = S (S L S)^-1 S. False (Mi untouched) when a diagonal entry is not
// positive or a scaled pivot falls below kMinScaledPivot: the caller then
// factorises in FP64. The FP32 path's preconditioner is stored in FP32, and
// a 1e-3 pivot bounds the FP32 factorisation's error in the inverse to about
// 1e-3 relative, which leaves the preconditioned iteration unchanged in
// practice; GB300 runs FP64 at 1/64 of the FP32 rate, and the FP64
// factorisation's square roots and divisions dominated this kernel.
template <int D>
__device__ __forceinline__ bool image_block_inverse_f32(const double (&L)[D][D + 1], double (&Mi)[D][D + 1],
                                                        float (&A)[D][D + 1], float *sc, float *inv, int lane) {
    bool pos = true;
    if (lane < D) {
        const double dd = L[lane][lane];
        pos = dd > 0.0 && isfinite(dd);
        sc[lane] = pos ? rsqrtf((float)dd) : 0.0f;
    }
    if (!__all_sync(0xffffffffu, pos)) return false;
    __syncwarp();
    for (int idx = lane; idx < D * D; idx += 32) {
        const int a = idx / D, b = idx - a * D;
        A[a][b] = (float)L[a][b] * sc[a] * sc[b];
    }
    __syncwarp();
    for (int j = 0; j < D; ++j) {
        const float d = A[j][j];
        if (!(d > kMinScaledPivot) || !isfinite(d)) return false;  // every lane read the same d
        const float sd = sqrtf(d);
        const float id = 1.0f / sd;
        __syncwarp();
        if (lane == 0) {
            A[j][j] = sd;
            inv[j] = id;
        }
        if (lane > j && lane < D) A[lane][j] *= id;
        __syncwarp();
        const int m = D - j - 1;
        for (int idx = lane; idx < m * m; idx += 32) {
            const int q = j + 1 + idx / m, c = j + 1 + idx % m;
            if (c <= q) A[q][c] = fmaf(-A[q][j], A[c][j], A[q][c]);
        }
        __syncwarp();
    }
    float col[D];
    if (lane < D) {
        const int c = lane;
#pragma unroll
        for (int q = 0; q < D; ++q) {
            float v = q == c ? 1.0f : 0.0f;
#pragma unroll
            for (int k = 0; k < q; ++k) v = fmaf(-A[q][k], col[k], v);
            col[q] = q < c ? 0.0f : v * inv[q];
        }
#pragma unroll
        for (int q = D - 1; q >= 0; --q) {
            float v = col[q];
#pragma unroll
            for (int k = q + 1; k < D; ++k) v = fmaf(-A[k][q], col[k], v);
            col[q] = v * inv[q];
        }
    }
    __syncwarp();
    if (lane < D)
#pragma unroll
        for (int q = 0; q < D; ++q) Mi[q][lane] = (double)(sc[q] * col[q] * sc[lane]);
    return true;
}

// Block-Jacobi preconditioner (exact image diagonal block of the Schur
// complement, Cholesky-inverted), reduced rhs and the PCG start vectors
// (x = 0, r = rhs, p = z = M^-1 r) of image i, from its MODE-1 partials.
// One warp per image: warp-cooperative Cholesky, one lane per column of the
// inverse with the triangular solves unrolled into registers.
template <typename T, int D>
__global__ void __launch_bounds__(128) k_mf_precond_finish(const T *__restrict__ part,
                                                           const int *__restrict__ ipart_off,
                                                           const double *__restrict__ img_H,
                                                           const double *__restrict__ img_b,
                                                           const int *__restrict__ img_active,
                                                           const int *__restrict__ img_pmask,
                                                           const LMState *__restrict__ st, int nI,
                                                           double *__restrict__ img_rhs, T *__restrict__ Minv_out,
                                                           T *__restrict__ x, T *__restrict__ r, T *__restrict__ z,
                                                           T *__restrict__ p, T *__restrict__ p4,
                                                           double *__restrict__ dots, int stride,
                                                           float *__restrict__ Hf) {
    constexpr int NH = D * (D + 1) / 2;
    constexpr int NV = NH + D;
    constexpr int WPB = 4;
    __shared__ double Ls[WPB][D][D + 1];
    __shared__ double Ms[WPB][D][D + 1];
    __shared__ double rvs[WPB][D];
    __shared__ double invd_s[WPB][D];
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i = blockIdx.x * WPB + wl;
    if (i >= nI) return;
    double(&L)[D][D + 1] = Ls[wl];
    double(&Mi)[D][D + 1] = Ms[wl];
    double *rv = rvs[wl];
    double *invd = invd_s[wl];
    const double lam = st->lambda;
    const int act = img_active[i];
    const int pm = img_pmask[i];  // the image's own block (a linked image's camera columns are not in it)
    const double *H = img_H + (size_t)i * D * D;
    const int p0 = ipart_off[i], p1 = ipart_off[i + 1];
    for (int e = lane; e < NV; e += 32) {
        double sum = 0.0;
        int k = p0;
        for (; k + 8 <= p1; k += 8) {  // eight loads in flight, added in partial order
            T w[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) w[u] = part[(size_t)(k + u) * stride + e];
#pragma unroll
            for (int u = 0; u < 8; ++u) sum += (double)w[u];
        }
        for (; k < p1; ++k) sum += (double)part[(size_t)k * stride + e];
        if (e < NH) {
            int t = e, a = 0;
            while (t >= D - a) { t -= D - a; ++a; }
            const int b = a + t;
            double v = H[a * D + b] - sum;
            if (a == b) v += H[a * D + a] * lam;
            const bool on = ((pm >> a) & 1) && ((pm >> b) & 1);
            if (!on) v = a == b ? 1.0 : 0.0;
            L[a][b] = v;
            L[b][a] = v;
            if (a == b) Mi[a][a] = v;  // keeps the diagonal for the Jacobi fallback
        } else {
            const int a = e - NH;
            const double rhs = ((act >> a) & 1) ? -img_b[(size_t)i * D + a] + sum : 0.0;
            rv[a] = rhs;
            img_rhs[(size_t)i * D + a] = rhs;
        }
    }
    if (Hf) {  // FP32 PCG: the damped image block for the CG kernel's (H_i + lambda diag H_i) p_i
        for (int idx = lane; idx < D * D; idx += 32) {
            const int a = idx / D, c = idx - a * D;
            double v = H[idx];
            if (a == c) v += H[idx] * lam;
            Hf[(size_t)i * D * D + idx] = (float)v;
        }
    }
    __syncwarp();
    bool done = false;  // FP32 path: Mi from the FP32 factorisation of the scaled block
    if constexpr (std::is_same<T, float>::value) {
        __shared__ float As[WPB][D][D + 1];
        __shared__ float scs[WPB][D], invs[WPB][D];
        done = image_block_inverse_f32<D>(L, Mi, As[wl], scs[wl], invs[wl], lane);
    }
    // Right-looking Cholesky of the D x D block in FP64, lower triangle in place.
    bool ok = !done;  // the FP64 factorisation ran and succeeded
    for (int j = 0; j < D && ok; ++j) {
        const double d = L[j][j];
        if (!(d > 0.0)) { ok = false; break; }
        const double sd = sqrt(d);
        const double id = 1.0 / sd;
        __syncwarp();
        if (lane == 0) { L[j][j] = sd; invd[j] = id; }
        if (lane > j && lane < D) L[lane][j] *= id;
        __syncwarp();
        const int m = D - j - 1;
        for (int idx = lane; idx < m * m; idx += 32) {
            const int q = j + 1 + idx / m, c = j + 1 + idx % m;
            if (c <= q) L[q][c] -= L[q][j] * L[c][j];
        }
        __syncwarp();
    }
    if (ok) {
        // Column c of the inverse: L y = e_c, then L^T x = y.
        double col[D];
        if (lane < D) {
            const int c = lane;
#pragma unroll
            for (int q = 0; q < D; ++q) {
                double v = q == c ? 1.0 : 0.0;
#pragma unroll
                for (int k = 0; k < q; ++k) v -= L[q][k] * col[k];
                col[q] = q < c ? 0.0 : v * invd[q];
            }
#pragma unroll
            for (int q = D - 1; q >= 0; --q) {
                double v = col[q];
#pragma unroll
                for (int k = q + 1; k < D; ++k) v -= L[k][q] * col[k];
                col[q] = v * invd[q];
            }
        }
        __syncwarp();
        if (lane < D)
#pragma unroll
            for (int q = 0; q < D; ++q) Mi[q][lane] = col[q];
    } else if (!done) {
        // Not SPD in FP64: Jacobi on the block's diagonal.
        double dl = 0.0;
        if (lane < D) dl = Mi[lane][lane];
        __syncwarp();
        if (lane < D)
            for (int q = 0; q < D; ++q) Mi[q][lane] = (q == lane && dl > 0.0) ? 1.0 / dl : 0.0;
    }
    __syncwarp();
    for (int idx = lane; idx < D * D; idx += 32) {
        const int a = idx / D, c = idx - a * D;
        const bool on = ((pm >> a) & 1) && ((pm >> c) & 1);
        if (!on) Mi[a][c] = 0.0;
        Minv_out[(size_t)i * D * D + idx] = (T)Mi[a][c];
    }
    __syncwarp();
    double rz = 0.0, rr = 0.0;
    if (lane < D) {
        double zc = 0.0;
#pragma unroll
        for (int d = 0; d < D; ++d) zc += Mi[lane][d] * rv[d];
        const size_t u = (size_t)i * D + lane;
        const T rt = (T)rv[lane], zt = (T)zc;
        x[u] = T(0);
        r[u] = rt;
        z[u] = zt;
        p[u] = zt;
        if (p4) store_dir(reinterpret_cast<float *>(p4), nI, i, lane, (float)zt);
        if ((pm >> lane) & 1) {  // a shared camera's entries are counted by launch_shared_precond
            rz = (double)rt * (double)zt;
            rr = (double)rt * (double)rt;
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        rz += __shfl_xor_sync(0xffffffffu, rz, off);
        rr += __shfl_xor_sync(0xffffffffu, rr, off);
    }
    if (lane == 0) {
        dots[i] = rz;
        dots[nI + i] = rr;
    }
}

// Launch variants of the two PCG passes, picked per device and problem
// shape by the autotuner in solver.cu: rounds of 32 observations computed
// per step (ILP) and the minimum resident blocks per SM the register
// allocation must allow. Every variant computes the same sums in the same
// order.
// Image-block vector entries of image i: from the FP32 mirror in planes
// (plane_index; D/4 rounded up vector loads, one per plane) when it exists,
// else from the D-strided vector.
template <typename T, int D>
__device__ __forceinline__ void load_image_vec(const T *__restrict__ v, const T *__restrict__ v4, int i, int nI,
                                               T (&out)[D]) {
    if constexpr (std::is_same<T, float>::value) {
        if (v4) {
            const float4 *q = reinterpret_cast<const float4 *>(v4);
#pragma unroll
            for (int k = 0; k < pad4(D) / 4; ++k) {
                const float4 t = __ldg(q + (size_t)k * nI + i);
                if (4 * k + 0 < D) out[4 * k + 0] = t.x;
                if (4 * k + 1 < D) out[4 * k + 1] = t.y;
                if (4 * k + 2 < D) out[4 * k + 2] = t.z;
                if (4 * k + 3 < D) out[4 * k + 3] = t.w;
            }
            return;
        }
    }
#pragma unroll
    for (int c = 0; c < D; ++c) out[c] = v[(size_t)i * D + c];
}

template <int V>
struct PassVariant {  // 0-3: one or two rounds x 3 or 4 blocks/SM; 4, 5: one round, 5 or 6 blocks/SM;
                      // 6-9: as 0-3 with the next step's records loaded ahead
    static constexpr int kBase = V >= 6 ? V - 6 : V;
    static constexpr int kILP = (kBase < 4 && (kBase & 1)) ? 2 : 1;
    static constexpr int kMinBlocks = kBase < 4 ? ((kBase & 2) ? 4 : 3) : kBase + 1;
    static constexpr bool kPF = V >= 6;
};

// PCG point pass: u_p = C_p^-1 sum_o Jx~^T (Jc~_o p_img(o)).
template <typename T, int D, bool RC, int V, int M>
__global__ void __launch_bounds__(256, PassVariant<V>::kMinBlocks)
    k_mf_points(JacSrc<T> J, const int *__restrict__ pchunk, int nchunks, const T *__restrict__ pt_Cinv,
                const unsigned char *__restrict__ pt_ok, const T *__restrict__ p, const T *__restrict__ p4,
                const LMState *__restrict__ st, T *__restrict__ u) {
    if (st->pcg_done) return;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= nchunks) return;
    point_chunk<T, 3, PassVariant<V>::kILP, PassVariant<V>::kPF>(
        J.obrec, pchunk[warp], pchunk[warp + 1], lane,
        [&](int o, int4 rc, T (&v)[3]) {
            T pv[D];
            load_image_vec<T, D>(p, p4, rc.x, J.nI, pv);
            T s0, s1;
            if constexpr (RC && mv_model<M>()) {
                MvOp<D, M> op;
                op.build(J, rc.x, rc.y, rc);
                op.jc_dot(pv, s0, s1);
                op.jx_t(s0, s1, v);
            } else {
                ObsOp<T, D, RC, M> op;
                make_op_point_major<T, D, RC>(J, o, rc, op);
                op.jc_dot(pv, s0, s1);
                op.jx_t(s0, s1, v);
            }
        },
        [&](int pt, const T (&v)[3]) {
            T u0 = 0, u1 = 0, u2 = 0;
            if (pt_ok[pt]) {
                const T *Ci = pt_Cinv + 6 * (size_t)pt;
                u0 = Ci[0] * v[0] + Ci[1] * v[1] + Ci[2] * v[2];
                u1 = Ci[1] * v[0] + Ci[3] * v[1] + Ci[4] * v[2];
                u2 = Ci[2] * v[0] + Ci[4] * v[1] + Ci[5] * v[2];
            }
            if constexpr (std::is_same<T, float>::value) {
                reinterpret_cast<float4 *>(u)[pt] = make_float4(u0, u1, u2, 0.0f);
            } else {
                T *uo = u + 4 * (size_t)pt;
                uo[0] = u0; uo[1] = u1; uo[2] = u2;
            }
        });
}

// PCG image pass: partial sums of Jc~^T (Jx~ u_p) per (chunk, image).
template <typename T, int D, bool RC, int V, int M>
__global__ void __launch_bounds__(256, PassVariant<V>::kMinBlocks)
    k_mf_images(JacSrc<T> J, long long nO, const int *__restrict__ img_start, const int *__restrict__ ipart_off,
                const T *__restrict__ u, const LMState *__restrict__ st, T *__restrict__ ipart) {
    constexpr int ILP = PassVariant<V>::kILP;
    if (st->pcg_done) return;
    const long long chunk = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const long long cs = chunk * kChunkObs;
    if (cs >= nO) return;
    const long long ce = cs + kChunkObs < nO ? cs + kChunkObs : nO;
    T acc[D];
#pragma unroll
    for (int c = 0; c < D; ++c) acc[c] = T(0);
    int cur = __ldg(J.isrec + cs).x;
    auto flush = [&](int img) {
#pragma unroll
        for (int c = 0; c < D; ++c) {
            T v = acc[c];
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
            acc[c] = v;
        }
        if (lane == 0) {
            T *dst = ipart + (size_t)partial_slot(ipart_off, img_start, img, chunk) * D;
#pragma unroll
            for (int c = 0; c < D; ++c) dst[c] = acc[c];
        }
#pragma unroll
        for (int c = 0; c < D; ++c) acc[c] = T(0);
    };
    // Jc~^T (Jx~ u_p) of image-major observation k (zero when invalid).
    auto contrib = [&](long long k, bool valid, int4 rc, T (&cv)[D]) {
#pragma unroll
        for (int c = 0; c < D; ++c) cv[c] = T(0);
        if (!valid) return;
        const int pt = rc.y;
        T u0, u1, u2;
        if constexpr (std::is_same<T, float>::value) {
            const float4 t = __ldg(reinterpret_cast<const float4 *>(u) + pt);
            u0 = t.x; u1 = t.y; u2 = t.z;
        } else {
            const T *up = u + 4 * (size_t)pt;
            u0 = up[0]; u1 = up[1]; u2 = up[2];
        }
        T z0, z1;
        if constexpr (RC && mv_model<M>()) {
            MvOp<D, M> op;
            op.build(J, rc.x, rc.y, rc);
            op.jx(u0, u1, u2, z0, z1);
            op.jc_t(z0, z1, cv);
        } else {
            ObsOp<T, D, RC, M> op;
            make_op_image_major<T, D, RC>(J, k, rc, op);
            op.jx(u0, u1, u2, z0, z1);
            op.jc_t(z0, z1, cv);
        }
    };
    auto accumulate = [&](bool valid, int img, const T (&cv)[D]) {
        while (true) {
            if (valid && img == cur) {
#pragma unroll
                for (int c = 0; c < D; ++c) acc[c] += cv[c];
            }
            const unsigned rest = __ballot_sync(0xffffffffu, valid && img > cur);
            if (!rest) break;
            flush(cur);
            cur = __shfl_sync(0xffffffffu, img, __ffs(rest) - 1);
        }
    };
    // ILP rounds of 32 observations per step, all computed before any is
    // accumulated (independent work overlaps; the sums are the same); with
    // PF the next step's records are loaded while this step computes.
    auto load = [&](long long base, int4 (&rc)[ILP]) {
#pragma unroll
        for (int r = 0; r < ILP; ++r) {
            const long long k = base + 32 * r + lane;
            rc[r] = make_int4(0x7fffffff, 0, 0, 0);
            if (k < ce) rc[r] = __ldg(J.isrec + k);
        }
    };
    int4 nx[ILP];
    if constexpr (PassVariant<V>::kPF) load(cs, nx);
    for (long long base = cs; base < ce; base += 32 * ILP) {
        int4 rc[ILP];
        if constexpr (PassVariant<V>::kPF) {
#pragma unroll
            for (int r = 0; r < ILP; ++r) rc[r] = nx[r];
            load(base + 32 * ILP, nx);
        } else {
            load(base, rc);
        }
        T cv[ILP][D];
#pragma unroll
        for (int r = 0; r < ILP; ++r) contrib(base + 32 * r + lane, base + 32 * r + lane < ce, rc[r], cv[r]);
#pragma unroll
        for (int r = 0; r < ILP; ++r) accumulate(base + 32 * r + lane < ce, rc[r].x, cv[r]);
    }
    flush(cur);
}

// Point back-substitution: delta_p = -C_p^-1 (g_p + sum_o Jx~^T (Jc~ delta_img)),
// trial point = p + delta_p (lib.rs:1100-1120, :1138-1141). Points without
// a usable inverse keep their value (points_trial is a copy beforehand).
template <typename T, int D, bool RC, int M>
__global__ void __launch_bounds__(256) k_mf_backsub(JacSrc<T> J, const int *__restrict__ pchunk, int nchunks,
                                                    const T *__restrict__ img_delta, const T *__restrict__ pt_Cinv,
                                                    const T *__restrict__ pt_g, const unsigned char *__restrict__ pt_ok,
                                                    const double *__restrict__ points,
                                                    double *__restrict__ points_trial) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= nchunks) return;
    point_chunk<T, 3, kPtPassILP<T>, kPtPassPF<T>>(
        J.obrec, pchunk[warp], pchunk[warp + 1], lane,
        [&](int o, int4 rc, T (&v)[3]) {
            ObsOp<T, D, RC, M> op;
            make_op_point_major<T, D, RC>(J, o, rc, op);
            T dv[D];
#pragma unroll
            for (int c = 0; c < D; ++c) dv[c] = img_delta[(size_t)rc.x * D + c];
            T t0, t1;
            op.jc_dot(dv, t0, t1);
            op.jx_t(t0, t1, v);
        },
        [&](int pt, const T (&v)[3]) {
            if (!pt_ok[pt]) return;
            const T *g = pt_g + 3 * (size_t)pt;
            const T a0 = g[0] + v[0], a1 = g[1] + v[1], a2 = g[2] + v[2];
            const T *Ci = pt_Cinv + 6 * (size_t)pt;
            const T d0 = Ci[0] * a0 + Ci[1] * a1 + Ci[2] * a2;
            const T d1 = Ci[1] * a0 + Ci[3] * a1 + Ci[4] * a2;
            const T d2 = Ci[2] * a0 + Ci[4] * a1 + Ci[5] * a2;
            const double *X = points + 3 * (size_t)pt;
            double *Y = points_trial + 3 * (size_t)pt;
            Y[0] = X[0] + (double)(-d0);
            Y[1] = X[1] + (double)(-d1);
            Y[2] = X[2] + (double)(-d2);
        });
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

// FP32 recomputes the Jacobian in every pass; FP64 reads stored records.
template <typename F>
void dispatch_TDR(const Bufs &b, F &&f) {
    dispatch_D(b.D, [&](auto dc) {
        constexpr int D = decltype(dc)::value;
        if (b.mixed) {
            // Recomputed FP32 Jacobians: the camera model as a compile-time
            // constant when every camera has the same model and D is its width.
            auto try_model = [&](auto mc) {
                constexpr int M = decltype(mc)::value;
                if constexpr (model_fits_width(M, D)) {
                    if (b.uniform_model == M) {
                        f((float)0, dc, std::true_type(), mc);
                        return true;
                    }
                }
                return false;
            };
            if (try_model(std::integral_constant<int, SFMBA_SIMPLE_PINHOLE>()) ||
                try_model(std::integral_constant<int, SFMBA_PINHOLE>()) ||
                try_model(std::integral_constant<int, SFMBA_SIMPLE_RADIAL>()) ||
                try_model(std::integral_constant<int, SFMBA_RADIAL>()) ||
                try_model(std::integral_constant<int, SFMBA_OPENCV>()) ||
                try_model(std::integral_constant<int, SFMBA_OPENCV_FISHEYE>()))
                return;
            f((float)0, dc, std::true_type(), std::integral_constant<int, -1>());
        } else {
            f((double)0, dc, std::false_type(), std::integral_constant<int, -1>());
        }
    });
}

template <typename T>
JacSrc<T> jac_src(const Bufs &b) {
    JacSrc<T> J;
    J.rec = (const T *)b.rec;
    J.img_lin = (const ImageLin<T> *)b.img_lin;
    J.points32 = b.points32;
    J.points64 = b.points;
    J.obrec = b.obrec;
    J.isrec = b.isrec;
    J.img_obs = b.img_obs;
    J.loss = b.loss;
    J.scale = (T)b.loss_scale;
    if constexpr (std::is_same<T, float>::value) J.rs = b.ob_rs;
    J.img_live = b.img_live;
    J.mv = b.img_mv;
    J.nI = b.nI;
    return J;
}

inline int warps_grid(long long warps, int threads) { return div_up(warps * 32, threads); }

}  // namespace

}  // namespace sfmba
