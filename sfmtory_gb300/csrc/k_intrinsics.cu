// refine_intrinsics (crates/sfm-ba/src/intrinsics.rs:116-238): every camera's
// parameters refined by its own dense LM with poses and points held fixed,
// one CTA per camera for the whole solve. Per iteration the CTA forms the
// k x k normal equations of the robustly weighted residuals with central
// finite-difference Jacobians (step 1e-6 on each parameter), reduced over
// its threads in FP64; one thread solves the damped system (Cholesky, LU
// fallback, else lambda x 3) and the CTA evaluates the trial cost; accept
// iff finite and lower (lambda / 3, floor 1e-12), at most 8 tries, stop
// when none is accepted. Cameras with fewer than 8 observations keep their
// parameters. All arithmetic FP64 (the reference's, with the cost's FP64
// projection).
#include "camera.cuh"
#include "kernels.cuh"

namespace sfmba {

namespace {

constexpr int kRefineThreads = 128;
constexpr double kFdStep = 1e-6;  // intrinsics.rs EPS

// Block sum in FP64, fixed order (warp shuffles, then the warps in order).
__device__ __forceinline__ double block_sum128(double v, double *sh) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    const double r = sh[0] + sh[1] + sh[2] + sh[3];
    return r;
}

__device__ __forceinline__ bool obs_residual(const double *poses, const double *points, const int *ob_img,
                                             const int *ob_pt, const double *ob_xy, int o, int model,
                                             const double *cam, double &rx, double &ry) {
    const int i = ob_img[o], p = ob_pt[o];
    const double *X = points + 3 * (size_t)p;
    return residual64(poses + 7 * (size_t)i, model, cam, X[0], X[1], X[2], ob_xy[2 * (size_t)o],
                      ob_xy[2 * (size_t)o + 1], rx, ry);
}

// Robust cost of camera parameters `cam` over observations [s, e) of cobs.
__device__ double camera_cost(const double *poses, const double *points, const int *ob_img, const int *ob_pt,
                              const double *ob_xy, const int *cobs, int s, int e, int model, const double *cam,
                              int loss, double scale, double *sh) {
    double sum = 0.0;
    for (int k = s + threadIdx.x; k < e; k += blockDim.x) {
        double rx, ry;
        if (obs_residual(poses, points, ob_img, ob_pt, ob_xy, cobs[k], model, cam, rx, ry)) {
            const double n = sqrt(rx * rx + ry * ry);
            sum += robust_weight<double>(n, loss, scale) * n * n;
        }
    }
    return block_sum128(sum, sh);
}

// Solves A x = b (n <= 8, row-major, A symmetric): Cholesky, else LU with
// partial pivoting; false if both fail.
__device__ bool solve_small(int n, const double *A, const double *b, double *x) {
    double L[64];
    bool chol = true;
    for (int j = 0; j < n && chol; ++j) {
        double d = A[j * n + j];
        for (int k = 0; k < j; ++k) d -= L[j * 8 + k] * L[j * 8 + k];
        if (!(d > 0.0)) { chol = false; break; }
        const double ljj = sqrt(d);
        L[j * 8 + j] = ljj;
        for (int i = j + 1; i < n; ++i) {
            double v = A[i * n + j];
            for (int k = 0; k < j; ++k) v -= L[i * 8 + k] * L[j * 8 + k];
            L[i * 8 + j] = v / ljj;
        }
    }
    if (chol) {
        double y[8];
        for (int i = 0; i < n; ++i) {
            double v = b[i];
            for (int k = 0; k < i; ++k) v -= L[i * 8 + k] * y[k];
            y[i] = v / L[i * 8 + i];
        }
        for (int i = n - 1; i >= 0; --i) {
            double v = y[i];
            for (int k = i + 1; k < n; ++k) v -= L[k * 8 + i] * x[k];
            x[i] = v / L[i * 8 + i];
        }
        return true;
    }
    double M[64], r[8];
    int perm[8];
    for (int i = 0; i < n; ++i) {
        perm[i] = i;
        r[i] = b[i];
        for (int j = 0; j < n; ++j) M[i * 8 + j] = A[i * n + j];
    }
    for (int k = 0; k < n; ++k) {
        int p = k;
        double best = fabs(M[k * 8 + k]);
        for (int i = k + 1; i < n; ++i)
            if (fabs(M[i * 8 + k]) > best) { best = fabs(M[i * 8 + k]); p = i; }
        if (best == 0.0) return false;
        if (p != k) {
            for (int j = 0; j < n; ++j) { const double t = M[k * 8 + j]; M[k * 8 + j] = M[p * 8 + j]; M[p * 8 + j] = t; }
            const double t = r[k]; r[k] = r[p]; r[p] = t;
            const int q = perm[k]; perm[k] = perm[p]; perm[p] = q;
        }
        for (int i = k + 1; i < n; ++i) {
            const double f = M[i * 8 + k] / M[k * 8 + k];
            for (int j = k; j < n; ++j) M[i * 8 + j] -= f * M[k * 8 + j];
            r[i] -= f * r[k];
        }
    }
    for (int i = n - 1; i >= 0; --i) {
        double v = r[i];
        for (int j = i + 1; j < n; ++j) v -= M[i * 8 + j] * x[j];
        x[i] = v / M[i * 8 + i];
    }
    return true;
}

__global__ void __launch_bounds__(kRefineThreads)
    k_refine_intrinsics(const double *poses, const double *points, const int *ob_img, const int *ob_pt,
                        const double *ob_xy, const int *cam_model, const int *cobs_start, const int *cobs,
                        int max_iterations, double lambda0, int loss, double scale, double *cams) {
    constexpr int NA = 8 * 9 / 2 + 8;  // upper triangle of J^T W J, then J^T W r
    __shared__ double sh[4];
    __shared__ double cur[8], trial[8], sys[NA];
    __shared__ int s_ok;
    const int c = blockIdx.x;
    const int s = cobs_start[c], e = cobs_start[c + 1];
    if (e - s < 8) return;  // intrinsics.rs:135-141: left as it is
    const int model = cam_model[c];
    const int np = model_dof(model);
    if (threadIdx.x < 8) cur[threadIdx.x] = cams[8 * (size_t)c + threadIdx.x];
    __syncthreads();
    double cost = camera_cost(poses, points, ob_img, ob_pt, ob_xy, cobs, s, e, model, cur, loss, scale, sh);
    double lambda = lambda0;
    for (int it = 0; it < max_iterations; ++it) {
        double acc[NA];
#pragma unroll
        for (int q = 0; q < NA; ++q) acc[q] = 0.0;
        for (int k = s + threadIdx.x; k < e; k += blockDim.x) {
            const int o = cobs[k];
            double r0x, r0y;
            if (!obs_residual(poses, points, ob_img, ob_pt, ob_xy, o, model, cur, r0x, r0y)) continue;
            const double w = robust_weight<double>(sqrt(r0x * r0x + r0y * r0y), loss, scale);
            double jx[8], jy[8], pp[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) pp[q] = cur[q];
#pragma unroll
            for (int a = 0; a < 8; ++a) {
                jx[a] = jy[a] = 0.0;
                if (a >= np) continue;
                double px = r0x, py = r0y, mx = r0x, my = r0y;
                pp[a] = cur[a] + kFdStep;
                if (!obs_residual(poses, points, ob_img, ob_pt, ob_xy, o, model, pp, px, py)) { px = r0x; py = r0y; }
                pp[a] = cur[a] - kFdStep;
                if (!obs_residual(poses, points, ob_img, ob_pt, ob_xy, o, model, pp, mx, my)) { mx = r0x; my = r0y; }
                pp[a] = cur[a];
                jx[a] = (px - mx) / (2.0 * kFdStep);
                jy[a] = (py - my) / (2.0 * kFdStep);
            }
            int q = 0;
#pragma unroll
            for (int a = 0; a < 8; ++a)
#pragma unroll
                for (int b = a; b < 8; ++b) acc[q++] += w * (jx[a] * jx[b] + jy[a] * jy[b]);
#pragma unroll
            for (int a = 0; a < 8; ++a) acc[q++] += w * (jx[a] * r0x + jy[a] * r0y);
        }
#pragma unroll
        for (int q = 0; q < NA; ++q) {
            const double v = block_sum128(acc[q], sh);
            if (threadIdx.x == 0) sys[q] = v;
        }
        __syncthreads();
        bool accepted = false;
        for (int t = 0; t < 8; ++t) {
            if (threadIdx.x == 0) {
                double A[64], rhs[8], dx[8];
                int q = 0;
                for (int a = 0; a < 8; ++a)
                    for (int b = a; b < 8; ++b, ++q)
                        if (a < np && b < np) A[a * np + b] = A[b * np + a] = sys[q];
                for (int a = 0; a < np; ++a) {
                    rhs[a] = -sys[36 + a];
                    A[a * np + a] += lambda * fmax(A[a * np + a], 1e-12);
                }
                s_ok = solve_small(np, A, rhs, dx) ? 1 : 0;
                for (int a = 0; a < 8; ++a) trial[a] = cur[a] + (s_ok && a < np ? dx[a] : 0.0);
            }
            __syncthreads();
            if (!s_ok) {  // intrinsics.rs:202-205
                lambda *= 3.0;
                continue;
            }
            const double tc = camera_cost(poses, points, ob_img, ob_pt, ob_xy, cobs, s, e, model, trial, loss, scale, sh);
            if (isfinite(tc) && tc < cost) {
                __syncthreads();
                if (threadIdx.x < 8) cur[threadIdx.x] = trial[threadIdx.x];
                __syncthreads();
                cost = tc;
                lambda = fmax(lambda / 3.0, 1e-12);
                accepted = true;
                break;
            }
            lambda *= 3.0;
            __syncthreads();
        }
        if (!accepted) break;
    }
    if (threadIdx.x < 8) cams[8 * (size_t)c + threadIdx.x] = cur[threadIdx.x];
}

}  // namespace

void launch_refine_intrinsics(const IntrinsicsBufs &q, int max_iterations, double lambda0, int loss, double scale,
                              cudaStream_t s) {
    if (q.nC == 0) return;
    k_refine_intrinsics<<<q.nC, kRefineThreads, 0, s>>>(q.poses, q.points, q.ob_img, q.ob_pt, q.ob_xy, q.cam_model,
                                                        q.cobs_start, q.cobs, max_iterations, lambda0, loss, scale,
                                                        q.cams);
    SFMBA_LAUNCH_CHECK();
}

}  // namespace sfmba
