// Camera registration by PnP (crates/sfm-geometry/src/pnp.rs, ransac.rs,
// linalg.rs) for many images at once, and the batched Gauss-Newton pose
// refinement it ends with.
//
// RANSAC (ransac.rs:72-131) is sequential only in its bookkeeping: every
// iteration consumes six values of one xorshift64 stream seeded 0xFACADE
// (the partial Fisher-Yates shuffle restarts from the identity each time),
// so hypothesis t depends on stream values 6t..6t+5 alone. Hypotheses are
// therefore formed and scored in parallel, a round of B per image at a
// time (one thread forms one 6-point DLT: conditioning test, 12 x 12
// one-sided Jacobi SVD, polar factor, scale), one warp scores one hypothesis
// against every correspondence, and one thread per image replays the
// reference's adaptive loop over the round in order (best model on a strict
// count improvement, the required iteration count re-estimated from the
// inlier ratio) - so the chosen model and the iteration count are the
// sequential loop's. Rounds repeat until every image's loop has ended. The
// local refit (DLT over all inliers, a 2m x 12 Jacobi SVD with CTA-wide
// column dot products), the never-regress checks and the two Gauss-Newton
// polish rounds (pnp.rs:236-306) run with one CTA per image. All FP64.
#include <climits>
#include <cstdint>

#include "kernels.cuh"

namespace sfmba {

namespace {

constexpr int kPnpThreads = 128;
constexpr int kSample = 6;  // pnp.rs:221 (sample size of the 12-unknown DLT)
constexpr double kFmax = 1.79769313486231570815e308;

struct PQuat {
    double w, x, y, z;
};

struct PPose {
    PQuat q;
    double t[3];
};

__device__ __forceinline__ PQuat qmul(const PQuat &a, const PQuat &b) {
    return {a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z, a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y,
            a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x, a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w};
}

// R X + t with R the unit quaternion's rotation: v + 2w (u x v) + 2 u x (u x v).
__device__ __forceinline__ void ptransform(const PPose &p, const double *X, double out[3]) {
    const PQuat &q = p.q;
    const double tx = 2.0 * (q.y * X[2] - q.z * X[1]);
    const double ty = 2.0 * (q.z * X[0] - q.x * X[2]);
    const double tz = 2.0 * (q.x * X[1] - q.y * X[0]);
    out[0] = X[0] + q.w * tx + (q.y * tz - q.z * ty) + p.t[0];
    out[1] = X[1] + q.w * ty + (q.z * tx - q.x * tz) + p.t[1];
    out[2] = X[2] + q.w * tz + (q.x * ty - q.y * tx) + p.t[2];
}

// UnitQuaternion::from_scaled_axis: rotation by |v| about v; identity at 0.
__device__ __forceinline__ PQuat from_scaled_axis(const double v[3]) {
    const double th = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (th == 0.0) return {1.0, 0.0, 0.0, 0.0};
    const double s = sin(0.5 * th) / th;
    return {cos(0.5 * th), s * v[0], s * v[1], s * v[2]};
}

// Quaternion of a rotation matrix (row-major): from the trace when positive,
// else from the largest diagonal entry.
__device__ PQuat from_rotation_matrix(const double m[9]) {
    const double tr = m[0] + m[4] + m[8];
    if (tr > 0.0) {
        const double d = sqrt(tr + 1.0) * 2.0;
        return {0.25 * d, (m[7] - m[5]) / d, (m[2] - m[6]) / d, (m[3] - m[1]) / d};
    }
    if (m[0] > m[4] && m[0] > m[8]) {
        const double d = sqrt(1.0 + m[0] - m[4] - m[8]) * 2.0;
        return {(m[7] - m[5]) / d, 0.25 * d, (m[1] + m[3]) / d, (m[2] + m[6]) / d};
    }
    if (m[4] > m[8]) {
        const double d = sqrt(1.0 + m[4] - m[0] - m[8]) * 2.0;
        return {(m[2] - m[6]) / d, (m[1] + m[3]) / d, 0.25 * d, (m[5] + m[7]) / d};
    }
    const double d = sqrt(1.0 + m[8] - m[0] - m[4]) * 2.0;
    return {(m[3] - m[1]) / d, (m[2] + m[6]) / d, (m[5] + m[7]) / d, 0.25 * d};
}

// pnp.rs:132-141: reprojection distance in normalised coordinates,
// f64::MAX behind the camera.
__device__ __forceinline__ double pnp_residual(const PPose &p, const double *X, const double *uv) {
    double pc[3];
    ptransform(p, X, pc);
    if (pc[2] <= 1e-9) return kFmax;
    const double dx = pc[0] / pc[2] - uv[0], dy = pc[1] / pc[2] - uv[1];
    return sqrt(dx * dx + dy * dy);
}

// One Jacobi rotation of columns (p, q) from their Gram entries: returns
// false when they are already orthogonal to 1e-15 relative.
__device__ __forceinline__ bool jacobi_cs(double al, double be, double ga, double &c, double &s) {
    if (fabs(ga) <= 1e-15 * sqrt(al * be) || ga == 0.0) return false;
    const double zeta = (be - al) / (2.0 * ga);
    const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
    c = 1.0 / sqrt(1.0 + t * t);
    s = c * t;
    return true;
}

// One-sided (Hestenes) Jacobi SVD of the column-major m x n matrix a, one
// thread: cyclic sweeps over p < q until no rotation happens (at most 60).
// On return the columns of a are U Sigma, v (column-major n x n) is V and
// sv the singular values (column norms).
template <int M, int N>
__device__ void jacobi_svd_serial(double *a, double *v, double *sv) {
    for (int i = 0; i < N * N; ++i) v[i] = 0.0;
    for (int i = 0; i < N; ++i) v[i * N + i] = 1.0;
    for (int sweep = 0; sweep < 60; ++sweep) {
        bool rotated = false;
        for (int p = 0; p < N - 1; ++p)
            for (int q = p + 1; q < N; ++q) {
                double al = 0.0, be = 0.0, ga = 0.0;
                double *ap = a + p * M, *aq = a + q * M;
                for (int r = 0; r < M; ++r) {
                    al += ap[r] * ap[r];
                    be += aq[r] * aq[r];
                    ga += ap[r] * aq[r];
                }
                double c, s;
                if (!jacobi_cs(al, be, ga, c, s)) continue;
                rotated = true;
                for (int r = 0; r < M; ++r) {
                    const double x = ap[r], y = aq[r];
                    ap[r] = c * x - s * y;
                    aq[r] = s * x + c * y;
                }
                double *vp = v + p * N, *vq = v + q * N;
                for (int r = 0; r < N; ++r) {
                    const double x = vp[r], y = vq[r];
                    vp[r] = c * x - s * y;
                    vq[r] = s * x + c * y;
                }
            }
        if (!rotated) break;
    }
    for (int j = 0; j < N; ++j) {
        double s = 0.0;
        for (int r = 0; r < M; ++r) s += a[j * M + r] * a[j * M + r];
        sv[j] = sqrt(s);
    }
}

// The DLT rows of correspondence (X, uv) (pnp.rs:28-47) as rows r, r + 1 of
// the column-major matrix a with leading dimension ld.
__device__ __forceinline__ void dlt_rows(const double *X, const double *uv, double *a, int ld, int r) {
    const double x = X[0], y = X[1], z = X[2], u = uv[0], w = uv[1];
#pragma unroll
    for (int c = 0; c < 12; ++c) {
        a[c * ld + r] = 0.0;
        a[c * ld + r + 1] = 0.0;
    }
    a[0 * ld + r] = x; a[1 * ld + r] = y; a[2 * ld + r] = z; a[3 * ld + r] = 1.0;
    a[8 * ld + r] = -u * x; a[9 * ld + r] = -u * y; a[10 * ld + r] = -u * z; a[11 * ld + r] = -u;
    a[4 * ld + r + 1] = x; a[5 * ld + r + 1] = y; a[6 * ld + r + 1] = z; a[7 * ld + r + 1] = 1.0;
    a[8 * ld + r + 1] = -w * x; a[9 * ld + r + 1] = -w * y; a[10 * ld + r + 1] = -w * z; a[11 * ld + r + 1] = -w;
}

// pnp.rs:49-112 after the null vector p (3 x 4 row-major): rotation from the
// polar factor of p[:, :3] (sign fixed to det > 0), scale by projection,
// translation p[:, 3] / scale. False where the reference returns None.
__device__ bool pose_from_projection(const double p[12], PPose &out) {
    for (int c = 0; c < 12; ++c)
        if (!isfinite(p[c])) return false;
    double a[9], v[9], sv[3];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) a[c * 3 + r] = p[r * 4 + c];
    const double rb[9] = {p[0], p[1], p[2], p[4], p[5], p[6], p[8], p[9], p[10]};
    jacobi_svd_serial<3, 3>(a, v, sv);
    double R[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k) {
                const double u = sv[k] > 0.0 ? a[k * 3 + r] / sv[k] : 0.0;
                s += u * v[k * 3 + c];
            }
            R[r * 3 + c] = s;
        }
    const double det = R[0] * (R[4] * R[8] - R[5] * R[7]) - R[1] * (R[3] * R[8] - R[5] * R[6]) +
                       R[2] * (R[3] * R[7] - R[4] * R[6]);
    if (det < 0.0)
        for (int k = 0; k < 9; ++k) R[k] = -R[k];
    double num = 0.0, den = 0.0;
    for (int k = 0; k < 9; ++k) {
        num += rb[k] * R[k];
        den += R[k] * R[k];
    }
    if (den < 1e-12) return false;
    const double lambda = num / den;
    if (fabs(lambda) < 1e-12) return false;
    out.q = from_rotation_matrix(R);
    out.t[0] = p[3] / lambda;
    out.t[1] = p[7] / lambda;
    out.t[2] = p[11] / lambda;
    return true;
}

// Eigenvalues of a symmetric 3 x 3 matrix by cyclic Jacobi.
__device__ void sym3_eigenvalues(double m[9], double ev[3]) {
    for (int sweep = 0; sweep < 50; ++sweep) {
        const double off = m[1] * m[1] + m[2] * m[2] + m[5] * m[5];
        if (off == 0.0) break;
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                const double apq = m[p * 3 + q];
                if (apq == 0.0) continue;
                const double app = m[p * 3 + p], aqq = m[q * 3 + q];
                const double theta = (aqq - app) / (2.0 * apq);
                const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < 3; ++k) {
                    const double x = m[k * 3 + p], y = m[k * 3 + q];
                    m[k * 3 + p] = c * x - s * y;
                    m[k * 3 + q] = s * x + c * y;
                }
                for (int k = 0; k < 3; ++k) {
                    const double x = m[p * 3 + k], y = m[q * 3 + k];
                    m[p * 3 + k] = c * x - s * y;
                    m[q * 3 + k] = s * x + c * y;
                }
                m[p * 3 + q] = m[q * 3 + p] = 0.0;
            }
    }
    ev[0] = m[0];
    ev[1] = m[4];
    ev[2] = m[8];
}

// pnp.rs:115-130: smallest / largest covariance eigenvalue of the sample > 1e-3.
__device__ bool well_conditioned(const double *X, const long long *idx) {
    double c[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < kSample; ++i)
        for (int d = 0; d < 3; ++d) c[d] += X[3 * idx[i] + d];
    for (int d = 0; d < 3; ++d) c[d] /= kSample;
    double cov[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = 0; i < kSample; ++i) {
        double e[3];
        for (int k = 0; k < 3; ++k) e[k] = X[3 * idx[i] + k] - c[k];
        for (int r = 0; r < 3; ++r)
            for (int k = 0; k < 3; ++k) cov[r * 3 + k] += e[r] * e[k];
    }
    double ev[3];
    sym3_eigenvalues(cov, ev);
    const double lo = fmin(ev[0], fmin(ev[1], ev[2])), hi = fmax(ev[0], fmax(ev[1], ev[2]));
    if (hi < 1e-12) return false;
    return lo / hi > 1e-3;
}

// Per-image RANSAC state (ransac.rs:90-131).
struct PnpState {
    double best[8];      // pose of the best model (qw qx qy qz tx ty tz)
    long long count;     // its inlier count
    long long needed;    // required iterations (starts at max_iterations)
    long long iter;      // iterations run
    int have;            // a model has been found
    int done;            // the adaptive loop has ended
};

// Hypothesis t = round_base + h of image k: sample, conditioning, DLT.
__global__ void __launch_bounds__(kPnpThreads) k_pnp_hypotheses(const long long *off, const double *X,
                                                                const double *uv, const unsigned long long *raw,
                                                                int P, int B, long long round_base,
                                                                long long max_it, const PnpState *st,
                                                                double *models, unsigned char *valid) {
    const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (g >= (long long)P * B) return;
    const int k = (int)(g / B), h = (int)(g - (long long)k * B);
    const long long t = round_base + h;
    valid[g] = 0;
    if (st[k].done || t >= max_it) return;
    const long long n = off[k + 1] - off[k];
    const double *Xk = X + 3 * off[k], *uvk = uv + 2 * off[k];
    // Partial Fisher-Yates over the identity (ransac.rs:63-71), the swapped
    // positions held in a small map.
    long long mpos[2 * kSample], mval[2 * kSample];
    int nm = 0;
    auto get = [&](long long pos) {
        for (int e = 0; e < nm; ++e)
            if (mpos[e] == pos) return mval[e];
        return pos;
    };
    auto set = [&](long long pos, long long val) {
        for (int e = 0; e < nm; ++e)
            if (mpos[e] == pos) { mval[e] = val; return; }
        mpos[nm] = pos;
        mval[nm] = val;
        ++nm;
    };
    for (int i = 0; i < kSample; ++i) {
        const long long j = i + (long long)(raw[kSample * t + i] % (unsigned long long)(n - i));
        const long long vi = get(i), vj = get(j);
        set(i, vj);
        set(j, vi);
    }
    long long idx[kSample];
    for (int i = 0; i < kSample; ++i) idx[i] = get(i);
    if (!well_conditioned(Xk, idx)) return;
    double a[12 * 12], v[12 * 12], sv[12];
    for (int i = 0; i < kSample; ++i) dlt_rows(Xk + 3 * idx[i], uvk + 2 * idx[i], a, 12, 2 * i);
    jacobi_svd_serial<12, 12>(a, v, sv);
    int best = 0;
    for (int j = 1; j < 12; ++j)
        if (sv[j] < sv[best]) best = j;
    double p[12];
    for (int c = 0; c < 12; ++c) p[c] = v[best * 12 + c];
    PPose m;
    if (!pose_from_projection(p, m)) return;
    double *o = models + 8 * g;
    o[0] = m.q.w; o[1] = m.q.x; o[2] = m.q.y; o[3] = m.q.z;
    o[4] = m.t[0]; o[5] = m.t[1]; o[6] = m.t[2]; o[7] = 0.0;
    valid[g] = 1;
}

__device__ __forceinline__ PPose load_pose8(const double *o) {
    PPose m;
    m.q = {o[0], o[1], o[2], o[3]};
    m.t[0] = o[4]; m.t[1] = o[5]; m.t[2] = o[6];
    return m;
}

// Inlier count of every valid hypothesis, one warp each.
__global__ void __launch_bounds__(256) k_pnp_score(const long long *off, const double *X, const double *uv,
                                                   int P, int B, double thr, const double *models,
                                                   const unsigned char *valid, long long *counts) {
    const long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= (long long)P * B) return;
    if (!valid[w]) return;
    const int k = (int)(w / B);
    const long long s = off[k], e = off[k + 1];
    const PPose m = load_pose8(models + 8 * w);
    long long c = 0;
    for (long long i = s + lane; i < e; i += 32) c += pnp_residual(m, X + 3 * i, uv + 2 * i) < thr;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (lane == 0) counts[w] = c;
}

// The reference's adaptive loop over one round, in order (ransac.rs:95-128).
__global__ void k_pnp_select(const long long *off, int P, int B, long long round_base, long long max_it,
                             const double *models, const unsigned char *valid, const long long *counts,
                             PnpState *st, int *active) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P) return;
    PnpState &S = st[k];
    if (S.done) return;
    const long long n = off[k + 1] - off[k];
    for (int h = 0; h < B; ++h) {
        const long long limit = min(max_it, max(S.needed, 1LL));
        if (S.iter >= limit) { S.done = 1; break; }
        const long long t = round_base + h;
        S.iter = t + 1;
        const long long g = (long long)k * B + h;
        if (!valid[g]) continue;
        const long long c = counts[g];
        if (!S.have || c > S.count) {
            S.have = 1;
            S.count = c;
            for (int q = 0; q < 8; ++q) S.best[q] = models[8 * g + q];
            const double ratio = fmax((double)c / (double)n, 1e-6);
            // f64::powi(6) as binary powering: x^2 * (x^2)^2.
            const double r2 = ratio * ratio;
            const double denom = log(fmax(1.0 - r2 * (r2 * r2), 1e-12));
            if (denom < 0.0) {
                const double est = ceil(log(1.0 - 0.999) / denom);
                if (isfinite(est) && est >= 0.0) S.needed = min((long long)est, max_it);
            }
        }
    }
    const long long limit = min(max_it, max(S.needed, 1LL));
    if (!S.done && S.iter >= limit) S.done = 1;
    if (!S.done) {
        atomicAdd(active, 1);
        atomicMax(active + 1, (int)min(limit - S.iter, (long long)INT_MAX));  // iterations still to run
    }
}

// FP64 block sum (kPnpThreads threads) of NV values per thread into out (all threads).
template <int NV>
__device__ void cta_sum(double (&v)[NV], double (*sh)[kPnpThreads / 32], double *out) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        double x = v[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) sh[q][w] = x;
    }
    __syncthreads();
    for (int q = threadIdx.x; q < NV; q += blockDim.x) {
        double s = 0.0;
        for (int ww = 0; ww < kPnpThreads / 32; ++ww) s += sh[q][ww];
        out[q] = s;
    }
    __syncthreads();
}

__device__ long long cta_count(long long c, long long *sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = c;
    __syncthreads();
    long long s = 0;
    for (int w = 0; w < kPnpThreads / 32; ++w) s += sh[w];
    __syncthreads();
    return s;
}

// Partial-pivot LU solve of a 6 x 6 system (first largest pivot; a zero
// pivot skips its column); false when U has a zero diagonal.
__device__ bool lu_solve6(double a[36], const double b[6], double x[6]) {
    int perm[6] = {0, 1, 2, 3, 4, 5};
    for (int i = 0; i < 6; ++i) {
        int piv = i;
        for (int r = i + 1; r < 6; ++r)
            if (fabs(a[r * 6 + i]) > fabs(a[piv * 6 + i])) piv = r;
        if (a[piv * 6 + i] == 0.0) continue;
        if (piv != i) {
            for (int c = 0; c < 6; ++c) {
                const double tmp = a[i * 6 + c];
                a[i * 6 + c] = a[piv * 6 + c];
                a[piv * 6 + c] = tmp;
            }
            const int tp = perm[i];
            perm[i] = perm[piv];
            perm[piv] = tp;
        }
        for (int r = i + 1; r < 6; ++r) {
            const double f = a[r * 6 + i] / a[i * 6 + i];
            a[r * 6 + i] = f;
            for (int c = i + 1; c < 6; ++c) a[r * 6 + c] -= f * a[i * 6 + c];
        }
    }
    double y[6];
    for (int r = 0; r < 6; ++r) {
        double s = b[perm[r]];
        for (int c = 0; c < r; ++c) s -= a[r * 6 + c] * y[c];
        y[r] = s;
    }
    for (int r = 5; r >= 0; --r) {
        if (a[r * 6 + r] == 0.0) return false;
        double s = y[r];
        for (int c = r + 1; c < 6; ++c) s -= a[r * 6 + c] * x[c];
        x[r] = s / a[r * 6 + r];
    }
    return true;
}

struct CtaShared {
    double red[27][kPnpThreads / 32];
    double sums[27];
    long long cnt[kPnpThreads / 32];
    double V[144];
    double gram[3];
    double cs[2];
    int flag;
    PPose pose;
};

// pnp.rs:151-206 by one CTA: `iterations` Gauss-Newton steps over the
// correspondences [0, n) of (X, uv) with mask[i] != 0 (mask NULL: all).
// Upper triangle of J^T J (21) and J^T r (6) reduced per step; thread 0
// solves and updates. sh.pose holds the pose in and out.
__device__ void cta_refine_gn(const double *X, const double *uv, const unsigned char *mask, long long n,
                              int iterations, CtaShared &sh) {
    for (int it = 0; it < iterations; ++it) {
        double v[27];
#pragma unroll
        for (int q = 0; q < 27; ++q) v[q] = 0.0;
        const PPose pose = sh.pose;
        for (long long i = threadIdx.x; i < n; i += blockDim.x) {
            if (mask && !mask[i]) continue;
            double pc[3];
            ptransform(pose, X + 3 * i, pc);
            if (pc[2] <= 1e-9) continue;
            const double iz = 1.0 / pc[2], x = pc[0] * iz, y = pc[1] * iz;
            const double dr[3][3] = {{0.0, pc[2], -pc[1]}, {-pc[2], 0.0, pc[0]}, {pc[1], -pc[0], 0.0}};
            double J[2][6];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                J[0][c] = iz * dr[0][c] - x * iz * dr[2][c];
                J[1][c] = iz * dr[1][c] - y * iz * dr[2][c];
            }
            J[0][3] = iz; J[0][4] = 0.0; J[0][5] = -x * iz;
            J[1][3] = 0.0; J[1][4] = iz; J[1][5] = -y * iz;
            const double r0 = x - uv[2 * i], r1 = y - uv[2 * i + 1];
            int e = 0;
#pragma unroll
            for (int a = 0; a < 6; ++a)
#pragma unroll
                for (int b = a; b < 6; ++b) v[e++] += J[0][a] * J[0][b] + J[1][a] * J[1][b];
#pragma unroll
            for (int a = 0; a < 6; ++a) v[21 + a] += J[0][a] * r0 + J[1][a] * r1;
        }
        cta_sum<27>(v, sh.red, sh.sums);
        if (threadIdx.x == 0) {
            double A[36], rhs[6], d[6];
            int e = 0;
            for (int a = 0; a < 6; ++a)
                for (int b = a; b < 6; ++b) A[a * 6 + b] = A[b * 6 + a] = sh.sums[e++];
            for (int a = 0; a < 6; ++a) {
                A[a * 6 + a] += 1e-9;
                rhs[a] = -sh.sums[21 + a];
            }
            bool ok = lu_solve6(A, rhs, d);
            for (int a = 0; a < 6 && ok; ++a) ok = isfinite(d[a]);
            sh.flag = ok;
            if (ok) {
                PPose p = sh.pose;
                p.q = qmul(from_scaled_axis(d), p.q);
                p.t[0] += d[3];
                p.t[1] += d[4];
                p.t[2] += d[5];
                sh.pose = p;
            }
        }
        __syncthreads();
        if (!sh.flag) break;
    }
}

// Inlier count of sh.pose (and the mask, when given) by one CTA.
__device__ long long cta_inliers(const double *X, const double *uv, long long n, double thr, unsigned char *mask,
                                 CtaShared &sh) {
    const PPose p = sh.pose;
    long long c = 0;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) {
        const bool ok = pnp_residual(p, X + 3 * i, uv + 2 * i) < thr;
        if (mask) mask[i] = ok;
        c += ok;
    }
    return cta_count(c, sh.cnt);
}

// DLT over the correspondences with inl[i] != 0 (m of them, m >= 6) by one
// CTA: the 2m x 12 system in scratch a (column-major), reduced to its 12 x 12
// R factor by Householder reflections (column norms and the 11 column dot
// products of each step reduced over the CTA), then thread 0 takes the
// one-sided Jacobi SVD of R (A and R share their right singular vectors) —
// the same steps as the oracle's restatement. Pose in sh.pose; false where
// pnp_dlt returns None.
__device__ bool cta_dlt(const double *X, const double *uv, const unsigned char *inl, long long n, long long m,
                        double *a, CtaShared &sh, long long *slot) {
    const long long M = 2 * m;
    // Rows in input order: slot[i] = rank of i among the inliers.
    if (threadIdx.x == 0) {
        long long r = 0;
        for (long long i = 0; i < n; ++i) slot[i] = inl[i] ? r++ : -1;
    }
    __syncthreads();
    for (long long i = threadIdx.x; i < n; i += blockDim.x)
        if (slot[i] >= 0) dlt_rows(X + 3 * i, uv + 2 * i, a, (int)M, (int)(2 * slot[i]));
    __syncthreads();
    // sh.V holds R (column-major 12 x 12) as it is produced; a 12 x 12
    // system (6 inliers) is its own R, as in the oracle.
    for (int q = threadIdx.x; q < 144; q += blockDim.x) sh.V[q] = M > 12 ? 0.0 : a[q];
    __syncthreads();
    for (int k = 0; k < 12 && M > 12; ++k) {
        double *x = a + k * M;
        double g[1] = {0.0};
        for (long long r = k + threadIdx.x; r < M; r += blockDim.x) g[0] += x[r] * x[r];
        cta_sum<1>(g, sh.red, sh.gram);
        const double s = sh.gram[0], x0 = x[k];
        const double nrm = sqrt(s);
        const double alpha = x0 >= 0.0 ? -nrm : nrm;
        const double v0 = x0 - alpha;
        const double beta = s - x0 * x0 + v0 * v0;
        __syncthreads();  // every thread has read x[k]
        if (threadIdx.x == 0) {
            x[k] = v0;
            sh.V[k * 12 + k] = beta > 0.0 ? alpha : x0;
        }
        __syncthreads();
        if (beta > 0.0 && k < 11) {
            double d[11];
#pragma unroll
            for (int j = 0; j < 11; ++j) d[j] = 0.0;
            for (long long r = k + threadIdx.x; r < M; r += blockDim.x) {
                const double vr = x[r];
#pragma unroll
                for (int j = 0; j < 11; ++j)
                    if (k + 1 + j < 12) d[j] += vr * a[(k + 1 + j) * M + r];
            }
            cta_sum<11>(d, sh.red, sh.sums);
            for (long long r = k + threadIdx.x; r < M; r += blockDim.x) {
                const double vr = x[r];
#pragma unroll
                for (int j = 0; j < 11; ++j)
                    if (k + 1 + j < 12) a[(k + 1 + j) * M + r] -= (2.0 * sh.sums[j] / beta) * vr;
            }
            __syncthreads();
        }
        if (threadIdx.x == 0)
            for (int j = k + 1; j < 12; ++j) sh.V[j * 12 + k] = a[j * M + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double R[144], V[144], sv[12];
        for (int q = 0; q < 144; ++q) R[q] = sh.V[q];
        jacobi_svd_serial<12, 12>(R, V, sv);
        int best = 0;
        for (int j = 1; j < 12; ++j)
            if (sv[j] < sv[best]) best = j;
        double p[12];
        for (int c = 0; c < 12; ++c) p[c] = V[best * 12 + c];
        PPose out;
        sh.flag = pose_from_projection(p, out);
        if (sh.flag) sh.pose = out;
    }
    __syncthreads();
    return sh.flag != 0;
}

// pnp.rs:221-306 after RANSAC, one CTA per image: inlier mask of the best
// model, the local refit kept only if it loses no inliers, two never-regress
// Gauss-Newton polish rounds of 10 iterations over the inliers.
__global__ void __launch_bounds__(kPnpThreads) k_pnp_finish(const long long *off, const double *X,
                                                            const double *uv, double thr, const PnpState *st,
                                                            double *dlt_scratch, long long *slot_scratch,
                                                            unsigned char *mask_a, unsigned char *mask_b,
                                                            double *poses_out, int *found_out) {
    __shared__ CtaShared sh;
    const int k = blockIdx.x;
    const long long s = off[k], n = off[k + 1] - s;
    const double *Xk = X + 3 * s, *uvk = uv + 2 * s;
    unsigned char *best_mask = mask_a + s, *trial = mask_b + s;
    if (threadIdx.x == 0) found_out[k] = 0;
    const PnpState &S = st[k];
    if (!S.have || S.count < kSample) {  // pnp.rs:235-237: None
        for (long long i = threadIdx.x; i < n; i += blockDim.x) best_mask[i] = 0;
        return;
    }
    if (threadIdx.x == 0) sh.pose = load_pose8(S.best);
    __syncthreads();
    long long best_count = cta_inliers(Xk, uvk, n, thr, best_mask, sh);
    PPose best_pose = sh.pose;
    // LO refit (pnp.rs:246-268).
    if (cta_dlt(Xk, uvk, best_mask, n, best_count, dlt_scratch + 24 * s, sh, slot_scratch + s)) {
        const long long c = cta_inliers(Xk, uvk, n, thr, trial, sh);
        if (c >= best_count) {
            best_count = c;
            best_pose = sh.pose;
            for (long long i = threadIdx.x; i < n; i += blockDim.x) best_mask[i] = trial[i];
        }
    }
    __syncthreads();
    // Gauss-Newton polish (pnp.rs:280-306).
    for (int round = 0; round < 2; ++round) {
        long long m = 0;
        for (long long i = threadIdx.x; i < n; i += blockDim.x) m += best_mask[i];
        m = cta_count(m, sh.cnt);
        if (m < kSample) break;
        if (threadIdx.x == 0) sh.pose = best_pose;
        __syncthreads();
        cta_refine_gn(Xk, uvk, best_mask, n, 10, sh);
        const long long c = cta_inliers(Xk, uvk, n, thr, trial, sh);
        if (c < best_count) break;
        const bool converged = c == best_count;
        best_pose = sh.pose;
        best_count = c;
        for (long long i = threadIdx.x; i < n; i += blockDim.x) best_mask[i] = trial[i];
        __syncthreads();
        if (converged) break;
    }
    if (threadIdx.x == 0) {
        double *o = poses_out + 7 * (size_t)k;
        o[0] = best_pose.q.w; o[1] = best_pose.q.x; o[2] = best_pose.q.y; o[3] = best_pose.q.z;
        o[4] = best_pose.t[0]; o[5] = best_pose.t[1]; o[6] = best_pose.t[2];
        found_out[k] = 1;
    }
}

// refine_pose_gauss_newton for every pose, one CTA each.
__global__ void __launch_bounds__(kPnpThreads) k_refine_pose_gn(const long long *off, const double *X,
                                                                const double *uv, int iterations,
                                                                double *poses) {
    __shared__ CtaShared sh;
    const int k = blockIdx.x;
    const long long s = off[k], n = off[k + 1] - s;
    double *o = poses + 7 * (size_t)k;
    if (threadIdx.x == 0) sh.pose = load_pose8(o);
    __syncthreads();
    cta_refine_gn(X + 3 * s, uv + 2 * s, nullptr, n, iterations, sh);
    if (threadIdx.x == 0) {
        const PPose p = sh.pose;
        o[0] = p.q.w; o[1] = p.q.x; o[2] = p.q.y; o[3] = p.q.z;
        o[4] = p.t[0]; o[5] = p.t[1]; o[6] = p.t[2];
    }
}

// ransac.rs:88-93 and pnp.rs:217-219: fewer than 6 correspondences (or no
// iterations) end the loop before it starts, with no model.
__global__ void k_pnp_init(const long long *off, int P, long long max_it, PnpState *st) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P) return;
    PnpState &S = st[k];
    for (int q = 0; q < 8; ++q) S.best[q] = 0.0;
    S.count = 0;
    S.needed = max_it;
    S.iter = 0;
    S.have = 0;
    S.done = (off[k + 1] - off[k] < kSample || max_it <= 0) ? 1 : 0;
}

}  // namespace

size_t pnp_state_bytes() { return sizeof(PnpState); }

void launch_pnp_init(const PnpBufs &q, cudaStream_t s) {
    if (q.P == 0) return;
    k_pnp_init<<<div_up(q.P, 128), 128, 0, s>>>(q.off, q.P, q.max_it, (PnpState *)q.state);
    SFMBA_LAUNCH_CHECK();
}

void launch_pnp_round(const PnpBufs &q, long long round_base, cudaStream_t s) {
    const long long total = (long long)q.P * q.B;
    k_pnp_hypotheses<<<div_up(total, kPnpThreads), kPnpThreads, 0, s>>>(
        q.off, q.X, q.uv, q.raw, q.P, q.B, round_base, q.max_it, (const PnpState *)q.state, q.models, q.valid);
    SFMBA_LAUNCH_CHECK();
    k_pnp_score<<<div_up(total * 32, 256), 256, 0, s>>>(q.off, q.X, q.uv, q.P, q.B, q.thr, q.models, q.valid,
                                                        q.counts);
    SFMBA_LAUNCH_CHECK();
    SFMBA_CUDA(cudaMemsetAsync(q.active, 0, 2 * sizeof(int), s));
    k_pnp_select<<<div_up(q.P, 128), 128, 0, s>>>(q.off, q.P, q.B, round_base, q.max_it, q.models, q.valid,
                                                  q.counts, (PnpState *)q.state, q.active);
    SFMBA_LAUNCH_CHECK();
}

void launch_pnp_finish(const PnpBufs &q, cudaStream_t s) {
    if (q.P == 0) return;
    k_pnp_finish<<<q.P, kPnpThreads, 0, s>>>(q.off, q.X, q.uv, q.thr, (const PnpState *)q.state, q.dlt_scratch,
                                             q.slot_scratch, q.mask, q.mask_trial, q.poses, q.found);
    SFMBA_LAUNCH_CHECK();
}

void launch_pnp_iterations(const PnpBufs &q, long long *iters, cudaStream_t s) {
    // iterations run per image: PnpState::iter, gathered with a strided copy.
    if (q.P == 0) return;
    SFMBA_CUDA(cudaMemcpy2DAsync(iters, sizeof(long long), (const char *)q.state + offsetof(PnpState, iter),
                                 sizeof(PnpState), sizeof(long long), q.P, cudaMemcpyDeviceToDevice, s));
}

void launch_refine_pose_gn(const long long *off, const double *X, const double *uv, int P, int iterations,
                           double *poses, cudaStream_t s) {
    if (P == 0) return;
    k_refine_pose_gn<<<P, kPnpThreads, 0, s>>>(off, X, uv, iterations, poses);
    SFMBA_LAUNCH_CHECK();
}

}  // namespace sfmba
