// TEST INFRASTRUCTURE ONLY - CPU FP64 restatement of sfmtory's PnP camera
// registration (crates/sfm-geometry/src/pnp.rs, ransac.rs, linalg.rs), the
// checker for the GPU `sfmba_pnp_ransac_batched` /
// `sfmba_refine_pose_gauss_newton_batched` entry points. Never linked into
// the product library.
//
// Third-party arithmetic the reference takes from nalgebra 0.33 (SVD,
// symmetric eigenvalues, LU, quaternion construction) is written here from
// the mathematics: one-sided (Hestenes) Jacobi SVD, cyclic Jacobi
// eigenvalues, partial-pivot LU, the trace/major-diagonal quaternion of a
// rotation matrix. Parity with the Rust binary is pinned only through the
// reference's known-answer test (pnp.rs:311-339); the singular vectors and
// eigenvalues agree with any correct SVD/eigen-solver up to rounding and
// the null vector's sign, which the DLT normalises away.
#include "../include/sfmba.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

struct Quat {
    double w, x, y, z;
};

Quat qmul(const Quat &a, const Quat &b) {
    return {a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z, a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y,
            a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x, a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w};
}

// v' = v + 2 w (u x v) + 2 u x (u x v) for the unit quaternion (w, u).
void qrot(const Quat &q, const double v[3], double out[3]) {
    const double tx = 2.0 * (q.y * v[2] - q.z * v[1]);
    const double ty = 2.0 * (q.z * v[0] - q.x * v[2]);
    const double tz = 2.0 * (q.x * v[1] - q.y * v[0]);
    out[0] = v[0] + q.w * tx + (q.y * tz - q.z * ty);
    out[1] = v[1] + q.w * ty + (q.z * tx - q.x * tz);
    out[2] = v[2] + q.w * tz + (q.x * ty - q.y * tx);
}

// UnitQuaternion::from_scaled_axis: angle |v| about v / |v|; zero -> identity.
Quat from_scaled_axis(const double v[3]) {
    const double th = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (th == 0.0) return {1.0, 0.0, 0.0, 0.0};
    const double s = std::sin(0.5 * th) / th;
    return {std::cos(0.5 * th), s * v[0], s * v[1], s * v[2]};
}

// Quaternion of a rotation matrix (row-major m): from the trace when it is
// positive, else from the largest diagonal entry.
Quat from_rotation_matrix(const double m[9]) {
    const double tr = m[0] + m[4] + m[8];
    if (tr > 0.0) {
        const double d = std::sqrt(tr + 1.0) * 2.0;
        return {0.25 * d, (m[7] - m[5]) / d, (m[2] - m[6]) / d, (m[3] - m[1]) / d};
    }
    if (m[0] > m[4] && m[0] > m[8]) {
        const double d = std::sqrt(1.0 + m[0] - m[4] - m[8]) * 2.0;
        return {(m[7] - m[5]) / d, 0.25 * d, (m[1] + m[3]) / d, (m[2] + m[6]) / d};
    }
    if (m[4] > m[8]) {
        const double d = std::sqrt(1.0 + m[4] - m[0] - m[8]) * 2.0;
        return {(m[2] - m[6]) / d, (m[1] + m[3]) / d, 0.25 * d, (m[5] + m[7]) / d};
    }
    const double d = std::sqrt(1.0 + m[8] - m[0] - m[4]) * 2.0;
    return {(m[3] - m[1]) / d, (m[2] + m[6]) / d, (m[5] + m[7]) / d, 0.25 * d};
}

struct Pose {
    Quat q;
    double t[3];
};

void transform(const Pose &p, const double X[3], double out[3]) {
    qrot(p.q, X, out);
    out[0] += p.t[0];
    out[1] += p.t[1];
    out[2] += p.t[2];
}

// One-sided Jacobi SVD of the m x n column-major matrix a (m >= n): on return
// the columns of a are U Sigma, v (n x n, column-major) holds V and sv the
// column norms (singular values). Cyclic sweeps over (p < q) until no
// rotation is larger than the relative threshold 1e-15, at most 60 sweeps.
void jacobi_svd(std::vector<double> &a, int m, int n, std::vector<double> &v, std::vector<double> &sv) {
    v.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) v[(size_t)i * n + i] = 1.0;
    for (int sweep = 0; sweep < 60; ++sweep) {
        bool rotated = false;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                double al = 0.0, be = 0.0, ga = 0.0;
                double *ap = &a[(size_t)p * m], *aq = &a[(size_t)q * m];
                for (int r = 0; r < m; ++r) {
                    al += ap[r] * ap[r];
                    be += aq[r] * aq[r];
                    ga += ap[r] * aq[r];
                }
                if (std::fabs(ga) <= 1e-15 * std::sqrt(al * be) || ga == 0.0) continue;
                rotated = true;
                const double zeta = (be - al) / (2.0 * ga);
                const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
                const double c = 1.0 / std::sqrt(1.0 + t * t), s = c * t;
                for (int r = 0; r < m; ++r) {
                    const double x = ap[r], y = aq[r];
                    ap[r] = c * x - s * y;
                    aq[r] = s * x + c * y;
                }
                double *vp = &v[(size_t)p * n], *vq = &v[(size_t)q * n];
                for (int r = 0; r < n; ++r) {
                    const double x = vp[r], y = vq[r];
                    vp[r] = c * x - s * y;
                    vq[r] = s * x + c * y;
                }
            }
        if (!rotated) break;
    }
    sv.assign(n, 0.0);
    for (int j = 0; j < n; ++j) {
        double s = 0.0;
        for (int r = 0; r < m; ++r) s += a[(size_t)j * m + r] * a[(size_t)j * m + r];
        sv[j] = std::sqrt(s);
    }
}

// Householder QR of the column-major m x n matrix a (m > n), returning the
// n x n upper-triangular R column-major: column k is reflected by
// v = x - alpha e1 with alpha = -sign(x0) |x| (x0 = 0 counts as positive).
// A and R have the same right singular vectors.
void householder_r(std::vector<double> &a, int m, int n, std::vector<double> &r) {
    r.assign((size_t)n * n, 0.0);
    for (int k = 0; k < n; ++k) {
        double *x = &a[(size_t)k * m];
        double s = 0.0;
        for (int i = k; i < m; ++i) s += x[i] * x[i];
        const double nrm = std::sqrt(s), x0 = x[k];
        const double alpha = x0 >= 0.0 ? -nrm : nrm;
        const double v0 = x0 - alpha;
        const double beta = s - x0 * x0 + v0 * v0;  // v.v
        x[k] = v0;
        if (beta > 0.0)
            for (int j = k + 1; j < n; ++j) {
                double *y = &a[(size_t)j * m];
                double d = 0.0;
                for (int i = k; i < m; ++i) d += x[i] * y[i];
                const double f = 2.0 * d / beta;
                for (int i = k; i < m; ++i) y[i] -= f * x[i];
            }
        r[(size_t)k * n + k] = beta > 0.0 ? alpha : x0;
        for (int j = k + 1; j < n; ++j) r[(size_t)j * n + k] = a[(size_t)j * m + k];
    }
}

// linalg.rs:11-20 (null_space_vector): the right singular vector of the
// smallest singular value (first one on ties). Rows of the 2n x 12 system
// of pnp.rs:28-47; a taller system is first reduced to its 12 x 12 R factor.
bool dlt_null_vector(const double *X, const double *uv, const long *idx, long n, double out[12]) {
    const int m = (int)(2 * n);
    std::vector<double> a((size_t)m * 12, 0.0), v, sv;
    auto A = [&](int r, int c) -> double & { return a[(size_t)c * m + r]; };
    for (long i = 0; i < n; ++i) {
        const long k = idx ? idx[i] : i;
        const double x = X[3 * k], y = X[3 * k + 1], z = X[3 * k + 2], u = uv[2 * k], w = uv[2 * k + 1];
        const int r0 = (int)(2 * i), r1 = r0 + 1;
        A(r0, 0) = x; A(r0, 1) = y; A(r0, 2) = z; A(r0, 3) = 1.0;
        A(r0, 8) = -u * x; A(r0, 9) = -u * y; A(r0, 10) = -u * z; A(r0, 11) = -u;
        A(r1, 4) = x; A(r1, 5) = y; A(r1, 6) = z; A(r1, 7) = 1.0;
        A(r1, 8) = -w * x; A(r1, 9) = -w * y; A(r1, 10) = -w * z; A(r1, 11) = -w;
    }
    if (m > 12) {
        std::vector<double> r;
        householder_r(a, m, 12, r);
        jacobi_svd(r, 12, 12, v, sv);
    } else {
        jacobi_svd(a, m, 12, v, sv);
    }
    int best = 0;
    for (int j = 1; j < 12; ++j)
        if (sv[j] < sv[best]) best = j;
    for (int c = 0; c < 12; ++c) out[c] = v[(size_t)best * 12 + c];
    for (int c = 0; c < 12; ++c)
        if (!std::isfinite(out[c])) return false;
    return true;
}

// pnp.rs:22-113 (pnp_dlt) over the correspondences idx (NULL: all n).
bool pnp_dlt(const double *X, const double *uv, const long *idx, long n, Pose &out) {
    if (n < 6) return false;
    double p[12];
    if (!dlt_null_vector(X, uv, idx, n, p)) return false;
    // r_block = p[:, :3]; candidate = U V^T of its SVD (the orthogonal polar
    // factor), negated if its determinant is negative.
    std::vector<double> a(9), v, sv;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) a[(size_t)c * 3 + r] = p[r * 4 + c];
    const double rb[9] = {p[0], p[1], p[2], p[4], p[5], p[6], p[8], p[9], p[10]};
    jacobi_svd(a, 3, 3, v, sv);
    double R[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k) {
                const double u = sv[k] > 0.0 ? a[(size_t)k * 3 + r] / sv[k] : 0.0;
                s += u * v[(size_t)k * 3 + c];
            }
            R[r * 3 + c] = s;
        }
    const double det = R[0] * (R[4] * R[8] - R[5] * R[7]) - R[1] * (R[3] * R[8] - R[5] * R[6]) +
                       R[2] * (R[3] * R[7] - R[4] * R[6]);
    if (det < 0.0)
        for (double &x : R) x = -x;
    double num = 0.0, den = 0.0;
    for (int k = 0; k < 9; ++k) {
        num += rb[k] * R[k];
        den += R[k] * R[k];
    }
    if (den < 1e-12) return false;
    const double lambda = num / den;
    if (std::fabs(lambda) < 1e-12) return false;
    out.q = from_rotation_matrix(R);
    out.t[0] = p[3] / lambda;
    out.t[1] = p[7] / lambda;
    out.t[2] = p[11] / lambda;
    return true;
}

// Eigenvalues of a symmetric 3x3 matrix (cyclic Jacobi).
void sym3_eigenvalues(double m[9], double ev[3]) {
    for (int sweep = 0; sweep < 50; ++sweep) {
        const double off = m[1] * m[1] + m[2] * m[2] + m[5] * m[5];
        if (off == 0.0) break;
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                const double apq = m[p * 3 + q];
                if (apq == 0.0) continue;
                const double app = m[p * 3 + p], aqq = m[q * 3 + q];
                const double theta = (aqq - app) / (2.0 * apq);
                const double t = (theta >= 0.0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < 3; ++k) {  // columns p, q
                    const double x = m[k * 3 + p], y = m[k * 3 + q];
                    m[k * 3 + p] = c * x - s * y;
                    m[k * 3 + q] = s * x + c * y;
                }
                for (int k = 0; k < 3; ++k) {  // rows p, q
                    const double x = m[p * 3 + k], y = m[q * 3 + k];
                    m[p * 3 + k] = c * x - s * y;
                    m[q * 3 + k] = s * x + c * y;
                }
                m[p * 3 + q] = m[q * 3 + p] = 0.0;
            }
    }
    ev[0] = m[0]; ev[1] = m[4]; ev[2] = m[8];
}

// pnp.rs:115-130 (is_well_conditioned_for_dlt).
bool well_conditioned(const double *X, const long *idx, int n) {
    double c[3] = {0, 0, 0};
    for (int i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) c[d] += X[3 * idx[i] + d];
    for (double &x : c) x /= n;
    double cov[9] = {0};
    for (int i = 0; i < n; ++i) {
        double d[3];
        for (int k = 0; k < 3; ++k) d[k] = X[3 * idx[i] + k] - c[k];
        for (int r = 0; r < 3; ++r)
            for (int k = 0; k < 3; ++k) cov[r * 3 + k] += d[r] * d[k];
    }
    double ev[3];
    sym3_eigenvalues(cov, ev);
    const double lo = std::min(ev[0], std::min(ev[1], ev[2])), hi = std::max(ev[0], std::max(ev[1], ev[2]));
    if (hi < 1e-12) return false;
    return lo / hi > 1e-3;
}

// pnp.rs:132-141 (reprojection_residual), normalised coordinates.
double residual(const Pose &p, const double *X, const double *uv) {
    double pc[3];
    transform(p, X, pc);
    if (pc[2] <= 1e-9) return 1.79769313486231570815e308;  // f64::MAX
    const double dx = pc[0] / pc[2] - uv[0], dy = pc[1] / pc[2] - uv[1];
    return std::sqrt(dx * dx + dy * dy);
}

// Partial-pivot LU solve of the 6x6 system a x = b (pivot: first largest
// magnitude in the column; a zero pivot skips the column). False when a
// diagonal of U is zero.
bool lu_solve6(double a[36], double b[6], double x[6]) {
    int perm[6] = {0, 1, 2, 3, 4, 5};
    for (int i = 0; i < 6; ++i) {
        int piv = i;
        for (int r = i + 1; r < 6; ++r)
            if (std::fabs(a[r * 6 + i]) > std::fabs(a[piv * 6 + i])) piv = r;
        if (a[piv * 6 + i] == 0.0) continue;
        if (piv != i) {
            for (int c = 0; c < 6; ++c) std::swap(a[i * 6 + c], a[piv * 6 + c]);
            std::swap(perm[i], perm[piv]);
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

// pnp.rs:151-206 (refine_pose_gauss_newton) over the correspondences idx
// (NULL: all n).
Pose refine_gn(const Pose &init, const double *X, const double *uv, const long *idx, long n, int iterations) {
    Pose pose = init;
    for (int it = 0; it < iterations; ++it) {
        double jtj[36] = {0}, jtr[6] = {0};
        for (long i = 0; i < n; ++i) {
            const long k = idx ? idx[i] : i;
            double pc[3];
            transform(pose, X + 3 * k, pc);
            if (pc[2] <= 1e-9) continue;
            const double iz = 1.0 / pc[2], x = pc[0] * iz, y = pc[1] * iz;
            // d(pc)/d(rot) = -skew(pc) (columns), d(pc)/d(t) = I.
            const double dr[3][3] = {{0.0, pc[2], -pc[1]}, {-pc[2], 0.0, pc[0]}, {pc[1], -pc[0], 0.0}};
            double J[2][6] = {{0}};
            for (int c = 0; c < 3; ++c) {
                const double dx = dr[0][c], dy = dr[1][c], dz = dr[2][c];
                J[0][c] = iz * dx - x * iz * dz;
                J[1][c] = iz * dy - y * iz * dz;
            }
            J[0][3] = iz;
            J[1][4] = iz;
            J[0][5] = -x * iz;
            J[1][5] = -y * iz;
            const double r[2] = {x - uv[2 * k], y - uv[2 * k + 1]};
            for (int a = 0; a < 6; ++a) {
                for (int b = 0; b < 6; ++b) jtj[a * 6 + b] += J[0][a] * J[0][b] + J[1][a] * J[1][b];
                jtr[a] += J[0][a] * r[0] + J[1][a] * r[1];
            }
        }
        for (int d = 0; d < 6; ++d) jtj[d * 6 + d] += 1e-9;
        double rhs[6], delta[6];
        for (int d = 0; d < 6; ++d) rhs[d] = -jtr[d];
        if (!lu_solve6(jtj, rhs, delta)) break;
        bool finite = true;
        for (double v : delta) finite = finite && std::isfinite(v);
        if (!finite) break;
        pose.q = qmul(from_scaled_axis(delta), pose.q);
        pose.t[0] += delta[3];
        pose.t[1] += delta[4];
        pose.t[2] += delta[5];
    }
    return pose;
}

struct Xorshift64 {  // ransac.rs:43-60
    uint64_t s;
    explicit Xorshift64(uint64_t seed) : s(seed | 1) {}
    uint64_t next() {
        uint64_t x = s;
        x ^= x << 13;
        x ^= x >> 7;
        x ^= x << 17;
        s = x;
        return x;
    }
    long below(long bound) { return (long)(next() % (uint64_t)bound); }
};

long count_inliers(const Pose &p, const double *X, const double *uv, long n, double thr, uint8_t *mask) {
    long c = 0;
    for (long i = 0; i < n; ++i) {
        const bool ok = residual(p, X + 3 * i, uv + 2 * i) < thr;
        if (mask) mask[i] = ok;
        c += ok;
    }
    return c;
}

Pose load(const double *p7) {
    Pose p;
    p.q = {p7[0], p7[1], p7[2], p7[3]};
    p.t[0] = p7[4]; p.t[1] = p7[5]; p.t[2] = p7[6];
    return p;
}

void store(const Pose &p, double *p7) {
    p7[0] = p.q.w; p7[1] = p.q.x; p7[2] = p.q.y; p7[3] = p.q.z;
    p7[4] = p.t[0]; p7[5] = p.t[1]; p7[6] = p.t[2];
}

}  // namespace

extern "C" {

// pnp.rs:151-206 for each pose k over its correspondences
// [offsets[k], offsets[k+1]). poses [num][7] (qw qx qy qz tx ty tz) in/out.
int oracle_refine_pose_gauss_newton(int num, const int64_t *offsets, const double *X, const double *uv,
                                    int iterations, double *poses) {
    if (num < 0 || !offsets || !poses) return SFMBA_ERR_INVALID_ARGUMENT;
    for (int k = 0; k < num; ++k) {
        const long a = offsets[k], n = offsets[k + 1] - a;
        const Pose r = refine_gn(load(poses + 7 * k), X + 3 * a, uv + 2 * a, nullptr, n, iterations);
        store(r, poses + 7 * k);
    }
    return SFMBA_OK;
}

// pnp.rs:211-309 (pnp_ransac) with ransac.rs:72-131 (seed 0xFACADE, sample
// size 6, confidence 0.999), for one correspondence set of n points.
// found = 0 (None) leaves pose and inliers untouched.
int oracle_pnp_ransac(long n, const double *X, const double *uv, double threshold, long max_iterations,
                      double *pose_out, uint8_t *inliers_out, int32_t *found, int64_t *iterations_out) {
    if (!found || n < 0) return SFMBA_ERR_INVALID_ARGUMENT;
    *found = 0;
    if (iterations_out) *iterations_out = 0;
    if (n < 6) return SFMBA_OK;
    const int k = 6;
    Xorshift64 rng(0xFACADEull);
    std::vector<long> buf((size_t)n);
    bool have = false;
    Pose best{};
    std::vector<uint8_t> best_mask((size_t)n), mask((size_t)n);
    long best_count = 0, needed = max_iterations, iter = 0;
    while (iter < std::min(max_iterations, std::max(needed, 1L))) {
        ++iter;
        for (long i = 0; i < n; ++i) buf[i] = i;
        for (int i = 0; i < k; ++i) std::swap(buf[i], buf[i + rng.below(n - i)]);
        if (!well_conditioned(X, buf.data(), k)) continue;
        Pose m;
        if (!pnp_dlt(X, uv, buf.data(), k, m)) continue;
        const long count = count_inliers(m, X, uv, n, threshold, mask.data());
        if (!have || count > best_count) {
            have = true;
            best = m;
            best_mask = mask;
            best_count = count;
            const double ratio = std::max((double)count / (double)n, 1e-6);
            // f64::powi(6) as binary powering: x^2 * (x^2)^2.
            const double r2 = ratio * ratio;
            const double denom = std::log(std::max(1.0 - r2 * (r2 * r2), 1e-12));
            if (denom < 0.0) {
                const double est = std::ceil(std::log(1.0 - 0.999) / denom);
                if (std::isfinite(est) && est >= 0.0) needed = std::min((long)est, max_iterations);
            }
        }
    }
    if (iterations_out) *iterations_out = iter;
    if (!have || best_count < 6) return SFMBA_OK;
    // LO refit on the inlier set, kept only if it loses no inliers.
    std::vector<long> in;
    for (long i = 0; i < n; ++i)
        if (best_mask[i]) in.push_back(i);
    Pose refit;
    if (pnp_dlt(X, uv, in.data(), (long)in.size(), refit)) {
        const long c = count_inliers(refit, X, uv, n, threshold, mask.data());
        if (c >= best_count) {
            best = refit;
            best_mask = mask;
            best_count = c;
        }
    }
    // Two Gauss-Newton polish rounds, never regressing.
    for (int round = 0; round < 2; ++round) {
        in.clear();
        for (long i = 0; i < n; ++i)
            if (best_mask[i]) in.push_back(i);
        if (in.size() < 6) break;
        const Pose r = refine_gn(best, X, uv, in.data(), (long)in.size(), 10);
        const long c = count_inliers(r, X, uv, n, threshold, mask.data());
        if (c < best_count) break;
        const bool converged = c == best_count;
        best = r;
        best_mask = mask;
        best_count = c;
        if (converged) break;
    }
    *found = 1;
    if (pose_out) store(best, pose_out);
    if (inliers_out) std::memcpy(inliers_out, best_mask.data(), (size_t)n);
    return SFMBA_OK;
}

}  // extern "C"
