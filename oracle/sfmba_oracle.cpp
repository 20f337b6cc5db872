// TEST INFRASTRUCTURE ONLY - never linked into or called by the product path.
//
// CPU FP64 restatement of sfmtory's `sfm-ba` crate (Rust; it cannot be built
// in this environment: no cargo/rustc). Only tests/, __graft_entry__.smoke()
// and bench.py's CPU-baseline leg load this library, as the checker.
//
// Every function names the reference lines it restates (paths inside the
// sfmtory project). Third-party arithmetic the reference takes from nalgebra
// 0.33.3 (Cargo.lock:1122-1124) is restated from the mathematics:
//   - UnitQuaternion::from_scaled_axis: (cos(t/2), sin(t/2) * w/t), identity
//     when |w| == 0;
//   - quaternion product (Hamilton) and vector rotation v + 2w(q x v) + 2 q x (q x v);
//   - to_rotation_matrix: the standard unit-quaternion rotation matrix;
//   - Matrix3::try_inverse: adjugate / determinant, None iff det == 0;
//   - Cholesky::new: left-looking column LL^T on the lower triangle, fails
//     iff a pivot is not > 0 (covers 0, negative and NaN);
//   - lu().solve: partial pivoting on max |a|, zero columns skipped, solve
//     fails iff a diagonal entry of U is 0.
// Parity status: pinned by the reference's own known-answer tests (analytic
// vs central-difference Jacobians for all six models at the reference's
// tolerances, and its convergence tests), ported in tests/test_oracle.py.
// The reference publishes no numeric golden outputs, so agreement with the
// Rust binary's exact numbers is unpinned.
#include "../include/sfmba.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double kFunctionTolerance = 1e-6;   // lib.rs:814
constexpr int kMaxDampingRetries = 8;         // lib.rs:914
constexpr long kParallelSchurMinPoints = 1500;  // lib.rs:981
constexpr double kMinDepth = 1e-9;            // lib.rs:256, 338
constexpr double kFdEps = 1e-6;               // lib.rs:272, intrinsics.rs:82

int model_dof(int model) {  // camera.rs:136-163 (params().len())
    static const int dof[6] = {3, 4, 4, 5, 8, 8};
    return (model >= 0 && model < 6) ? dof[model] : 0;
}

struct Quat {
    double w, x, y, z;
};

Quat qmul(const Quat &a, const Quat &b) {
    return {a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z,
            a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y,
            a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x,
            a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w};
}

// UnitQuaternion * Vector3: v + w*t + q_v x t with t = 2 q_v x v.
void qrotate(const Quat &q, const double v[3], double out[3]) {
    double tx = 2.0 * (q.y * v[2] - q.z * v[1]);
    double ty = 2.0 * (q.z * v[0] - q.x * v[2]);
    double tz = 2.0 * (q.x * v[1] - q.y * v[0]);
    out[0] = v[0] + q.w * tx + (q.y * tz - q.z * ty);
    out[1] = v[1] + q.w * ty + (q.z * tx - q.x * tz);
    out[2] = v[2] + q.w * tz + (q.x * ty - q.y * tx);
}

void qmatrix(const Quat &q, double R[9]) {
    double ww = q.w * q.w, xx = q.x * q.x, yy = q.y * q.y, zz = q.z * q.z;
    double xy = 2 * q.x * q.y, wz = 2 * q.w * q.z, wy = 2 * q.w * q.y;
    double xz = 2 * q.x * q.z, yz = 2 * q.y * q.z, wx = 2 * q.w * q.x;
    R[0] = ww + xx - yy - zz; R[1] = xy - wz;           R[2] = wy + xz;
    R[3] = wz + xy;           R[4] = ww - xx + yy - zz; R[5] = yz - wx;
    R[6] = xz - wy;           R[7] = wx + yz;           R[8] = ww - xx - yy + zz;
}

Quat quat_from_scaled_axis(const double w[3]) {
    double t = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
    if (!(t > 0.0)) return {1.0, 0.0, 0.0, 0.0};
    double s = std::sin(0.5 * t) / t;
    return {std::cos(0.5 * t), w[0] * s, w[1] * s, w[2] * s};
}

struct Pose {
    Quat q;
    double t[3];
};

Pose load_pose(const double *p) { return {{p[0], p[1], p[2], p[3]}, {p[4], p[5], p[6]}}; }
void store_pose(const Pose &p, double *o) {
    o[0] = p.q.w; o[1] = p.q.x; o[2] = p.q.y; o[3] = p.q.z;
    o[4] = p.t[0]; o[5] = p.t[1]; o[6] = p.t[2];
}

// pose.rs:46-48
void transform_point(const Pose &P, const double X[3], double pc[3]) {
    double r[3];
    qrotate(P.q, X, r);
    pc[0] = r[0] + P.t[0]; pc[1] = r[1] + P.t[1]; pc[2] = r[2] + P.t[2];
}

// lib.rs:263-269 (perturb_pose): R <- exp(w) R, t <- t + dt.
Pose perturb_pose(const Pose &P, const double d[6]) {
    Pose out;
    out.q = qmul(quat_from_scaled_axis(d), P.q);
    out.t[0] = P.t[0] + d[3]; out.t[1] = P.t[1] + d[4]; out.t[2] = P.t[2] + d[5];
    return out;
}

// camera.rs:204-244 (CameraModel::project).
void project(int model, const double *c, const double pc[3], double uv[2]) {
    double x = pc[0] / pc[2], y = pc[1] / pc[2];
    switch (model) {
    case SFMBA_SIMPLE_PINHOLE:
        uv[0] = c[0] * x + c[1]; uv[1] = c[0] * y + c[2]; return;
    case SFMBA_PINHOLE:
        uv[0] = c[0] * x + c[2]; uv[1] = c[1] * y + c[3]; return;
    case SFMBA_SIMPLE_RADIAL: {
        double r2 = x * x + y * y, d = 1.0 + c[3] * r2;
        uv[0] = c[0] * (x * d) + c[1]; uv[1] = c[0] * (y * d) + c[2]; return;
    }
    case SFMBA_RADIAL: {
        double r2 = x * x + y * y, d = 1.0 + c[3] * r2 + c[4] * r2 * r2;
        uv[0] = c[0] * (x * d) + c[1]; uv[1] = c[0] * (y * d) + c[2]; return;
    }
    case SFMBA_OPENCV: {
        double k1 = c[4], k2 = c[5], p1 = c[6], p2 = c[7];
        double r2 = x * x + y * y, rad = 1.0 + k1 * r2 + k2 * r2 * r2;
        double xd = x * rad + 2.0 * p1 * x * y + p2 * (r2 + 2.0 * x * x);
        double yd = y * rad + p1 * (r2 + 2.0 * y * y) + 2.0 * p2 * x * y;
        uv[0] = c[0] * xd + c[2]; uv[1] = c[1] * yd + c[3]; return;
    }
    default: {  // OPENCV_FISHEYE
        double r = std::max(std::sqrt(x * x + y * y), 1e-12);
        double th = std::atan(r), t2 = th * th;
        double thd = th * (1.0 + c[4] * t2 + c[5] * t2 * t2 + c[6] * t2 * t2 * t2 +
                           c[7] * t2 * t2 * t2 * t2);
        double s = thd / r;
        uv[0] = c[0] * (x * s) + c[2]; uv[1] = c[1] * (y * s) + c[3]; return;
    }
    }
}

// lib.rs:249-261 (reprojection_residual). Returns false when z <= 1e-9.
bool residual(const Pose &P, int model, const double *c, const double X[3], double ox, double oy,
              double r[2]) {
    double pc[3];
    transform_point(P, X, pc);
    if (pc[2] <= kMinDepth) return false;
    double uv[2];
    project(model, c, pc, uv);
    r[0] = uv[0] - ox; r[1] = uv[1] - oy;
    return true;
}

struct Jac {
    double r[2];
    double jp[2][6];
    double jx[2][3];
    double jc[2][8];
};

// lib.rs:282-310 (pose_point_jacobians) + lib.rs:327-590 (analytic_jacobians).
// The model-specific part yields the 2x2 derivative of the pixel w.r.t. the
// normalised coordinates (xp, yp) and the 2xk derivative w.r.t. the params;
// the chain rule through pc = R X + t is shared.
bool analytic(const Pose &P, int model, const double *c, const double X[3], double ox, double oy,
              Jac &J) {
    double pc[3];
    transform_point(P, X, pc);
    if (pc[2] <= kMinDepth) return false;
    const double iz = 1.0 / pc[2];
    const double xp = pc[0] * iz, yp = pc[1] * iz;
    double u = 0, v = 0;
    double a00 = 0, a01 = 0, a10 = 0, a11 = 0;  // d(u,v)/d(xp,yp)
    std::memset(J.jc, 0, sizeof(J.jc));
    switch (model) {
    case SFMBA_SIMPLE_PINHOLE: {
        double f = c[0];
        u = f * xp + c[1]; v = f * yp + c[2];
        a00 = f; a11 = f;
        J.jc[0][0] = xp; J.jc[0][1] = 1.0;
        J.jc[1][0] = yp; J.jc[1][2] = 1.0;
        break;
    }
    case SFMBA_PINHOLE: {
        u = c[0] * xp + c[2]; v = c[1] * yp + c[3];
        a00 = c[0]; a11 = c[1];
        J.jc[0][0] = xp; J.jc[0][2] = 1.0;
        J.jc[1][1] = yp; J.jc[1][3] = 1.0;
        break;
    }
    case SFMBA_SIMPLE_RADIAL:
    case SFMBA_RADIAL: {
        double f = c[0], k1 = c[3], k2 = (model == SFMBA_RADIAL) ? c[4] : 0.0;
        double r2 = xp * xp + yp * yp;
        double d = (model == SFMBA_RADIAL) ? 1.0 + k1 * r2 + k2 * r2 * r2 : 1.0 + k1 * r2;
        double dd = (model == SFMBA_RADIAL) ? k1 + 2.0 * k2 * r2 : k1;  // d(d)/d(r2)
        u = f * xp * d + c[1]; v = f * yp * d + c[2];
        a00 = f * (d + 2.0 * dd * xp * xp);
        a01 = 2.0 * f * dd * xp * yp;
        a10 = a01;
        a11 = f * (d + 2.0 * dd * yp * yp);
        J.jc[0][0] = xp * d; J.jc[0][1] = 1.0; J.jc[0][3] = f * xp * r2;
        J.jc[1][0] = yp * d; J.jc[1][2] = 1.0; J.jc[1][3] = f * yp * r2;
        if (model == SFMBA_RADIAL) {
            J.jc[0][4] = f * xp * r2 * r2;
            J.jc[1][4] = f * yp * r2 * r2;
        }
        break;
    }
    case SFMBA_OPENCV: {
        double fx = c[0], fy = c[1], k1 = c[4], k2 = c[5], p1 = c[6], p2 = c[7];
        double r2 = xp * xp + yp * yp;
        double rad = 1.0 + k1 * r2 + k2 * r2 * r2;
        double xd = xp * rad + 2.0 * p1 * xp * yp + p2 * (r2 + 2.0 * xp * xp);
        double yd = yp * rad + p1 * (r2 + 2.0 * yp * yp) + 2.0 * p2 * xp * yp;
        u = fx * xd + c[2]; v = fy * yd + c[3];
        double kr = k1 + 2.0 * k2 * r2;
        double dxx = rad + 2.0 * kr * xp * xp + 2.0 * p1 * yp + 6.0 * p2 * xp;
        double dxy = 2.0 * kr * xp * yp + 2.0 * p1 * xp + 2.0 * p2 * yp;
        double dyy = rad + 2.0 * kr * yp * yp + 6.0 * p1 * yp + 2.0 * p2 * xp;
        a00 = fx * dxx; a01 = fx * dxy; a10 = fy * dxy; a11 = fy * dyy;
        J.jc[0][0] = xd; J.jc[0][2] = 1.0;
        J.jc[0][4] = fx * xp * r2; J.jc[0][5] = fx * xp * r2 * r2;
        J.jc[0][6] = fx * 2.0 * xp * yp; J.jc[0][7] = fx * (r2 + 2.0 * xp * xp);
        J.jc[1][1] = yd; J.jc[1][3] = 1.0;
        J.jc[1][4] = fy * yp * r2; J.jc[1][5] = fy * yp * r2 * r2;
        J.jc[1][6] = fy * (r2 + 2.0 * yp * yp); J.jc[1][7] = fy * 2.0 * xp * yp;
        break;
    }
    default: {  // OPENCV_FISHEYE
        double fx = c[0], fy = c[1], k1 = c[4], k2 = c[5], k3 = c[6], k4 = c[7];
        double r = std::max(std::sqrt(xp * xp + yp * yp), 1e-12);
        double th = std::atan(r), t2 = th * th, t4 = t2 * t2, t6 = t4 * t2, t8 = t4 * t4;
        double poly = 1.0 + k1 * t2 + k2 * t4 + k3 * t6 + k4 * t8;
        double thd = th * poly, s = thd / r;
        u = fx * (xp * s) + c[2]; v = fy * (yp * s) + c[3];
        double dpoly = k1 + 2.0 * k2 * t2 + 3.0 * k3 * t4 + 4.0 * k4 * t6;  // d(poly)/d(t2)
        double dthd = poly + 2.0 * t2 * dpoly;
        double dth_dr = 1.0 / (1.0 + r * r);
        double ds_dr = (dthd * dth_dr * r - thd) / (r * r);
        double dsx = ds_dr * (xp / r), dsy = ds_dr * (yp / r);
        a00 = fx * (s + xp * dsx); a01 = fx * xp * dsy;
        a10 = fy * yp * dsx;       a11 = fy * (s + yp * dsy);
        J.jc[0][0] = xp * s; J.jc[0][2] = 1.0;
        J.jc[1][1] = yp * s; J.jc[1][3] = 1.0;
        double tk[4] = {th * t2, th * t4, th * t6, th * t8};
        for (int i = 0; i < 4; ++i) {
            J.jc[0][4 + i] = fx * xp * tk[i] / r;
            J.jc[1][4 + i] = fy * yp * tk[i] / r;
        }
        break;
    }
    }
    J.r[0] = u - ox; J.r[1] = v - oy;
    // d(u,v)/d(pc) through xp = pc.x/z, yp = pc.y/z.
    double du[3] = {a00 * iz, a01 * iz, -(a00 * pc[0] + a01 * pc[1]) * iz * iz};
    double dv[3] = {a10 * iz, a11 * iz, -(a10 * pc[0] + a11 * pc[1]) * iz * iz};
    double R[9];
    qmatrix(P.q, R);
    for (int k = 0; k < 3; ++k) {  // J_point = R^T d
        J.jx[0][k] = R[0 * 3 + k] * du[0] + R[1 * 3 + k] * du[1] + R[2 * 3 + k] * du[2];
        J.jx[1][k] = R[0 * 3 + k] * dv[0] + R[1 * 3 + k] * dv[1] + R[2 * 3 + k] * dv[2];
    }
    // J_pose = [skew(q) d, d] with q = pc - t (left rotation perturbation).
    double q[3] = {pc[0] - P.t[0], pc[1] - P.t[1], pc[2] - P.t[2]};
    const double *dr[2] = {du, dv};
    for (int row = 0; row < 2; ++row) {
        const double *d = dr[row];
        J.jp[row][0] = -q[2] * d[1] + q[1] * d[2];
        J.jp[row][1] = q[2] * d[0] - q[0] * d[2];
        J.jp[row][2] = -q[1] * d[0] + q[0] * d[1];
        J.jp[row][3] = d[0]; J.jp[row][4] = d[1]; J.jp[row][5] = d[2];
    }
    return true;
}

// lib.rs:677-694 (robust_weight).
double robust_weight(double n, int loss, double scale) {
    double s = std::max(scale, 1e-9);
    if (loss == SFMBA_LOSS_HUBER) return n <= s ? 1.0 : s / n;
    if (loss == SFMBA_LOSS_CAUCHY) {
        double t = n / s;
        return 1.0 / (1.0 + t * t);
    }
    return 1.0;
}

// Owned, fully padded copy of an sfmba_problem.
struct Problem {
    long nI = 0, nC = 0, nP = 0, nO = 0;
    std::vector<int> cam_of_img, model;
    std::vector<double> cam;     // nC * 8
    std::vector<double> poses;   // nI * 7
    std::vector<double> points;  // nP * 3
    std::vector<int> ob_img, ob_pt;
    std::vector<double> ob_xy;
    std::vector<uint8_t> fixed_pose, fixed_cam, fixed_cp;  // nI, nC, nC*8
};

bool load(const sfmba_problem *p, Problem &P) {
    if (!p || p->num_images < 0 || p->num_cameras < 0 || p->num_points < 0 ||
        p->num_observations < 0)
        return false;
    P.nI = p->num_images; P.nC = p->num_cameras; P.nP = p->num_points; P.nO = p->num_observations;
    P.cam_of_img.assign(p->camera_of_image, p->camera_of_image + P.nI);
    P.model.assign(p->camera_model, p->camera_model + P.nC);
    P.cam.assign(p->camera_params, p->camera_params + P.nC * 8);
    P.poses.assign(p->poses, p->poses + P.nI * 7);
    P.points.assign(p->points, p->points + P.nP * 3);
    P.ob_img.assign(p->obs_image, p->obs_image + P.nO);
    P.ob_pt.assign(p->obs_point, p->obs_point + P.nO);
    P.ob_xy.assign(p->obs_xy, p->obs_xy + P.nO * 2);
    P.fixed_pose.assign(P.nI, 0);
    P.fixed_cam.assign(P.nC, 0);
    P.fixed_cp.assign(P.nC * 8, 0);
    if (p->fixed_poses) P.fixed_pose.assign(p->fixed_poses, p->fixed_poses + P.nI);
    if (p->fixed_cameras) P.fixed_cam.assign(p->fixed_cameras, p->fixed_cameras + P.nC);
    if (p->fixed_camera_params)
        P.fixed_cp.assign(p->fixed_camera_params, p->fixed_camera_params + P.nC * 8);
    for (long c = 0; c < P.nC; ++c)
        if (model_dof(P.model[c]) == 0) return false;
    for (long i = 0; i < P.nI; ++i)
        if (P.cam_of_img[i] < 0 || P.cam_of_img[i] >= P.nC) return false;
    for (long o = 0; o < P.nO; ++o)
        if (P.ob_img[o] < 0 || P.ob_img[o] >= P.nI || P.ob_pt[o] < 0 || P.ob_pt[o] >= P.nP)
            return false;
    return true;
}

// lib.rs:727-745 (total_cost).
double total_cost(const Problem &P, const std::vector<double> &poses,
                  const std::vector<double> &cams, const std::vector<double> &pts, int loss,
                  double scale) {
    double sum = 0.0;
#pragma omp parallel for reduction(+ : sum) schedule(static)
    for (long o = 0; o < P.nO; ++o) {
        int i = P.ob_img[o], c = P.cam_of_img[i];
        double r[2];
        if (residual(load_pose(&poses[i * 7]), P.model[c], &cams[c * 8], &pts[P.ob_pt[o] * 3],
                     P.ob_xy[2 * o], P.ob_xy[2 * o + 1], r)) {
            double n = std::sqrt(r[0] * r[0] + r[1] * r[1]);
            sum += robust_weight(n, loss, scale) * n * n;
        }
    }
    return sum;
}

// Dense LL^T (nalgebra Cholesky::new semantics) on the lower triangle of a
// row-major n x n matrix, in place. Returns false iff a pivot is not > 0.
bool cholesky(std::vector<double> &A, long n) {
    for (long j = 0; j < n; ++j) {
        for (long k = 0; k < j; ++k) {
            double f = A[j * n + k];
            if (f == 0.0) continue;
            for (long i = j; i < n; ++i) A[i * n + j] -= f * A[i * n + k];
        }
        double d = A[j * n + j];
        if (!(d > 0.0)) return false;
        double s = std::sqrt(d);
        A[j * n + j] = s;
        for (long i = j + 1; i < n; ++i) A[i * n + j] /= s;
    }
    return true;
}

void cholesky_solve(const std::vector<double> &L, long n, std::vector<double> &x) {
    for (long i = 0; i < n; ++i) {
        double s = x[i];
        for (long k = 0; k < i; ++k) s -= L[i * n + k] * x[k];
        x[i] = s / L[i * n + i];
    }
    for (long i = n - 1; i >= 0; --i) {
        double s = x[i];
        for (long k = i + 1; k < n; ++k) s -= L[k * n + i] * x[k];
        x[i] = s / L[i * n + i];
    }
}

// nalgebra lu().solve: partial pivoting; returns false iff U has a zero diagonal.
bool lu_solve(std::vector<double> A, long n, std::vector<double> &b) {
    std::vector<long> perm_a, perm_b;
    for (long i = 0; i < n; ++i) {
        long piv = i;
        double best = std::fabs(A[i * n + i]);
        for (long r = i + 1; r < n; ++r) {
            double v = std::fabs(A[r * n + i]);
            if (v > best) { best = v; piv = r; }
        }
        double diag = A[piv * n + i];
        if (diag == 0.0) continue;
        if (piv != i) {
            perm_a.push_back(i); perm_b.push_back(piv);
            for (long c = 0; c < n; ++c) std::swap(A[i * n + c], A[piv * n + c]);
        }
        for (long r = i + 1; r < n; ++r) {
            double f = A[r * n + i] / diag;
            A[r * n + i] = f;
            if (f == 0.0) continue;
            for (long c = i + 1; c < n; ++c) A[r * n + c] -= f * A[i * n + c];
        }
    }
    for (size_t k = 0; k < perm_a.size(); ++k) std::swap(b[perm_a[k]], b[perm_b[k]]);
    for (long i = 0; i < n; ++i) {  // unit lower
        double s = b[i];
        for (long k = 0; k < i; ++k) s -= A[i * n + k] * b[k];
        b[i] = s;
    }
    for (long i = n - 1; i >= 0; --i) {
        double d = A[i * n + i];
        if (d == 0.0) return false;
        double s = b[i];
        for (long k = i + 1; k < n; ++k) s -= A[i * n + k] * b[k];
        b[i] = s / d;
    }
    return true;
}

// nalgebra Matrix3::try_inverse: adjugate over determinant; None iff det == 0.
bool inverse3(const double m[9], double out[9]) {
    double c00 = m[4] * m[8] - m[5] * m[7];
    double c01 = m[5] * m[6] - m[3] * m[8];
    double c02 = m[3] * m[7] - m[4] * m[6];
    double det = m[0] * c00 + m[1] * c01 + m[2] * c02;
    if (det == 0.0) return false;
    double id = 1.0 / det;
    out[0] = c00 * id;
    out[1] = (m[2] * m[7] - m[1] * m[8]) * id;
    out[2] = (m[1] * m[5] - m[2] * m[4]) * id;
    out[3] = c01 * id;
    out[4] = (m[0] * m[8] - m[2] * m[6]) * id;
    out[5] = (m[2] * m[3] - m[0] * m[5]) * id;
    out[6] = c02 * id;
    out[7] = (m[1] * m[6] - m[0] * m[7]) * id;
    out[8] = (m[0] * m[4] - m[1] * m[3]) * id;
    return true;
}

// One point-coupling block (lib.rs:101-104, EBlock): rows x 3, row-major.
struct EBlock {
    int slot;  // offset in the reduced system
    int rows;  // 6 for a pose, k for a camera
    double E[8 * 3];
};

// lib.rs:114-211 (accumulate_point_schur): S -= E_i C^-1 E_j^T over every
// unordered pair of the point's blocks (mirrored when i != j), rhs += E_i C^-1 g.
void accumulate_point(const double Ci[9], const std::vector<EBlock> &L, const double g[3],
                      double *S, double *rhs, long n) {
    for (size_t a = 0; a < L.size(); ++a) {
        const EBlock &A = L[a];
        double EC[8 * 3];
        for (int r = 0; r < A.rows; ++r)
            for (int c = 0; c < 3; ++c)
                EC[r * 3 + c] = A.E[r * 3 + 0] * Ci[0 * 3 + c] + A.E[r * 3 + 1] * Ci[1 * 3 + c] +
                                A.E[r * 3 + 2] * Ci[2 * 3 + c];
        for (size_t b = a; b < L.size(); ++b) {
            const EBlock &B = L[b];
            for (int r = 0; r < A.rows; ++r)
                for (int c = 0; c < B.rows; ++c) {
                    double v = EC[r * 3 + 0] * B.E[c * 3 + 0] + EC[r * 3 + 1] * B.E[c * 3 + 1] +
                               EC[r * 3 + 2] * B.E[c * 3 + 2];
                    S[(long)(A.slot + r) * n + (B.slot + c)] -= v;
                    if (b != a) S[(long)(B.slot + c) * n + (A.slot + r)] -= v;
                }
        }
    }
    double h[3];
    for (int r = 0; r < 3; ++r) h[r] = Ci[r * 3 + 0] * g[0] + Ci[r * 3 + 1] * g[1] + Ci[r * 3 + 2] * g[2];
    for (const EBlock &A : L)
        for (int r = 0; r < A.rows; ++r)
            rhs[A.slot + r] += A.E[r * 3 + 0] * h[0] + A.E[r * 3 + 1] * h[1] + A.E[r * 3 + 2] * h[2];
}

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

// Phase timers of the last oracle_bundle_adjust call (seconds), for the CPU
// baseline: 0 jacobians, 1 assembly, 2 system build + Schur, 3 factor+solve,
// 4 back-substitution + trial update, 5 trial cost.
thread_local double g_phase[8];

int g_threads_override = 0;

}  // namespace

extern "C" {

void oracle_set_threads(int n) { g_threads_override = n; }

int oracle_threads(void) {
#ifdef _OPENMP
    return g_threads_override > 0 ? g_threads_override : omp_get_max_threads();
#else
    return 1;
#endif
}

void oracle_phase_seconds(double out[8]) { std::memcpy(out, g_phase, sizeof(g_phase)); }

int oracle_project(int model, const double *params, const double *pc, double *uv) {
    if (model_dof(model) == 0) return 1;
    project(model, params, pc, uv);
    return 0;
}

void oracle_perturb_pose(const double *pose7, const double *delta6, double *out7) {
    store_pose(perturb_pose(load_pose(pose7), delta6), out7);
}

void oracle_transform_point(const double *pose7, const double *X, double *pc) {
    transform_point(load_pose(pose7), X, pc);
}

// Analytic Jacobians of one observation (lib.rs:327-590). Returns 1 if the
// point is in front of the camera, 0 otherwise.
int oracle_analytic_jacobians(const double *pose7, int model, const double *params,
                              const double *X, double ox, double oy, double *r, double *jp,
                              double *jx, double *jc) {
    Jac J;
    if (!analytic(load_pose(pose7), model, params, X, ox, oy, J)) return 0;
    std::memcpy(r, J.r, sizeof(J.r));
    std::memcpy(jp, J.jp, sizeof(J.jp));
    std::memcpy(jx, J.jx, sizeof(J.jx));
    std::memcpy(jc, J.jc, sizeof(J.jc));
    return 1;
}

// Central-difference Jacobians (lib.rs:600-670, observation_jacobians and
// camera_jacobian; step 1e-6, perturbation through perturb_pose / params[k]).
int oracle_numerical_jacobians(const double *pose7, int model, const double *params,
                               const double *X, double ox, double oy, double *r, double *jp,
                               double *jx, double *jc) {
    Pose P = load_pose(pose7);
    double r0[2];
    if (!residual(P, model, params, X, ox, oy, r0)) return 0;
    r[0] = r0[0]; r[1] = r0[1];
    auto col = [&](const double rp[2], const double rm[2], double *dst, int stride, int k) {
        dst[0 * stride + k] = (rp[0] - rm[0]) / (2.0 * kFdEps);
        dst[1 * stride + k] = (rp[1] - rm[1]) / (2.0 * kFdEps);
    };
    for (int k = 0; k < 6; ++k) {
        double dp[6] = {0}, dm[6] = {0};
        dp[k] = kFdEps; dm[k] = -kFdEps;
        double rp[2], rm[2];
        if (!residual(perturb_pose(P, dp), model, params, X, ox, oy, rp)) { rp[0] = r0[0]; rp[1] = r0[1]; }
        if (!residual(perturb_pose(P, dm), model, params, X, ox, oy, rm)) { rm[0] = r0[0]; rm[1] = r0[1]; }
        col(rp, rm, jp, 6, k);
    }
    for (int k = 0; k < 3; ++k) {
        double Xp[3] = {X[0], X[1], X[2]}, Xm[3] = {X[0], X[1], X[2]};
        Xp[k] += kFdEps; Xm[k] -= kFdEps;
        double rp[2], rm[2];
        if (!residual(P, model, params, Xp, ox, oy, rp)) { rp[0] = r0[0]; rp[1] = r0[1]; }
        if (!residual(P, model, params, Xm, ox, oy, rm)) { rm[0] = r0[0]; rm[1] = r0[1]; }
        col(rp, rm, jx, 3, k);
    }
    int nk = model_dof(model);
    for (int i = 0; i < 16; ++i) jc[i] = 0.0;
    for (int k = 0; k < nk; ++k) {
        double cp[8], cm[8];
        std::memcpy(cp, params, sizeof(cp)); std::memcpy(cm, params, sizeof(cm));
        cp[k] += kFdEps; cm[k] -= kFdEps;
        double rp[2], rm[2];
        if (!residual(P, model, cp, X, ox, oy, rp)) { rp[0] = r0[0]; rp[1] = r0[1]; }
        if (!residual(P, model, cm, X, ox, oy, rm)) { rm[0] = r0[0]; rm[1] = r0[1]; }
        col(rp, rm, jc, 8, k);
    }
    return 1;
}

// Jacobians of every observation of a problem, in input order, for checks
// over a whole scene. mode 0: analytic (lib.rs:327-590). mode 1: central
// differences as lib.rs:600-670 but with a step relative to the parameter,
// h = h_rel * max(1, |value|) (pose increments are taken at 0, so their step
// is h_rel). Outputs r[nO][2], jp[nO][2][6], jx[nO][2][3], jc[nO][2][8]
// (columns past the model's parameter count 0), valid[nO].
int oracle_jacobians_batch(const sfmba_problem *p, int mode, double h_rel, double *r, double *jp, double *jx,
                           double *jc, uint8_t *valid) {
    Problem P;
    if (!load(p, P) || (mode != 0 && mode != 1) || !(h_rel > 0.0)) return SFMBA_ERR_INVALID_ARGUMENT;
#pragma omp parallel for schedule(static)
    for (long o = 0; o < P.nO; ++o) {
        const int i = P.ob_img[o], c = P.cam_of_img[i], model = P.model[c];
        const Pose pose = load_pose(&P.poses[(size_t)i * 7]);
        const double *cp = &P.cam[(size_t)c * 8];
        const double *X = &P.points[(size_t)P.ob_pt[o] * 3];
        const double ox = P.ob_xy[2 * o], oy = P.ob_xy[2 * o + 1];
        double *ro = r + 2 * o, *jpo = jp + 12 * o, *jxo = jx + 6 * o, *jco = jc + 16 * o;
        for (int k = 0; k < 16; ++k) jco[k] = 0.0;
        if (mode == 0) {
            Jac J;
            valid[o] = analytic(pose, model, cp, X, ox, oy, J) ? 1 : 0;
            if (!valid[o]) continue;
            std::memcpy(ro, J.r, sizeof(J.r));
            std::memcpy(jpo, J.jp, sizeof(J.jp));
            std::memcpy(jxo, J.jx, sizeof(J.jx));
            std::memcpy(jco, J.jc, sizeof(J.jc));
            continue;
        }
        double r0[2];
        valid[o] = residual(pose, model, cp, X, ox, oy, r0) ? 1 : 0;
        if (!valid[o]) continue;
        ro[0] = r0[0]; ro[1] = r0[1];
        auto col = [&](const double rp[2], const double rm[2], double h, double *dst, int stride, int k) {
            dst[0 * stride + k] = (rp[0] - rm[0]) / (2.0 * h);
            dst[1 * stride + k] = (rp[1] - rm[1]) / (2.0 * h);
        };
        auto res_or_r0 = [&](const Pose &Q, const double *cc, const double *XX, double out[2]) {
            if (!residual(Q, model, cc, XX, ox, oy, out)) { out[0] = r0[0]; out[1] = r0[1]; }
        };
        for (int k = 0; k < 6; ++k) {
            double dp[6] = {0}, dm[6] = {0};
            dp[k] = h_rel; dm[k] = -h_rel;
            double rp[2], rm[2];
            res_or_r0(perturb_pose(pose, dp), cp, X, rp);
            res_or_r0(perturb_pose(pose, dm), cp, X, rm);
            col(rp, rm, h_rel, jpo, 6, k);
        }
        for (int k = 0; k < 3; ++k) {
            const double h = h_rel * std::max(1.0, std::fabs(X[k]));
            double Xp[3] = {X[0], X[1], X[2]}, Xm[3] = {X[0], X[1], X[2]};
            Xp[k] += h; Xm[k] -= h;
            double rp[2], rm[2];
            res_or_r0(pose, cp, Xp, rp);
            res_or_r0(pose, cp, Xm, rm);
            col(rp, rm, (Xp[k] - Xm[k]) * 0.5, jxo, 3, k);
        }
        for (int k = 0; k < model_dof(model); ++k) {
            const double h = h_rel * std::max(1.0, std::fabs(cp[k]));
            double cpp[8], cpm[8];
            std::memcpy(cpp, cp, sizeof(cpp)); std::memcpy(cpm, cp, sizeof(cpm));
            cpp[k] += h; cpm[k] -= h;
            double rp[2], rm[2];
            res_or_r0(pose, cpp, X, rp);
            res_or_r0(pose, cpm, X, rm);
            col(rp, rm, (cpp[k] - cpm[k]) * 0.5, jco, 8, k);
        }
    }
    return SFMBA_OK;
}

double oracle_robust_weight(double n, int loss, double scale) { return robust_weight(n, loss, scale); }

int oracle_total_cost(const sfmba_problem *p, const sfmba_options *o, double *out) {
    Problem P;
    if (!load(p, P) || !o || !out) return SFMBA_ERR_INVALID_ARGUMENT;
    *out = total_cost(P, P.poses, P.cam, P.points, o->robust_loss, o->loss_scale_px);
    return SFMBA_OK;
}

// lib.rs:708-725 (mean_reprojection_error).
int oracle_mean_reprojection_error(const sfmba_problem *p, double *out) {
    Problem P;
    if (!load(p, P) || !out) return SFMBA_ERR_INVALID_ARGUMENT;
    double sum = 0.0;
    long count = 0;
#pragma omp parallel for reduction(+ : sum, count)
    for (long o = 0; o < P.nO; ++o) {
        int i = P.ob_img[o], c = P.cam_of_img[i];
        double r[2];
        if (residual(load_pose(&P.poses[i * 7]), P.model[c], &P.cam[c * 8], &P.points[P.ob_pt[o] * 3],
                     P.ob_xy[2 * o], P.ob_xy[2 * o + 1], r)) {
            sum += std::sqrt(r[0] * r[0] + r[1] * r[1]);
            count += 1;
        }
    }
    *out = count == 0 ? 0.0 : sum / (double)count;
    return SFMBA_OK;
}

// intrinsics.rs:33-61 (principal_point_indices, default_fixed_params_mask).
int oracle_default_fixed_params_mask(int64_t n, const int32_t *models, uint8_t *out) {
    for (int64_t c = 0; c < n; ++c) {
        int m = models[c];
        if (model_dof(m) == 0) return SFMBA_ERR_INVALID_ARGUMENT;
        std::memset(out + c * 8, 0, 8);
        bool simple = (m == SFMBA_SIMPLE_PINHOLE || m == SFMBA_SIMPLE_RADIAL || m == SFMBA_RADIAL);
        int a = simple ? 1 : 2;
        out[c * 8 + a] = 1;
        out[c * 8 + a + 1] = 1;
    }
    return SFMBA_OK;
}

// lib.rs:747-1232 (bundle_adjust), restated step by step.
int oracle_bundle_adjust(const sfmba_problem *p, const sfmba_options *opt, sfmba_result *res) {
    double t_start = now_s();
    Problem P;
    if (!load(p, P) || !opt || !res) return SFMBA_ERR_INVALID_ARGUMENT;
    std::memset(g_phase, 0, sizeof(g_phase));
    const int loss = opt->robust_loss;
    const double scale = opt->loss_scale_px;

    // lib.rs:753-776: slots for free poses (6 each), then free cameras (k each).
    std::vector<long> pose_slot(P.nI, -1), cam_slot(P.nC, -1);
    long n = 0;
    for (long i = 0; i < P.nI; ++i)
        if (!P.fixed_pose[i]) { pose_slot[i] = n; n += 6; }
    for (long c = 0; c < P.nC; ++c)
        if (!P.fixed_cam[c]) { cam_slot[c] = n; n += model_dof(P.model[c]); }

    std::vector<double> poses = P.poses, cams = P.cam, pts = P.points;
    auto finish = [&](double init, double fin, int iters) {
        if (res->poses) std::memcpy(res->poses, poses.data(), poses.size() * sizeof(double));
        if (res->points) std::memcpy(res->points, pts.data(), pts.size() * sizeof(double));
        if (res->camera_params) std::memcpy(res->camera_params, cams.data(), cams.size() * sizeof(double));
        res->initial_cost = init;
        res->final_cost = fin;
        res->iterations_run = iters;
        res->status = SFMBA_OK;
        res->solver_used = SFMBA_SOLVER_DENSE;
        res->reduced_dim = n;
        res->seconds = now_s() - t_start;
        return SFMBA_OK;
    };
    res->damping_retries = 0;
    res->linear_iterations = 0;
    if (n == 0) {  // lib.rs:777-787
        double c0 = total_cost(P, poses, cams, pts, loss, scale);
        return finish(c0, c0, 0);
    }

    std::vector<double> S((size_t)n * n), rhs(n);
    const double initial_cost = total_cost(P, poses, cams, pts, loss, scale);
    double lambda = opt->initial_lambda, nu = 2.0, cost = initial_cost;
    int iterations_run = 0;
    const int nthreads = oracle_threads();

    struct Prepared {
        int img, cam, pt;
        Jac J;
        double w;
    };
    std::vector<Prepared> prep(P.nO);
    std::vector<char> prep_ok(P.nO);

    for (int outer = 0; outer < opt->max_iterations; ++outer) {
        ++iterations_run;
        const double cost_before = cost;
        double t0 = now_s();
        // lib.rs:832-853: Jacobians, parallel over observations, order kept.
#pragma omp parallel for schedule(static) num_threads(nthreads)
        for (long o = 0; o < P.nO; ++o) {
            int i = P.ob_img[o], c = P.cam_of_img[i];
            Prepared &q = prep[o];
            q.img = i; q.cam = c; q.pt = P.ob_pt[o];
            prep_ok[o] = analytic(load_pose(&poses[i * 7]), P.model[c], &cams[c * 8],
                                  &pts[q.pt * 3], P.ob_xy[2 * o], P.ob_xy[2 * o + 1], q.J);
            if (prep_ok[o])
                q.w = robust_weight(std::sqrt(q.J.r[0] * q.J.r[0] + q.J.r[1] * q.J.r[1]), loss, scale);
        }
        long nprep = 0;
        for (long o = 0; o < P.nO; ++o) nprep += prep_ok[o];
        double t1 = now_s();
        g_phase[0] += t1 - t0;
        if (nprep == 0) break;  // lib.rs:855-857

        // lib.rs:859-909: serial normal-equation assembly in observation order.
        std::vector<double> Bp(P.nI * 36, 0.0), bp(P.nI * 6, 0.0);
        std::vector<double> Bc(P.nC * 64, 0.0), bc(P.nC * 8, 0.0);
        std::vector<double> X(P.nI * 48, 0.0);  // pose x camera cross, 6 x 8
        std::vector<double> Cd(P.nP * 9, 0.0), Cg(P.nP * 3, 0.0);
        std::vector<std::vector<EBlock>> p2o(P.nP);
        for (long o = 0; o < P.nO; ++o) {
            if (!prep_ok[o]) continue;
            const Prepared &q = prep[o];
            const double w = q.w;
            const int k = model_dof(P.model[q.cam]);
            for (int a = 0; a < 3; ++a) {
                for (int b = 0; b < 3; ++b)
                    Cd[q.pt * 9 + a * 3 + b] += w * (q.J.jx[0][a] * q.J.jx[0][b] + q.J.jx[1][a] * q.J.jx[1][b]);
                Cg[q.pt * 3 + a] += w * (q.J.jx[0][a] * q.J.r[0] + q.J.jx[1][a] * q.J.r[1]);
            }
            const bool pf = pose_slot[q.img] >= 0, cf = cam_slot[q.cam] >= 0;
            if (pf) {
                EBlock e;
                e.slot = (int)pose_slot[q.img]; e.rows = 6;
                for (int a = 0; a < 6; ++a) {
                    for (int b = 0; b < 6; ++b)
                        Bp[q.img * 36 + a * 6 + b] += w * (q.J.jp[0][a] * q.J.jp[0][b] + q.J.jp[1][a] * q.J.jp[1][b]);
                    bp[q.img * 6 + a] += w * (q.J.jp[0][a] * q.J.r[0] + q.J.jp[1][a] * q.J.r[1]);
                    for (int b = 0; b < 3; ++b)
                        e.E[a * 3 + b] = w * (q.J.jp[0][a] * q.J.jx[0][b] + q.J.jp[1][a] * q.J.jx[1][b]);
                }
                p2o[q.pt].push_back(e);
            }
            if (cf) {
                EBlock e;
                e.slot = (int)cam_slot[q.cam]; e.rows = k;
                for (int a = 0; a < k; ++a) {
                    for (int b = 0; b < k; ++b)
                        Bc[q.cam * 64 + a * 8 + b] += w * (q.J.jc[0][a] * q.J.jc[0][b] + q.J.jc[1][a] * q.J.jc[1][b]);
                    bc[q.cam * 8 + a] += w * (q.J.jc[0][a] * q.J.r[0] + q.J.jc[1][a] * q.J.r[1]);
                    for (int b = 0; b < 3; ++b)
                        e.E[a * 3 + b] = w * (q.J.jc[0][a] * q.J.jx[0][b] + q.J.jc[1][a] * q.J.jx[1][b]);
                }
                p2o[q.pt].push_back(e);
            }
            if (pf && cf)
                for (int a = 0; a < 6; ++a)
                    for (int b = 0; b < k; ++b)
                        X[q.img * 48 + a * 8 + b] += w * (q.J.jp[0][a] * q.J.jc[0][b] + q.J.jp[1][a] * q.J.jc[1][b]);
        }
        double t2 = now_s();
        g_phase[1] += t2 - t1;

        bool accepted = false;
        for (int inner = 0; inner < kMaxDampingRetries; ++inner) {
            ++res->damping_retries;
            double r0 = now_s();
            // lib.rs:918-956: damped diagonal blocks, -b, undamped cross blocks.
            std::fill(S.begin(), S.end(), 0.0);
            std::fill(rhs.begin(), rhs.end(), 0.0);
            for (long i = 0; i < P.nI; ++i) {
                long off = pose_slot[i];
                if (off < 0) continue;
                for (int a = 0; a < 6; ++a) {
                    for (int b = 0; b < 6; ++b) S[(off + a) * n + off + b] = Bp[i * 36 + a * 6 + b];
                    S[(off + a) * n + off + a] += Bp[i * 36 + a * 6 + a] * lambda;
                    rhs[off + a] = -bp[i * 6 + a];
                }
            }
            for (long c = 0; c < P.nC; ++c) {
                long off = cam_slot[c];
                int k = model_dof(P.model[c]);
                if (off < 0) continue;
                for (int a = 0; a < k; ++a) {
                    for (int b = 0; b < k; ++b) S[(off + a) * n + off + b] = Bc[c * 64 + a * 8 + b];
                    S[(off + a) * n + off + a] += Bc[c * 64 + a * 8 + a] * lambda;
                    rhs[off + a] = -bc[c * 8 + a];
                }
            }
            for (long i = 0; i < P.nI; ++i) {
                int c = P.cam_of_img[i];
                long po = pose_slot[i], co = cam_slot[c];
                int k = model_dof(P.model[c]);
                if (po < 0 || co < 0) continue;
                for (int a = 0; a < 6; ++a)
                    for (int b = 0; b < k; ++b) {
                        S[(po + a) * n + co + b] = X[i * 48 + a * 8 + b];
                        S[(co + b) * n + po + a] = X[i * 48 + a * 8 + b];
                    }
            }
            // lib.rs:958-965: damped point inverses for points with E blocks.
            std::vector<double> Ci(P.nP * 9);
            std::vector<char> ci_ok(P.nP, 0);
            for (long q = 0; q < P.nP; ++q) {
                if (p2o[q].empty()) continue;
                double m[9];
                for (int a = 0; a < 9; ++a) m[a] = Cd[q * 9 + a];
                for (int a = 0; a < 3; ++a) m[a * 4] += Cd[q * 9 + a * 4] * lambda;
                ci_ok[q] = inverse3(m, &Ci[q * 9]);
            }
            // lib.rs:981-1043: Schur accumulation, chunked per thread above 1500 points.
            if (P.nP >= kParallelSchurMinPoints && nthreads > 1) {
                long chunk = (P.nP + nthreads - 1) / nthreads;
                std::vector<std::vector<double>> accS(nthreads), accR(nthreads);
#pragma omp parallel num_threads(nthreads)
                {
                    int t = 0;
#ifdef _OPENMP
                    t = omp_get_thread_num();
#endif
                    accS[t].assign((size_t)n * n, 0.0);
                    accR[t].assign(n, 0.0);
                    long lo = std::min(P.nP, t * chunk), hi = std::min(P.nP, (t + 1) * chunk);
                    for (long q = lo; q < hi; ++q)
                        if (ci_ok[q]) accumulate_point(&Ci[q * 9], p2o[q], &Cg[q * 3], accS[t].data(), accR[t].data(), n);
                }
                for (int t = 0; t < nthreads; ++t) {
#pragma omp parallel for num_threads(nthreads)
                    for (long e = 0; e < n * n; ++e) S[e] += accS[t][e];
                    for (long e = 0; e < n; ++e) rhs[e] += accR[t][e];
                }
            } else {
                for (long q = 0; q < P.nP; ++q)
                    if (ci_ok[q]) accumulate_point(&Ci[q * 9], p2o[q], &Cg[q * 3], S.data(), rhs.data(), n);
            }
            // lib.rs:1051-1070: per-parameter masks of free cameras.
            for (long c = 0; c < P.nC; ++c) {
                int k = model_dof(P.model[c]);
                if (cam_slot[c] < 0) continue;
                for (int a = 0; a < k; ++a) {
                    if (!P.fixed_cp[c * 8 + a]) continue;
                    long row = cam_slot[c] + a;
                    for (long col = 0; col < n; ++col) { S[row * n + col] = 0.0; S[col * n + row] = 0.0; }
                    S[row * n + row] = 1.0;
                    rhs[row] = 0.0;
                }
            }
            // lib.rs:1074: S = (S + S^T) / 2.
            for (long a = 0; a < n; ++a)
                for (long b = a + 1; b < n; ++b) {
                    double v = 0.5 * (S[a * n + b] + S[b * n + a]);
                    S[a * n + b] = v; S[b * n + a] = v;
                }
            double r1 = now_s();
            g_phase[2] += r1 - r0;
            // lib.rs:1081-1094: Cholesky, LU fallback, else grow lambda.
            std::vector<double> delta = rhs;
            std::vector<double> L = S;
            bool solved = cholesky(L, n);
            if (solved) cholesky_solve(L, n, delta);
            else {
                delta = rhs;
                solved = lu_solve(S, n, delta);
            }
            double r2 = now_s();
            g_phase[3] += r2 - r1;
            if (!solved) {
                lambda *= nu; nu *= 2.0;
                continue;
            }
            // lib.rs:1100-1120: delta_p = -C^-1 (g + sum E^T delta).
            std::vector<double> tpts = pts;
            for (long q = 0; q < P.nP; ++q) {
                if (!ci_ok[q]) continue;
                double acc[3] = {Cg[q * 3], Cg[q * 3 + 1], Cg[q * 3 + 2]};
                for (const EBlock &e : p2o[q])
                    for (int r = 0; r < e.rows; ++r)
                        for (int c = 0; c < 3; ++c) acc[c] += e.E[r * 3 + c] * delta[e.slot + r];
                for (int a = 0; a < 3; ++a)
                    tpts[q * 3 + a] += -(Ci[q * 9 + a * 3 + 0] * acc[0] + Ci[q * 9 + a * 3 + 1] * acc[1] + Ci[q * 9 + a * 3 + 2] * acc[2]);
            }
            // lib.rs:1122-1164: trial poses, points, cameras.
            std::vector<double> tposes = poses, tcams = cams;
            for (long i = 0; i < P.nI; ++i) {
                double d[6] = {0, 0, 0, 0, 0, 0};
                if (pose_slot[i] >= 0)
                    for (int a = 0; a < 6; ++a) d[a] = delta[pose_slot[i] + a];
                store_pose(perturb_pose(load_pose(&poses[i * 7]), d), &tposes[i * 7]);
            }
            for (long c = 0; c < P.nC; ++c) {
                if (cam_slot[c] < 0) continue;
                int k = model_dof(P.model[c]);
                for (int a = 0; a < k; ++a) tcams[c * 8 + a] += delta[cam_slot[c] + a];
            }
            double r3 = now_s();
            g_phase[4] += r3 - r2;
            // lib.rs:1176-1212: trial cost and the accept / reject rule.
            double trial = total_cost(P, tposes, tcams, tpts, loss, scale);
            g_phase[5] += now_s() - r3;
            if (std::isfinite(trial) && trial < cost) {
                poses.swap(tposes); pts.swap(tpts); cams.swap(tcams);
                cost = trial;
                lambda = std::max(lambda / 3.0, 1e-12);
                nu = 2.0;
                accepted = true;
                break;
            }
            lambda *= nu; nu *= 2.0;
        }
        if (!accepted) break;
        double rel = (cost_before - cost) / std::max(cost_before, 1e-12);
        if (rel < kFunctionTolerance) break;
        if (opt->target_cost > 0.0 && cost <= opt->target_cost) break;
    }
    return finish(initial_cost, cost, iterations_run);
}


// CPU baseline sample of ONE Levenberg-Marquardt iteration of the reference
// algorithm on the full problem (lib.rs:816-1176), for problems whose dense
// reduced system is too large to run whole in a bounded time. Phases:
//   out[0] Jacobians of every observation (parallel, lib.rs:832-853)
//   out[1] serial normal-equation assembly of every observation (:859-909)
//   out[2] Schur accumulation of every `point_stride`-th point into the dense
//          n x n system, one thread (:114-211); scale by stride / threads
//   out[3] unblocked LL^T of a chol_dim x chol_dim SPD matrix, one thread
//          like nalgebra (:1081); scale by (n / chol_dim)^3
//   out[4] point back-substitution + trial update of every point (:1100-1164)
//   out[5] trial cost of every observation (parallel, :1176)
//   out[6] points in the Schur sample, out[7] threads used.
int oracle_lm_iteration_sample(const sfmba_problem *p, const sfmba_options *opt, int point_stride,
                               int chol_dim, double *out) {
    Problem P;
    if (!load(p, P) || !opt || !out || point_stride < 1 || chol_dim < 1) return SFMBA_ERR_INVALID_ARGUMENT;
    const int loss = opt->robust_loss;
    const double scale = opt->loss_scale_px;
    const int nthreads = oracle_threads();
    std::vector<long> pose_slot(P.nI, -1), cam_slot(P.nC, -1);
    long n = 0;
    for (long i = 0; i < P.nI; ++i)
        if (!P.fixed_pose[i]) { pose_slot[i] = n; n += 6; }
    for (long c = 0; c < P.nC; ++c)
        if (!P.fixed_cam[c]) { cam_slot[c] = n; n += model_dof(P.model[c]); }
    for (int k = 0; k < 8; ++k) out[k] = 0.0;
    double t0 = now_s();
    std::vector<Jac> J(P.nO);
    std::vector<double> W(P.nO);
    std::vector<char> ok(P.nO);
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (long o = 0; o < P.nO; ++o) {
        int i = P.ob_img[o], c = P.cam_of_img[i];
        ok[o] = analytic(load_pose(&P.poses[i * 7]), P.model[c], &P.cam[c * 8], &P.points[P.ob_pt[o] * 3],
                         P.ob_xy[2 * o], P.ob_xy[2 * o + 1], J[o]);
        if (ok[o]) W[o] = robust_weight(std::sqrt(J[o].r[0] * J[o].r[0] + J[o].r[1] * J[o].r[1]), loss, scale);
    }
    double t1 = now_s();
    out[0] = t1 - t0;
    std::vector<double> Cd(P.nP * 9, 0.0), Cg(P.nP * 3, 0.0);
    std::vector<std::vector<EBlock>> p2o(P.nP);
    std::vector<double> Bp(P.nI * 36, 0.0), bc(P.nC * 8, 0.0);
    for (long o = 0; o < P.nO; ++o) {
        if (!ok[o]) continue;
        const Jac &q = J[o];
        const double w = W[o];
        const int i = P.ob_img[o], c = P.cam_of_img[i], pt = P.ob_pt[o], k = model_dof(P.model[c]);
        for (int a = 0; a < 3; ++a) {
            for (int b = 0; b < 3; ++b) Cd[pt * 9 + a * 3 + b] += w * (q.jx[0][a] * q.jx[0][b] + q.jx[1][a] * q.jx[1][b]);
            Cg[pt * 3 + a] += w * (q.jx[0][a] * q.r[0] + q.jx[1][a] * q.r[1]);
        }
        if (pose_slot[i] >= 0) {
            EBlock e;
            e.slot = (int)pose_slot[i]; e.rows = 6;
            for (int a = 0; a < 6; ++a) {
                for (int b = 0; b < 6; ++b) Bp[i * 36 + a * 6 + b] += w * (q.jp[0][a] * q.jp[0][b] + q.jp[1][a] * q.jp[1][b]);
                for (int b = 0; b < 3; ++b) e.E[a * 3 + b] = w * (q.jp[0][a] * q.jx[0][b] + q.jp[1][a] * q.jx[1][b]);
            }
            p2o[pt].push_back(e);
        }
        if (cam_slot[c] >= 0) {
            EBlock e;
            e.slot = (int)cam_slot[c]; e.rows = k;
            for (int a = 0; a < k; ++a) {
                bc[c * 8 + a] += w * (q.jc[0][a] * q.r[0] + q.jc[1][a] * q.r[1]);
                for (int b = 0; b < 3; ++b) e.E[a * 3 + b] = w * (q.jc[0][a] * q.jx[0][b] + q.jc[1][a] * q.jx[1][b]);
            }
            p2o[pt].push_back(e);
        }
    }
    double t2 = now_s();
    out[1] = t2 - t1;
    {
        std::vector<double> S((size_t)n * n, 0.0), rhs(n, 0.0);
        std::vector<double> Ci(9);
        long sampled = 0;
        double ts = now_s();
        for (long q = 0; q < P.nP; q += point_stride) {
            if (p2o[q].empty()) continue;
            double m[9];
            for (int a = 0; a < 9; ++a) m[a] = Cd[q * 9 + a];
            for (int a = 0; a < 3; ++a) m[a * 4] += Cd[q * 9 + a * 4] * opt->initial_lambda;
            if (!inverse3(m, Ci.data())) continue;
            accumulate_point(Ci.data(), p2o[q], &Cg[q * 3], S.data(), rhs.data(), n);
            ++sampled;
        }
        out[2] = now_s() - ts;
        out[6] = (double)sampled;
    }
    {
        const long m = std::min<long>(chol_dim, std::max<long>(n, 1));
        std::vector<double> A((size_t)m * m);
        for (long a = 0; a < m; ++a)
            for (long b = 0; b < m; ++b) A[a * m + b] = (a == b ? (double)m : 0.0) + 1.0 / (1.0 + (double)(a > b ? a - b : b - a));
        double tc = now_s();
        cholesky(A, m);
        out[3] = now_s() - tc;
    }
    double t4 = now_s();
    std::vector<double> delta(n, 1e-9), tpts = P.points, tposes = P.poses, tcams = P.cam;
    for (long q = 0; q < P.nP; ++q) {
        if (p2o[q].empty()) continue;
        double m[9], ci[9];
        for (int a = 0; a < 9; ++a) m[a] = Cd[q * 9 + a];
        for (int a = 0; a < 3; ++a) m[a * 4] += Cd[q * 9 + a * 4] * opt->initial_lambda;
        if (!inverse3(m, ci)) continue;
        double acc[3] = {Cg[q * 3], Cg[q * 3 + 1], Cg[q * 3 + 2]};
        for (const EBlock &e : p2o[q])
            for (int r = 0; r < e.rows; ++r)
                for (int c = 0; c < 3; ++c) acc[c] += e.E[r * 3 + c] * delta[e.slot + r];
        for (int a = 0; a < 3; ++a) tpts[q * 3 + a] -= ci[a * 3] * acc[0] + ci[a * 3 + 1] * acc[1] + ci[a * 3 + 2] * acc[2];
    }
    for (long i = 0; i < P.nI; ++i) {
        double d[6] = {0, 0, 0, 0, 0, 0};
        if (pose_slot[i] >= 0)
            for (int a = 0; a < 6; ++a) d[a] = delta[pose_slot[i] + a];
        store_pose(perturb_pose(load_pose(&P.poses[i * 7]), d), &tposes[i * 7]);
    }
    double t5 = now_s();
    out[4] = t5 - t4;
    volatile double c = total_cost(P, tposes, tcams, tpts, loss, scale);
    (void)c;
    out[5] = now_s() - t5;
    out[7] = nthreads;
    return SFMBA_OK;
}

// crates/sfm-reconstruction/src/lib.rs:1722-1768 (filter_and_reoptimize):
// bundle adjustment, then up to two rounds (FILTER_ROUNDS) of dropping the
// observations behind their camera (z <= 1e-9) or farther than threshold_px
// from their projection under the previous output, and adjusting again from
// that output; a round that drops nothing, or leaves fewer than 12
// observations (MIN_OBSERVATIONS), ends the loop without another adjustment.
// res holds the last adjustment's output; keep[o] = 1 for the input
// observations that adjustment used (may be NULL).
int oracle_filter_and_reoptimize(const sfmba_problem *p, const sfmba_options *opt, double threshold_px,
                                 sfmba_result *res, uint8_t *keep) {
    Problem P;
    if (!load(p, P) || !opt || !res) return SFMBA_ERR_INVALID_ARGUMENT;
    const long nO = P.nO;
    std::vector<int32_t> img(p->obs_image, p->obs_image + nO), pt(p->obs_point, p->obs_point + nO);
    std::vector<double> xy(p->obs_xy, p->obs_xy + 2 * nO);
    std::vector<long> orig(nO);
    for (long o = 0; o < nO; ++o) orig[o] = o;
    std::vector<double> out_poses(P.nI * 7), out_points(P.nP * 3), out_cams(P.nC * 8);
    std::vector<double> in_poses, in_points, in_cams;
    sfmba_result r = *res;
    r.poses = out_poses.data();
    r.points = out_points.data();
    r.camera_params = out_cams.data();
    sfmba_problem cur = *p;
    int st = oracle_bundle_adjust(&cur, opt, &r);
    if (st != SFMBA_OK) return st;
    std::vector<long> used = orig;
    for (int round = 0; round < 2; ++round) {
        std::vector<int32_t> ni, np;
        std::vector<double> nxy;
        std::vector<long> norig;
        for (size_t k = 0; k < img.size(); ++k) {
            const int c = P.cam_of_img[img[k]];
            double rr[2];
            if (!residual(load_pose(&out_poses[(size_t)img[k] * 7]), P.model[c], &out_cams[(size_t)c * 8],
                          &out_points[(size_t)pt[k] * 3], xy[2 * k], xy[2 * k + 1], rr))
                continue;
            if (std::sqrt(rr[0] * rr[0] + rr[1] * rr[1]) <= threshold_px) {
                ni.push_back(img[k]);
                np.push_back(pt[k]);
                nxy.push_back(xy[2 * k]);
                nxy.push_back(xy[2 * k + 1]);
                norig.push_back(orig[k]);
            }
        }
        const bool same = ni.size() == img.size();
        img.swap(ni); pt.swap(np); xy.swap(nxy); orig.swap(norig);
        if (same || img.size() < 12) break;
        in_poses = out_poses;
        in_points = out_points;
        in_cams = out_cams;
        cur.poses = in_poses.data();
        cur.points = in_points.data();
        cur.camera_params = in_cams.data();
        cur.num_observations = (int64_t)img.size();
        cur.obs_image = img.data();
        cur.obs_point = pt.data();
        cur.obs_xy = xy.data();
        st = oracle_bundle_adjust(&cur, opt, &r);
        if (st != SFMBA_OK) return st;
        used = orig;
    }
    if (res->poses) std::memcpy(res->poses, out_poses.data(), out_poses.size() * sizeof(double));
    if (res->points) std::memcpy(res->points, out_points.data(), out_points.size() * sizeof(double));
    if (res->camera_params) std::memcpy(res->camera_params, out_cams.data(), out_cams.size() * sizeof(double));
    res->initial_cost = r.initial_cost;
    res->final_cost = r.final_cost;
    res->iterations_run = r.iterations_run;
    res->status = r.status;
    if (keep) {
        std::memset(keep, 0, (size_t)nO);
        for (long o : used) keep[o] = 1;
    }
    return SFMBA_OK;
}

// crates/sfm-reconstruction/src/lib.rs:1567-1708 (the intrinsics handling of
// run_bundle_adjustment over a built problem): mode 0 (Fixed) adjusts with
// every camera fixed; mode 1 (Free) adjusts once with the cameras that have
// >= 5 images and are not fixed by the caller left free (:1598-1621); mode 2
// (FreeGuarded) runs filter_and_reoptimize with every camera fixed and, if
// some camera has >= 5 images, with those cameras free, and keeps the free
// result iff every camera's opencv_distortion() coefficient is below 0.5 in
// magnitude (:1672-1677) and its plain mean reprojection error over all the
// input observations (:1567-1578) is below the fixed result's (:1691-1695).
// chose_free = 1 when the free result was taken; errors[2] = the two mean
// errors (NaN for a candidate not run); keep as in filter_and_reoptimize.
int oracle_adjust_global(const sfmba_problem *p, const sfmba_options *opt, int mode, double threshold_px,
                         sfmba_result *res, uint8_t *keep, int32_t *chose_free, double *errors) {
    Problem P;
    if (!load(p, P) || !opt || !res || mode < 0 || mode > 2) return SFMBA_ERR_INVALID_ARGUMENT;
    std::vector<int> per_cam(P.nC, 0);
    for (long i = 0; i < P.nI; ++i) per_cam[P.cam_of_img[i]] += 1;
    std::vector<uint8_t> all_fixed(P.nC, 1), free_fixed(P.nC, 0);
    bool any_eligible = false;
    for (long c = 0; c < P.nC; ++c) {
        const bool user = p->fixed_cameras && p->fixed_cameras[c];
        free_fixed[c] = (per_cam[c] < 5 || user) ? 1 : 0;
        if (per_cam[c] >= 5) any_eligible = true;
    }
    struct Cand {
        std::vector<double> poses, points, cams;
        std::vector<uint8_t> keep;
        sfmba_result r{};
        double err = std::numeric_limits<double>::quiet_NaN();
    };
    auto run = [&](const std::vector<uint8_t> &fc, Cand &c) {
        sfmba_problem q = *p;
        q.fixed_cameras = fc.data();
        c.poses.assign(P.nI * 7, 0.0);
        c.points.assign(P.nP * 3, 0.0);
        c.cams.assign(P.nC * 8, 0.0);
        c.keep.assign((size_t)P.nO + 1, 1);
        c.r = sfmba_result{};
        c.r.poses = c.poses.data();
        c.r.points = c.points.data();
        c.r.camera_params = c.cams.data();
        return mode == 2 ? oracle_filter_and_reoptimize(&q, opt, threshold_px, &c.r, c.keep.data())
                         : oracle_bundle_adjust(&q, opt, &c.r);
    };
    auto eval_error = [&](Cand &c) {
        sfmba_problem q = *p;
        q.poses = c.poses.data();
        q.points = c.points.data();
        q.camera_params = c.cams.data();
        q.fixed_poses = nullptr;
        q.fixed_cameras = nullptr;
        q.fixed_camera_params = nullptr;
        return oracle_mean_reprojection_error(&q, &c.err);
    };
    Cand fixed, free;
    Cand *chosen = nullptr;
    int st = SFMBA_OK;
    if (mode == 1) {
        if ((st = run(free_fixed, free)) != SFMBA_OK) return st;
        chosen = &free;
    } else {
        if ((st = run(all_fixed, fixed)) != SFMBA_OK) return st;
        chosen = &fixed;
        if (mode == 2 && any_eligible) {
            if ((st = run(free_fixed, free)) != SFMBA_OK) return st;
            bool plausible = true;
            for (long c = 0; c < P.nC; ++c) {
                const double *k = &free.cams[(size_t)c * 8];
                double d[6] = {0, 0, 0, 0, 0, 0};
                switch (P.model[c]) {
                case 2: d[0] = k[3]; break;
                case 3: d[0] = k[3]; d[1] = k[4]; break;
                case 4: d[0] = k[4]; d[1] = k[5]; d[2] = k[6]; d[3] = k[7]; break;
                case 5: d[0] = k[4]; d[1] = k[5]; d[4] = k[6]; d[5] = k[7]; break;
                default: break;
                }
                for (double v : d) plausible = plausible && std::fabs(v) < 0.5;
            }
            if ((st = eval_error(fixed)) != SFMBA_OK) return st;
            if ((st = eval_error(free)) != SFMBA_OK) return st;
            if (plausible && free.err < fixed.err) chosen = &free;
        }
    }
    if (res->poses) std::memcpy(res->poses, chosen->poses.data(), chosen->poses.size() * sizeof(double));
    if (res->points) std::memcpy(res->points, chosen->points.data(), chosen->points.size() * sizeof(double));
    if (res->camera_params)
        std::memcpy(res->camera_params, chosen->cams.data(), chosen->cams.size() * sizeof(double));
    res->initial_cost = chosen->r.initial_cost;
    res->final_cost = chosen->r.final_cost;
    res->iterations_run = chosen->r.iterations_run;
    res->status = SFMBA_OK;
    if (keep && P.nO) std::memcpy(keep, chosen->keep.data(), (size_t)P.nO);
    if (chose_free) *chose_free = chosen == &free ? 1 : 0;
    if (errors) {
        errors[0] = fixed.err;
        errors[1] = free.err;
    }
    return SFMBA_OK;
}

// intrinsics.rs:116-238 (refine_intrinsics, refine_one_camera): per-camera
// dense LM over that camera's own parameters with central-difference
// Jacobians; cameras with fewer than 8 observations are left untouched.
int oracle_refine_intrinsics(const sfmba_problem *p, const sfmba_options *opt, double *cam_inout) {
    Problem P;
    if (!load(p, P) || !opt || !cam_inout) return SFMBA_ERR_INVALID_ARGUMENT;
    std::vector<std::vector<long>> by_cam(P.nC);
    for (long o = 0; o < P.nO; ++o) by_cam[P.cam_of_img[P.ob_img[o]]].push_back(o);
    std::vector<double> out = P.cam;
#pragma omp parallel for schedule(dynamic)
    for (long c = 0; c < P.nC; ++c) {
        const std::vector<long> &obs = by_cam[c];
        if (obs.size() < 8) continue;
        const int m = P.model[c], k = model_dof(m);
        double cur[8];
        std::memcpy(cur, &P.cam[c * 8], sizeof(cur));
        auto cost_of = [&](const double *cp) {
            double s = 0.0;
            for (long o : obs) {
                double r[2];
                if (residual(load_pose(&P.poses[P.ob_img[o] * 7]), m, cp, &P.points[P.ob_pt[o] * 3],
                             P.ob_xy[2 * o], P.ob_xy[2 * o + 1], r)) {
                    double nn = std::sqrt(r[0] * r[0] + r[1] * r[1]);
                    s += robust_weight(nn, opt->robust_loss, opt->loss_scale_px) * nn * nn;
                }
            }
            return s;
        };
        double cost = cost_of(cur), lambda = opt->initial_lambda;
        for (int it = 0; it < opt->max_iterations; ++it) {
            std::vector<double> jtj(k * k, 0.0), jtr(k, 0.0);
            for (long o : obs) {
                Pose Pi = load_pose(&P.poses[P.ob_img[o] * 7]);
                const double *X = &P.points[P.ob_pt[o] * 3];
                double ox = P.ob_xy[2 * o], oy = P.ob_xy[2 * o + 1], r0[2];
                if (!residual(Pi, m, cur, X, ox, oy, r0)) continue;
                double w = robust_weight(std::sqrt(r0[0] * r0[0] + r0[1] * r0[1]), opt->robust_loss, opt->loss_scale_px);
                double jac[8][2];
                for (int a = 0; a < k; ++a) {
                    double cp[8], cm[8], rp[2], rm[2];
                    std::memcpy(cp, cur, sizeof(cp)); std::memcpy(cm, cur, sizeof(cm));
                    cp[a] += kFdEps; cm[a] -= kFdEps;
                    if (!residual(Pi, m, cp, X, ox, oy, rp)) { rp[0] = r0[0]; rp[1] = r0[1]; }
                    if (!residual(Pi, m, cm, X, ox, oy, rm)) { rm[0] = r0[0]; rm[1] = r0[1]; }
                    jac[a][0] = (rp[0] - rm[0]) / (2.0 * kFdEps);
                    jac[a][1] = (rp[1] - rm[1]) / (2.0 * kFdEps);
                }
                for (int a = 0; a < k; ++a) {
                    jtr[a] += w * (jac[a][0] * r0[0] + jac[a][1] * r0[1]);
                    for (int b = 0; b < k; ++b) jtj[a * k + b] += w * (jac[a][0] * jac[b][0] + jac[a][1] * jac[b][1]);
                }
            }
            bool accepted = false;
            for (int inner = 0; inner < kMaxDampingRetries; ++inner) {
                std::vector<double> A = jtj, d(k);
                for (int a = 0; a < k; ++a) {
                    A[a * k + a] += lambda * std::max(jtj[a * k + a], 1e-12);
                    d[a] = -jtr[a];
                }
                std::vector<double> L = A;
                bool ok = cholesky(L, k);
                if (ok) cholesky_solve(L, k, d);
                else {
                    for (int a = 0; a < k; ++a) d[a] = -jtr[a];
                    ok = lu_solve(A, k, d);
                }
                if (!ok) { lambda *= 3.0; continue; }
                double trial[8];
                std::memcpy(trial, cur, sizeof(trial));
                for (int a = 0; a < k; ++a) trial[a] += d[a];
                double tc = cost_of(trial);
                if (std::isfinite(tc) && tc < cost) {
                    std::memcpy(cur, trial, sizeof(cur));
                    cost = tc;
                    lambda = std::max(lambda / 3.0, 1e-12);
                    accepted = true;
                    break;
                }
                lambda *= 3.0;
            }
            if (!accepted) break;
        }
        std::memcpy(&out[c * 8], cur, sizeof(cur));
    }
    std::memcpy(cam_inout, out.data(), out.size() * sizeof(double));
    return SFMBA_OK;
}

}  // extern "C"
