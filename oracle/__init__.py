"""TEST INFRASTRUCTURE ONLY: ctypes loader for the CPU FP64 oracle
(``oracle/sfmba_oracle.cpp``), a restatement of sfmtory's sfm-ba.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import this module, and only as the checker / CPU baseline. The
product path (:mod:`sfmtory_gb300`) never imports it.

Parity status: pinned by the reference's own known-answer tests (analytic vs
central-difference Jacobians for all six camera models, convergence tests);
the Rust reference cannot be built here and publishes no numeric golden
outputs, so exact agreement with its binary is unpinned.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

from sfmtory_gb300.abi import PackedProblem, ResultBuffers, SfmbaOptions, default_options

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle_sfmba.so")
_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++ -fopenmp)."""
    srcs = [os.path.join(_HERE, f) for f in ("sfmba_oracle.cpp", "pnp_oracle.cpp", "Makefile")]
    if force or not os.path.exists(_LIB_PATH) or any(os.path.getmtime(_LIB_PATH) < os.path.getmtime(s)
                                                     for s in srcs):
        subprocess.run(["make", "-C", _HERE, "-B" if force else "liboracle_sfmba.so"], check=True,
                       stdout=subprocess.DEVNULL)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(_LIB_PATH)
            vp, dp, i32, i64 = C.c_void_p, C.POINTER(C.c_double), C.c_int32, C.c_int64
            L.oracle_bundle_adjust.argtypes = [vp, vp, vp]
            L.oracle_total_cost.argtypes = [vp, vp, dp]
            L.oracle_mean_reprojection_error.argtypes = [vp, dp]
            L.oracle_default_fixed_params_mask.argtypes = [i64, vp, vp]
            L.oracle_refine_intrinsics.argtypes = [vp, vp, vp]
            L.oracle_filter_and_reoptimize.argtypes = [vp, vp, C.c_double, vp, vp]
            L.oracle_adjust_global.argtypes = [vp, vp, C.c_int, C.c_double, vp, vp, vp, vp]
            L.oracle_refine_pose_gauss_newton.argtypes = [C.c_int, vp, vp, vp, C.c_int, vp]
            L.oracle_pnp_ransac.argtypes = [C.c_long, vp, vp, C.c_double, C.c_long, vp, vp, vp, vp]
            for f in (L.oracle_analytic_jacobians, L.oracle_numerical_jacobians):
                f.argtypes = [vp, C.c_int, vp, vp, C.c_double, C.c_double, vp, vp, vp, vp]
                f.restype = C.c_int
            L.oracle_project.argtypes = [C.c_int, vp, vp, vp]
            L.oracle_perturb_pose.argtypes = [vp, vp, vp]
            L.oracle_transform_point.argtypes = [vp, vp, vp]
            L.oracle_robust_weight.argtypes = [C.c_double, C.c_int, C.c_double]
            L.oracle_robust_weight.restype = C.c_double
            L.oracle_set_threads.argtypes = [C.c_int]
            L.oracle_threads.restype = C.c_int
            L.oracle_phase_seconds.argtypes = [vp]
            L.oracle_lm_iteration_sample.argtypes = [vp, vp, C.c_int, C.c_int, vp]
            L.oracle_jacobians_batch.argtypes = [vp, C.c_int, C.c_double, vp, vp, vp, vp, vp]
            _lib = L
    return _lib


def set_threads(n: int) -> None:
    lib().oracle_set_threads(int(n))


def threads() -> int:
    return int(lib().oracle_threads())


def phase_seconds() -> np.ndarray:
    out = np.zeros(8)
    lib().oracle_phase_seconds(out.ctypes.data)
    return out


def _opts(options=None, **kw):
    if options is None:
        options = default_options(**kw)
    elif kw:
        for k, v in kw.items():
            setattr(options, k, v)
    return options


class OracleResult:
    def __init__(self, buffers: ResultBuffers):
        r = buffers.struct
        self.poses = buffers.poses
        self.points = buffers.points
        self.camera_params = buffers.camera_params
        self.initial_cost = r.initial_cost
        self.final_cost = r.final_cost
        self.iterations_run = r.iterations_run
        self.damping_retries = r.damping_retries
        self.reduced_dim = r.reduced_dim
        self.seconds = r.seconds


def bundle_adjust(problem, options: SfmbaOptions | None = None, **kw) -> OracleResult:
    packed = PackedProblem(problem)
    buf = ResultBuffers(packed)
    o = _opts(options, **kw)
    st = lib().oracle_bundle_adjust(C.byref(packed.struct), C.byref(o), C.byref(buf.struct))
    if st != 0:
        raise ValueError(f"oracle_bundle_adjust failed with status {st}")
    return OracleResult(buf)


def total_cost(problem, options: SfmbaOptions | None = None, **kw) -> float:
    packed = PackedProblem(problem)
    out = C.c_double()
    st = lib().oracle_total_cost(C.byref(packed.struct), C.byref(_opts(options, **kw)), C.byref(out))
    if st != 0:
        raise ValueError(f"oracle_total_cost failed with status {st}")
    return out.value


def mean_reprojection_error(problem) -> float:
    packed = PackedProblem(problem)
    out = C.c_double()
    st = lib().oracle_mean_reprojection_error(C.byref(packed.struct), C.byref(out))
    if st != 0:
        raise ValueError(f"oracle_mean_reprojection_error failed with status {st}")
    return out.value


def default_fixed_params_mask(models) -> np.ndarray:
    models = np.ascontiguousarray(models, dtype=np.int32)
    out = np.zeros((len(models), 8), dtype=np.uint8)
    st = lib().oracle_default_fixed_params_mask(len(models), models.ctypes.data, out.ctypes.data)
    if st != 0:
        raise ValueError("invalid camera model")
    return out.astype(bool)


def filter_and_reoptimize(problem, threshold_px: float, options: SfmbaOptions | None = None, **kw):
    """crates/sfm-reconstruction/src/lib.rs:1722-1768. Returns (result of the
    last adjustment, keep mask of the input observations it used)."""
    packed = PackedProblem(problem)
    buf = ResultBuffers(packed)
    keep = np.zeros(max(packed.struct.num_observations, 1), dtype=np.uint8)
    st = lib().oracle_filter_and_reoptimize(C.byref(packed.struct), C.byref(_opts(options, **kw)),
                                            C.c_double(threshold_px), C.byref(buf.struct), keep.ctypes.data)
    if st != 0:
        raise ValueError(f"oracle_filter_and_reoptimize failed with status {st}")
    return OracleResult(buf), keep[: packed.struct.num_observations].astype(bool)


def adjust_global(problem, mode: int, threshold_px: float, options: SfmbaOptions | None = None, **kw):
    """crates/sfm-reconstruction/src/lib.rs:1567-1708 (fixed-vs-free
    intrinsics handling). Returns (result, keep mask, chose_free, (fixed
    mean error, free mean error))."""
    packed = PackedProblem(problem)
    buf = ResultBuffers(packed)
    keep = np.zeros(max(packed.struct.num_observations, 1), dtype=np.uint8)
    chose = C.c_int32(-1)
    errs = np.full(2, np.nan)
    st = lib().oracle_adjust_global(C.byref(packed.struct), C.byref(_opts(options, **kw)), int(mode),
                                    C.c_double(threshold_px), C.byref(buf.struct), keep.ctypes.data,
                                    C.byref(chose), errs.ctypes.data)
    if st != 0:
        raise ValueError(f"oracle_adjust_global failed with status {st}")
    return (OracleResult(buf), keep[: packed.struct.num_observations].astype(bool), bool(chose.value),
            (float(errs[0]), float(errs[1])))


def refine_intrinsics(problem, options: SfmbaOptions | None = None, **kw) -> np.ndarray:
    """intrinsics.rs refine_intrinsics defaults: 30 iterations, lambda 1e-3, Huber 2 px."""
    base = dict(max_iterations=30)
    base.update(kw)
    packed = PackedProblem(problem)
    cams = packed.camera_params.copy()
    st = lib().oracle_refine_intrinsics(C.byref(packed.struct), C.byref(_opts(options, **base)),
                                        cams.ctypes.data)
    if st != 0:
        raise ValueError(f"oracle_refine_intrinsics failed with status {st}")
    return cams


def _jac(fn, pose7, model, params, X, obs):
    pose7 = np.ascontiguousarray(pose7, dtype=np.float64)
    p = np.zeros(8)
    p[: len(params)] = params
    X = np.ascontiguousarray(X, dtype=np.float64)
    r, jp, jx, jc = np.zeros(2), np.zeros((2, 6)), np.zeros((2, 3)), np.zeros((2, 8))
    ok = fn(pose7.ctypes.data, int(model), p.ctypes.data, X.ctypes.data, float(obs[0]), float(obs[1]),
            r.ctypes.data, jp.ctypes.data, jx.ctypes.data, jc.ctypes.data)
    if not ok:
        return None
    return r, jp, jx, jc


def analytic_jacobians(pose7, model, params, X, obs):
    """(r, J_pose 2x6, J_point 2x3, J_cam 2x8) or None (lib.rs:327-590)."""
    return _jac(lib().oracle_analytic_jacobians, pose7, model, params, X, obs)


def numerical_jacobians(pose7, model, params, X, obs):
    """Central differences, step 1e-6 (lib.rs:600-670)."""
    return _jac(lib().oracle_numerical_jacobians, pose7, model, params, X, obs)


def jacobians_batch(problem, numerical: bool = False, h_rel: float = 1e-6):
    """Residuals and Jacobians of every observation in input order: analytic
    (lib.rs:327-590) or central differences with step h_rel * max(1, |value|)
    per parameter (pose increments at 0: step h_rel). Returns (r [nO,2],
    J_pose [nO,2,6], J_point [nO,2,3], J_cam [nO,2,8], valid [nO])."""
    packed = PackedProblem(problem)
    n = int(packed.struct.num_observations)
    r, jp, jx = np.zeros((n, 2)), np.zeros((n, 2, 6)), np.zeros((n, 2, 3))
    jc, valid = np.zeros((n, 2, 8)), np.zeros(max(n, 1), np.uint8)
    st = lib().oracle_jacobians_batch(C.byref(packed.struct), 1 if numerical else 0, C.c_double(h_rel),
                                      r.ctypes.data, jp.ctypes.data, jx.ctypes.data, jc.ctypes.data,
                                      valid.ctypes.data)
    if st != 0:
        raise ValueError(f"oracle_jacobians_batch failed with status {st}")
    return r, jp, jx, jc, valid[:n].astype(bool)


def perturb_pose(pose7, delta6) -> np.ndarray:
    pose7 = np.ascontiguousarray(pose7, dtype=np.float64)
    delta6 = np.ascontiguousarray(delta6, dtype=np.float64)
    out = np.zeros(7)
    lib().oracle_perturb_pose(pose7.ctypes.data, delta6.ctypes.data, out.ctypes.data)
    return out


def transform_point(pose7, X) -> np.ndarray:
    pose7 = np.ascontiguousarray(pose7, dtype=np.float64)
    X = np.ascontiguousarray(X, dtype=np.float64)
    out = np.zeros(3)
    lib().oracle_transform_point(pose7.ctypes.data, X.ctypes.data, out.ctypes.data)
    return out


def project(model, params, pc) -> np.ndarray:
    p = np.zeros(8)
    p[: len(params)] = params
    pc = np.ascontiguousarray(pc, dtype=np.float64)
    out = np.zeros(2)
    lib().oracle_project(int(model), p.ctypes.data, pc.ctypes.data, out.ctypes.data)
    return out


def lm_iteration_sample(problem, point_stride: int, chol_dim: int, options: SfmbaOptions | None = None, **kw):
    """Phase times of one reference LM iteration on the full problem, with the
    Schur accumulation and the dense Cholesky timed on samples (see
    oracle_lm_iteration_sample). Returns a dict with the raw times and the
    extrapolated seconds per LM iteration."""
    packed = PackedProblem(problem)
    out = np.zeros(8)
    st = lib().oracle_lm_iteration_sample(C.byref(packed.struct), C.byref(_opts(options, **kw)),
                                          int(point_stride), int(chol_dim), out.ctypes.data)
    if st != 0:
        raise ValueError(f"oracle_lm_iteration_sample failed with status {st}")
    n = problem.reduced_dim()
    threads_used = max(1.0, out[7])
    n_pts_free = max(out[6], 1.0)
    schur_scale = (problem.num_points / point_stride) / n_pts_free * point_stride / threads_used
    chol_scale = (n / max(1, min(chol_dim, n))) ** 3
    est = out[0] + out[1] + out[2] * schur_scale + out[3] * chol_scale + out[4] + out[5]
    return {
        "jacobians_s": out[0], "assembly_s": out[1], "schur_sample_s": out[2], "schur_points": int(out[6]),
        "cholesky_sample_s": out[3], "chol_dim": int(min(chol_dim, n)), "backsub_update_s": out[4],
        "trial_cost_s": out[5], "threads": int(out[7]), "reduced_dim": n,
        "schur_scale": schur_scale, "cholesky_scale": chol_scale, "seconds_per_iteration": est,
        "measured_s": float(out[:6].sum()),
    }


def refine_pose_gauss_newton(poses, points3d_list, points2d_list, iterations: int) -> np.ndarray:
    """crates/sfm-geometry/src/pnp.rs:151-206 for each pose (rows of
    ``poses``, qw qx qy qz tx ty tz) over its own correspondences."""
    poses = np.ascontiguousarray(poses, dtype=np.float64).copy()
    off = np.concatenate([[0], np.cumsum([len(p) for p in points3d_list])]).astype(np.int64)
    X = np.ascontiguousarray(np.concatenate([np.asarray(p, np.float64).reshape(-1, 3) for p in points3d_list])
                             if len(points3d_list) else np.zeros((0, 3)))
    uv = np.ascontiguousarray(np.concatenate([np.asarray(p, np.float64).reshape(-1, 2) for p in points2d_list])
                              if len(points2d_list) else np.zeros((0, 2)))
    st = lib().oracle_refine_pose_gauss_newton(len(poses), off.ctypes.data, X.ctypes.data, uv.ctypes.data,
                                               int(iterations), poses.ctypes.data)
    if st != 0:
        raise ValueError(f"oracle_refine_pose_gauss_newton failed with status {st}")
    return poses


def pnp_ransac(points3d, points2d_norm, threshold: float, max_iterations: int):
    """crates/sfm-geometry/src/pnp.rs:211-309. Returns None or (pose [7],
    inlier mask, RANSAC iterations run)."""
    X = np.ascontiguousarray(points3d, dtype=np.float64).reshape(-1, 3)
    uv = np.ascontiguousarray(points2d_norm, dtype=np.float64).reshape(-1, 2)
    n = len(X)
    pose = np.zeros(7)
    mask = np.zeros(max(n, 1), np.uint8)
    found = C.c_int32(0)
    iters = C.c_int64(0)
    st = lib().oracle_pnp_ransac(n, X.ctypes.data, uv.ctypes.data, C.c_double(threshold), int(max_iterations),
                                 pose.ctypes.data, mask.ctypes.data, C.byref(found), C.byref(iters))
    if st != 0:
        raise ValueError(f"oracle_pnp_ransac failed with status {st}")
    if not found.value:
        return None
    return pose, mask[:n].astype(bool), int(iters.value)
