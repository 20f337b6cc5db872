"""ctypes binding of libsfmba_gb300.so (the C ABI in include/sfmba.h).

There is no fallback: if the CUDA library is missing or no GPU is present,
every call raises. Build the library with ``python -m sfmtory_gb300.build``
(or ``__graft_entry__.build()``).
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

from .abi import (
    STATUS_NAMES,
    PackedProblem,
    ResultBuffers,
    SfmbaOptions,
    SfmbaProblem,
    SfmbaResult,
    default_options,
)

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libsfmba_gb300.so")
_lock = threading.Lock()
_lib = None

#: Every entry point declared in include/sfmba.h.
EXPORTED_SYMBOLS = (
    "sfmba_default_options",
    "sfmba_bundle_adjust",
    "sfmba_bundle_adjust_device",
    "sfmba_mean_reprojection_error",
    "sfmba_total_cost",
    "sfmba_default_fixed_params_mask",
    "sfmba_refine_intrinsics",
    "sfmba_bundle_adjust_batched",
    "sfmba_filter_and_reoptimize",
    "sfmba_adjust_global",
    "sfmba_refine_pose_gauss_newton_batched",
    "sfmba_pnp_ransac_batched",
    "sfmba_local_windows",
    "sfmba_colmap_refine",
    "sfmba_colmap_rewrite",
    "sfmba_colmap_model_stats",
    "sfmba_residuals_jacobians",
    "sfmba_total_cost_noalloc",
    "sfmba_measure_peaks",
    "sfmba_dense_cholesky",
    "sfmba_profile_enable",
    "sfmba_profile_report",
    "sfmba_last_error",
    "sfmba_version",
)


class SfmbaError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def load(path: str | None = None):
    """Load the library (no compute call). Raises if it is missing."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise RuntimeError(
                f"{p} is missing: the CUDA bundle adjuster has not been built "
                "(run `python -m sfmtory_gb300.build`); there is no CPU fallback")
        L = C.CDLL(p)
        vp = C.c_void_p
        L.sfmba_default_options.argtypes = [vp]
        L.sfmba_default_options.restype = None
        for name in ("sfmba_bundle_adjust",):
            getattr(L, name).argtypes = [vp, vp, vp]
        L.sfmba_bundle_adjust_device.argtypes = [vp, vp, vp, vp]
        L.sfmba_mean_reprojection_error.argtypes = [vp, vp]
        L.sfmba_total_cost.argtypes = [vp, vp, vp]
        L.sfmba_default_fixed_params_mask.argtypes = [C.c_int64, vp, vp]
        L.sfmba_refine_intrinsics.argtypes = [vp, vp, vp]
        L.sfmba_bundle_adjust_batched.argtypes = [C.c_int32, vp, vp, vp]
        L.sfmba_filter_and_reoptimize.argtypes = [vp, vp, C.c_double, vp, vp]
        L.sfmba_adjust_global.argtypes = [vp, vp, C.c_int32, C.c_double, vp, vp, vp, vp]
        L.sfmba_refine_pose_gauss_newton_batched.argtypes = [C.c_int32, vp, vp, vp, C.c_int32, vp]
        L.sfmba_pnp_ransac_batched.argtypes = [C.c_int32, vp, vp, vp, C.c_double, C.c_int32, vp, vp, vp, vp]
        L.sfmba_colmap_refine.argtypes = [C.c_char_p, C.c_char_p, vp, C.c_int32, vp]
        L.sfmba_colmap_rewrite.argtypes = [C.c_char_p, C.c_char_p]
        L.sfmba_colmap_model_stats.argtypes = [C.c_char_p, vp, vp]
        L.sfmba_residuals_jacobians.argtypes = [vp, C.c_int32, vp, vp, vp, vp, vp]
        L.sfmba_total_cost_noalloc.argtypes = [vp, vp, vp, vp]
        L.sfmba_local_windows.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, vp, vp, vp]
        L.sfmba_measure_peaks.argtypes = [vp]
        L.sfmba_dense_cholesky.argtypes = [C.c_int64, vp, vp, C.c_int32, vp]
        L.sfmba_profile_enable.argtypes = [C.c_int32]
        L.sfmba_profile_report.argtypes = [C.c_char_p, C.c_int64]
        L.sfmba_last_error.restype = C.c_char_p
        L.sfmba_version.restype = C.c_char_p
        _lib = L
        return L


def _check(status: int):
    if status != 0:
        msg = load().sfmba_last_error().decode(errors="replace")
        raise SfmbaError(status, msg)


def options(**kw) -> SfmbaOptions:
    return default_options(**kw)


class Result:
    """Outputs of one solve (the fields of sfm-ba's BaOutput plus solver stats)."""

    def __init__(self, buf: ResultBuffers):
        r = buf.struct
        self.poses = buf.poses
        self.points = buf.points
        self.camera_params = buf.camera_params
        self.initial_cost = r.initial_cost
        self.final_cost = r.final_cost
        self.iterations_run = r.iterations_run
        self.damping_retries = r.damping_retries
        self.solver_used = r.solver_used
        self.polish_iteration = r.polish_iteration
        self.linear_iterations = r.linear_iterations
        self.reduced_dim = r.reduced_dim
        self.valid_observations = r.valid_observations
        self.seconds = r.seconds


def bundle_adjust_arrays(problem, opts: SfmbaOptions | None = None, **kw) -> Result:
    """Solve a :class:`~sfmtory_gb300.problem.Problem` through sfmba_bundle_adjust."""
    L = load()
    packed = PackedProblem(problem)
    buf = ResultBuffers(packed)
    o = opts if opts is not None else default_options(**kw)
    if opts is not None and kw:
        for k, v in kw.items():
            setattr(o, k, v)
    _check(L.sfmba_bundle_adjust(C.byref(packed.struct), C.byref(o), C.byref(buf.struct)))
    return Result(buf)


def total_cost(problem, opts: SfmbaOptions | None = None, **kw) -> float:
    L = load()
    packed = PackedProblem(problem)
    out = C.c_double()
    o = opts if opts is not None else default_options(**kw)
    _check(L.sfmba_total_cost(C.byref(packed.struct), C.byref(o), C.byref(out)))
    return out.value


def mean_reprojection_error_arrays(problem) -> float:
    L = load()
    packed = PackedProblem(problem)
    out = C.c_double()
    _check(L.sfmba_mean_reprojection_error(C.byref(packed.struct), C.byref(out)))
    return out.value


def default_fixed_params_mask_arrays(models) -> np.ndarray:
    L = load()
    models = np.ascontiguousarray(models, dtype=np.int32)
    out = np.zeros((len(models), 8), dtype=np.uint8)
    _check(L.sfmba_default_fixed_params_mask(len(models), models.ctypes.data, out.ctypes.data))
    return out.astype(bool)


def refine_intrinsics_arrays(problem, opts: SfmbaOptions | None = None, **kw) -> np.ndarray:
    L = load()
    packed = PackedProblem(problem)
    cams = packed.camera_params.copy()
    base = dict(max_iterations=30)
    base.update(kw)
    o = opts if opts is not None else default_options(**base)
    _check(L.sfmba_refine_intrinsics(C.byref(packed.struct), C.byref(o), cams.ctypes.data))
    return cams


def residuals_jacobians(problem, fp32: bool = False):
    """(r [n,2], J_pose [n,2,6], J_point [n,2,3], J_cam [n,2,8], valid [n]) from the GPU kernels."""
    L = load()
    packed = PackedProblem(problem)
    n = len(packed.obs_image)
    r = np.zeros((n, 2))
    jp = np.zeros((n, 2, 6))
    jx = np.zeros((n, 2, 3))
    jc = np.zeros((n, 2, 8))
    valid = np.zeros(n, np.uint8)
    _check(L.sfmba_residuals_jacobians(C.byref(packed.struct), 1 if fp32 else 0, r.ctypes.data,
                                       jp.ctypes.data, jx.ctypes.data, jc.ctypes.data, valid.ctypes.data))
    return r, jp, jx, jc, valid.astype(bool)


def local_windows(rec, centers, seed_image: int = -1, num_free_neighbours: int = 6):
    """BaScope::Local windows (crates/sfm-reconstruction/src/lib.rs:1336-1473)
    of a :class:`~sfmtory_gb300.problem.Reconstruction` for each centre image,
    through sfmba_local_windows. Returns, per centre, None where the
    reference makes no solve, else (Problem, image_ids, camera_ids,
    point_ids) with the reconstruction indices of the window's entries."""
    from .abi import SfmbaReconstruction, SfmbaWindowBuffers
    from .problem import Problem

    L = load()
    keep = []

    def ptr(a, dtype):
        a = np.ascontiguousarray(a, dtype=dtype)
        keep.append(a)
        return a.ctypes.data

    R = SfmbaReconstruction()
    R.num_images, R.num_cameras, R.num_points = len(rec.poses), len(rec.camera_model), len(rec.points)
    R.camera_of_image = ptr(rec.camera_of_image, np.int32)
    R.camera_model = ptr(rec.camera_model, np.int32)
    cp = np.zeros((len(rec.camera_model), 8))
    cp[:, : np.asarray(rec.camera_params).shape[1]] = rec.camera_params
    R.camera_params = ptr(cp, np.float64)
    R.poses = ptr(rec.poses, np.float64)
    R.registered = ptr(rec.registered, np.uint8)
    R.pose_fixed = ptr(rec.pose_fixed, np.uint8) if rec.pose_fixed is not None else None
    R.points = ptr(rec.points, np.float64)
    R.track_offsets = ptr(rec.track_offsets, np.int64)
    R.track_image = ptr(rec.track_image, np.int32)
    R.track_xy = ptr(np.asarray(rec.track_xy, np.float64).reshape(-1, 2), np.float64)
    cen = np.ascontiguousarray(centers, dtype=np.int32)
    counts = np.zeros((len(cen), 4), np.int64)
    _check(L.sfmba_local_windows(C.byref(R), int(seed_image), int(num_free_neighbours), len(cen), cen.ctypes.data,
                                 counts.ctypes.data, None))
    bufs = (SfmbaWindowBuffers * max(1, len(cen)))()
    arrays = []
    for k, (nI, nC, nP, nO) in enumerate(counts):
        a = dict(image_ids=np.zeros(nI, np.int32), camera_ids=np.zeros(nC, np.int32), point_ids=np.zeros(nP, np.int32),
                 camera_of_image=np.zeros(nI, np.int32), camera_model=np.zeros(nC, np.int32),
                 camera_params=np.zeros((nC, 8)), poses=np.zeros((nI, 7)), points=np.zeros((nP, 3)),
                 obs_image=np.zeros(nO, np.int32), obs_point=np.zeros(nO, np.int32), obs_xy=np.zeros((nO, 2)),
                 fixed_poses=np.zeros(nI, np.uint8), fixed_cameras=np.zeros(nC, np.uint8),
                 fixed_camera_params=np.zeros((nC, 8), np.uint8))
        for name, arr in a.items():
            setattr(bufs[k], name, arr.ctypes.data if arr.size else None)
        arrays.append(a)
    _check(L.sfmba_local_windows(C.byref(R), int(seed_image), int(num_free_neighbours), len(cen), cen.ctypes.data,
                                 counts.ctypes.data, bufs))
    out = []
    for k, a in enumerate(arrays):
        if counts[k, 3] == 0:
            out.append(None)
            continue
        prob = Problem(camera_of_image=a["camera_of_image"], camera_model=a["camera_model"],
                       camera_params=a["camera_params"], poses=a["poses"], points=a["points"],
                       obs_image=a["obs_image"], obs_point=a["obs_point"], obs_xy=a["obs_xy"],
                       fixed_poses=a["fixed_poses"].astype(bool), fixed_cameras=a["fixed_cameras"].astype(bool),
                       fixed_camera_params=a["fixed_camera_params"].astype(bool),
                       meta={"name": "local_window", "center": int(cen[k])})
        out.append((prob, a["image_ids"], a["camera_ids"], a["point_ids"]))
    return out


def bundle_adjust_batched_arrays(problems, opts: SfmbaOptions | None = None, **kw) -> list[Result]:
    L = load()
    packs = [PackedProblem(p) for p in problems]
    bufs = [ResultBuffers(p) for p in packs]
    arr = (SfmbaProblem * len(packs))(*[p.struct for p in packs])
    res = (SfmbaResult * len(bufs))(*[b.struct for b in bufs])
    o = opts if opts is not None else default_options(**kw)
    _check(L.sfmba_bundle_adjust_batched(len(packs), arr, C.byref(o), res))
    out = []
    for k, b in enumerate(bufs):
        b.struct = res[k]
        out.append(Result(b))
    return out


def filter_and_reoptimize_arrays(problem, threshold_px: float, opts: SfmbaOptions | None = None, **kw):
    """crates/sfm-reconstruction/src/lib.rs:1722-1768 on the GPU: returns the
    last adjustment's Result and the keep mask of the input observations it
    used."""
    L = load()
    packed = PackedProblem(problem)
    buf = ResultBuffers(packed)
    o = opts if opts is not None else default_options(**kw)
    keep = np.zeros(max(packed.struct.num_observations, 1), dtype=np.uint8)
    _check(L.sfmba_filter_and_reoptimize(C.byref(packed.struct), C.byref(o), C.c_double(threshold_px),
                                         C.byref(buf.struct), keep.ctypes.data))
    return Result(buf), keep[: packed.struct.num_observations].astype(bool)


def adjust_global_arrays(problem, mode: int, threshold_px: float, opts: SfmbaOptions | None = None, **kw):
    """The fixed-vs-free intrinsics handling of the reference's global
    adjustment (crates/sfm-reconstruction/src/lib.rs:1567-1708) on the GPU.
    Returns (Result of the chosen adjustment, keep mask, chose_free,
    (fixed mean error, free mean error))."""
    L = load()
    packed = PackedProblem(problem)
    buf = ResultBuffers(packed)
    o = opts if opts is not None else default_options(**kw)
    keep = np.zeros(max(packed.struct.num_observations, 1), dtype=np.uint8)
    chose = C.c_int32(-1)
    errs = np.full(2, np.nan)
    _check(L.sfmba_adjust_global(C.byref(packed.struct), C.byref(o), C.c_int32(mode), C.c_double(threshold_px),
                                 C.byref(buf.struct), keep.ctypes.data, C.byref(chose), errs.ctypes.data))
    return (Result(buf), keep[: packed.struct.num_observations].astype(bool), bool(chose.value),
            (float(errs[0]), float(errs[1])))


def _pack_correspondences(points3d_list, points2d_list):
    if len(points3d_list) != len(points2d_list):
        raise ValueError("points3d and points2d lists differ in length")
    n = [len(p) for p in points3d_list]
    if any(len(b) != a for a, b in zip(n, points2d_list)):
        raise ValueError("a 3D/2D correspondence set differs in length")
    off = np.concatenate([[0], np.cumsum(n)]).astype(np.int64)
    X = np.ascontiguousarray(np.concatenate([np.asarray(p, np.float64).reshape(-1, 3) for p in points3d_list])
                             if n and off[-1] else np.zeros((1, 3)))
    uv = np.ascontiguousarray(np.concatenate([np.asarray(p, np.float64).reshape(-1, 2) for p in points2d_list])
                              if n and off[-1] else np.zeros((1, 2)))
    return off, X, uv


def refine_pose_gauss_newton_batched(poses, points3d_list, points2d_list, iterations: int) -> np.ndarray:
    """crates/sfm-geometry/src/pnp.rs:151-206 on the GPU for every pose
    (rows qw qx qy qz tx ty tz) over its own correspondences."""
    L = load()
    off, X, uv = _pack_correspondences(points3d_list, points2d_list)
    out = np.ascontiguousarray(poses, dtype=np.float64).reshape(-1, 7).copy()
    if len(out) != len(off) - 1:
        raise ValueError("one pose per correspondence set")
    _check(L.sfmba_refine_pose_gauss_newton_batched(len(out), off.ctypes.data, X.ctypes.data, uv.ctypes.data,
                                                    int(iterations), out.ctypes.data))
    return out


def pnp_ransac_batched(points3d_list, points2d_list, threshold: float, max_iterations: int):
    """crates/sfm-geometry/src/pnp.rs:211-309 on the GPU for many images.
    Returns, per image, None or (pose [7], inlier mask, RANSAC iterations)."""
    L = load()
    off, X, uv = _pack_correspondences(points3d_list, points2d_list)
    P = len(off) - 1
    poses = np.zeros((max(P, 1), 7))
    mask = np.zeros(max(int(off[-1]), 1), np.uint8)
    found = np.zeros(max(P, 1), np.int32)
    iters = np.zeros(max(P, 1), np.int64)
    _check(L.sfmba_pnp_ransac_batched(P, off.ctypes.data, X.ctypes.data, uv.ctypes.data, C.c_double(threshold),
                                      int(max_iterations), poses.ctypes.data, mask.ctypes.data,
                                      found.ctypes.data, iters.ctypes.data))
    out = []
    for k in range(P):
        if not found[k]:
            out.append(None)
        else:
            out.append((poses[k].copy(), mask[off[k]:off[k + 1]].astype(bool), int(iters[k])))
    return out


def colmap_refine(dir_in: str, dir_out: str | None = None, refine_intrinsics: bool = False,
                  opts: SfmbaOptions | None = None, **kw) -> dict:
    """`sfmtory refine` (crates/sfm-cli/src/main.rs:946-1130) on the COLMAP
    text model in ``dir_in``, written to ``dir_out`` (default: in place).
    Without options the reference's Huber loss and 200 iterations; keyword
    arguments override option fields. Returns the report as a dict."""
    from .abi import SfmbaRefineReport

    L = load()
    o = opts
    if o is None and kw:
        base = dict(robust_loss=1, max_iterations=200)
        base.update(kw)
        o = default_options(**base)
    rep = SfmbaRefineReport()
    _check(L.sfmba_colmap_refine(os.fsencode(dir_in), os.fsencode(dir_out or dir_in),
                                 C.byref(o) if o is not None else None, 1 if refine_intrinsics else 0,
                                 C.byref(rep)))
    return {f: getattr(rep, f) for f, _ in SfmbaRefineReport._fields_ if not f.startswith("reserved")}


def colmap_rewrite(dir_in: str, dir_out: str) -> None:
    """crates/sfm-io/src/colmap.rs read_model then write_model."""
    _check(load().sfmba_colmap_rewrite(os.fsencode(dir_in), os.fsencode(dir_out)))


def colmap_model_stats(dir: str) -> dict:
    """Counts of the text model in ``dir`` and its
    Reconstruction::mean_reprojection_error."""
    counts = np.zeros(5, np.int64)
    err = C.c_double(0.0)
    _check(load().sfmba_colmap_model_stats(os.fsencode(dir), counts.ctypes.data, C.byref(err)))
    keys = ("cameras", "images", "points3d", "track_elements", "keypoints")
    out = {k: int(v) for k, v in zip(keys, counts)}
    out["mean_reprojection_error"] = err.value
    return out


def measure_peaks() -> dict:
    """TFLOP/s of the GPU's FP64 FMA, FP64 mma.sync and BF16 mma.sync units."""
    out = np.zeros(3)
    _check(load().sfmba_measure_peaks(out.ctypes.data))
    return {"dfma_tflops": float(out[0]), "dmma_tflops": float(out[1]), "bf16_mma_tflops": float(out[2])}


def dense_cholesky(A: np.ndarray, tensor_update: bool = True):
    """(L, seconds): the dense solver's blocked Cholesky of the SPD matrix A on the GPU."""
    A = np.ascontiguousarray(A, dtype=np.float64)
    n = A.shape[0]
    L = np.zeros_like(A)
    sec = C.c_double(0.0)
    _check(load().sfmba_dense_cholesky(n, A.ctypes.data, L.ctypes.data, 1 if tensor_update else 0,
                                       C.byref(sec)))
    return L, sec.value


def profile_enable(on: bool = True) -> None:
    """Per-phase CUDA-event timing of later solves on this thread (clears totals)."""
    _check(load().sfmba_profile_enable(1 if on else 0))


def profile_report() -> dict:
    """{phase: {"ms": device milliseconds, "launches": count}} since profile_enable."""
    import json

    size = 1 << 16
    while True:
        buf = C.create_string_buffer(size)
        st = load().sfmba_profile_report(buf, len(buf))
        if st == 0:
            return json.loads(buf.value.decode())
        msg = load().sfmba_last_error().decode(errors="replace")
        if "need" not in msg or size >= 1 << 26:
            _check(st)
        size *= 4


def version() -> str:
    return load().sfmba_version().decode()
