"""ctypes mirror of ``include/sfmba.h`` (the C ABI of libsfmba_gb300.so).

Only type definitions and the array-packing helpers live here; loading the
library is in :mod:`sfmtory_gb300.native`.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

MAX_CAMERA_PARAMS = 8
POSE_STRIDE = 7

# COLMAP model ids (crates/sfm-core/src/camera.rs:74-83).
SIMPLE_PINHOLE, PINHOLE, SIMPLE_RADIAL, RADIAL, OPENCV, OPENCV_FISHEYE = range(6)
MODEL_NAMES = ("SIMPLE_PINHOLE", "PINHOLE", "SIMPLE_RADIAL", "RADIAL", "OPENCV", "OPENCV_FISHEYE")
MODEL_DOF = (3, 4, 4, 5, 8, 8)  # camera.rs:136-163, params().len()

LOSS_NONE, LOSS_HUBER, LOSS_CAUCHY = range(3)
PRECISION_FP64, PRECISION_MIXED = range(2)
SOLVER_AUTO, SOLVER_DENSE, SOLVER_PCG = range(3)
# sfmba_intrinsics_mode (crates/sfm-reconstruction/src/lib.rs:1300-1316).
INTRINSICS_FIXED, INTRINSICS_FREE, INTRINSICS_FREE_GUARDED = range(3)

STATUS_NAMES = {
    0: "OK",
    1: "INVALID_ARGUMENT",
    2: "CUDA",
    3: "OUT_OF_MEMORY",
    4: "NO_DEVICE",
    5: "UNSUPPORTED",
    6: "INTERNAL",
}

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_up = C.POINTER(C.c_uint8)


class SfmbaProblem(C.Structure):
    _fields_ = [
        ("num_images", C.c_int64),
        ("num_cameras", C.c_int64),
        ("num_points", C.c_int64),
        ("num_observations", C.c_int64),
        ("camera_of_image", C.c_void_p),
        ("camera_model", C.c_void_p),
        ("camera_params", C.c_void_p),
        ("poses", C.c_void_p),
        ("points", C.c_void_p),
        ("obs_image", C.c_void_p),
        ("obs_point", C.c_void_p),
        ("obs_xy", C.c_void_p),
        ("fixed_poses", C.c_void_p),
        ("fixed_cameras", C.c_void_p),
        ("fixed_camera_params", C.c_void_p),
    ]


class SfmbaReconstruction(C.Structure):
    _fields_ = [
        ("num_images", C.c_int64),
        ("num_cameras", C.c_int64),
        ("num_points", C.c_int64),
        ("camera_of_image", C.c_void_p),
        ("camera_model", C.c_void_p),
        ("camera_params", C.c_void_p),
        ("poses", C.c_void_p),
        ("registered", C.c_void_p),
        ("pose_fixed", C.c_void_p),
        ("points", C.c_void_p),
        ("track_offsets", C.c_void_p),
        ("track_image", C.c_void_p),
        ("track_xy", C.c_void_p),
    ]


class SfmbaWindowBuffers(C.Structure):
    _fields_ = [(name, C.c_void_p) for name in (
        "image_ids", "camera_ids", "point_ids", "camera_of_image", "camera_model", "camera_params", "poses",
        "points", "obs_image", "obs_point", "obs_xy", "fixed_poses", "fixed_cameras", "fixed_camera_params")]


class SfmbaOptions(C.Structure):
    _fields_ = [
        ("max_iterations", C.c_int32),
        ("initial_lambda", C.c_double),
        ("robust_loss", C.c_int32),
        ("loss_scale_px", C.c_double),
        ("precision", C.c_int32),
        ("solver", C.c_int32),
        ("pcg_max_iterations", C.c_int32),
        ("pcg_tolerance", C.c_double),
        ("refinement_steps", C.c_int32),
        ("target_cost", C.c_double),
        ("dense_max_dim", C.c_int32),
        ("fp64_polish", C.c_int32),
        ("kernel_variant", C.c_int32),
        ("pcg_coarse_clusters", C.c_int32),
        ("dense_fp64_fma", C.c_int32),
        ("reserved", C.c_int32 * 3),
    ]


class SfmbaResult(C.Structure):
    _fields_ = [
        ("poses", C.c_void_p),
        ("points", C.c_void_p),
        ("camera_params", C.c_void_p),
        ("initial_cost", C.c_double),
        ("final_cost", C.c_double),
        ("iterations_run", C.c_int32),
        ("status", C.c_int32),
        ("damping_retries", C.c_int32),
        ("solver_used", C.c_int32),
        ("polish_iteration", C.c_int32),
        ("reserved_i", C.c_int32),
        ("linear_iterations", C.c_int64),
        ("reduced_dim", C.c_int64),
        ("valid_observations", C.c_int64),
        ("seconds", C.c_double),
        ("reserved", C.c_double * 4),
    ]


class SfmbaRefineReport(C.Structure):
    """sfmba_refine_report (statistics of crates/sfm-cli/src/main.rs cmd_refine)."""

    _fields_ = [
        ("num_images", C.c_int64),
        ("num_cameras", C.c_int64),
        ("num_points3d", C.c_int64),
        ("num_observations", C.c_int64),
        ("initial_cost", C.c_double),
        ("final_cost", C.c_double),
        ("iterations_run", C.c_int32),
        ("reserved_i", C.c_int32),
        ("mean_error_before_px", C.c_double),
        ("mean_error_after_px", C.c_double),
        ("seconds", C.c_double),
        ("reserved", C.c_double * 4),
    ]


def default_options(**overrides) -> SfmbaOptions:
    """Reference BaParams::default() (crates/sfm-ba/src/lib.rs:229-238) plus
    the GB300 solver controls; keyword arguments override fields."""
    o = SfmbaOptions()
    o.max_iterations = 50
    o.initial_lambda = 1e-3
    o.robust_loss = LOSS_HUBER
    o.loss_scale_px = 2.0
    o.precision = PRECISION_FP64
    o.solver = SOLVER_AUTO
    o.pcg_max_iterations = 100
    o.pcg_tolerance = 0.1
    o.refinement_steps = 1
    o.target_cost = 0.0
    o.dense_max_dim = 6000
    o.fp64_polish = 0
    for k, v in overrides.items():
        if not hasattr(o, k):
            raise AttributeError(f"sfmba_options has no field {k!r}")
        setattr(o, k, v)
    return o


def _ptr(a):
    return None if a is None else a.ctypes.data


class PackedProblem:
    """Contiguous typed arrays of one problem plus the sfmba_problem struct
    that points at them (host pointers). Keeps the arrays alive."""

    def __init__(self, p):
        self.camera_of_image = np.ascontiguousarray(p.camera_of_image, dtype=np.int32)
        self.camera_model = np.ascontiguousarray(p.camera_model, dtype=np.int32)
        cp = np.zeros((len(self.camera_model), MAX_CAMERA_PARAMS), dtype=np.float64)
        src = np.asarray(p.camera_params, dtype=np.float64)
        if src.size:
            src = src.reshape(len(self.camera_model), -1)
            cp[:, : src.shape[1]] = src
        self.camera_params = cp
        self.poses = np.ascontiguousarray(p.poses, dtype=np.float64).reshape(-1, POSE_STRIDE)
        self.points = np.ascontiguousarray(p.points, dtype=np.float64).reshape(-1, 3)
        self.obs_image = np.ascontiguousarray(p.obs_image, dtype=np.int32)
        self.obs_point = np.ascontiguousarray(p.obs_point, dtype=np.int32)
        self.obs_xy = np.ascontiguousarray(p.obs_xy, dtype=np.float64).reshape(-1, 2)
        self.fixed_poses = _mask(p.fixed_poses, len(self.poses))
        self.fixed_cameras = _mask(p.fixed_cameras, len(self.camera_model))
        self.fixed_camera_params = _param_mask(p.fixed_camera_params, len(self.camera_model))
        s = SfmbaProblem()
        s.num_images = len(self.poses)
        s.num_cameras = len(self.camera_model)
        s.num_points = len(self.points)
        s.num_observations = len(self.obs_image)
        s.camera_of_image = _ptr(self.camera_of_image)
        s.camera_model = _ptr(self.camera_model)
        s.camera_params = _ptr(self.camera_params)
        s.poses = _ptr(self.poses)
        s.points = _ptr(self.points)
        s.obs_image = _ptr(self.obs_image)
        s.obs_point = _ptr(self.obs_point)
        s.obs_xy = _ptr(self.obs_xy)
        s.fixed_poses = _ptr(self.fixed_poses)
        s.fixed_cameras = _ptr(self.fixed_cameras)
        s.fixed_camera_params = _ptr(self.fixed_camera_params)
        self.struct = s


def _mask(m, n):
    """Vec<bool> read with `.get(i).unwrap_or(false)`: shorter means false."""
    if m is None:
        return None
    out = np.zeros(n, dtype=np.uint8)
    m = np.asarray(m, dtype=bool).reshape(-1)[:n]
    out[: len(m)] = m
    return out


def _param_mask(m, n):
    """Vec<Vec<bool>> padded to [n][8]; missing rows/entries are false."""
    if m is None:
        return None
    out = np.zeros((n, MAX_CAMERA_PARAMS), dtype=np.uint8)
    if isinstance(m, np.ndarray) and m.ndim == 2:
        r, c = min(m.shape[0], n), min(m.shape[1], MAX_CAMERA_PARAMS)
        out[:r, :c] = m[:r, :c]
        return out
    for c, row in enumerate(list(m)[:n]):
        row = np.asarray(row, dtype=bool).reshape(-1)[:MAX_CAMERA_PARAMS]
        out[c, : len(row)] = row
    return out


class ResultBuffers:
    """Caller-owned output arrays of one solve plus the sfmba_result struct."""

    def __init__(self, packed: PackedProblem):
        self.poses = np.zeros_like(packed.poses)
        self.points = np.zeros_like(packed.points)
        self.camera_params = np.zeros_like(packed.camera_params)
        r = SfmbaResult()
        r.poses = _ptr(self.poses)
        r.points = _ptr(self.points)
        r.camera_params = _ptr(self.camera_params)
        self.struct = r
