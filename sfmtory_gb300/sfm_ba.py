"""The public interface of sfmtory's ``sfm-ba`` crate, over the GB300 C ABI.

Names, fields and defaults follow the Rust crate so a caller (or a test
written like the crate's own tests) reads the same:

* ``CameraModel`` - crates/sfm-core/src/camera.rs:21-244 (COLMAP names, ids,
  ``params()`` order, ``from_name_and_params``, ``project``);
* ``Pose`` - crates/sfm-core/src/pose.rs:15-81 (world-to-camera, Hamilton
  quaternion w, x, y, z);
* ``Observation``, ``BaInput``, ``RobustLoss``, ``BaParams``, ``BaOutput``,
  ``bundle_adjust``, ``mean_reprojection_error`` - crates/sfm-ba/src/lib.rs:56-247, :708, :747;
* ``default_fixed_params_mask``, ``IntrinsicsRefineParams``,
  ``refine_intrinsics`` - crates/sfm-ba/src/intrinsics.rs:49-147.

The solve itself runs on the GPU (libsfmba_gb300.so); there is no CPU path.
"""
from __future__ import annotations

import enum
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import abi, native
from .problem import Problem, project as _project, quat_rotate

_NAMES = abi.MODEL_NAMES
_PARAM_NAMES = (
    ("f", "cx", "cy"),
    ("fx", "fy", "cx", "cy"),
    ("f", "cx", "cy", "k"),
    ("f", "cx", "cy", "k1", "k2"),
    ("fx", "fy", "cx", "cy", "k1", "k2", "p1", "p2"),
    ("fx", "fy", "cx", "cy", "k1", "k2", "k3", "k4"),
)


@dataclass(frozen=True)
class CameraModel:
    """One camera's intrinsics: COLMAP model id and its parameter vector."""

    model_id: int
    param_values: tuple

    @staticmethod
    def from_name_and_params(name: str, params: Sequence[float]) -> Optional["CameraModel"]:
        if name not in _NAMES:
            return None
        m = _NAMES.index(name)
        k = abi.MODEL_DOF[m]
        return CameraModel(m, tuple(float(x) for x in list(params)[:k]))

    @staticmethod
    def simple_pinhole(f, cx, cy):
        return CameraModel(abi.SIMPLE_PINHOLE, (f, cx, cy))

    @staticmethod
    def pinhole(fx, fy, cx, cy):
        return CameraModel(abi.PINHOLE, (fx, fy, cx, cy))

    @staticmethod
    def simple_radial(f, cx, cy, k):
        return CameraModel(abi.SIMPLE_RADIAL, (f, cx, cy, k))

    @staticmethod
    def radial(f, cx, cy, k1, k2):
        return CameraModel(abi.RADIAL, (f, cx, cy, k1, k2))

    @staticmethod
    def opencv(fx, fy, cx, cy, k1, k2, p1, p2):
        return CameraModel(abi.OPENCV, (fx, fy, cx, cy, k1, k2, p1, p2))

    @staticmethod
    def opencv_fisheye(fx, fy, cx, cy, k1, k2, k3, k4):
        return CameraModel(abi.OPENCV_FISHEYE, (fx, fy, cx, cy, k1, k2, k3, k4))

    def name(self) -> str:
        return _NAMES[self.model_id]

    def params(self) -> List[float]:
        return list(self.param_values)

    def __getattr__(self, item):
        names = _PARAM_NAMES[object.__getattribute__(self, "model_id")]
        if item in names:
            return self.param_values[names.index(item)]
        raise AttributeError(item)

    def project(self, p_camera) -> tuple:
        pc = np.asarray(p_camera, dtype=np.float64).reshape(1, 3)
        row = np.zeros((1, 8))
        row[0, : len(self.param_values)] = self.param_values
        uv = _project(np.array([self.model_id]), row, pc)[0]
        return float(uv[0]), float(uv[1])


@dataclass(frozen=True)
class Pose:
    """World-to-camera pose: X_cam = R X_world + t, R a unit quaternion (w, x, y, z)."""

    rotation: tuple = (1.0, 0.0, 0.0, 0.0)
    translation: tuple = (0.0, 0.0, 0.0)

    @staticmethod
    def identity() -> "Pose":
        return Pose()

    @staticmethod
    def from_quaternion_wxyz_translation(q, t) -> "Pose":
        q = np.asarray(q, dtype=np.float64)
        q = q / np.linalg.norm(q)
        return Pose(tuple(float(x) for x in q), tuple(float(x) for x in t))

    @staticmethod
    def from_rotation_translation(q, t) -> "Pose":
        return Pose.from_quaternion_wxyz_translation(q, t)

    def quaternion_wxyz(self):
        return list(self.rotation)

    def transform_point(self, p):
        return quat_rotate(np.asarray(self.rotation), np.asarray(p, dtype=np.float64)) + np.asarray(self.translation)

    def camera_center(self):
        q = np.asarray(self.rotation)
        qi = q * np.array([1.0, -1.0, -1.0, -1.0])
        return -quat_rotate(qi, np.asarray(self.translation))

    def as_array(self) -> np.ndarray:
        return np.array(list(self.rotation) + list(self.translation))


@dataclass(frozen=True)
class Observation:
    image_idx: int
    point_idx: int
    x: float
    y: float


class RobustLoss(enum.IntEnum):
    NONE = abi.LOSS_NONE
    HUBER = abi.LOSS_HUBER
    CAUCHY = abi.LOSS_CAUCHY


@dataclass
class BaParams:
    """crates/sfm-ba/src/lib.rs:220-238; the remaining fields select the GB300 path."""

    max_iterations: int = 50
    initial_lambda: float = 1e-3
    robust_loss: RobustLoss = RobustLoss.HUBER
    loss_scale_px: float = 2.0
    precision: int = abi.PRECISION_FP64
    solver: int = abi.SOLVER_AUTO
    pcg_max_iterations: int = 100
    pcg_tolerance: float = 0.1
    refinement_steps: int = 1
    target_cost: float = 0.0
    fp64_polish: bool = False

    def to_options(self) -> abi.SfmbaOptions:
        return abi.default_options(
            max_iterations=int(self.max_iterations), initial_lambda=float(self.initial_lambda),
            robust_loss=int(self.robust_loss), loss_scale_px=float(self.loss_scale_px),
            precision=int(self.precision), solver=int(self.solver),
            pcg_max_iterations=int(self.pcg_max_iterations), pcg_tolerance=float(self.pcg_tolerance),
            refinement_steps=int(self.refinement_steps), target_cost=float(self.target_cost),
            fp64_polish=int(bool(self.fp64_polish)))


@dataclass
class BaInput:
    camera_of_image: List[int]
    cameras: List[CameraModel]
    poses: List[Pose]
    points: List[Sequence[float]]
    observations: List[Observation]
    fixed_poses: List[bool] = field(default_factory=list)
    fixed_cameras: List[bool] = field(default_factory=list)
    fixed_camera_params: List[List[bool]] = field(default_factory=list)

    def to_problem(self) -> Problem:
        cp = np.zeros((len(self.cameras), 8))
        for c, cam in enumerate(self.cameras):
            cp[c, : len(cam.param_values)] = cam.param_values
        obs = self.observations
        return Problem(
            camera_of_image=np.asarray(self.camera_of_image, np.int32),
            camera_model=np.asarray([c.model_id for c in self.cameras], np.int32),
            camera_params=cp,
            poses=np.asarray([p.as_array() for p in self.poses], np.float64).reshape(-1, 7),
            points=np.asarray(self.points, np.float64).reshape(-1, 3),
            obs_image=np.asarray([o.image_idx for o in obs], np.int32),
            obs_point=np.asarray([o.point_idx for o in obs], np.int32),
            obs_xy=np.asarray([(o.x, o.y) for o in obs], np.float64).reshape(-1, 2),
            fixed_poses=np.asarray(self.fixed_poses, bool) if len(self.fixed_poses) else None,
            fixed_cameras=np.asarray(self.fixed_cameras, bool) if len(self.fixed_cameras) else None,
            fixed_camera_params=self.fixed_camera_params if len(self.fixed_camera_params) else None,
        )


@dataclass
class BaOutput:
    poses: List[Pose]
    points: List[np.ndarray]
    cameras: List[CameraModel]
    initial_cost: float
    final_cost: float
    iterations_run: int


def bundle_adjust(input: BaInput, params: BaParams = BaParams()) -> BaOutput:
    """crates/sfm-ba/src/lib.rs:747 - joint pose/point/intrinsics LM on the GPU."""
    p = input.to_problem()
    r = native.bundle_adjust_arrays(p, params.to_options())
    cams = [CameraModel(c.model_id, tuple(float(x) for x in r.camera_params[k, : len(c.param_values)]))
            for k, c in enumerate(input.cameras)]
    poses = [Pose(tuple(map(float, r.poses[i, :4])), tuple(map(float, r.poses[i, 4:])))
             for i in range(len(input.poses))]
    return BaOutput(poses, [r.points[k].copy() for k in range(len(r.points))], cams,
                    r.initial_cost, r.final_cost, r.iterations_run)


def bundle_adjust_batched(inputs: Sequence[BaInput], params: BaParams = BaParams()) -> List[BaOutput]:
    """Many independent windows (sfm-reconstruction's BaScope::Local calls,
    crates/sfm-reconstruction/src/lib.rs:1287-1299) in one GPU solve, each
    window with its own damping and stopping; one BaOutput per window, as
    ``bundle_adjust`` would return it."""
    problems = [inp.to_problem() for inp in inputs]
    res = native.bundle_adjust_batched_arrays(problems, params.to_options())
    out = []
    for inp, r in zip(inputs, res):
        cams = [CameraModel(c.model_id, tuple(float(x) for x in r.camera_params[k, : len(c.param_values)]))
                for k, c in enumerate(inp.cameras)]
        poses = [Pose(tuple(map(float, r.poses[i, :4])), tuple(map(float, r.poses[i, 4:])))
                 for i in range(len(inp.poses))]
        out.append(BaOutput(poses, [r.points[k].copy() for k in range(len(r.points))], cams,
                            r.initial_cost, r.final_cost, r.iterations_run))
    return out


def filter_and_reoptimize(input: BaInput, params: BaParams, threshold_px: float) -> BaOutput:
    """crates/sfm-reconstruction/src/lib.rs:1722-1768 - adjust, drop
    observations behind their camera or beyond ``threshold_px``, adjust
    again (at most two filter rounds, never below 12 observations); all on
    the GPU."""
    r, _ = native.filter_and_reoptimize_arrays(input.to_problem(), threshold_px, params.to_options())
    cams = [CameraModel(c.model_id, tuple(float(x) for x in r.camera_params[k, : len(c.param_values)]))
            for k, c in enumerate(input.cameras)]
    poses = [Pose(tuple(map(float, r.poses[i, :4])), tuple(map(float, r.poses[i, 4:])))
             for i in range(len(input.poses))]
    return BaOutput(poses, [r.points[k].copy() for k in range(len(r.points))], cams,
                    r.initial_cost, r.final_cost, r.iterations_run)


class IntrinsicsMode(enum.IntEnum):
    """crates/sfm-reconstruction/src/lib.rs:1300-1316."""

    FIXED = 0
    FREE = 1
    FREE_GUARDED = 2


#: max_iterations the reference's run_bundle_adjustment gives each mode
#: (crates/sfm-reconstruction/src/lib.rs:1494-1520).
GLOBAL_MAX_ITERATIONS = {IntrinsicsMode.FREE_GUARDED: 200, IntrinsicsMode.FREE: 50, IntrinsicsMode.FIXED: 50}


def adjust_global(input: BaInput, params: BaParams, intrinsics: IntrinsicsMode,
                  max_reprojection_error_px: float) -> Tuple[BaOutput, bool]:
    """The intrinsics handling of the reference's global bundle adjustment
    (crates/sfm-reconstruction/src/lib.rs:1567-1708) over a built BaInput:
    FIXED holds every camera; FREE frees the cameras seen by >= 5 images
    that ``input.fixed_cameras`` does not fix; FREE_GUARDED runs
    ``filter_and_reoptimize`` both ways and keeps the free result only if
    its distortion is plausible (|d| < 0.5) and its plain mean reprojection
    error is lower. ``params`` is used as given (the reference's caller
    picks ``max_iterations`` per mode, see GLOBAL_MAX_ITERATIONS). Returns
    the chosen output and whether it is the intrinsics-free one."""
    r, _, chose_free, _ = native.adjust_global_arrays(input.to_problem(), int(intrinsics),
                                                      max_reprojection_error_px, params.to_options())
    cams = [CameraModel(c.model_id, tuple(float(x) for x in r.camera_params[k, : len(c.param_values)]))
            for k, c in enumerate(input.cameras)]
    poses = [Pose(tuple(map(float, r.poses[i, :4])), tuple(map(float, r.poses[i, 4:])))
             for i in range(len(input.poses))]
    return BaOutput(poses, [r.points[k].copy() for k in range(len(r.points))], cams,
                    r.initial_cost, r.final_cost, r.iterations_run), chose_free


def mean_reprojection_error(input: BaInput) -> float:
    """crates/sfm-ba/src/lib.rs:708-725."""
    return native.mean_reprojection_error_arrays(input.to_problem())


def default_fixed_params_mask(cameras: Sequence[CameraModel]) -> List[List[bool]]:
    """crates/sfm-ba/src/intrinsics.rs:49-61."""
    m = native.default_fixed_params_mask_arrays([c.model_id for c in cameras])
    return [list(map(bool, m[k, : len(c.param_values)])) for k, c in enumerate(cameras)]


@dataclass
class IntrinsicsRefineParams:
    """crates/sfm-ba/src/intrinsics.rs:66-83."""

    max_iterations: int = 30
    initial_lambda: float = 1e-3
    robust_loss: RobustLoss = RobustLoss.HUBER
    loss_scale_px: float = 2.0


def refine_intrinsics(cameras: List[CameraModel], camera_of_image: Sequence[int], poses: Sequence[Pose],
                      points, observations: Sequence[Observation],
                      params: IntrinsicsRefineParams = IntrinsicsRefineParams()) -> None:
    """crates/sfm-ba/src/intrinsics.rs:116-147 - updates ``cameras`` in place."""
    inp = BaInput(list(camera_of_image), list(cameras), list(poses), list(points), list(observations))
    o = abi.default_options(max_iterations=params.max_iterations, initial_lambda=params.initial_lambda,
                            robust_loss=int(params.robust_loss), loss_scale_px=params.loss_scale_px)
    out = native.refine_intrinsics_arrays(inp.to_problem(), o)
    for k, c in enumerate(cameras):
        cameras[k] = CameraModel(c.model_id, tuple(float(x) for x in out[k, : len(c.param_values)]))
