"""Array form of a bundle-adjustment problem (the data of sfm-ba's ``BaInput``,
crates/sfm-ba/src/lib.rs:64-96) and vectorised numpy geometry used to build
synthetic scenes. Nothing here is on the solve path; the solver is the CUDA
library behind :mod:`sfmtory_gb300.native`."""
from __future__ import annotations

from dataclasses import dataclass, field, replace
from typing import Optional

import numpy as np

from .abi import MAX_CAMERA_PARAMS, MODEL_DOF, OPENCV, OPENCV_FISHEYE, PINHOLE, RADIAL, SIMPLE_PINHOLE, SIMPLE_RADIAL


@dataclass
class Problem:
    """One bundle-adjustment problem in structure-of-arrays form.

    poses: [nI, 7] world-to-camera (qw, qx, qy, qz, tx, ty, tz);
    camera_params: [nC, 8] in ``CameraModel::params()`` order, zero padded;
    observations: image index, point index, pixel (x, y).
    Masks follow the Rust semantics: ``None`` or a short array means False.
    """

    camera_of_image: np.ndarray
    camera_model: np.ndarray
    camera_params: np.ndarray
    poses: np.ndarray
    points: np.ndarray
    obs_image: np.ndarray
    obs_point: np.ndarray
    obs_xy: np.ndarray
    fixed_poses: Optional[np.ndarray] = None
    fixed_cameras: Optional[np.ndarray] = None
    fixed_camera_params: Optional[np.ndarray] = None
    meta: dict = field(default_factory=dict)

    @property
    def num_images(self) -> int:
        return len(self.poses)

    @property
    def num_cameras(self) -> int:
        return len(self.camera_model)

    @property
    def num_points(self) -> int:
        return len(self.points)

    @property
    def num_observations(self) -> int:
        return len(self.obs_image)

    def copy(self, **changes) -> "Problem":
        def c(a):
            return None if a is None else np.array(a, copy=True)

        base = replace(
            self,
            camera_of_image=c(self.camera_of_image),
            camera_model=c(self.camera_model),
            camera_params=c(self.camera_params),
            poses=c(self.poses),
            points=c(self.points),
            obs_image=c(self.obs_image),
            obs_point=c(self.obs_point),
            obs_xy=c(self.obs_xy),
            fixed_poses=c(self.fixed_poses),
            fixed_cameras=c(self.fixed_cameras),
            fixed_camera_params=c(self.fixed_camera_params),
            meta=dict(self.meta),
        )
        return replace(base, **changes) if changes else base

    def block_width(self) -> int:
        """Width D of the solver's per-image block: 6 pose columns plus the
        widest free camera, rounded to the widths the kernels are built for."""
        fc = np.zeros(self.num_cameras, bool)
        if self.fixed_cameras is not None:
            m = np.asarray(self.fixed_cameras, bool)[: self.num_cameras]
            fc[: len(m)] = m
        ks = [MODEL_DOF[m] for c, m in enumerate(self.camera_model) if not fc[c]]
        k = max(ks) if ks else 0
        return 6 if k == 0 else 9 if k <= 3 else 10 if k <= 4 else 11 if k <= 5 else 14

    def reduced_dim(self) -> int:
        """Size of the reduced camera system under the reference's slotting
        (crates/sfm-ba/src/lib.rs:753-776)."""
        fp = np.zeros(self.num_images, bool)
        if self.fixed_poses is not None:
            m = np.asarray(self.fixed_poses, bool)[: self.num_images]
            fp[: len(m)] = m
        fc = np.zeros(self.num_cameras, bool)
        if self.fixed_cameras is not None:
            m = np.asarray(self.fixed_cameras, bool)[: self.num_cameras]
            fc[: len(m)] = m
        dof = np.array([MODEL_DOF[m] for m in self.camera_model], dtype=np.int64)
        return int(6 * (~fp).sum() + dof[~fc].sum())


# ---------------------------------------------------------------- quaternions

@dataclass
class Reconstruction:
    """A reconstruction in progress, as sfm-reconstruction holds it while it
    grows (crates/sfm-reconstruction/src/lib.rs:126-129 `PointWork`: a
    point's position and its track of (image, keypoint)), in array form:
    tracks are CSR (``track_offsets`` [nP+1]) with each element's image and
    keypoint pixel; ``registered`` images have valid poses; ``pose_fixed``
    marks poses the caller pinned."""

    camera_of_image: np.ndarray
    camera_model: np.ndarray
    camera_params: np.ndarray
    poses: np.ndarray
    registered: np.ndarray
    points: np.ndarray
    track_offsets: np.ndarray
    track_image: np.ndarray
    track_xy: np.ndarray
    pose_fixed: Optional[np.ndarray] = None
    meta: dict = field(default_factory=dict)


def quat_from_euler(roll: float, pitch: float, yaw: float) -> np.ndarray:
    """Unit quaternion (w, x, y, z) of R = Rz(yaw) Ry(pitch) Rx(roll): the
    roll-pitch-yaw convention of nalgebra's UnitQuaternion::from_euler_angles,
    which the reference tests use for their fixtures."""
    cr, sr = np.cos(roll * 0.5), np.sin(roll * 0.5)
    cp, sp = np.cos(pitch * 0.5), np.sin(pitch * 0.5)
    cy, sy = np.cos(yaw * 0.5), np.sin(yaw * 0.5)
    return np.array([
        cr * cp * cy + sr * sp * sy,
        sr * cp * cy - cr * sp * sy,
        cr * sp * cy + sr * cp * sy,
        cr * cp * sy - sr * sp * cy,
    ])


def quat_mul(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Hamilton product of (..., 4) arrays."""
    aw, ax, ay, az = np.moveaxis(a, -1, 0)
    bw, bx, by, bz = np.moveaxis(b, -1, 0)
    return np.stack([
        aw * bw - ax * bx - ay * by - az * bz,
        aw * bx + ax * bw + ay * bz - az * by,
        aw * by - ax * bz + ay * bw + az * bx,
        aw * bz + ax * by - ay * bx + az * bw,
    ], axis=-1)


def quat_from_scaled_axis(w: np.ndarray) -> np.ndarray:
    """exp of a rotation vector, (..., 3) -> (..., 4); identity at 0."""
    w = np.asarray(w, dtype=np.float64)
    t = np.linalg.norm(w, axis=-1, keepdims=True)
    safe = np.where(t > 0, t, 1.0)
    s = np.where(t > 0, np.sin(0.5 * t) / safe, 0.0)
    return np.concatenate([np.where(t > 0, np.cos(0.5 * t), 1.0), w * s], axis=-1)


def quat_rotate(q: np.ndarray, v: np.ndarray) -> np.ndarray:
    """Rotate (..., 3) vectors by (..., 4) unit quaternions."""
    qv = q[..., 1:]
    t = 2.0 * np.cross(qv, v)
    return v + q[..., :1] * t + np.cross(qv, t)


def quat_to_matrix(q: np.ndarray) -> np.ndarray:
    w, x, y, z = np.moveaxis(np.asarray(q, dtype=np.float64), -1, 0)
    return np.stack([
        np.stack([w * w + x * x - y * y - z * z, 2 * (x * y - w * z), 2 * (w * y + x * z)], -1),
        np.stack([2 * (w * z + x * y), w * w - x * x + y * y - z * z, 2 * (y * z - w * x)], -1),
        np.stack([2 * (x * z - w * y), 2 * (w * x + y * z), w * w - x * x - y * y + z * z], -1),
    ], -2)


def quat_from_matrix(R: np.ndarray) -> np.ndarray:
    """Unit quaternion (w, x, y, z) of rotation matrices (..., 3, 3)."""
    R = np.asarray(R, dtype=np.float64)
    tr = R[..., 0, 0] + R[..., 1, 1] + R[..., 2, 2]
    w = np.sqrt(np.maximum(0.0, 1.0 + tr)) / 2
    x = np.sqrt(np.maximum(0.0, 1.0 + R[..., 0, 0] - R[..., 1, 1] - R[..., 2, 2])) / 2
    y = np.sqrt(np.maximum(0.0, 1.0 - R[..., 0, 0] + R[..., 1, 1] - R[..., 2, 2])) / 2
    z = np.sqrt(np.maximum(0.0, 1.0 - R[..., 0, 0] - R[..., 1, 1] + R[..., 2, 2])) / 2
    x = np.copysign(x, R[..., 2, 1] - R[..., 1, 2])
    y = np.copysign(y, R[..., 0, 2] - R[..., 2, 0])
    z = np.copysign(z, R[..., 1, 0] - R[..., 0, 1])
    q = np.stack([w, x, y, z], -1)
    return q / np.linalg.norm(q, axis=-1, keepdims=True)


def perturb_pose(pose7: np.ndarray, delta6: np.ndarray) -> np.ndarray:
    """R <- exp(w) R, t <- t + dt (crates/sfm-ba/src/lib.rs:263-269)."""
    pose7 = np.asarray(pose7, dtype=np.float64)
    delta6 = np.asarray(delta6, dtype=np.float64)
    q = quat_mul(quat_from_scaled_axis(delta6[..., :3]), pose7[..., :4])
    return np.concatenate([q, pose7[..., 4:] + delta6[..., 3:]], axis=-1)


def look_at_pose(center: np.ndarray, target: np.ndarray, up=(0.0, 0.0, 1.0)) -> np.ndarray:
    """World-to-camera pose (COLMAP axes: +x right, +y down, +z forward) of a
    camera at ``center`` looking at ``target``; vectorised over rows."""
    center = np.atleast_2d(np.asarray(center, dtype=np.float64))
    target = np.broadcast_to(np.asarray(target, dtype=np.float64), center.shape)
    up = np.broadcast_to(np.asarray(up, dtype=np.float64), center.shape)
    z = target - center
    z /= np.linalg.norm(z, axis=1, keepdims=True)
    x = np.cross(z, -up)
    bad = np.linalg.norm(x, axis=1) < 1e-9
    if bad.any():
        x[bad] = np.cross(z[bad], np.array([1.0, 0.0, 0.0]))
    x /= np.linalg.norm(x, axis=1, keepdims=True)
    y = np.cross(z, x)
    R = np.stack([x, y, z], axis=1)  # rows: camera axes in world coordinates
    q = quat_from_matrix(R)
    t = -np.einsum("nij,nj->ni", R, center)
    return np.concatenate([q, t], axis=1)


# ----------------------------------------------------------------- projection

def project(model: np.ndarray, params: np.ndarray, pc: np.ndarray) -> np.ndarray:
    """Pixel coordinates of camera-frame points (crates/sfm-core/src/camera.rs:204-244),
    vectorised: ``model`` [n], ``params`` [n, 8], ``pc`` [n, 3] -> [n, 2]."""
    model = np.broadcast_to(np.asarray(model), pc.shape[:1])
    params = np.broadcast_to(np.asarray(params, dtype=np.float64), pc.shape[:1] + (MAX_CAMERA_PARAMS,))
    x = pc[:, 0] / pc[:, 2]
    y = pc[:, 1] / pc[:, 2]
    out = np.empty((len(pc), 2))
    c = params
    for m in np.unique(model):
        s = model == m
        xs, ys, cs = x[s], y[s], c[s]
        if m == SIMPLE_PINHOLE:
            u, v = cs[:, 0] * xs + cs[:, 1], cs[:, 0] * ys + cs[:, 2]
        elif m == PINHOLE:
            u, v = cs[:, 0] * xs + cs[:, 2], cs[:, 1] * ys + cs[:, 3]
        elif m in (SIMPLE_RADIAL, RADIAL):
            r2 = xs * xs + ys * ys
            d = 1.0 + cs[:, 3] * r2 + (cs[:, 4] * r2 * r2 if m == RADIAL else 0.0)
            u, v = cs[:, 0] * (xs * d) + cs[:, 1], cs[:, 0] * (ys * d) + cs[:, 2]
        elif m == OPENCV:
            k1, k2, p1, p2 = cs[:, 4], cs[:, 5], cs[:, 6], cs[:, 7]
            r2 = xs * xs + ys * ys
            rad = 1.0 + k1 * r2 + k2 * r2 * r2
            xd = xs * rad + 2.0 * p1 * xs * ys + p2 * (r2 + 2.0 * xs * xs)
            yd = ys * rad + p1 * (r2 + 2.0 * ys * ys) + 2.0 * p2 * xs * ys
            u, v = cs[:, 0] * xd + cs[:, 2], cs[:, 1] * yd + cs[:, 3]
        elif m == OPENCV_FISHEYE:
            r = np.maximum(np.sqrt(xs * xs + ys * ys), 1e-12)
            th = np.arctan(r)
            t2 = th * th
            thd = th * (1 + cs[:, 4] * t2 + cs[:, 5] * t2**2 + cs[:, 6] * t2**3 + cs[:, 7] * t2**4)
            sc = thd / r
            u, v = cs[:, 0] * (xs * sc) + cs[:, 2], cs[:, 1] * (ys * sc) + cs[:, 3]
        else:
            raise ValueError(f"unknown camera model {m}")
        out[s, 0], out[s, 1] = u, v
    return out


def camera_frame(poses: np.ndarray, points: np.ndarray) -> np.ndarray:
    """pc = R X + t for matching rows of poses [n, 7] and points [n, 3]."""
    return quat_rotate(poses[:, :4], points) + poses[:, 4:]


def reprojection_residuals(p: Problem) -> tuple[np.ndarray, np.ndarray]:
    """(residuals [nO, 2], valid [nO]) in float64 numpy - for scene
    construction and reporting only."""
    img = p.obs_image
    cam = p.camera_of_image[img]
    pc = camera_frame(p.poses[img], p.points[p.obs_point])
    valid = pc[:, 2] > 1e-9
    r = np.zeros((len(img), 2))
    if valid.any():
        r[valid] = project(p.camera_model[cam][valid], p.camera_params[cam][valid], pc[valid]) - p.obs_xy[valid]
    return r, valid


def rms_reprojection_error(p: Problem) -> float:
    r, valid = reprojection_residuals(p)
    if not valid.any():
        return 0.0
    return float(np.sqrt(np.mean(np.sum(r[valid] ** 2, axis=1))))


def camera_centers(poses: np.ndarray) -> np.ndarray:
    """World position of each camera, C = -R^T t, for poses [n, 7]."""
    q = np.asarray(poses[:, :4], np.float64)
    qc = q * np.array([1.0, -1.0, -1.0, -1.0])
    return -quat_rotate(qc, np.asarray(poses[:, 4:], np.float64))


def _rel(a: np.ndarray, b: np.ndarray) -> float:
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    if a.size == 0:
        return 0.0
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0)))


def parameter_errors(poses, points, camera_params, ref_poses, ref_points, ref_camera_params,
                     anchor: int = 0, second: int = 1) -> dict:
    """Errors of one solution's parameters against a reference solution.

    raw: max over entries of |a - b| / max(|b|, 1), per group (poses, points,
    cameras). normalized: the same after removing the free scale of a problem
    whose gauge is fixed by one pose (crates/sfm-ba/src/lib.rs:1454-1460):
    each solution's camera centres and points are taken relative to the
    anchor camera's centre C0 and divided by that solution's |C1 - C0|
    (C1: the centre of image ``second``); rotations and intrinsics are
    scale-free and compared as they are (quaternions sign-aligned).
    """
    out = {"raw": {"poses": _rel(poses, ref_poses), "points": _rel(points, ref_points),
                   "cameras": _rel(camera_params, ref_camera_params)}}
    ca, cb = camera_centers(np.asarray(poses)), camera_centers(np.asarray(ref_poses))
    sa = np.linalg.norm(ca[second] - ca[anchor]) if len(ca) > max(anchor, second) else 1.0
    sb = np.linalg.norm(cb[second] - cb[anchor]) if len(cb) > max(anchor, second) else 1.0
    sa, sb = (sa if sa > 0 else 1.0), (sb if sb > 0 else 1.0)
    qa, qb = np.asarray(poses, np.float64)[:, :4], np.asarray(ref_poses, np.float64)[:, :4]
    qa = qa * np.where(np.sum(qa * qb, axis=1, keepdims=True) < 0, -1.0, 1.0)
    pa = (np.asarray(points, np.float64) - ca[anchor]) / sa
    pb = (np.asarray(ref_points, np.float64) - cb[anchor]) / sb
    out["normalized"] = {
        "rotations": _rel(qa, qb),
        "centers": _rel((ca - ca[anchor]) / sa, (cb - cb[anchor]) / sb),
        "points": _rel(pa, pb),
        "cameras": _rel(camera_params, ref_camera_params),
    }
    out["raw_max"] = max(out["raw"].values())
    out["normalized_max"] = max(out["normalized"].values())
    out["scale_ratio"] = float(sa / sb)
    return out


def rms_of(p: Problem, poses, points, camera_params) -> float:
    """RMS reprojection error (px) of p's observations under the given parameters."""
    return rms_reprojection_error(p.copy(poses=np.asarray(poses), points=np.asarray(points),
                                         camera_params=np.asarray(camera_params)))
