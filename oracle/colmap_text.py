"""TEST INFRASTRUCTURE ONLY: a Python restatement of sfmtory's COLMAP text
model reader/writer (crates/sfm-io/src/colmap.rs:24-305) and of the
`sfmtory refine` driver (crates/sfm-cli/src/main.rs:946-1130) on top of the
CPU oracle's bundle_adjust. It writes test models, parses the GPU library's
output and computes what the reference would write, as the checker for
`sfmba_colmap_refine` / `sfmba_colmap_rewrite`. The product path never
imports it.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

MODEL_NAMES = ("SIMPLE_PINHOLE", "PINHOLE", "SIMPLE_RADIAL", "RADIAL", "OPENCV", "OPENCV_FISHEYE")
MODEL_DOF = (3, 4, 4, 5, 8, 8)


@dataclass
class Camera:
    id: int
    model: int
    width: int
    height: int
    params: list


@dataclass
class Image:
    id: int
    q: list  # qw qx qy qz
    t: list
    camera_id: int
    name: str
    keypoints: list = field(default_factory=list)  # (x, y) as float32 values
    point3d_ids: list = field(default_factory=list)  # -1: none


@dataclass
class Point:
    id: int
    xyz: list
    color: tuple
    error: float
    track: list = field(default_factory=list)  # (image id, keypoint index)


@dataclass
class Model:
    cameras: dict = field(default_factory=dict)
    images: dict = field(default_factory=dict)
    points: dict = field(default_factory=dict)

    def mean_reprojection_error(self) -> float:
        """crates/sfm-core/src/model.rs:84-97."""
        total = count = 0.0
        for p in self.points.values():
            n = float(len(p.track))
            total += p.error * n
            count += n
        return total / count if count > 0.0 else 0.0


def _fixed(v: float, d: int) -> str:
    """Rust's `{:.d}` of an f64."""
    if math.isnan(v):
        return "NaN"
    if math.isinf(v):
        return "inf" if v > 0 else "-inf"
    return f"{v:.{d}f}"


def write_model(m: Model, d: str) -> None:
    """colmap.rs:24-31, :43-67, :113-148, :221-249."""
    os.makedirs(d, exist_ok=True)
    out = ["# Camera list with one line of data per camera:\n", "#   CAMERA_ID, MODEL, WIDTH, HEIGHT, PARAMS[]\n",
           f"# Number of cameras: {len(m.cameras)}\n"]
    for cid in sorted(m.cameras):
        c = m.cameras[cid]
        ps = " ".join(_fixed(float(v), 10) for v in c.params[: MODEL_DOF[c.model]])
        out.append(f"{c.id} {MODEL_NAMES[c.model]} {c.width} {c.height} {ps}\n")
    open(os.path.join(d, "cameras.txt"), "w").write("".join(out))
    total = sum(len(im.keypoints) for im in m.images.values())
    mean_obs = total / len(m.images) if m.images else 0.0
    out = ["# Image list with two lines of data per image:\n",
           "#   IMAGE_ID, QW, QX, QY, QZ, TX, TY, TZ, CAMERA_ID, NAME\n",
           "#   POINTS2D[] as (X, Y, POINT3D_ID)\n",
           f"# Number of images: {len(m.images)}, mean observations per image: {_fixed(mean_obs, 1)}\n"]
    for iid in sorted(m.images):
        im = m.images[iid]
        head = " ".join([str(im.id)] + [_fixed(float(v), 10) for v in list(im.q) + list(im.t)] +
                        [str(im.camera_id), im.name])
        out.append(head + "\n")
        out.append(" ".join(f"{_fixed(float(x), 3)} {_fixed(float(y), 3)} {int(p) if p >= 0 else -1}"
                            for (x, y), p in zip(im.keypoints, im.point3d_ids)) + "\n")
    open(os.path.join(d, "images.txt"), "w").write("".join(out))
    out = ["# 3D point list with one line of data per point:\n",
           "#   POINT3D_ID, X, Y, Z, R, G, B, ERROR, TRACK[] as (IMAGE_ID, POINT2D_IDX)\n",
           f"# Number of points: {len(m.points)}\n"]
    for pid in sorted(m.points):
        p = m.points[pid]
        tr = " ".join(f"{a} {b}" for a, b in p.track)
        out.append(f"{p.id} {_fixed(p.xyz[0], 10)} {_fixed(p.xyz[1], 10)} {_fixed(p.xyz[2], 10)} "
                   f"{p.color[0]} {p.color[1]} {p.color[2]} {_fixed(p.error, 6)} {tr}\n")
    open(os.path.join(d, "points3D.txt"), "w").write("".join(out))


def _data_lines(path):
    for line in open(path).read().split("\n"):
        t = line.strip()
        if t and not t.startswith("#"):
            yield t


def read_model(d: str) -> Model:
    """colmap.rs:33-41, :70-111, :150-219, :251-305 (well-formed files)."""
    m = Model()
    for t in _data_lines(os.path.join(d, "cameras.txt")):
        tok = t.split()
        model = MODEL_NAMES.index(tok[1])
        ps = [float(v) for v in tok[4:]][: MODEL_DOF[model]]
        m.cameras[int(tok[0])] = Camera(int(tok[0]), model, int(tok[2]), int(tok[3]), ps + [0.0] * (8 - len(ps)))
    lines = list(_data_lines(os.path.join(d, "images.txt")))
    k = 0
    while k < len(lines):
        tok = lines[k].split()
        q = np.array([float(v) for v in tok[1:5]])
        q = q / math.sqrt(q[1] ** 2 + q[2] ** 2 + q[3] ** 2 + q[0] ** 2)
        im = Image(int(tok[0]), list(q), [float(v) for v in tok[5:8]], int(tok[8]), tok[9])
        pt = lines[k + 1].split() if k + 1 < len(lines) else []
        for j in range(0, len(pt) - 2, 3):
            im.keypoints.append((float(np.float32(pt[j])), float(np.float32(pt[j + 1]))))
            pid = int(pt[j + 2])
            im.point3d_ids.append(pid if pid >= 0 else -1)
        m.images[im.id] = im
        k += 2
    for t in _data_lines(os.path.join(d, "points3D.txt")):
        tok = t.split()
        tr = [(int(tok[j]), int(tok[j + 1])) for j in range(8, len(tok) - 1, 2)]
        m.points[int(tok[0])] = Point(int(tok[0]), [float(v) for v in tok[1:4]],
                                      tuple(int(v) for v in tok[4:7]), float(tok[7]), tr)
    return m


def refine_input(m: Model, refine_intrinsics: bool):
    """The BaInput of cmd_refine (main.rs:969-1047) as a Problem, plus the
    id maps: images in id order, cameras in first-use order, points in id
    order, observations point by point in track order."""
    from sfmtory_gb300.abi import MAX_CAMERA_PARAMS
    from sfmtory_gb300.problem import Problem
    import oracle

    image_ids = sorted(m.images)
    image_pos = {iid: k for k, iid in enumerate(image_ids)}
    cam_ids, cam_index, cam_of_img = [], {}, []
    for iid in image_ids:
        cid = m.images[iid].camera_id
        if cid not in cam_index:
            cam_index[cid] = len(cam_ids)
            cam_ids.append(cid)
        cam_of_img.append(cam_index[cid])
    point_ids = sorted(m.points)
    img, pt, xy, pt_obs = [], [], [], [0]
    for k, pid in enumerate(point_ids):
        for a, b in m.points[pid].track:
            if a not in image_pos or b >= len(m.images[a].keypoints):
                continue
            img.append(image_pos[a])
            pt.append(k)
            xy.append(m.images[a].keypoints[b])
        pt_obs.append(len(img))
    models = np.array([m.cameras[c].model for c in cam_ids], np.int32)
    params = np.array([list(m.cameras[c].params) + [0.0] * (MAX_CAMERA_PARAMS - len(m.cameras[c].params))
                       for c in cam_ids])
    fixed_poses = np.zeros(len(image_ids), bool)
    fixed_poses[0] = True
    prob = Problem(
        camera_of_image=np.array(cam_of_img, np.int32), camera_model=models, camera_params=params,
        poses=np.array([list(m.images[i].q) + list(m.images[i].t) for i in image_ids]),
        points=np.array([m.points[p].xyz for p in point_ids], np.float64).reshape(-1, 3),
        obs_image=np.array(img, np.int32), obs_point=np.array(pt, np.int32),
        obs_xy=np.array(xy, np.float64).reshape(-1, 2), fixed_poses=fixed_poses,
        fixed_cameras=np.full(len(cam_ids), not refine_intrinsics),
        fixed_camera_params=(oracle.default_fixed_params_mask(models) if refine_intrinsics else None),
        meta={"name": "colmap"})
    return prob, image_ids, cam_ids, point_ids, np.array(pt_obs)


def refine(m: Model, refine_intrinsics: bool, **options):
    """What cmd_refine writes (main.rs:1058-1100), with the oracle's
    bundle_adjust: returns (refined model, BA result, error before, error
    after)."""
    import copy

    import oracle
    from sfmtory_gb300.problem import reprojection_residuals

    prob, image_ids, cam_ids, point_ids, pt_obs = refine_input(m, refine_intrinsics)
    before = m.mean_reprojection_error()
    r = oracle.bundle_adjust(prob, **options)
    out = copy.deepcopy(m)
    for k, iid in enumerate(image_ids):
        out.images[iid].q = list(r.poses[k, :4])
        out.images[iid].t = list(r.poses[k, 4:])
    for k, pid in enumerate(point_ids):
        out.points[pid].xyz = list(r.points[k])
    if refine_intrinsics:
        for k, cid in enumerate(cam_ids):
            out.cameras[cid].params = list(r.camera_params[k])
    res, valid = reprojection_residuals(prob.copy(poses=r.poses, points=r.points,
                                                  camera_params=r.camera_params if refine_intrinsics
                                                  else prob.camera_params))
    norm = np.linalg.norm(res, axis=1)
    for k, pid in enumerate(point_ids):
        s, e = pt_obs[k], pt_obs[k + 1]
        v = valid[s:e]
        if v.any():
            out.points[pid].error = float(norm[s:e][v].sum() / v.sum())
    return out, r, before, out.mean_reprojection_error()
