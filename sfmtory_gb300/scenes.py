"""Seeded synthetic bundle-adjustment problems.

Two families:

* the fixtures of sfm-ba's own unit tests (crates/sfm-ba/src/lib.rs:1245-1592,
  crates/sfm-ba/src/intrinsics.rs:252-383), rebuilt from their formulas;
* the benchmark workloads: ``ring16`` (16 PINHOLE cameras, 2000 points),
  ``opencv47`` (47 OPENCV cameras, 20k points, 5 % outliers),
  ``radial500`` (500 SIMPLE_RADIAL cameras, 200k points),
  ``radial2000`` (2000 RADIAL cameras, 1M points, power-law tracks) and
  ``windows512`` (512 independent local windows).

Every generator takes a seed and a ``scale`` that shrinks the point count
(and the camera count where stated) for fast tests while keeping the
per-point statistics. Observations are rounded to float32, as keypoints are
in the real pipeline (crates/sfm-core/src/features.rs:12-13).
"""
from __future__ import annotations

import numpy as np

from .abi import MAX_CAMERA_PARAMS, OPENCV, OPENCV_FISHEYE, PINHOLE, RADIAL, SIMPLE_PINHOLE, SIMPLE_RADIAL
from .problem import (
    Problem,
    camera_frame,
    look_at_pose,
    perturb_pose,
    project,
    quat_from_euler,
    quat_from_scaled_axis,
    quat_to_matrix,
)


def _pad(params):
    out = np.zeros(MAX_CAMERA_PARAMS)
    out[: len(params)] = params
    return out


def _pose(euler, t):
    return np.concatenate([quat_from_euler(*euler), np.asarray(t, dtype=np.float64)])


IDENTITY_POSE = np.array([1.0, 0, 0, 0, 0, 0, 0])


# ------------------------------------------------------- reference fixtures

#: Camera parameters of the per-model analytic-vs-numerical Jacobian tests
#: (crates/sfm-ba/src/lib.rs:1297-1363).
JACOBIAN_TEST_CAMERAS = {
    SIMPLE_PINHOLE: [1420.0, 320.0, 240.0],
    PINHOLE: [1420.0, 1390.0, 320.0, 240.0],
    SIMPLE_RADIAL: [1420.0, 320.0, 240.0, -0.45],
    RADIAL: [1420.0, 320.0, 240.0, -0.35, 0.12],
    OPENCV: [1420.0, 1390.0, 320.0, 240.0, -0.28, 0.09, 0.015, -0.02],
    OPENCV_FISHEYE: [900.0, 880.0, 320.0, 240.0, -0.05, 0.02, -0.01, 0.005],
}


def jacobian_test_fixture():
    """Pose, point and observation of assert_analytic_matches_numerical
    (crates/sfm-ba/src/lib.rs:1252-1258)."""
    return _pose((0.15, -0.3, 0.08), (0.6, -0.2, 1.3)), np.array([0.35, -0.18, 2.7]), (410.0, 260.0)


def _observe(cam_model, cam_params, poses, points, min_z):
    img, pt, xy = [], [], []
    for p_idx, X in enumerate(points):
        for i, P in enumerate(poses):
            pc = camera_frame(P[None], X[None])
            if pc[0, 2] <= min_z:
                continue
            uv = project(np.array([cam_model]), cam_params[None], pc)[0]
            img.append(i)
            pt.append(p_idx)
            xy.append(uv)
    return np.array(img, np.int32), np.array(pt, np.int32), np.array(xy, np.float64).reshape(-1, 2)


def recovers_ground_truth_fixture() -> Problem:
    """recovers_ground_truth_from_perturbed_initialization
    (crates/sfm-ba/src/lib.rs:1368-1476): 2 images, 25 noiseless points,
    pose 0 and the camera fixed; run with max_iterations = 30."""
    cam = _pad([700.0, 320.0, 240.0])
    true_poses = np.stack([IDENTITY_POSE, _pose((0.02, 0.2, -0.01), (0.8, 0.05, 0.1))])
    t = np.arange(25, dtype=np.float64)
    true_pts = np.stack([0.5 * np.sin(t * 0.6), 0.4 * np.cos(t * 0.4), 3.0 + 0.1 * t], 1)
    img, pt, xy = _observe(SIMPLE_PINHOLE, cam, true_poses, true_pts, 0.0)
    init_poses = true_poses.copy()
    init_poses[1] = perturb_pose(true_poses[1], np.array([0.03, -0.02, 0.01, 0.05, -0.03, 0.04]))
    s = t
    init_pts = true_pts + np.stack([0.05 * np.sin(s * 1.1), -0.04 * np.cos(s * 0.7), 0.06 * np.sin(s * 0.3)], 1)
    return Problem(
        camera_of_image=np.array([0, 0], np.int32),
        camera_model=np.array([SIMPLE_PINHOLE], np.int32),
        camera_params=cam[None].copy(),
        poses=init_poses,
        points=init_pts,
        obs_image=img,
        obs_point=pt,
        obs_xy=xy,
        fixed_poses=np.array([True, False]),
        fixed_cameras=np.array([True]),
        fixed_camera_params=None,
        meta={"name": "recovers_ground_truth", "true_poses": true_poses, "true_points": true_pts},
    )


def shared_focal_fixture(wrong_f: float = 1000.0) -> Problem:
    """joint_optimization_recovers_shared_camera_focal_length
    (crates/sfm-ba/src/lib.rs:1487-1592): 4 images sharing one SIMPLE_PINHOLE
    camera (true f = 1500), 60 noiseless points, observations with z > 0.1.
    Returned with the wrong focal length, true poses/points, pose 0 fixed and
    the camera fixed (the pre-convergence solve); the joint solve frees it."""
    true_cam = _pad([1500.0, 500.0, 400.0])
    true_poses = np.stack([
        IDENTITY_POSE,
        _pose((0.0, 0.25, 0.0), (1.2, 0.1, -0.3)),
        _pose((0.1, -0.3, 0.05), (-0.9, 0.4, 0.5)),
        _pose((-0.05, 0.4, -0.1), (0.5, -0.6, 1.1)),
    ])
    t = np.arange(60, dtype=np.float64)
    true_pts = np.stack([0.8 * np.sin(t * 0.31), 0.7 * np.cos(t * 0.47), 2.5 + 0.15 * t], 1)
    img, pt, xy = _observe(SIMPLE_PINHOLE, true_cam, true_poses, true_pts, 0.1)
    return Problem(
        camera_of_image=np.zeros(4, np.int32),
        camera_model=np.array([SIMPLE_PINHOLE], np.int32),
        camera_params=_pad([wrong_f, 500.0, 400.0])[None].copy(),
        poses=true_poses.copy(),
        points=true_pts.copy(),
        obs_image=img,
        obs_point=pt,
        obs_xy=xy,
        fixed_poses=np.array([True, False, False, False]),
        fixed_cameras=np.array([True]),
        meta={"name": "shared_focal", "true_f": 1500.0},
    )


def intrinsics_fixture(n_points: int = 40, wrong_f: float = 960.0) -> Problem:
    """recovers_true_focal_length_from_wrong_initial_guess
    (crates/sfm-ba/src/intrinsics.rs:262-305): one identity pose, points
    (0.4 sin 0.6t, 0.3 cos 0.4t, 3 + 0.05t), true SIMPLE_PINHOLE f = 1500 on a
    1000x800 image, starting from f = 960."""
    true_cam = _pad([1500.0, 500.0, 400.0])
    t = np.arange(n_points, dtype=np.float64)
    pts = np.stack([0.4 * np.sin(t * 0.6), 0.3 * np.cos(t * 0.4), 3.0 + 0.05 * t], 1)
    img, pt, xy = _observe(SIMPLE_PINHOLE, true_cam, IDENTITY_POSE[None], pts, -np.inf)
    return Problem(
        camera_of_image=np.zeros(1, np.int32),
        camera_model=np.array([SIMPLE_PINHOLE], np.int32),
        camera_params=_pad([wrong_f, 500.0, 400.0])[None].copy(),
        poses=IDENTITY_POSE[None].copy(),
        points=pts,
        obs_image=img,
        obs_point=pt,
        obs_xy=xy,
        meta={"name": "intrinsics", "true_f": 1500.0},
    )


# ------------------------------------------------------ benchmark workloads

def _finish_scene(rng, *, cam_model, cam_true, image_wh, poses_true, pts_true, views_img, views_pt,
                  noise_px, outlier_frac, fixed_first_pose, rot_deg, trans_abs, point_rel, focal_rel,
                  mask_principal_point, name, extra_meta=None):
    """Project the chosen (image, point) pairs, keep the visible ones, add
    noise/outliers, round to float32 and perturb the initial guess."""
    cam_of_img = np.arange(len(poses_true), dtype=np.int32)
    cam_idx = cam_of_img[views_img]
    pc = camera_frame(poses_true[views_img], pts_true[views_pt])
    ok = pc[:, 2] > 1e-3
    uv = np.zeros((len(views_img), 2))
    uv[ok] = project(cam_model[cam_idx][ok], cam_true[cam_idx][ok], pc[ok])
    w, h = image_wh[cam_idx, 0], image_wh[cam_idx, 1]
    ok &= (uv[:, 0] >= 0) & (uv[:, 0] < w) & (uv[:, 1] >= 0) & (uv[:, 1] < h)
    img, pt, uv = views_img[ok], views_pt[ok], uv[ok]
    # Points need at least two views.
    cnt = np.bincount(pt, minlength=len(pts_true))
    keep_pt = cnt >= 2
    sel = keep_pt[pt]
    img, pt, uv = img[sel], pt[sel], uv[sel]
    remap = -np.ones(len(pts_true), np.int64)
    remap[keep_pt] = np.arange(keep_pt.sum())
    pt = remap[pt].astype(np.int32)
    pts_true = pts_true[keep_pt]

    obs = uv + rng.normal(0.0, noise_px, uv.shape)
    n_out = int(round(outlier_frac * len(obs)))
    if n_out:
        idx = rng.choice(len(obs), n_out, replace=False)
        ci = img[idx]
        obs[idx, 0] = rng.uniform(0, image_wh[ci, 0])
        obs[idx, 1] = rng.uniform(0, image_wh[ci, 1])
    obs = obs.astype(np.float32).astype(np.float64)

    n_img = len(poses_true)
    poses = poses_true.copy()
    axis = rng.normal(size=(n_img, 3))
    axis /= np.linalg.norm(axis, axis=1, keepdims=True)
    tdir = rng.normal(size=(n_img, 3))
    tdir /= np.linalg.norm(tdir, axis=1, keepdims=True)
    delta = np.concatenate([axis * np.deg2rad(rot_deg), tdir * trans_abs], 1)
    if fixed_first_pose:
        delta[0] = 0.0
    poses = perturb_pose(poses_true, delta)

    # Point perturbation: a random direction, 1 % of the depth in the first observing image.
    first = np.full(len(pts_true), -1, np.int64)
    order = np.argsort(pt, kind="stable")
    starts = np.searchsorted(pt[order], np.arange(len(pts_true)))
    first = img[order[starts]]
    depth = camera_frame(poses_true[first], pts_true)[:, 2]
    pdir = rng.normal(size=pts_true.shape)
    pdir /= np.linalg.norm(pdir, axis=1, keepdims=True)
    points = pts_true + pdir * (point_rel * np.abs(depth))[:, None]

    cams = cam_true.copy()
    sign = rng.choice([-1.0, 1.0], size=len(cams))
    focal_cols = np.where(np.isin(cam_model, [PINHOLE, OPENCV, OPENCV_FISHEYE]), 2, 1)
    for c in range(len(cams)):
        cams[c, : focal_cols[c]] *= 1.0 + focal_rel * sign[c]

    fixed_poses = np.zeros(n_img, bool)
    fixed_poses[0] = fixed_first_pose
    mask = None
    if mask_principal_point:
        mask = np.zeros((len(cams), MAX_CAMERA_PARAMS), bool)
        simple = np.isin(cam_model, [SIMPLE_PINHOLE, SIMPLE_RADIAL, RADIAL])
        mask[simple, 1:3] = True
        mask[~simple, 2:4] = True
    meta = {
        "name": name,
        "true_poses": poses_true,
        "true_points": pts_true,
        "true_camera_params": cam_true,
        "image_wh": image_wh,
    }
    if extra_meta:
        meta.update(extra_meta)
    return Problem(
        camera_of_image=cam_of_img,
        camera_model=cam_model.astype(np.int32),
        camera_params=cams,
        poses=poses,
        points=points,
        obs_image=img.astype(np.int32),
        obs_point=pt,
        obs_xy=obs,
        fixed_poses=fixed_poses,
        fixed_cameras=np.zeros(len(cams), bool),
        fixed_camera_params=mask,
        meta=meta,
    )


def ring16(seed: int = 0, scale: float = 1.0) -> Problem:
    """16 PINHOLE cameras (fx = fy = 1200, cx = 800, cy = 600, 1600x1200) on a
    20 degree arc of radius 10 looking at the origin; 2000 points uniform in
    the 4x4x4 cube, each seen by every camera whose frustum holds it;
    sigma = 0.5 px; init: rotations 1 deg, translations 2 % of the radius,
    points 1 % of depth, focal 3 %; pose 0 fixed, principal point masked.
    Solve with squared loss and 50 iterations."""
    rng = np.random.default_rng(seed)
    n_cam = 16
    ang = np.deg2rad(np.linspace(-10.0, 10.0, n_cam))
    centers = np.stack([10.0 * np.cos(ang), 10.0 * np.sin(ang), np.zeros(n_cam)], 1)
    poses_true = look_at_pose(centers, np.zeros(3))
    n_pts = max(8, int(round(2000 * scale)))
    pts = rng.uniform(-2.0, 2.0, size=(n_pts, 3))
    views_img = np.tile(np.arange(n_cam, dtype=np.int64), n_pts)
    views_pt = np.repeat(np.arange(n_pts, dtype=np.int64), n_cam)
    cam_true = np.tile(_pad([1200.0, 1200.0, 800.0, 600.0]), (n_cam, 1))
    return _finish_scene(
        rng, cam_model=np.full(n_cam, PINHOLE), cam_true=cam_true,
        image_wh=np.tile([1600.0, 1200.0], (n_cam, 1)), poses_true=poses_true, pts_true=pts,
        views_img=views_img, views_pt=views_pt, noise_px=0.5, outlier_frac=0.0,
        fixed_first_pose=True, rot_deg=1.0, trans_abs=0.2, point_rel=0.01, focal_rel=0.03,
        mask_principal_point=True, name="ring16", extra_meta={"seed": seed, "scale": scale})


def _contiguous_views(rng, n_cam, counts, loop):
    """For each point, ``counts[p]`` consecutive cameras along the path
    starting at a random camera (wrapping if the path is a loop)."""
    counts = np.minimum(counts, n_cam)
    if loop:
        start = rng.integers(0, n_cam, size=len(counts))
    else:
        start = (rng.random(len(counts)) * (n_cam - counts + 1)).astype(np.int64)
    pt = np.repeat(np.arange(len(counts), dtype=np.int64), counts)
    offs = np.arange(counts.sum()) - np.repeat(np.cumsum(counts) - counts, counts)
    img = np.repeat(start, counts) + offs
    if loop:
        img %= n_cam
    return img.astype(np.int64), pt


def opencv47(seed: int = 0, scale: float = 1.0) -> Problem:
    """47 OPENCV cameras (f ~ 1200, k1 U[-0.1,0.1], k2 U[-0.02,0.02],
    p1,p2 U[-1e-3,1e-3], 1600x1200) on a ring of radius 10 at three
    elevations; 20k points in a radius-2.5 ball, ~6 consecutive views each
    (2 + Poisson(4)); sigma = 0.5 px plus 5 % outliers uniform over the image.
    Solve with Huber at 1 px."""
    rng = np.random.default_rng(seed)
    n_cam = 47
    az = np.linspace(0, 2 * np.pi, n_cam, endpoint=False)
    elev = np.deg2rad(np.array([10.0, 25.0, 40.0]))[np.arange(n_cam) % 3]
    centers = 10.0 * np.stack([np.cos(az) * np.cos(elev), np.sin(az) * np.cos(elev), np.sin(elev)], 1)
    poses_true = look_at_pose(centers, np.zeros(3))
    fx = rng.uniform(1150, 1250, n_cam)
    cam_true = np.zeros((n_cam, MAX_CAMERA_PARAMS))
    cam_true[:, 0] = fx
    cam_true[:, 1] = fx * rng.uniform(0.99, 1.01, n_cam)
    cam_true[:, 2], cam_true[:, 3] = 800.0, 600.0
    cam_true[:, 4] = rng.uniform(-0.1, 0.1, n_cam)
    cam_true[:, 5] = rng.uniform(-0.02, 0.02, n_cam)
    cam_true[:, 6:8] = rng.uniform(-1e-3, 1e-3, (n_cam, 2))
    n_pts = max(16, int(round(20000 * scale)))
    d = rng.normal(size=(n_pts, 3))
    pts = d / np.linalg.norm(d, axis=1, keepdims=True) * (2.5 * rng.random(n_pts) ** (1 / 3))[:, None]
    counts = 2 + rng.poisson(4.0, n_pts)
    views_img, views_pt = _contiguous_views(rng, n_cam, counts, loop=True)
    return _finish_scene(
        rng, cam_model=np.full(n_cam, OPENCV), cam_true=cam_true,
        image_wh=np.tile([1600.0, 1200.0], (n_cam, 1)), poses_true=poses_true, pts_true=pts,
        views_img=views_img, views_pt=views_pt, noise_px=0.5, outlier_frac=0.05,
        fixed_first_pose=True, rot_deg=1.0, trans_abs=0.2, point_rel=0.01, focal_rel=0.03,
        mask_principal_point=True, name="opencv47", extra_meta={"seed": seed, "scale": scale})


def _smooth_loop(rng, n_cam, radius, height, wobble):
    """Camera centres on a closed loop with smooth random radius/height
    variation, all looking near the origin."""
    s = np.linspace(0, 2 * np.pi, n_cam, endpoint=False)
    r = np.full(n_cam, radius)
    z = np.full(n_cam, height)
    for k in range(1, 4):
        r += wobble * radius * rng.normal() / k * np.sin(k * s + rng.uniform(0, 2 * np.pi))
        z += wobble * radius * rng.normal() / k * np.sin(k * s + rng.uniform(0, 2 * np.pi))
    centers = np.stack([r * np.cos(s), r * np.sin(s), z], 1)
    look = rng.normal(0.0, 0.05 * radius, size=(n_cam, 3))
    return look_at_pose(centers, look)


def radial500(seed: int = 0, scale: float = 1.0) -> Problem:
    """500 SIMPLE_RADIAL cameras (f U[900,1500], k U[-0.05,0.05], 1600x1200)
    on a smooth random loop of radius ~16; 200k points in a radius-3 ball,
    view counts 2 + Geometric(mean 4) over consecutive cameras (~1.2M
    observations); sigma = 0.5 px; init as ring16."""
    rng = np.random.default_rng(seed)
    n_cam = 500 if scale >= 1 else max(16, int(round(500 * scale ** 0.5)))
    poses_true = _smooth_loop(rng, n_cam, 16.0, 2.0, 0.06)
    cam_true = np.zeros((n_cam, MAX_CAMERA_PARAMS))
    cam_true[:, 0] = rng.uniform(900, 1500, n_cam)
    cam_true[:, 1], cam_true[:, 2] = 800.0, 600.0
    cam_true[:, 3] = rng.uniform(-0.05, 0.05, n_cam)
    n_pts = max(16, int(round(200000 * scale)))
    d = rng.normal(size=(n_pts, 3))
    pts = d / np.linalg.norm(d, axis=1, keepdims=True) * (3.0 * rng.random(n_pts) ** (1 / 3))[:, None]
    counts = 2 + rng.geometric(1.0 / 5.0, n_pts) - 1
    views_img, views_pt = _contiguous_views(rng, n_cam, counts, loop=True)
    return _finish_scene(
        rng, cam_model=np.full(n_cam, SIMPLE_RADIAL), cam_true=cam_true,
        image_wh=np.tile([1600.0, 1200.0], (n_cam, 1)), poses_true=poses_true, pts_true=pts,
        views_img=views_img, views_pt=views_pt, noise_px=0.5, outlier_frac=0.0,
        fixed_first_pose=True, rot_deg=1.0, trans_abs=0.32, point_rel=0.01, focal_rel=0.03,
        mask_principal_point=True, name="radial500", extra_meta={"seed": seed, "scale": scale})


def power_law_counts(rng, n, alpha=2.5, lo=2, hi=200):
    """Track lengths with density ~ m^-alpha on [lo, hi], rounded up."""
    u = rng.random(n)
    a = 1.0 - alpha
    x = (lo**a + u * (hi**a - lo**a)) ** (1.0 / a)
    return np.minimum(np.ceil(x).astype(np.int64), hi)


def radial2000(seed: int = 0, scale: float = 1.0) -> Problem:
    """2000 RADIAL cameras (f U[900,1500], k1 U[-0.05,0.05], k2 U[-0.01,0.01],
    1600x1200) on a smooth random loop of radius ~20; 1M points in a
    radius-3 ball; power-law track lengths (exponent 2.5, 2..200) over
    consecutive cameras (~5.9M observations); sigma = 0.5 px; init as ring16.
    ``scale`` shrinks points and cameras together."""
    rng = np.random.default_rng(seed)
    n_cam = 2000 if scale >= 1 else max(16, int(round(2000 * scale ** 0.5)))
    poses_true = _smooth_loop(rng, n_cam, 20.0, 2.0, 0.05)
    cam_true = np.zeros((n_cam, MAX_CAMERA_PARAMS))
    cam_true[:, 0] = rng.uniform(900, 1500, n_cam)
    cam_true[:, 1], cam_true[:, 2] = 800.0, 600.0
    cam_true[:, 3] = rng.uniform(-0.05, 0.05, n_cam)
    cam_true[:, 4] = rng.uniform(-0.01, 0.01, n_cam)
    n_pts = max(16, int(round(1_000_000 * scale)))
    d = rng.normal(size=(n_pts, 3))
    pts = d / np.linalg.norm(d, axis=1, keepdims=True) * (3.0 * rng.random(n_pts) ** (1 / 3))[:, None]
    counts = power_law_counts(rng, n_pts, hi=min(200, n_cam))
    views_img, views_pt = _contiguous_views(rng, n_cam, counts, loop=True)
    return _finish_scene(
        rng, cam_model=np.full(n_cam, RADIAL), cam_true=cam_true,
        image_wh=np.tile([1600.0, 1200.0], (n_cam, 1)), poses_true=poses_true, pts_true=pts,
        views_img=views_img, views_pt=views_pt, noise_px=0.5, outlier_frac=0.0,
        fixed_first_pose=True, rot_deg=1.0, trans_abs=0.4, point_rel=0.01, focal_rel=0.03,
        mask_principal_point=True, name="radial2000", extra_meta={"seed": seed, "scale": scale})


def reconstruction_in_progress(seed: int = 0, n_images: int = 60, n_points: int = 6000, n_cameras: int = 3,
                               unregistered: float = 0.15, pinned: int = 2):
    """A reconstruction part way through incremental growth, for the local
    bundle-adjustment windows (crates/sfm-reconstruction/src/lib.rs:
    1287-1299, :1336-1473): ``n_images`` on a 120 degree arc of radius 8
    around a radius-2 ball of points, taken with ``n_cameras`` physical
    cameras (PINHOLE / SIMPLE_RADIAL / RADIAL, consecutive runs of images);
    each point's track covers a run of 1 + Poisson(4) consecutive images (so
    some tracks have a single element); a fraction ``unregistered`` of the
    images is not registered yet (their track elements stay in the tracks);
    ``pinned`` registered images carry caller-pinned poses. Keypoints are the
    true projections plus 0.5 px noise, rounded to float32; poses and points
    are perturbed as in the benchmark scenes."""
    from .problem import Reconstruction

    rng = np.random.default_rng(seed)
    ang = np.deg2rad(np.linspace(-60.0, 60.0, n_images))
    centers = np.stack([8.0 * np.cos(ang), 8.0 * np.sin(ang), rng.uniform(-0.5, 0.5, n_images)], 1)
    poses_true = look_at_pose(centers, np.zeros(3))
    group = (np.arange(n_images) * n_cameras // n_images).astype(np.int32)
    models = np.array([(PINHOLE, SIMPLE_RADIAL, RADIAL)[c % 3] for c in range(n_cameras)], np.int32)
    cams = np.zeros((n_cameras, MAX_CAMERA_PARAMS))
    for c, m in enumerate(models):
        f = rng.uniform(1000, 1400)
        cams[c, :(4 if m != RADIAL else 5)] = {PINHOLE: [f, f * 1.01, 800, 600], SIMPLE_RADIAL: [f, 800, 600, 0.01],
                                   RADIAL: [f, 800, 600, 0.01, -0.002]}[int(m)]
    d = rng.normal(size=(n_points, 3))
    pts_true = d / np.linalg.norm(d, axis=1, keepdims=True) * (2.0 * rng.random(n_points) ** (1 / 3))[:, None]
    lens = 1 + rng.poisson(4.0, n_points)
    start = rng.integers(0, n_images, n_points)
    off = [0]
    t_img, t_xy = [], []
    for p in range(n_points):
        imgs = [int(start[p]) + k for k in range(lens[p])]
        imgs = [i for i in imgs if i < n_images]
        pc = camera_frame(poses_true[imgs], np.repeat(pts_true[p:p + 1], len(imgs), 0))
        ok = pc[:, 2] > 0.1
        imgs = [i for i, o in zip(imgs, ok) if o]
        if not imgs:
            off.append(off[-1])
            continue
        pc = camera_frame(poses_true[imgs], np.repeat(pts_true[p:p + 1], len(imgs), 0))
        uv = project(models[group[imgs]], cams[group[imgs]], pc)
        uv = (uv + rng.normal(0.0, 0.5, uv.shape)).astype(np.float32).astype(np.float64)
        t_img.extend(imgs)
        t_xy.extend(uv.tolist())
        off.append(off[-1] + len(imgs))
    registered = rng.random(n_images) >= unregistered
    registered[0] = True
    axis = rng.normal(size=(n_images, 3))
    axis /= np.linalg.norm(axis, axis=1, keepdims=True)
    tdir = rng.normal(size=(n_images, 3))
    tdir /= np.linalg.norm(tdir, axis=1, keepdims=True)
    delta = np.concatenate([axis * np.deg2rad(0.5), tdir * 0.05], 1)
    delta[0] = 0.0
    poses = perturb_pose(poses_true, delta)
    pdir = rng.normal(size=pts_true.shape)
    pdir /= np.linalg.norm(pdir, axis=1, keepdims=True)
    points = pts_true + pdir * 0.02
    pose_fixed = np.zeros(n_images, bool)
    reg_idx = np.flatnonzero(registered)
    if pinned:
        pose_fixed[rng.choice(reg_idx[1:], min(pinned, len(reg_idx) - 1), replace=False)] = True
    return Reconstruction(camera_of_image=group, camera_model=models, camera_params=cams, poses=poses,
                          registered=registered, points=points, track_offsets=np.asarray(off, np.int64),
                          track_image=np.asarray(t_img, np.int32),
                          track_xy=np.asarray(t_xy, np.float64).reshape(-1, 2), pose_fixed=pose_fixed,
                          meta={"name": "reconstruction_in_progress", "seed": seed})


def shared_radial(seed: int = 0, scale: float = 1.0, n_cameras: int = 1) -> Problem:
    """radial2000's geometry (2000 images on a smooth loop, 1M points,
    power-law tracks; ``scale`` shrinks points and images together) taken
    with ``n_cameras`` physical RADIAL cameras, each used by a consecutive
    run of images: the global adjustment of a sequence shot with one or a
    few cameras, where every camera is one free block shared by many images
    (crates/sfm-reconstruction/src/lib.rs:1489-1520). Observations are
    projected with the shared true cameras (f U[900,1500], k1 U[-0.05,0.05],
    k2 U[-0.01,0.01]); each camera starts with a 3 % focal error; principal
    points masked; pose 0 fixed."""
    rng = np.random.default_rng(seed)
    n_img = 2000 if scale >= 1 else max(16, int(round(2000 * scale ** 0.5)))
    n_cameras = max(1, min(n_cameras, n_img))
    poses_true = _smooth_loop(rng, n_img, 20.0, 2.0, 0.05)
    group = (np.arange(n_img) * n_cameras // n_img).astype(np.int32)
    phys = np.zeros((n_cameras, MAX_CAMERA_PARAMS))
    phys[:, 0] = rng.uniform(900, 1500, n_cameras)
    phys[:, 1], phys[:, 2] = 800.0, 600.0
    phys[:, 3] = rng.uniform(-0.05, 0.05, n_cameras)
    phys[:, 4] = rng.uniform(-0.01, 0.01, n_cameras)
    cam_true = phys[group]
    n_pts = max(16, int(round(1_000_000 * scale)))
    d = rng.normal(size=(n_pts, 3))
    pts = d / np.linalg.norm(d, axis=1, keepdims=True) * (3.0 * rng.random(n_pts) ** (1 / 3))[:, None]
    counts = power_law_counts(rng, n_pts, hi=min(200, n_img))
    views_img, views_pt = _contiguous_views(rng, n_img, counts, loop=True)
    p = _finish_scene(
        rng, cam_model=np.full(n_img, RADIAL), cam_true=cam_true,
        image_wh=np.tile([1600.0, 1200.0], (n_img, 1)), poses_true=poses_true, pts_true=pts,
        views_img=views_img, views_pt=views_pt, noise_px=0.5, outlier_frac=0.0,
        fixed_first_pose=True, rot_deg=1.0, trans_abs=0.4, point_rel=0.01, focal_rel=0.03,
        mask_principal_point=True, name="shared_radial",
        extra_meta={"seed": seed, "scale": scale, "n_cameras": n_cameras})
    first = np.searchsorted(group, np.arange(n_cameras))
    return p.copy(camera_of_image=group, camera_model=p.camera_model[first], camera_params=p.camera_params[first],
                  fixed_cameras=np.zeros(n_cameras, bool), fixed_camera_params=p.fixed_camera_params[first],
                  meta=dict(p.meta, true_camera_params=phys))


def local_window(rng, n_cam, n_pts, views=5.0, models=(PINHOLE, SIMPLE_RADIAL, OPENCV)) -> Problem:
    """One local-BA window: ``n_cam`` cameras on a 60 degree arc of radius 8
    looking at a radius-2 ball of ``n_pts`` points, each seen by
    2 + Poisson(views - 2) consecutive cameras; camera models drawn from
    ``models``; pose 0 fixed, principal point masked."""
    ang = np.deg2rad(np.linspace(-30.0, 30.0, n_cam)) + rng.uniform(0, 2 * np.pi)
    centers = np.stack([8.0 * np.cos(ang), 8.0 * np.sin(ang), rng.uniform(-1, 1, n_cam)], 1)
    poses_true = look_at_pose(centers, np.zeros(3))
    model = rng.choice(np.asarray(models), size=n_cam)
    cam_true = np.zeros((n_cam, MAX_CAMERA_PARAMS))
    f = rng.uniform(1000, 1400, n_cam)
    for c in range(n_cam):
        m = model[c]
        if m == PINHOLE:
            cam_true[c, :4] = [f[c], f[c] * rng.uniform(0.99, 1.01), 800.0, 600.0]
        elif m == SIMPLE_RADIAL:
            cam_true[c, :4] = [f[c], 800.0, 600.0, rng.uniform(-0.05, 0.05)]
        elif m == SIMPLE_PINHOLE:
            cam_true[c, :3] = [f[c], 800.0, 600.0]
        elif m == RADIAL:
            cam_true[c, :5] = [f[c], 800.0, 600.0, rng.uniform(-0.05, 0.05), rng.uniform(-0.01, 0.01)]
        else:
            cam_true[c, :8] = [f[c], f[c] * rng.uniform(0.99, 1.01), 800.0, 600.0,
                               rng.uniform(-0.1, 0.1), rng.uniform(-0.02, 0.02),
                               rng.uniform(-1e-3, 1e-3), rng.uniform(-1e-3, 1e-3)]
    d = rng.normal(size=(n_pts, 3))
    pts = d / np.linalg.norm(d, axis=1, keepdims=True) * (2.0 * rng.random(n_pts) ** (1 / 3))[:, None]
    counts = 2 + rng.poisson(max(views - 2.0, 0.0), n_pts)
    views_img, views_pt = _contiguous_views(rng, n_cam, counts, loop=False)
    return _finish_scene(
        rng, cam_model=model, cam_true=cam_true, image_wh=np.tile([1600.0, 1200.0], (n_cam, 1)),
        poses_true=poses_true, pts_true=pts, views_img=views_img, views_pt=views_pt, noise_px=0.5,
        outlier_frac=0.0, fixed_first_pose=True, rot_deg=1.0, trans_abs=0.16, point_rel=0.01,
        focal_rel=0.03, mask_principal_point=True, name="window")


def windows512(seed: int = 0, scale: float = 1.0, num_windows: int = 512) -> list[Problem]:
    """512 independent local windows: cameras U[8,64], points U[500,20000]
    (times ``scale``), ~5 views per point, mixed PINHOLE / SIMPLE_RADIAL /
    OPENCV cameras."""
    rng = np.random.default_rng(seed)
    out = []
    for w in range(num_windows):
        n_cam = int(rng.integers(8, 65))
        n_pts = max(20, int(round(rng.integers(500, 20001) * scale)))
        p = local_window(rng, n_cam, n_pts)
        p.meta["window"] = w
        out.append(p)
    return out


WORKLOADS = {
    "ring16": ring16,
    "opencv47": opencv47,
    "radial500": radial500,
    "radial2000": radial2000,
}


def shared_ring(seed: int = 0, scale: float = 0.1, images_per_camera=(8, 8), model: int = PINHOLE,
                k: float = 0.0) -> Problem:
    """ring16's geometry with its 16 images sharing a few physical cameras
    (``images_per_camera[c]`` consecutive images each), for the fixed-vs-free
    intrinsics handling of the global adjustment. PINHOLE keeps ring16's
    observations; SIMPLE_RADIAL re-projects them with distortion ``k``
    (true f = 1200, cx = 800, cy = 600) plus 0.5 px noise, and starts from
    the true k. Each camera starts with its first image's 3 % focal error."""
    base = ring16(seed=seed, scale=scale)
    assert sum(images_per_camera) == 16
    cam_of_img = np.repeat(np.arange(len(images_per_camera), dtype=np.int32), images_per_camera)
    first = np.concatenate([[0], np.cumsum(images_per_camera)[:-1]])
    n_cam = len(images_per_camera)
    obs = base.obs_xy
    if model == SIMPLE_RADIAL:
        true = _pad([1200.0, 800.0, 600.0, k])
        pc = camera_frame(base.meta["true_poses"][base.obs_image], base.meta["true_points"][base.obs_point])
        rng = np.random.default_rng(seed + 1000)
        obs = project(np.full(len(pc), SIMPLE_RADIAL), np.tile(true, (len(pc), 1)), pc)
        obs = (obs + rng.normal(0.0, 0.5, obs.shape)).astype(np.float32).astype(np.float64)
        cams = np.tile(true, (n_cam, 1))
        cams[:, 0] = base.camera_params[first, 0]
        mask = np.zeros((n_cam, MAX_CAMERA_PARAMS), bool)
        mask[:, 1:3] = True
    else:
        cams = base.camera_params[first].copy()
        mask = base.fixed_camera_params[first].copy()
    return base.copy(camera_of_image=cam_of_img, camera_model=np.full(n_cam, model, np.int32),
                     camera_params=cams, obs_xy=obs, fixed_cameras=np.zeros(n_cam, bool),
                     fixed_camera_params=mask,
                     meta=dict(base.meta, name="shared_ring", images_per_camera=tuple(images_per_camera)))


def pnp_known_pose_fixture():
    """recovers_known_pose_from_synthetic_correspondences
    (crates/sfm-geometry/src/pnp.rs:311-339): true pose from Euler angles
    (0.05, -0.1, 0.02) and t = (0.2, -0.1, 0.5); 30 points
    (0.5 sin 0.5t, 0.5 cos 0.3t, 5 + 0.2t) and their exact normalised
    projections. Returns (pose [7], points [30, 3], uv [30, 2])."""
    pose = np.concatenate([quat_from_euler(0.05, -0.1, 0.02), [0.2, -0.1, 0.5]])
    t = np.arange(30, dtype=np.float64)
    X = np.stack([0.5 * np.sin(t * 0.5), 0.5 * np.cos(t * 0.3), 5.0 + 0.2 * t], 1)
    pc = camera_frame(np.tile(pose, (30, 1)), X)
    return pose, X, pc[:, :2] / pc[:, 2:3]


def pnp_batch(seed: int = 0, num_images: int = 64, n_min: int = 200, n_max: int = 2000, outlier_frac: float = 0.3,
              noise_px: float = 0.5, focal: float = 1200.0):
    """Registration of many images at once, as the incremental pipeline
    registers them (crates/sfm-reconstruction/src/lib.rs:654-676): per image
    n ~ U[n_min, n_max] 2D-3D correspondences of points 4-12 units in front
    of the camera inside a 60 degree cone, normalised observations with
    ``noise_px`` / focal noise, a fraction replaced by uniform outliers.
    Returns (true poses [num_images, 7], list of points [n, 3], list of
    uv [n, 2], threshold = 8 px / focal)."""
    rng = np.random.default_rng(seed)
    poses, Xs, uvs = [], [], []
    for _ in range(num_images):
        ax = rng.normal(size=3)
        ax *= rng.uniform(0.0, 0.5) / np.linalg.norm(ax)
        q = quat_from_scaled_axis(ax)
        t = rng.uniform(-2.0, 2.0, 3)
        pose = np.concatenate([q, t])
        n = int(rng.integers(n_min, n_max + 1))
        d = rng.uniform(4.0, 12.0, n)
        xy = rng.uniform(-0.55, 0.55, (n, 2))
        pc = np.concatenate([xy * d[:, None], d[:, None]], 1)
        # world point X with R X + t = pc
        R = quat_to_matrix(q)
        X = (pc - t) @ R
        uv = xy + rng.normal(0.0, noise_px / focal, (n, 2))
        k = int(round(outlier_frac * n))
        idx = rng.choice(n, k, replace=False)
        uv[idx] = rng.uniform(-0.6, 0.6, (k, 2))
        poses.append(pose)
        Xs.append(X)
        uvs.append(uv)
    return np.array(poses), Xs, uvs, 8.0 / focal
