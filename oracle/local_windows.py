"""TEST INFRASTRUCTURE ONLY: a restatement of sfm-reconstruction's local
bundle-adjustment window construction (BaScope::Local), the checker of the
library's sfmba_local_windows.

Follows crates/sfm-reconstruction/src/lib.rs:1336-1473 (run_bundle_adjustment
with BaScope::Local and IntrinsicsMode::Fixed) step by step on the array
form of a reconstruction (sfmtory_gb300.problem.Reconstruction):
free points :1345-1352, co-visibility ranking :1353-1376 (LOCAL_BA_NUM_IMAGES
= 6, :1320), window images :1385-1406, cameras in first-use order
:1408-1420, fixed poses :1427-1456, observations :1458-1473, the
principal-point mask of default_fixed_params_mask (crates/sfm-ba/src/
intrinsics.rs:33-61, :1489). Pure Python loops; only tests import it.
"""
from __future__ import annotations

import numpy as np

LOCAL_BA_NUM_IMAGES = 6


def local_window(rec, center: int, seed_image: int = -1, num_free: int = LOCAL_BA_NUM_IMAGES):
    """None where the reference returns without a solve, else a dict of the
    window's arrays and the reconstruction indices of its entries."""
    off, timg, txy = rec.track_offsets, rec.track_image, rec.track_xy
    registered = [bool(x) for x in rec.registered]
    n_pts = len(off) - 1
    tracks = [[(int(timg[e]), e) for e in range(off[p], off[p + 1])] for p in range(n_pts)]
    point_ids = [p for p in range(n_pts) if len(tracks[p]) >= 2 and any(img == center for img, _ in tracks[p])]
    covis: dict[int, int] = {}
    for p in point_ids:
        for img, _ in tracks[p]:
            if img != center and registered[img]:
                covis[img] = covis.get(img, 0) + 1
    ranked = sorted(covis.items(), key=lambda kv: (-kv[1], kv[0]))
    free = {img for img, _ in ranked[:num_free]}
    free.add(center)
    seen = [False] * len(registered)
    for p in point_ids:
        for img, _ in tracks[p]:
            if registered[img]:
                seen[img] = True
    image_ids = [i for i in range(len(registered)) if seen[i]]
    if len(image_ids) < 2:
        return None
    image_pos = {orig: k for k, orig in enumerate(image_ids)}
    camera_of_image, camera_ids, cam_index = [], [], {}
    for orig in image_ids:
        c = int(rec.camera_of_image[orig])
        if c not in cam_index:
            cam_index[c] = len(camera_ids)
            camera_ids.append(c)
        camera_of_image.append(cam_index[c])
    pinned = rec.pose_fixed if rec.pose_fixed is not None else np.zeros(len(registered), bool)
    fixed = [orig == seed_image or orig not in free for orig in image_ids]
    fixed = [f or bool(pinned[orig]) for f, orig in zip(fixed, image_ids)]
    if not any(fixed):
        fixed[0] = True
    obs_image, obs_point, obs_xy = [], [], []
    for cp, p in enumerate(point_ids):
        for img, e in tracks[p]:
            if img not in image_pos:
                continue
            obs_image.append(image_pos[img])
            obs_point.append(cp)
            obs_xy.append((float(txy[e][0]), float(txy[e][1])))
    if not obs_image:
        return None
    models = [int(rec.camera_model[c]) for c in camera_ids]
    mask = np.zeros((len(camera_ids), 8), bool)
    for k, m in enumerate(models):
        a = 1 if m in (0, 2, 3) else 2  # SIMPLE_PINHOLE, SIMPLE_RADIAL, RADIAL: (1, 2); else (2, 3)
        mask[k, a] = mask[k, a + 1] = True
    cams = np.zeros((len(camera_ids), 8))
    cp_src = np.asarray(rec.camera_params)
    for k, c in enumerate(camera_ids):
        cams[k, : cp_src.shape[1]] = cp_src[c]
    return {
        "image_ids": np.array(image_ids, np.int32), "camera_ids": np.array(camera_ids, np.int32),
        "point_ids": np.array(point_ids, np.int32), "camera_of_image": np.array(camera_of_image, np.int32),
        "camera_model": np.array(models, np.int32), "camera_params": cams,
        "poses": np.asarray(rec.poses)[image_ids], "points": np.asarray(rec.points)[point_ids],
        "obs_image": np.array(obs_image, np.int32), "obs_point": np.array(obs_point, np.int32),
        "obs_xy": np.array(obs_xy, np.float64).reshape(-1, 2), "fixed_poses": np.array(fixed, bool),
        "fixed_cameras": np.ones(len(camera_ids), bool), "fixed_camera_params": mask,
    }
