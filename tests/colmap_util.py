"""Test models in COLMAP text form built from the seeded scenes."""
import numpy as np

from oracle.colmap_text import Camera, Image, Model, Point


def model_from_problem(p, seed=0, extra_keypoints=2, dangling=3):
    """A COLMAP model of a Problem with scattered ids: each image's keypoints
    are its observations (plus unmatched ones), tracks reference them; a few
    track elements point at a missing image or keypoint (skipped by refine)."""
    rng = np.random.default_rng(seed)
    m = Model()
    cam_ids = [5 + 4 * c for c in range(p.num_cameras)]
    for c, cid in enumerate(cam_ids):
        m.cameras[cid] = Camera(cid, int(p.camera_model[c]), 1600, 1200, list(p.camera_params[c]))
    img_ids = [10 + 3 * i for i in range(p.num_images)]
    pt_ids = [1000 + 7 * k for k in range(p.num_points)]
    for i, iid in enumerate(img_ids):
        m.images[iid] = Image(iid, list(p.poses[i, :4]), list(p.poses[i, 4:]), cam_ids[p.camera_of_image[i]],
                              f"img_{i:04d}.jpg")
    for k, pid in enumerate(pt_ids):
        m.points[pid] = Point(pid, list(p.points[k]), tuple(int(v) for v in rng.integers(0, 256, 3)),
                              float(rng.uniform(0.1, 2.0)))
    for o in range(p.num_observations):
        im = m.images[img_ids[p.obs_image[o]]]
        for _ in range(int(rng.integers(0, extra_keypoints + 1))):
            im.keypoints.append(tuple(float(np.float32(v)) for v in rng.uniform(0, 1000, 2)))
            im.point3d_ids.append(-1)
        im.keypoints.append((float(np.float32(p.obs_xy[o, 0])), float(np.float32(p.obs_xy[o, 1]))))
        im.point3d_ids.append(pt_ids[p.obs_point[o]])
        m.points[pt_ids[p.obs_point[o]]].track.append((im.id, len(im.keypoints) - 1))
    for _ in range(dangling):
        pt = m.points[pt_ids[int(rng.integers(0, p.num_points))]]
        pt.track.append((999999, 0) if rng.random() < 0.5 else (img_ids[0], 10 ** 6))
    return m


def sample_recon():
    """The reference's round-trip fixture (crates/sfm-io/src/colmap.rs:311-351)."""
    m = Model()
    m.cameras[1] = Camera(1, 2, 1920, 1080, [1600.0, 960.0, 540.0, -0.05])
    q = np.array([0.98, 0.1, 0.05, 0.02])
    q = q / np.sqrt(q[1] ** 2 + q[2] ** 2 + q[3] ** 2 + q[0] ** 2)  # Pose::from_quaternion_wxyz_translation
    m.images[1] = Image(1, list(q), [0.1, -0.2, 1.5], 1, "img_0001.jpg",
                        [(100.5, 200.25), (300.0, 400.0)], [1, -1])
    m.points[1] = Point(1, [1.0, 2.0, 3.0], (255, 128, 0), 0.42, [(1, 0)])
    return m
