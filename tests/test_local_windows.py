"""Local bundle-adjustment windows (sfm-reconstruction's BaScope::Local,
crates/sfm-reconstruction/src/lib.rs:1287-1299, :1336-1473) built by the
library's host code (sfmba_local_windows), against the restated builder in
oracle/local_windows.py: every index set and copied value bit-exact. Host
computation only: runs without a GPU."""
import numpy as np
import pytest

from oracle import local_windows as O
from sfmtory_gb300 import native, scenes
from sfmtory_gb300.problem import Reconstruction


def _compare(got, exp):
    if exp is None:
        assert got is None
        return
    assert got is not None
    prob, image_ids, camera_ids, point_ids = got
    assert np.array_equal(image_ids, exp["image_ids"])
    assert np.array_equal(camera_ids, exp["camera_ids"])
    assert np.array_equal(point_ids, exp["point_ids"])
    for name in ("camera_of_image", "camera_model", "obs_image", "obs_point"):
        assert np.array_equal(getattr(prob, name), exp[name]), name
    for name in ("camera_params", "poses", "points", "obs_xy"):
        assert np.array_equal(getattr(prob, name), exp[name]), name  # copied, bit for bit
    for name in ("fixed_poses", "fixed_cameras", "fixed_camera_params"):
        assert np.array_equal(np.asarray(getattr(prob, name), bool), exp[name]), name


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_local_windows_match_restated_builder(seed):
    rec = scenes.reconstruction_in_progress(seed=seed)
    centers = list(range(len(rec.poses)))  # registered and unregistered centres alike
    got = native.local_windows(rec, centers, seed_image=0)
    for c, g in zip(centers, got):
        _compare(g, O.local_window(rec, c, seed_image=0))


def test_local_windows_neighbour_count_and_no_seed():
    rec = scenes.reconstruction_in_progress(seed=4, n_images=30, n_points=2000, n_cameras=2)
    for k in (0, 1, 6, 40):
        got = native.local_windows(rec, [3, 15, 29], seed_image=-1, num_free_neighbours=k)
        for c, g in zip([3, 15, 29], got):
            _compare(g, O.local_window(rec, c, seed_image=-1, num_free=k))


def test_local_window_structure():
    """The centre and at most six co-visible images are free, every other
    window image is fixed, the pinned poses stay fixed, intrinsics are held
    with the principal point masked."""
    rec = scenes.reconstruction_in_progress(seed=5)
    c = int(np.flatnonzero(rec.registered)[10])
    prob, image_ids, camera_ids, point_ids = native.local_windows(rec, [c], seed_image=0)[0]
    free = ~np.asarray(prob.fixed_poses, bool)
    assert 1 <= free.sum() <= 7
    assert c in image_ids[free] or rec.pose_fixed[c]
    assert not free[np.isin(image_ids, np.flatnonzero(rec.pose_fixed))].any()
    assert np.all(rec.registered[image_ids])
    assert np.all(prob.fixed_cameras)
    for p in point_ids:  # every free point is seen by the centre and has >= 2 elements
        tr = rec.track_image[rec.track_offsets[p]:rec.track_offsets[p + 1]]
        assert len(tr) >= 2 and c in tr


def test_local_windows_empty_cases():
    """No window where the reference makes no solve: a centre with no
    points, a window of a single image."""
    rec = scenes.reconstruction_in_progress(seed=6, n_images=10, n_points=300)
    n = len(rec.poses)
    lone = Reconstruction(camera_of_image=np.zeros(2, np.int32), camera_model=rec.camera_model[:1],
                          camera_params=rec.camera_params[:1], poses=rec.poses[:2],
                          registered=np.array([True, False]), points=rec.points[:1],
                          track_offsets=np.array([0, 2], np.int64), track_image=np.array([0, 1], np.int32),
                          track_xy=np.zeros((2, 2)))
    assert native.local_windows(lone, [0, 1])[0] is None  # one registered image only
    assert O.local_window(lone, 0) is None
    empty = Reconstruction(camera_of_image=rec.camera_of_image, camera_model=rec.camera_model,
                           camera_params=rec.camera_params, poses=rec.poses, registered=rec.registered,
                           points=np.zeros((0, 3)), track_offsets=np.zeros(1, np.int64),
                           track_image=np.zeros(0, np.int32), track_xy=np.zeros((0, 2)))
    assert native.local_windows(empty, list(range(n))) == [None] * n


def test_local_windows_reject_bad_input():
    rec = scenes.reconstruction_in_progress(seed=7, n_images=10, n_points=300)
    with pytest.raises(native.SfmbaError) as e:
        native.local_windows(rec, [10])
    assert e.value.status == 1
    bad = Reconstruction(**{**rec.__dict__, "track_image": np.where(np.arange(len(rec.track_image)) == 3, 99,
                                                                   rec.track_image).astype(np.int32)})
    with pytest.raises(native.SfmbaError):
        native.local_windows(bad, [0])
