"""COLMAP text model I/O (crates/sfm-io/src/colmap.rs) through the C ABI:
host code only, so these run without a GPU. The checker is the Python
restatement in oracle/colmap_text.py."""
import os

import numpy as np
import pytest

from oracle import colmap_text as ct
from sfmtory_gb300 import native

from colmap_util import model_from_problem, sample_recon


def _read(d, name):
    return open(os.path.join(d, name)).read()


def test_round_trips_through_text_files(tmp_path):
    """round_trips_through_text_files (colmap.rs:353-383), read and written
    by the library: the reference's assertions, and the library's output is
    byte-identical to the reference writer's."""
    a, b = str(tmp_path / "a"), str(tmp_path / "b")
    ct.write_model(sample_recon(), a)
    native.colmap_rewrite(a, b)
    for f in ("cameras.txt", "images.txt", "points3D.txt"):
        assert _read(a, f) == _read(b, f), f
    back = ct.read_model(b)
    assert len(back.cameras) == 1 and len(back.images) == 1 and len(back.points) == 1
    assert ct.MODEL_NAMES[back.cameras[1].model] == "SIMPLE_RADIAL" and back.cameras[1].width == 1920
    img = back.images[1]
    assert img.name == "img_0001.jpg" and len(img.keypoints) == 2 and img.point3d_ids == [1, -1]
    p = back.points[1]
    assert p.color == (255, 128, 0) and len(p.track) == 1 and abs(p.xyz[0] - 1.0) < 1e-6
    st = native.colmap_model_stats(b)
    assert (st["cameras"], st["images"], st["points3d"], st["track_elements"], st["keypoints"]) == (1, 1, 1, 1, 2)
    assert st["mean_reprojection_error"] == pytest.approx(0.42, abs=1e-12)


def test_rewrite_of_a_scene_model_matches_reference_writer(tmp_path):
    """A larger model with scattered ids, unmatched keypoints and dangling
    track elements; the quaternions of the input are not normalised (read
    normalises them, pose.rs:74-80)."""
    from sfmtory_gb300 import scenes

    m = model_from_problem(scenes.shared_ring(0, 0.05), seed=1)
    for im in m.images.values():
        im.q = [2.0 * v for v in im.q]
    a, b, c = str(tmp_path / "a"), str(tmp_path / "b"), str(tmp_path / "c")
    ct.write_model(m, a)
    native.colmap_rewrite(a, b)
    ct.write_model(ct.read_model(a), c)
    for f in ("cameras.txt", "images.txt", "points3D.txt"):
        assert _read(b, f) == _read(c, f), f


@pytest.mark.parametrize("fname,bad", [
    ("cameras.txt", "1 PINHOLE 100\n"),
    ("cameras.txt", "1 NOT_A_MODEL 100 100 1 2 3\n"),
    ("cameras.txt", "1 PINHOLE 100 100 1 2 3\n"),
    ("cameras.txt", "x PINHOLE 100 100 1 2 3 4\n"),
    ("cameras.txt", "1 PINHOLE -5 100 1 2 3 4\n"),
    ("images.txt", "1 1 0 0 0 0 0 0 1\n\n"),
    ("images.txt", "1 1 0 0 0 0 0 0 1 a.jpg\n"),
    ("images.txt", "1 1 0 0 q 0 0 0 1 a.jpg\n1 2 3\n"),
    ("images.txt", "1 1 0 0 0 0 0 0 1 a.jpg\n1.0 2.0 z\n"),
    ("points3D.txt", "1 0 0 0 1 2 3\n"),
    ("points3D.txt", "1 0 0 0 1 2 300 0.5\n"),
    ("points3D.txt", "1 0 0 0 1 2 3 0.5 1 -2\n"),
])
def test_malformed_files_are_errors(tmp_path, fname, bad):
    d = str(tmp_path / "m")
    ct.write_model(sample_recon(), d)
    open(os.path.join(d, fname), "w").write("# comment\n" + bad)
    with pytest.raises(native.SfmbaError) as e:
        native.colmap_rewrite(d, str(tmp_path / "out"))
    assert e.value.status == 1


def test_missing_model_is_an_error(tmp_path):
    with pytest.raises(native.SfmbaError):
        native.colmap_model_stats(str(tmp_path / "nothing"))
