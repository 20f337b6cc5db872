"""`sfmtory refine` (crates/sfm-cli/src/main.rs:946-1130) on a COLMAP text
model, on the GPU, against the Python restatement of that command on the CPU
oracle (oracle/colmap_text.py).

Bars (FP64): final cost 1e-6 relative and the same iteration count; the
written poses, points and cameras within 1e-6 relative to max(|x|, 1) (the
files carry 10 decimals); every point's recomputed error within 1e-6 px
(6 decimals in the file); the mean errors before and after within 1e-6."""
import numpy as np
import pytest

from oracle import colmap_text as ct
from sfmtory_gb300 import abi, native, scenes

from colmap_util import model_from_problem

pytestmark = pytest.mark.gpu


def _close(a, b, tol):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return (np.abs(a - b) / np.maximum(np.abs(b), 1.0)).max() <= tol


@pytest.mark.parametrize("refine_intrinsics", [False, True])
def test_refine_matches_oracle(tmp_path, oracle_lib, refine_intrinsics):
    p = scenes.shared_ring(0, 0.1, images_per_camera=(6, 5, 5))
    d_in, d_out = str(tmp_path / "in"), str(tmp_path / "out")
    ct.write_model(model_from_problem(p, seed=3), d_in)
    kw = dict(robust_loss=abi.LOSS_HUBER, max_iterations=200)
    rep = native.colmap_refine(d_in, d_out, refine_intrinsics, solver=abi.SOLVER_DENSE, **kw)
    ref, r, before, after = ct.refine(ct.read_model(d_in), refine_intrinsics, **kw)
    got = ct.read_model(d_out)
    assert rep["iterations_run"] == r.iterations_run
    assert abs(rep["final_cost"] - r.final_cost) <= 1e-6 * r.final_cost
    assert abs(rep["mean_error_before_px"] - before) <= 1e-9
    assert abs(rep["mean_error_after_px"] - after) <= 1e-6
    assert rep["num_images"] == 16 and rep["num_points3d"] == len(ref.points)
    for iid, im in ref.images.items():
        g = got.images[iid]
        assert _close(g.t, im.t, 1e-6)
        assert min(np.abs(np.array(g.q) - im.q).max(), np.abs(np.array(g.q) + im.q).max()) <= 1e-6
        assert g.keypoints == im.keypoints and g.point3d_ids == im.point3d_ids and g.name == im.name
    for pid, pt in ref.points.items():
        g = got.points[pid]
        assert _close(g.xyz, pt.xyz, 1e-6)
        assert abs(g.error - pt.error) <= 1e-6 + 1e-9
        assert g.track == pt.track and g.color == pt.color
    for cid, c in ref.cameras.items():
        assert _close(got.cameras[cid].params, c.params, 1e-6)
        if not refine_intrinsics:
            assert _close(got.cameras[cid].params, ct.read_model(d_in).cameras[cid].params, 0.0)


def test_refine_in_place_and_default_options(tmp_path):
    """dir_out = dir_in rewrites the model; with no options the reference's
    Huber loss and 200 iterations are used."""
    p = scenes.shared_ring(1, 0.05)
    d = str(tmp_path / "m")
    ct.write_model(model_from_problem(p, seed=4), d)
    rep = native.colmap_refine(d)
    assert rep["final_cost"] < rep["initial_cost"]
    assert rep["mean_error_after_px"] < rep["mean_error_before_px"]
    assert native.colmap_model_stats(d)["mean_reprojection_error"] == pytest.approx(rep["mean_error_after_px"])


def test_refine_rejects_what_the_reference_rejects(tmp_path):
    """Fewer than 2 images, no points, no usable observation: errors."""
    p = scenes.shared_ring(0, 0.05)
    m = model_from_problem(p, seed=5)
    one = ct.Model(cameras=m.cameras, images={k: v for k, v in list(m.images.items())[:1]}, points=m.points)
    d = str(tmp_path / "one")
    ct.write_model(one, d)
    with pytest.raises(native.SfmbaError):
        native.colmap_refine(d, str(tmp_path / "o1"))
    nopts = ct.Model(cameras=m.cameras, images=m.images, points={})
    d = str(tmp_path / "nopts")
    ct.write_model(nopts, d)
    with pytest.raises(native.SfmbaError):
        native.colmap_refine(d, str(tmp_path / "o2"))
    dangling = ct.Model(cameras=m.cameras, images=m.images,
                        points={k: ct.Point(k, v.xyz, v.color, v.error, [(999999, 0)]) for k, v in m.points.items()})
    d = str(tmp_path / "dangling")
    ct.write_model(dangling, d)
    with pytest.raises(native.SfmbaError):
        native.colmap_refine(d, str(tmp_path / "o3"))
