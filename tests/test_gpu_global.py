"""The fixed-vs-free intrinsics handling of the global adjustment
(crates/sfm-reconstruction/src/lib.rs:1567-1708) on the GPU against the
oracle's restatement.

Bars (FP64 path): the same candidate chosen, the same observations kept,
final cost 1e-6 relative, both candidates' plain mean reprojection errors
1e-9 relative (a pure function of the outputs, so it inherits their
agreement), parameters 1e-5 relative to max(|x|, 1) (the free camera's
focal length is weakly observed on this 20 degree arc: the cost is flat
along it, and summation order moves it by ~1e-6 while the cost agrees to
1e-9). FP32 path: the same candidate, final cost 1e-6 relative."""
import numpy as np
import pytest

from sfmtory_gb300 import abi, native, scenes

pytestmark = pytest.mark.gpu

KW = dict(robust_loss=abi.LOSS_HUBER, loss_scale_px=1.0, max_iterations=50)


def _with_outliers(p, frac=0.03, seed=7):
    rng = np.random.default_rng(seed)
    q = p.copy()
    idx = rng.choice(q.num_observations, int(frac * q.num_observations), replace=False)
    q.obs_xy[idx] = rng.uniform([0.0, 0.0], [1600.0, 1200.0], size=(len(idx), 2))
    return q


CASES = {
    "pinhole_outliers": lambda: _with_outliers(scenes.shared_ring(0, 0.1)),
    "few_images": lambda: scenes.shared_ring(1, 0.1, images_per_camera=(12, 4)),
    "implausible_k": lambda: scenes.shared_ring(2, 0.1, model=abi.SIMPLE_RADIAL, k=0.6),
}


@pytest.mark.parametrize("mode", [abi.INTRINSICS_FIXED, abi.INTRINSICS_FREE, abi.INTRINSICS_FREE_GUARDED])
@pytest.mark.parametrize("case", list(CASES))
def test_adjust_global_fp64_matches_oracle(oracle_lib, case, mode):
    p = CASES[case]()
    g, gk, gc, ge = native.adjust_global_arrays(p, mode, 4.0, solver=abi.SOLVER_DENSE, **KW)
    r, rk, rc, re = oracle_lib.adjust_global(p, mode, 4.0, **KW)
    assert gc == rc
    assert np.array_equal(gk, rk)
    assert abs(g.final_cost - r.final_cost) <= 1e-6 * r.final_cost
    for a, b in zip(ge, re):
        assert (np.isnan(a) and np.isnan(b)) or abs(a - b) <= 1e-9 * b
    for a, b in ((g.points, r.points), (g.poses, r.poses), (g.camera_params, r.camera_params)):
        assert (np.abs(a - b) / np.maximum(np.abs(b), 1.0)).max() <= 1e-5
    if mode == abi.INTRINSICS_FIXED:
        assert np.array_equal(g.camera_params, p.camera_params)
    if case == "implausible_k" and mode == abi.INTRINSICS_FREE_GUARDED:
        assert not gc and ge[1] < ge[0]  # lower error, rejected by the distortion bound


def test_adjust_global_mixed_same_choice(oracle_lib):
    p = CASES["pinhole_outliers"]()
    g, gk, gc, _ = native.adjust_global_arrays(p, abi.INTRINSICS_FREE_GUARDED, 4.0,
                                               precision=abi.PRECISION_MIXED, solver=abi.SOLVER_DENSE, **KW)
    r, rk, rc, _ = oracle_lib.adjust_global(p, abi.INTRINSICS_FREE_GUARDED, 4.0, **KW)
    assert gc == rc
    if np.array_equal(gk, rk):
        assert abs(g.final_cost - r.final_cost) <= 1e-6 * r.final_cost


def test_adjust_global_rejects_unknown_mode():
    p = scenes.shared_ring(0, 0.05)
    with pytest.raises(native.SfmbaError):
        native.adjust_global_arrays(p, 7, 4.0)
