"""Batched local windows (sfmba_bundle_adjust_batched) against the CPU FP64
oracle run on each window alone, and against single-window GPU solves.

Bars (written in each test): FP64 - initial cost 1e-12 relative, final
cost and parameters 1e-6 relative, same iteration count per window; mixed
FP32/FP64 - final cost 1e-6 relative and RMS 1e-4 px per window; window
order and batch composition do not change a window's result (1e-12)."""
import numpy as np
import pytest

from sfmtory_gb300 import abi, native, scenes
from sfmtory_gb300.problem import Problem, rms_reprojection_error

pytestmark = pytest.mark.gpu

KW = dict(robust_loss=abi.LOSS_HUBER, loss_scale_px=2.0, max_iterations=30)


def _windows(seed, count, cams=(8, 20), pts=(150, 500)):
    rng = np.random.default_rng(seed)
    return [scenes.local_window(rng, int(rng.integers(*cams)), int(rng.integers(*pts))) for _ in range(count)]


def _check_window(g, r, cost_rtol=1e-6, param_rtol=1e-6, same_iters=True):
    assert abs(g.initial_cost - r.initial_cost) <= 1e-12 * abs(r.initial_cost) + 1e-300
    assert abs(g.final_cost - r.final_cost) <= cost_rtol * abs(r.final_cost) + 1e-12
    if same_iters:
        assert g.iterations_run == r.iterations_run
    for a, b in ((g.points, r.points), (g.poses, r.poses), (g.camera_params, r.camera_params)):
        if b.size:
            err = np.abs(a - b) / np.maximum(np.abs(b), 1.0)
            assert err.max() <= param_rtol, err.max()


def test_batched_fp64_matches_oracle_per_window(oracle_lib):
    wins = _windows(11, 6)
    res = native.bundle_adjust_batched_arrays(wins, **KW)
    assert len(res) == len(wins)
    for p, g in zip(wins, res):
        r = oracle_lib.bundle_adjust(p, **KW)
        _check_window(g, r)
        assert g.final_cost < g.initial_cost
        assert g.reduced_dim == p.reduced_dim()


def test_batched_mixed_reaches_oracle_cost(oracle_lib):
    """FP32 linearisation and Schur, FP64 cost, Cholesky and refinement,
    FP64 polish: every window's final cost within 1e-6 relative of the
    oracle and its RMS within 1e-4 px."""
    wins = _windows(12, 6)
    res = native.bundle_adjust_batched_arrays(wins, precision=abi.PRECISION_MIXED, **KW)
    for p, g in zip(wins, res):
        r = oracle_lib.bundle_adjust(p, **KW)
        assert abs(g.final_cost - r.final_cost) <= 1e-6 * r.final_cost
        rg = rms_reprojection_error(p.copy(poses=g.poses, points=g.points, camera_params=g.camera_params))
        rr = rms_reprojection_error(p.copy(poses=r.poses, points=r.points, camera_params=r.camera_params))
        assert abs(rg - rr) < 1e-4


def test_batched_equals_single_window_solves():
    """Each window of a batch ends where the single-problem GPU path does."""
    wins = _windows(13, 4)
    res = native.bundle_adjust_batched_arrays(wins, **KW)
    for p, g in zip(wins, res):
        s = native.bundle_adjust_arrays(p, solver=abi.SOLVER_DENSE, **KW)
        _check_window(g, s, cost_rtol=1e-9, param_rtol=1e-7)


def test_batched_window_order_does_not_matter():
    """Windows are independent: reversing the batch and dropping windows
    leaves every remaining window's result unchanged."""
    wins = _windows(14, 5)
    a = native.bundle_adjust_batched_arrays(wins, precision=abi.PRECISION_MIXED, **KW)
    b = native.bundle_adjust_batched_arrays(wins[::-1], precision=abi.PRECISION_MIXED, **KW)[::-1]
    c = native.bundle_adjust_batched_arrays(wins[1:2], precision=abi.PRECISION_MIXED, **KW)
    for x, y in zip(a, b):
        assert x.iterations_run == y.iterations_run
        assert abs(x.final_cost - y.final_cost) <= 1e-12 * x.final_cost
        assert np.allclose(x.points, y.points, rtol=0, atol=1e-12 * max(1.0, np.abs(x.points).max()))
    assert a[1].iterations_run == c[0].iterations_run
    assert abs(a[1].final_cost - c[0].final_cost) <= 1e-12 * a[1].final_cost


def _empty_window():
    return Problem(camera_of_image=np.zeros(0, np.int32), camera_model=np.zeros(0, np.int32),
                   camera_params=np.zeros((0, 8)), poses=np.zeros((0, 7)), points=np.zeros((0, 3)),
                   obs_image=np.zeros(0, np.int32), obs_point=np.zeros(0, np.int32), obs_xy=np.zeros((0, 2)))


def test_batched_degenerate_windows(oracle_lib):
    """Windows the reference returns from early sit beside normal ones:
    an empty window, one with every parameter fixed (no unknowns,
    lib.rs:777-787), one with every point behind its cameras (no valid
    observation, lib.rs:855-857) and one with an unobserved free camera
    (singular system: Cholesky and LU fail, damping grows)."""
    rng = np.random.default_rng(15)
    normal = scenes.local_window(rng, 10, 300)
    fixed = scenes.local_window(rng, 8, 200)
    fixed = fixed.copy(fixed_poses=np.ones(fixed.num_images, bool), fixed_cameras=np.ones(fixed.num_cameras, bool))
    behind = scenes.recovers_ground_truth_fixture()
    behind = behind.copy(points=behind.points * np.array([1, 1, -1.0]))
    lonely = scenes.local_window(rng, 9, 250)
    keep = lonely.obs_image != 4
    lonely = lonely.copy(obs_image=lonely.obs_image[keep], obs_point=lonely.obs_point[keep],
                         obs_xy=lonely.obs_xy[keep])
    wins = [normal, _empty_window(), fixed, behind, lonely]
    res = native.bundle_adjust_batched_arrays(wins, **KW)
    assert res[1].iterations_run == 0 and res[1].final_cost == 0.0
    assert res[2].iterations_run == 0 and res[2].final_cost == res[2].initial_cost
    assert np.array_equal(res[2].points, fixed.points)
    for k in (0, 2, 3, 4):
        r = oracle_lib.bundle_adjust(wins[k], **KW)
        _check_window(res[k], r)
