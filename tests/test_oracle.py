"""The reference's own sfm-ba tests, run against the CPU FP64 oracle.

These pin the oracle before it is trusted as the parity reference for the GPU
path: crates/sfm-ba/src/lib.rs:1245-1592 (6 analytic-vs-numerical Jacobian
tests, 2 convergence tests) and crates/sfm-ba/src/intrinsics.rs:252-383
(3 intrinsics tests), with the reference's fixtures and tolerances.
"""
import numpy as np
import pytest

from sfmtory_gb300 import abi, scenes

MODELS = list(scenes.JACOBIAN_TEST_CAMERAS)


@pytest.mark.parametrize("model", MODELS, ids=[abi.MODEL_NAMES[m] for m in MODELS])
def test_analytic_matches_numerical(oracle_lib, model):
    """assert_analytic_matches_numerical (lib.rs:1252-1295): residual < 1e-9,
    pose/point Jacobian Frobenius < 1e-5, camera Jacobian < 1e-4."""
    pose, X, obs = scenes.jacobian_test_fixture()
    params = scenes.JACOBIAN_TEST_CAMERAS[model]
    num = oracle_lib.numerical_jacobians(pose, model, params, X, obs)
    an = oracle_lib.analytic_jacobians(pose, model, params, X, obs)
    assert num is not None and an is not None, "point in front of camera"
    assert np.linalg.norm(num[0] - an[0]) < 1e-9
    assert np.linalg.norm(num[1] - an[1]) < 1e-5
    assert np.linalg.norm(num[2] - an[2]) < 1e-5
    assert np.linalg.norm(num[3] - an[3]) < 1e-4
    # Columns past the model's parameter count are zero.
    assert np.all(an[3][:, abi.MODEL_DOF[model]:] == 0)


def test_recovers_ground_truth_from_perturbed_initialization(oracle_lib):
    """lib.rs:1368-1476."""
    p = scenes.recovers_ground_truth_fixture()
    out = oracle_lib.bundle_adjust(p, max_iterations=30)
    assert out.final_cost < out.initial_cost * 0.01
    mean_sq = out.final_cost / (len(out.poses) * 25)
    assert np.sqrt(mean_sq) < 0.5
    t = out.poses[1, 4:]
    tt = p.meta["true_poses"][1, 4:]
    cos = np.dot(t / np.linalg.norm(t), tt / np.linalg.norm(tt))
    assert cos > 0.999
    assert abs(np.linalg.norm(t) / np.linalg.norm(tt) - 1.0) < 0.1


def test_joint_optimization_recovers_shared_camera_focal_length(oracle_lib):
    """lib.rs:1487-1592: pre-converge with the wrong focal fixed, then solve
    jointly with the shared camera free."""
    p = scenes.shared_focal_fixture()
    pre = oracle_lib.bundle_adjust(p, max_iterations=50)
    joint = p.copy(poses=pre.poses, points=pre.points, fixed_cameras=np.array([False]))
    out = oracle_lib.bundle_adjust(joint, max_iterations=50)
    f = out.camera_params[0, 0]
    assert abs(f - 1500.0) / 1500.0 < 0.02, f


def test_recovers_true_focal_length_from_wrong_initial_guess(oracle_lib):
    """intrinsics.rs:262-305."""
    p = scenes.intrinsics_fixture()
    cams = oracle_lib.refine_intrinsics(p)
    assert abs(cams[0, 0] - 1500.0) < 1.0, cams[0, 0]


def test_leaves_camera_unchanged_with_too_few_observations(oracle_lib):
    """intrinsics.rs:307-340: one observation (< 8) leaves the camera as is."""
    p = scenes.intrinsics_fixture(n_points=1)
    p = p.copy(points=np.array([[0.1, 0.1, 3.0]]))
    from sfmtory_gb300.problem import project

    p.obs_xy = project(np.array([abi.SIMPLE_PINHOLE]), np.array([[1500.0, 500, 400, 0, 0, 0, 0, 0]]),
                       p.points)
    cams = oracle_lib.refine_intrinsics(p)
    assert np.array_equal(cams, p.camera_params)


def test_improves_overall_reprojection_cost_end_to_end(oracle_lib):
    """intrinsics.rs:342-382: refinement cuts the camera cost 100x."""
    p = scenes.intrinsics_fixture(n_points=30)
    before = oracle_lib.total_cost(p)
    cams = oracle_lib.refine_intrinsics(p)
    after = oracle_lib.total_cost(p.copy(camera_params=cams))
    assert after < before * 0.01


def test_default_fixed_params_mask(oracle_lib):
    """intrinsics.rs:33-61: principal point is [1,2] for SP/SR/R, [2,3] otherwise."""
    m = oracle_lib.default_fixed_params_mask(list(range(6)))
    expect = {0: [1, 2], 1: [2, 3], 2: [1, 2], 3: [1, 2], 4: [2, 3], 5: [2, 3]}
    for model, idx in expect.items():
        row = np.zeros(8, bool)
        row[idx] = True
        assert np.array_equal(m[model], row)


def test_perturb_pose_left_multiplies(oracle_lib):
    """perturb_pose (lib.rs:263-269) agrees with the numpy restatement used
    by the scene generators, and zero delta leaves the pose bit-identical."""
    from sfmtory_gb300.problem import perturb_pose

    pose, _, _ = scenes.jacobian_test_fixture()
    d = np.array([0.01, -0.02, 0.03, 0.1, 0.2, -0.3])
    assert np.allclose(oracle_lib.perturb_pose(pose, d), perturb_pose(pose, d), atol=1e-15)
    assert np.array_equal(oracle_lib.perturb_pose(pose, np.zeros(6)), pose)


def test_projection_matches_numpy(oracle_lib):
    from sfmtory_gb300.problem import project

    rng = np.random.default_rng(1)
    for m, params in scenes.JACOBIAN_TEST_CAMERAS.items():
        for _ in range(5):
            pc = rng.normal(size=3) + np.array([0, 0, 3.0])
            p = np.zeros(8)
            p[: len(params)] = params
            a = oracle_lib.project(m, params, pc)
            b = project(np.array([m]), p[None], pc[None])[0]
            assert np.allclose(a, b, rtol=0, atol=1e-9)


def test_total_cost_and_mean_error_semantics(oracle_lib):
    """total_cost = sum w |r|^2 skipping z <= 1e-9 (lib.rs:727-745);
    mean error = mean |r| over valid observations (lib.rs:708-725)."""
    from sfmtory_gb300.problem import reprojection_residuals

    p = scenes.ring16(seed=3, scale=0.05)
    r, valid = reprojection_residuals(p)
    n = np.linalg.norm(r[valid], axis=1)
    assert np.isclose(oracle_lib.total_cost(p, robust_loss=abi.LOSS_NONE), np.sum(n**2), rtol=1e-12)
    w = np.where(n <= 2.0, 1.0, 2.0 / n)
    assert np.isclose(oracle_lib.total_cost(p), np.sum(w * n**2), rtol=1e-12)
    s = 1.5
    w = 1.0 / (1.0 + (n / s) ** 2)
    assert np.isclose(oracle_lib.total_cost(p, robust_loss=abi.LOSS_CAUCHY, loss_scale_px=s),
                      np.sum(w * n**2), rtol=1e-12)
    assert np.isclose(oracle_lib.mean_reprojection_error(p), n.mean(), rtol=1e-12)
    # A point pushed behind every camera drops out of both.
    q = p.copy()
    q.points[0] = np.array([50.0, 0.0, 0.0])
    r2, v2 = reprojection_residuals(q)
    assert v2.sum() < valid.sum()
    assert np.isclose(oracle_lib.mean_reprojection_error(q), np.linalg.norm(r2[v2], axis=1).mean())


def test_total_dim_zero_returns_initial_cost(oracle_lib):
    """lib.rs:777-787: every pose and camera fixed -> no iterations."""
    p = scenes.recovers_ground_truth_fixture().copy(fixed_poses=np.array([True, True]))
    out = oracle_lib.bundle_adjust(p)
    assert out.iterations_run == 0
    assert out.final_cost == out.initial_cost
    assert np.array_equal(out.points, p.points)


def test_ring16_converges(oracle_lib):
    p = scenes.ring16(seed=0, scale=0.1)
    out = oracle_lib.bundle_adjust(p, robust_loss=abi.LOSS_NONE, max_iterations=50)
    assert out.final_cost < 0.05 * out.initial_cost
    n_obs = p.num_observations
    # Noise sigma 0.5 px -> E|r|^2 ~ 2 * 0.25 per observation.
    assert out.final_cost / n_obs < 0.6


def test_oracle_filter_and_reoptimize_semantics(oracle_lib):
    """lib.rs:1722-1768: with a threshold no observation exceeds and every
    point in front, the filter keeps everything and the result is the plain
    adjustment; with 5 % outliers and a 3 px threshold it drops some and the
    last adjustment's observations all fit the previous output."""
    from sfmtory_gb300 import abi, scenes

    p = scenes.recovers_ground_truth_fixture()
    plain = oracle_lib.bundle_adjust(p, max_iterations=30)
    r, keep = oracle_lib.filter_and_reoptimize(p, 1e9, max_iterations=30)
    assert keep.all() and r.final_cost == plain.final_cost
    q = scenes.opencv47(seed=3, scale=0.05)
    kw = dict(robust_loss=abi.LOSS_HUBER, loss_scale_px=1.0, max_iterations=30)
    r, keep = oracle_lib.filter_and_reoptimize(q, 3.0, **kw)
    assert 0.8 * q.num_observations < keep.sum() < q.num_observations
    assert r.final_cost < oracle_lib.bundle_adjust(q, **kw).final_cost


def _with_outliers(p, frac=0.03, seed=7):
    rng = np.random.default_rng(seed)
    q = p.copy()
    idx = rng.choice(q.num_observations, int(frac * q.num_observations), replace=False)
    q.obs_xy[idx] = rng.uniform([0.0, 0.0], [1600.0, 1200.0], size=(len(idx), 2))
    return q


def test_oracle_adjust_global_semantics(oracle_lib):
    """crates/sfm-reconstruction/src/lib.rs:1567-1708 restated: FIXED holds
    every camera; FREE leaves a camera with < 5 images held; FREE_GUARDED
    filters, takes the free result when its plain mean error is lower, and
    rejects it when a distortion coefficient reaches 0.5 even though its
    error is lower."""
    kw = dict(robust_loss=abi.LOSS_HUBER, loss_scale_px=1.0, max_iterations=50)
    p = _with_outliers(scenes.shared_ring(0, 0.1))
    r, keep, chose, errs = oracle_lib.adjust_global(p, 0, 4.0, **kw)
    assert not chose and keep.all() and np.isnan(errs).all()
    assert np.array_equal(r.camera_params, p.camera_params)
    r, keep, chose, errs = oracle_lib.adjust_global(p, 2, 4.0, **kw)
    assert chose and errs[1] < errs[0]
    assert 0.95 * p.num_observations < keep.sum() < p.num_observations  # outliers filtered
    few = scenes.shared_ring(0, 0.1, images_per_camera=(12, 4))
    r, _, chose, _ = oracle_lib.adjust_global(few, 1, 4.0, **kw)
    assert chose and np.array_equal(r.camera_params[1], few.camera_params[1])
    assert not np.array_equal(r.camera_params[0], few.camera_params[0])
    # A user-fixed camera stays held too.
    held = few.copy(fixed_cameras=np.array([True, False]))
    r, _, _, _ = oracle_lib.adjust_global(held, 1, 4.0, **kw)
    assert np.array_equal(r.camera_params, few.camera_params)
    rad = scenes.shared_ring(0, 0.1, model=abi.SIMPLE_RADIAL, k=0.6)
    r, _, chose, errs = oracle_lib.adjust_global(rad, 2, 4.0, **kw)
    assert not chose and errs[1] < errs[0]
    assert np.array_equal(r.camera_params, rad.camera_params)


def test_oracle_pnp_recovers_known_pose(oracle_lib):
    """recovers_known_pose_from_synthetic_correspondences (crates/sfm-geometry/
    src/pnp.rs:311-339): threshold 0.01, 500 iterations; every point an
    inlier, rotation and translation errors below 1e-4."""
    from sfmtory_gb300.problem import quat_to_matrix

    pose, X, uv = scenes.pnp_known_pose_fixture()
    r = oracle_lib.pnp_ransac(X, uv, 0.01, 500)
    assert r is not None
    p, inl, _ = r
    assert inl.all()
    Rt, Re = quat_to_matrix(pose[:4]), quat_to_matrix(p[:4])
    assert np.arccos(np.clip((np.trace(Rt.T @ Re) - 1) / 2, -1, 1)) < 1e-4
    assert np.linalg.norm(p[4:] - pose[4:]) < 1e-4


def test_oracle_pnp_none_cases(oracle_lib):
    """pnp.rs:217-219 / ransac.rs:88: fewer than 6 correspondences or no
    iterations give None; coplanar points fail the conditioning test of
    every sample (pnp.rs:115-130), so no model is ever found."""
    pose, X, uv = scenes.pnp_known_pose_fixture()
    assert oracle_lib.pnp_ransac(X[:5], uv[:5], 0.01, 500) is None
    assert oracle_lib.pnp_ransac(X, uv, 0.01, 0) is None
    flat = X.copy()
    flat[:, 2] = 5.0
    assert oracle_lib.pnp_ransac(flat, uv, 0.01, 50) is None


def test_oracle_refine_pose_converges_on_exact_data(oracle_lib):
    """refine_pose_gauss_newton (pnp.rs:151-206) from a perturbed pose on
    noise-free correspondences returns to the true pose."""
    pose, X, uv = scenes.pnp_known_pose_fixture()
    init = pose.copy()
    init[4:] += [0.02, -0.01, 0.03]
    out = oracle_lib.refine_pose_gauss_newton(init[None], [X], [uv], 10)[0]
    assert np.abs(out[4:] - pose[4:]).max() < 1e-9
    assert min(np.abs(out[:4] - pose[:4]).max(), np.abs(out[:4] + pose[:4]).max()) < 1e-9
