"""GPU parity: the CUDA path through the C ABI against the CPU FP64 oracle.

Bars (written in each test): FP64 path - initial cost 1e-12 relative,
final cost / parameters 1e-6 relative, same iteration count; FP32 path -
residuals/Jacobians to FP32 accuracy, final cost 1e-6 relative.
"""
import numpy as np
import pytest

from sfmtory_gb300 import abi, native, scenes

pytestmark = pytest.mark.gpu

MODELS = list(scenes.JACOBIAN_TEST_CAMERAS)


def _single_obs_problem(model, params, pose, X, obs):
    from sfmtory_gb300.problem import Problem

    cp = np.zeros((1, 8))
    cp[0, : len(params)] = params
    return Problem(
        camera_of_image=np.array([0], np.int32), camera_model=np.array([model], np.int32), camera_params=cp,
        poses=np.asarray(pose)[None], points=np.asarray(X)[None], obs_image=np.array([0], np.int32),
        obs_point=np.array([0], np.int32), obs_xy=np.array([obs], np.float64))


@pytest.mark.parametrize("model", MODELS, ids=[abi.MODEL_NAMES[m] for m in MODELS])
def test_jacobians_match_oracle_and_fd(oracle_lib, model):
    """Device adjoint Jacobians on the reference fixture (lib.rs:1252-1295):
    FP64 equals the oracle's analytic Jacobian to 1e-9 relative and meets the
    reference's FD tolerances; FP32 is within 1e-4 relative of it."""
    pose, X, obs = scenes.jacobian_test_fixture()
    params = scenes.JACOBIAN_TEST_CAMERAS[model]
    p = _single_obs_problem(model, params, pose, X, obs)
    an = oracle_lib.analytic_jacobians(pose, model, params, X, obs)
    num = oracle_lib.numerical_jacobians(pose, model, params, X, obs)
    r, jp, jx, jc, valid = native.residuals_jacobians(p, fp32=False)
    assert valid[0]
    scale = max(1.0, np.abs(an[1]).max(), np.abs(an[3]).max())
    assert np.abs(r[0] - an[0]).max() < 1e-9
    assert np.abs(jp[0] - an[1]).max() < 1e-9 * scale
    assert np.abs(jx[0] - an[2]).max() < 1e-9 * scale
    assert np.abs(jc[0] - an[3]).max() < 1e-9 * scale
    assert np.linalg.norm(jp[0] - num[1]) < 1e-5
    assert np.linalg.norm(jx[0] - num[2]) < 1e-5
    assert np.linalg.norm(jc[0] - num[3]) < 1e-4
    r32, jp32, jx32, jc32, v32 = native.residuals_jacobians(p, fp32=True)
    assert v32[0]
    for a, b in ((jp32[0], an[1]), (jx32[0], an[2]), (jc32[0], an[3])):
        assert np.abs(a - b).max() <= 1e-4 * max(1.0, np.abs(b).max())
    # pixel residual: FP32 rounding of ~1e3 px coordinates
    assert np.abs(r32[0] - an[0]).max() < 2e-3


def test_jacobians_random_observations(oracle_lib):
    """Many random poses/points per model, FP64 device vs oracle (1e-9 rel)."""
    rng = np.random.default_rng(7)
    from sfmtory_gb300.problem import Problem, quat_from_scaled_axis

    for model, params in scenes.JACOBIAN_TEST_CAMERAS.items():
        n = 64
        cp = np.zeros((n, 8))
        cp[:, : len(params)] = params
        q = quat_from_scaled_axis(rng.normal(0, 0.3, (n, 3)))
        poses = np.concatenate([q, rng.normal(0, 0.5, (n, 3))], 1)
        pts = rng.normal(0, 0.5, (n, 3)) + np.array([0, 0, 4.0])
        obs = rng.uniform(0, 600, (n, 2))
        p = Problem(camera_of_image=np.arange(n, dtype=np.int32), camera_model=np.full(n, model, np.int32),
                    camera_params=cp, poses=poses, points=pts, obs_image=np.arange(n, dtype=np.int32),
                    obs_point=np.arange(n, dtype=np.int32), obs_xy=obs)
        r, jp, jx, jc, valid = native.residuals_jacobians(p)
        for k in range(n):
            an = oracle_lib.analytic_jacobians(poses[k], model, params, pts[k], obs[k])
            assert (an is not None) == bool(valid[k])
            if an is None:
                continue
            s = max(1.0, np.abs(an[1]).max(), np.abs(an[3]).max())
            assert np.abs(r[k] - an[0]).max() < 1e-8
            assert np.abs(jp[k] - an[1]).max() < 1e-9 * s
            assert np.abs(jx[k] - an[2]).max() < 1e-9 * s
            assert np.abs(jc[k] - an[3]).max() < 1e-9 * s


@pytest.mark.parametrize("loss", [abi.LOSS_NONE, abi.LOSS_HUBER, abi.LOSS_CAUCHY])
def test_total_cost_and_mean_error(oracle_lib, loss):
    p = scenes.opencv47(seed=1, scale=0.1)
    a = native.total_cost(p, robust_loss=loss, loss_scale_px=1.0)
    b = oracle_lib.total_cost(p, robust_loss=loss, loss_scale_px=1.0)
    assert abs(a - b) <= 1e-12 * abs(b)
    assert abs(native.mean_reprojection_error_arrays(p) - oracle_lib.mean_reprojection_error(p)) < 1e-12


def _compare(gpu, ref, *, cost_rtol=1e-6, param_rtol=1e-6, same_iters=True):
    assert abs(gpu.initial_cost - ref.initial_cost) <= 1e-12 * abs(ref.initial_cost) + 1e-300
    assert abs(gpu.final_cost - ref.final_cost) <= cost_rtol * abs(ref.final_cost) + 1e-12
    if same_iters:
        assert gpu.iterations_run == ref.iterations_run
    for a, b in ((gpu.points, ref.points), (gpu.poses, ref.poses), (gpu.camera_params, ref.camera_params)):
        err = np.abs(a - b) / np.maximum(np.abs(b), 1.0)
        assert err.max() <= param_rtol, err.max()


def test_fp64_recovers_ground_truth_matches_oracle(oracle_lib):
    p = scenes.recovers_ground_truth_fixture()
    g = native.bundle_adjust_arrays(p, max_iterations=30)
    r = oracle_lib.bundle_adjust(p, max_iterations=30)
    # noiseless problem: final cost ~1e-25, compare the absolute level
    assert g.final_cost < 1e-12 and r.final_cost < 1e-12
    assert g.final_cost < 0.01 * g.initial_cost
    assert abs(g.initial_cost - r.initial_cost) < 1e-10 * r.initial_cost
    assert np.allclose(g.poses, r.poses, atol=1e-8)
    assert np.allclose(g.points, r.points, atol=1e-8)


def test_fp64_shared_focal_joint_matches_oracle(oracle_lib):
    """A camera shared by four images (slot fold with several pre-images)."""
    p = scenes.shared_focal_fixture()
    pre_g = native.bundle_adjust_arrays(p, max_iterations=50)
    pre_r = oracle_lib.bundle_adjust(p, max_iterations=50)
    assert np.allclose(pre_g.points, pre_r.points, atol=1e-7)
    joint = p.copy(poses=pre_r.poses, points=pre_r.points, fixed_cameras=np.array([False]))
    g = native.bundle_adjust_arrays(joint, max_iterations=50)
    r = oracle_lib.bundle_adjust(joint, max_iterations=50)
    assert abs(g.camera_params[0, 0] - 1500.0) / 1500.0 < 0.02
    assert abs(g.camera_params[0, 0] - r.camera_params[0, 0]) < 1e-6 * 1500


@pytest.mark.parametrize("scale", [0.05, 0.25])
def test_fp64_ring16_matches_oracle(oracle_lib, scale):
    p = scenes.ring16(seed=2, scale=scale)
    kw = dict(robust_loss=abi.LOSS_NONE, max_iterations=50)
    g = native.bundle_adjust_arrays(p, **kw)
    r = oracle_lib.bundle_adjust(p, **kw)
    _compare(g, r)


def test_fp64_opencv47_huber_matches_oracle(oracle_lib):
    p = scenes.opencv47(seed=3, scale=0.05)
    kw = dict(robust_loss=abi.LOSS_HUBER, loss_scale_px=1.0, max_iterations=30)
    g = native.bundle_adjust_arrays(p, **kw)
    r = oracle_lib.bundle_adjust(p, **kw)
    _compare(g, r)


def test_mixed_ring16_reaches_oracle_cost(oracle_lib):
    """FP32 linearisation + Schur, FP64 cost and Cholesky: final cost within
    1e-6 relative and RMS within 1e-4 px of the FP64 oracle."""
    from sfmtory_gb300.problem import rms_reprojection_error

    p = scenes.ring16(seed=4, scale=0.25)
    kw = dict(robust_loss=abi.LOSS_NONE, max_iterations=50)
    g = native.bundle_adjust_arrays(p, precision=abi.PRECISION_MIXED, **kw)
    r = oracle_lib.bundle_adjust(p, **kw)
    assert abs(g.final_cost - r.final_cost) <= 1e-6 * r.final_cost
    rg = rms_reprojection_error(p.copy(poses=g.poses, points=g.points, camera_params=g.camera_params))
    rr = rms_reprojection_error(p.copy(poses=r.poses, points=r.points, camera_params=r.camera_params))
    assert abs(rg - rr) < 1e-4


def test_total_dim_zero(oracle_lib):
    p = scenes.recovers_ground_truth_fixture().copy(fixed_poses=np.array([True, True]))
    g = native.bundle_adjust_arrays(p)
    assert g.iterations_run == 0
    assert g.final_cost == g.initial_cost
    assert np.array_equal(g.points, p.points)


def test_no_valid_observations_stops(oracle_lib):
    """Every point behind its camera: total_cost 0, loop exits at once (lib.rs:855-857)."""
    p = scenes.recovers_ground_truth_fixture()
    p = p.copy(points=p.points * np.array([1, 1, -1.0]))
    g = native.bundle_adjust_arrays(p)
    r = oracle_lib.bundle_adjust(p)
    assert g.initial_cost == 0.0 and r.initial_cost == 0.0
    assert g.iterations_run == r.iterations_run == 1
    assert np.array_equal(g.points, p.points)


def test_empty_problem():
    from sfmtory_gb300.problem import Problem

    p = Problem(camera_of_image=np.zeros(0, np.int32), camera_model=np.zeros(0, np.int32),
                camera_params=np.zeros((0, 8)), poses=np.zeros((0, 7)), points=np.zeros((0, 3)),
                obs_image=np.zeros(0, np.int32), obs_point=np.zeros(0, np.int32), obs_xy=np.zeros((0, 2)))
    g = native.bundle_adjust_arrays(p)
    assert g.iterations_run == 0 and g.final_cost == 0.0


def test_shuffled_observation_order_same_result(oracle_lib):
    """The device sorts observations by point; input order must not matter."""
    p = scenes.ring16(seed=5, scale=0.05)
    rng = np.random.default_rng(0)
    perm = rng.permutation(p.num_observations)
    q = p.copy(obs_image=p.obs_image[perm], obs_point=p.obs_point[perm], obs_xy=p.obs_xy[perm])
    kw = dict(robust_loss=abi.LOSS_NONE, max_iterations=20)
    a = native.bundle_adjust_arrays(p, **kw)
    b = native.bundle_adjust_arrays(q, **kw)
    assert abs(a.final_cost - b.final_cost) <= 1e-9 * a.final_cost
    assert np.allclose(a.points, b.points, rtol=0, atol=1e-9)


def test_pcg_fp64_matches_oracle(oracle_lib):
    """Matrix-free PCG solved tightly follows the dense reference trajectory."""
    p = scenes.ring16(seed=6, scale=0.1)
    kw = dict(robust_loss=abi.LOSS_NONE, max_iterations=50)
    g = native.bundle_adjust_arrays(p, solver=abi.SOLVER_PCG, pcg_tolerance=1e-12, pcg_max_iterations=1000, **kw)
    r = oracle_lib.bundle_adjust(p, **kw)
    assert g.solver_used == abi.SOLVER_PCG and g.linear_iterations > 0
    assert abs(g.final_cost - r.final_cost) <= 1e-6 * r.final_cost
    assert abs(g.initial_cost - r.initial_cost) <= 1e-12 * r.initial_cost


def test_pcg_mixed_radial_reaches_oracle_cost(oracle_lib):
    """FP32 PCG on a scaled-down power-law RADIAL scene reaches the FP64
    oracle's final cost to 1e-6 relative."""
    p = scenes.radial2000(seed=1, scale=0.002)
    kw = dict(robust_loss=abi.LOSS_NONE, max_iterations=50)
    r = oracle_lib.bundle_adjust(p, **kw)
    g = native.bundle_adjust_arrays(p, solver=abi.SOLVER_PCG, precision=abi.PRECISION_MIXED,
                                    pcg_tolerance=1e-6, pcg_max_iterations=200, **kw)
    assert g.final_cost <= r.final_cost * (1 + 1e-6)
    g64 = native.bundle_adjust_arrays(p, solver=abi.SOLVER_PCG, pcg_tolerance=1e-8, pcg_max_iterations=400, **kw)
    assert abs(g64.final_cost - r.final_cost) <= 1e-6 * r.final_cost


def test_pcg_shared_free_camera_matches_oracle(oracle_lib):
    """The reference's joint-focal test scene (one camera shared by four
    images, lib.rs:1487-1592) on the PCG solver: the shared camera is one
    unknown block, as in the reference's slotting (lib.rs:753-787)."""
    p = scenes.shared_focal_fixture()
    pre = oracle_lib.bundle_adjust(p, max_iterations=50)
    joint = p.copy(poses=pre.poses, points=pre.points, fixed_cameras=np.array([False]))
    r = oracle_lib.bundle_adjust(joint, max_iterations=50)
    g = native.bundle_adjust_arrays(joint, max_iterations=50, solver=abi.SOLVER_PCG, pcg_tolerance=1e-12,
                                    pcg_max_iterations=500)
    assert g.solver_used == abi.SOLVER_PCG
    assert abs(g.camera_params[0, 0] - 1500.0) / 1500.0 < 0.02
    assert abs(g.camera_params[0, 0] - r.camera_params[0, 0]) < 1e-6 * 1500
    assert abs(g.final_cost - r.final_cost) <= 1e-6 * r.final_cost + 1e-12


def test_profile_report_counts_phases():
    p = scenes.ring16(seed=7, scale=0.05)
    native.profile_enable(True)
    native.bundle_adjust_arrays(p, robust_loss=abi.LOSS_NONE, max_iterations=3)
    rep = native.profile_report()
    native.profile_enable(False)
    assert rep["linearize"]["launches"] >= 1 and rep["cholesky"]["ms"] > 0
    assert rep["kernel_launches"] > 10


@pytest.mark.parametrize("models", [(m,) for m in range(6)] + [(abi.PINHOLE, abi.SIMPLE_RADIAL, abi.OPENCV)],
                         ids=[abi.MODEL_NAMES[m] for m in range(6)] + ["mixed"])
def test_pcg_mixed_each_camera_model_reaches_oracle_cost(oracle_lib, models):
    """The FP32 PCG passes are compiled with the camera model as a constant
    when every camera shares it (one case per model) and keep the runtime
    switch otherwise (mixed); each reaches the FP64 oracle's final cost to
    1e-6 relative with the FP64 polish and to 1e-5 alone."""
    p = scenes.local_window(np.random.default_rng(11), 24, 1500, models=models)
    kw = dict(robust_loss=abi.LOSS_HUBER, loss_scale_px=2.0, max_iterations=40)
    r = oracle_lib.bundle_adjust(p, **kw)
    for polish, bar in ((1, 1e-6), (0, 1e-5)):
        g = native.bundle_adjust_arrays(p, solver=abi.SOLVER_PCG, precision=abi.PRECISION_MIXED, fp64_polish=polish,
                                        pcg_tolerance=1e-6, pcg_max_iterations=300, **kw)
        assert g.solver_used == abi.SOLVER_PCG
        assert g.final_cost <= r.final_cost * (1 + bar), (polish, g.final_cost, r.final_cost)


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_MIXED])
def test_pcg_coarse_correction_cuts_iterations(precision):
    """The coarse correction of the PCG preconditioner (clusters of
    consecutive images, A_c = Z^T S Z) changes only the Krylov iteration:
    solved tightly, both preconditioners follow the dense FP64 solve's LM
    trajectory (itself held to the oracle by the tests above; same cost to
    1e-6), and the two-level one needs fewer iterations on a long camera
    sequence (283 cameras)."""
    p = scenes.radial2000(seed=2, scale=0.02)
    kw = dict(robust_loss=abi.LOSS_NONE, max_iterations=6)
    ref = native.bundle_adjust_arrays(p, solver=abi.SOLVER_DENSE, dense_max_dim=10000, **kw)
    pk = dict(kw, solver=abi.SOLVER_PCG, precision=precision, pcg_tolerance=1e-6, pcg_max_iterations=3000)
    bj = native.bundle_adjust_arrays(p, pcg_coarse_clusters=-1, **pk)
    co = native.bundle_adjust_arrays(p, pcg_coarse_clusters=32, **pk)
    assert ref.solver_used == abi.SOLVER_DENSE
    for g in (bj, co):
        assert abs(g.final_cost - ref.final_cost) <= 1e-6 * ref.final_cost, (g.final_cost, ref.final_cost)
    assert co.linear_iterations < bj.linear_iterations, (co.linear_iterations, bj.linear_iterations)


@pytest.mark.parametrize("models", [(m,) for m in range(6)] + [(abi.PINHOLE, abi.SIMPLE_RADIAL, abi.OPENCV)],
                         ids=[abi.MODEL_NAMES[m] for m in range(6)] + ["mixed"])
@pytest.mark.parametrize("loss", [abi.LOSS_NONE, abi.LOSS_HUBER])
def test_mixed_cost_double_float_matches_fp64(oracle_lib, models, loss):
    """The FP32 path evaluates the cost with the projection in double-float
    arithmetic (FP32 pairs; OPENCV_FISHEYE cameras keep FP64): its initial
    cost is the FP64 oracle's to 1e-10 relative, and the final cost it
    reports is the FP64 cost of the parameters it returns to 1e-10."""
    p = scenes.local_window(np.random.default_rng(12), 24, 1500, models=models)
    kw = dict(robust_loss=loss, loss_scale_px=2.0)
    ref0 = oracle_lib.total_cost(p, **kw)
    g = native.bundle_adjust_arrays(p, solver=abi.SOLVER_PCG, precision=abi.PRECISION_MIXED, max_iterations=4, **kw)
    assert abs(g.initial_cost - ref0) <= 1e-10 * ref0, (g.initial_cost, ref0)
    out = p.copy(poses=g.poses, points=g.points, camera_params=g.camera_params)
    ref1 = oracle_lib.total_cost(out, **kw)
    assert abs(g.final_cost - ref1) <= 1e-10 * ref1, (g.final_cost, ref1)


def test_auto_solver_switch_over_point_matches_oracle(oracle_lib):
    """SOLVER_AUTO picks the dense reduced-camera solve up to dense_max_dim
    unknowns and the matrix-free PCG above it. At the switch-over point (the
    problem's own reduced dimension n: dense at dense_max_dim = n, PCG at
    n - 1) both FP64 solves follow the oracle's LM iterations: the same
    iteration count and final cost to 1e-6 (PCG solved tightly, so it is an
    exact linear solve up to its tolerance)."""
    p = scenes.ring16(seed=9, scale=0.25)
    n = p.reduced_dim()
    kw = dict(robust_loss=abi.LOSS_NONE, max_iterations=20)
    r = oracle_lib.bundle_adjust(p, **kw)
    dense = native.bundle_adjust_arrays(p, solver=abi.SOLVER_AUTO, dense_max_dim=n, **kw)
    pcg = native.bundle_adjust_arrays(p, solver=abi.SOLVER_AUTO, dense_max_dim=n - 1, pcg_tolerance=1e-10,
                                      pcg_max_iterations=2000, **kw)
    assert dense.solver_used == abi.SOLVER_DENSE and pcg.solver_used == abi.SOLVER_PCG
    for g in (dense, pcg):
        assert g.iterations_run == r.iterations_run, (g.solver_used, g.iterations_run, r.iterations_run)
        assert abs(g.final_cost - r.final_cost) <= 1e-6 * r.final_cost, (g.solver_used, g.final_cost, r.final_cost)
