"""The benchmark configurations at their stated sizes, against the FP64 oracle
(through the C ABI).

* ring16 full size (16 PINHOLE cameras, 2000 points, squared loss, 50
  iterations; reduced dimension 154).
* opencv47 full size (47 OPENCV cameras, 20k points, ~120k observations, 5 %
  outliers, Huber at 1 px): FP32 and FP64 residuals and Jacobians of every
  observation against the oracle's analytic Jacobians and central
  differences with a relative step of 1e-6, and the solve.
* radial500 full size (500 SIMPLE_RADIAL cameras, 200k points, ~1.2M
  observations, reduced dimension 4994): against the oracle solve stored in
  tests/golden/radial500_full.npz (made by make_config_golden.py).

Bars: the plain FP64 path follows the oracle's trajectory - initial cost
1e-12 relative, the same iteration count, final cost and every parameter
1e-6 relative. The FP32+adjoint (mixed) path: final cost 1e-6 relative and
RMS reprojection error 1e-4 px against the oracle. Its parameters are
stated raw and with the free scale removed (parity_report.errors) and held
beside the oracle's own last iteration: the reference stops when an
iteration lowers the cost by less than 1e-6 relative (lib.rs:814,
:1218-1221), and in that last iteration its own parameters still move by
~1e-3 (ring16: 2.1e-3 raw) along the problem's flat directions, so two
correct solves that stop at different iterates differ there by far more
than 1e-6. The mixed path's parameter error must be within that movement
(the stopping rule's own resolution; measured: 0.13-0.18 % of it on ring16
and opencv47, 13 % on radial500, where the mixed path's last step lands
1.1e-8 below the oracle's cost).

opencv47 (Huber at 1 px, 5 % outliers): the reference's own trajectory is
not reproducible past ~30 iterations - the oracle run with 8 and with 1
thread (only the summation order of its parallel sums differs) agrees to
1e-11 after 30 iterations and differs by up to 2.5 in a point coordinate
after 50, where one run stops after 36 iterations (no damped step
accepted) and the other runs all 50, 4.4e-4 apart in cost (iteratively
reweighted Huber steps amplify rounding once observations sit at the loss
threshold). The trajectory bars are therefore applied at 30 iterations; the
50-iteration solve is held to the oracle's cost to 1e-3 and its errors are
stated beside the oracle's own spread.
"""
import os
import sys

import numpy as np
import pytest

import parity_report as R
from sfmtory_gb300 import abi, native, scenes
from sfmtory_gb300.problem import parameter_errors, rms_of

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b)) / np.maximum(np.abs(np.asarray(b)), 1.0)))


def _fp64_follows(g, ref_initial, ref_final, ref_iters, ref_poses, ref_points, ref_cams, points=None):
    assert abs(g.initial_cost - ref_initial) <= 1e-12 * abs(ref_initial)
    assert g.iterations_run == ref_iters, (g.iterations_run, ref_iters)
    assert abs(g.final_cost - ref_final) <= 1e-6 * abs(ref_final), (g.final_cost, ref_final)
    pts = g.points if points is None else g.points[points]
    assert _rel(g.poses, ref_poses) <= 1e-6
    assert _rel(pts, ref_points) <= 1e-6
    assert _rel(g.camera_params, ref_cams) <= 1e-6


def _last_step(oracle_lib, p, r, kw):
    """Raw parameter movement of the oracle's last iteration."""
    prev = oracle_lib.bundle_adjust(p, **dict(kw, max_iterations=r.iterations_run - 1))
    return parameter_errors(prev.poses, prev.points, prev.camera_params, r.poses, r.points, r.camera_params)


def _mixed_bars(e, last_raw):
    e["oracle_last_step_raw"] = last_raw
    e["param_raw_over_last_step"] = e["param_raw_max"] / last_raw if last_raw > 0 else None
    assert e["meets"]["cost"], e
    assert e["meets"]["rms"], e
    assert e["param_raw_max"] <= last_raw, e


# ---------------------------------------------------------------- ring16 (C0)

RING16 = dict(robust_loss=abi.LOSS_NONE, max_iterations=50)


@pytest.fixture(scope="module")
def ring16_full(oracle_lib):
    p = scenes.ring16(seed=0, scale=1.0)
    r = oracle_lib.bundle_adjust(p, **RING16)
    return p, r, _last_step(oracle_lib, p, r, RING16)


def test_ring16_full_fp64_follows_oracle(ring16_full):
    p, r, _ = ring16_full
    assert p.reduced_dim() == 154
    g = native.bundle_adjust_arrays(p, **RING16)
    _fp64_follows(g, r.initial_cost, r.final_cost, r.iterations_run, r.poses, r.points, r.camera_params)
    R.record("ring16_full_fp64", R.errors(p, g, r.poses, r.points, r.camera_params, r.final_cost,
                                          rms_of(p, r.poses, r.points, r.camera_params)))


@pytest.mark.parametrize("solver", [abi.SOLVER_DENSE, abi.SOLVER_PCG], ids=["dense", "pcg"])
def test_ring16_full_mixed_errors(ring16_full, solver):
    p, r, last = ring16_full
    kw = dict(RING16, precision=abi.PRECISION_MIXED, solver=solver)
    if solver == abi.SOLVER_PCG:
        kw.update(pcg_tolerance=1e-6, pcg_max_iterations=500)
    g = native.bundle_adjust_arrays(p, **kw)
    e = R.errors(p, g, r.poses, r.points, r.camera_params, r.final_cost, rms_of(p, r.poses, r.points, r.camera_params))
    try:
        _mixed_bars(e, last["raw_max"])
    finally:
        R.record(f"ring16_full_mixed_{'dense' if solver == abi.SOLVER_DENSE else 'pcg'}", e)


# -------------------------------------------------------------- opencv47 (C1)

OPENCV47 = dict(robust_loss=abi.LOSS_HUBER, loss_scale_px=1.0)


@pytest.fixture(scope="module")
def opencv47_full():
    p = scenes.opencv47(seed=0, scale=1.0)
    assert p.num_observations > 100_000
    return p


def _jac_err(a, b):
    """Per observation: max |a - b| over the entries of a Jacobian block."""
    return np.max(np.abs(a - b).reshape(len(a), -1), axis=1)


def test_opencv47_full_jacobians(oracle_lib, opencv47_full):
    """Every observation of the 120k-observation scene: the FP64 kernels equal
    the oracle's analytic Jacobians to 1e-9 (relative to the observation's
    largest entry) and the FP32 kernels to 1e-4; both agree with central
    differences of step 1e-6 x max(1, |parameter|) to the same FP32 bar,
    and the FP64 ones to the reference's own FD tolerances (1e-5 pose and
    point, 1e-4 camera)."""
    p = opencv47_full
    an = oracle_lib.jacobians_batch(p)
    fd = oracle_lib.jacobians_batch(p, numerical=True, h_rel=1e-6)
    g64 = native.residuals_jacobians(p, fp32=False)
    g32 = native.residuals_jacobians(p, fp32=True)
    assert np.array_equal(an[4], g64[4]) and np.array_equal(an[4], g32[4]) and np.array_equal(an[4], fd[4])
    v = an[4]
    assert v.mean() > 0.99
    scale = np.maximum(1.0, np.maximum.reduce([np.abs(an[k][v]).reshape(v.sum(), -1).max(1) for k in (1, 2, 3)]))
    stats = {}
    for name, g, bar in (("fp64_vs_analytic", g64, 1e-9), ("fp32_vs_analytic", g32, 1e-4),
                         ("fp32_vs_fd", g32, 1e-4), ("fp64_vs_fd", g64, 1e-4)):
        ref = fd if name.endswith("fd") else an
        worst = 0.0
        for k in (1, 2, 3):
            worst = max(worst, float(np.max(_jac_err(g[k][v], ref[k][v]) / scale)))
        stats[name] = worst
        assert worst <= bar, (name, worst)
    stats["fp32_residual_px"] = float(np.max(np.abs(g32[0][v] - an[0][v])))
    stats["fp64_residual_px"] = float(np.max(np.abs(g64[0][v] - an[0][v])))
    assert stats["fp64_residual_px"] < 1e-9
    assert stats["fp32_residual_px"] < 2e-3  # FP32 rounding of ~1e3 px coordinates
    # the reference's own FD bars (lib.rs:1266-1294), Frobenius norms of the blocks
    fro = lambda a, b: np.sqrt(np.sum((a - b) ** 2, axis=(1, 2)))  # noqa: E731
    stats["fp64_fd_frobenius_rel"] = {
        "pose": float((fro(g64[1][v], fd[1][v]) / scale).max()),
        "point": float((fro(g64[2][v], fd[2][v]) / scale).max()),
        "camera": float((fro(g64[3][v], fd[3][v]) / scale).max()),
    }
    assert np.all(fro(g64[1][v], fd[1][v]) / scale < 1e-5)
    assert np.all(fro(g64[2][v], fd[2][v]) / scale < 1e-5)
    assert np.all(fro(g64[3][v], fd[3][v]) / scale < 1e-4)
    R.record("opencv47_full_jacobians", {"observations": int(v.size), "valid": int(v.sum()), **stats})


@pytest.fixture(scope="module")
def opencv47_oracle30(oracle_lib, opencv47_full):
    kw = dict(OPENCV47, max_iterations=30)
    r = oracle_lib.bundle_adjust(opencv47_full, **kw)
    return r, _last_step(oracle_lib, opencv47_full, r, kw)


def test_opencv47_full_fp64_follows_oracle_30_iterations(opencv47_full, opencv47_oracle30):
    p, (r, _) = opencv47_full, opencv47_oracle30
    g = native.bundle_adjust_arrays(p, max_iterations=30, **OPENCV47)
    R.record("opencv47_full_fp64_30it", R.errors(p, g, r.poses, r.points, r.camera_params, r.final_cost,
                                                 rms_of(p, r.poses, r.points, r.camera_params)))
    _fp64_follows(g, r.initial_cost, r.final_cost, r.iterations_run, r.poses, r.points, r.camera_params)


def test_opencv47_full_mixed_errors_30_iterations(opencv47_full, opencv47_oracle30):
    p, (r, last) = opencv47_full, opencv47_oracle30
    g = native.bundle_adjust_arrays(p, precision=abi.PRECISION_MIXED, max_iterations=30, **OPENCV47)
    e = R.errors(p, g, r.poses, r.points, r.camera_params, r.final_cost, rms_of(p, r.poses, r.points, r.camera_params))
    try:
        _mixed_bars(e, last["raw_max"])
    finally:
        R.record("opencv47_full_mixed_30it", e)


def test_opencv47_full_50_iterations_within_oracle_spread(oracle_lib, opencv47_full):
    """The stated 50-iteration solve: the oracle with 8 and with 1 thread
    gives its own spread; the GPU's FP64 and mixed results are held to its
    cost to 1e-3 relative and their errors stated beside that spread."""
    p = opencv47_full
    kw = dict(OPENCV47, max_iterations=50)
    oracle_lib.set_threads(8)
    r8 = oracle_lib.bundle_adjust(p, **kw)
    oracle_lib.set_threads(1)
    r1 = oracle_lib.bundle_adjust(p, **kw)
    oracle_lib.set_threads(0)
    spread = parameter_errors(r1.poses, r1.points, r1.camera_params, r8.poses, r8.points, r8.camera_params)
    out = {"oracle_threads_spread": {"cost_rel": (r1.final_cost - r8.final_cost) / r8.final_cost,
                                     "param_raw_max": spread["raw_max"], "iterations": [r8.iterations_run,
                                                                                        r1.iterations_run]}}
    rms8 = rms_of(p, r8.poses, r8.points, r8.camera_params)
    for name, prec in (("fp64", abi.PRECISION_FP64), ("mixed", abi.PRECISION_MIXED)):
        g = native.bundle_adjust_arrays(p, precision=prec, **kw)
        e = R.errors(p, g, r8.poses, r8.points, r8.camera_params, r8.final_cost, rms8)
        e["iterations"] = g.iterations_run
        out[name] = e
        assert g.final_cost < 0.6 * g.initial_cost
        assert e["cost_rel"] <= 1e-3, (name, e)
    R.record("opencv47_full_50it", out)


# ------------------------------------------------------------- radial500 (C2)

@pytest.fixture(scope="module")
def radial500_golden():
    if GOLDEN not in sys.path:
        sys.path.insert(0, GOLDEN)
    import make_config_golden as M

    z = np.load(os.path.join(GOLDEN, "radial500_full.npz"))
    p = scenes.radial500(seed=int(z["seed"]), scale=float(z["scale"]))
    got = M.input_checksums(p)
    # the scene generator must rebuild the stored scene (same seeded streams)
    assert np.allclose(got, z["input_checksums"], rtol=1e-12, atol=0), (got, z["input_checksums"])
    return p, z


def _radial500_kw(z):
    o = z["options"]
    return dict(max_iterations=int(o[0]), robust_loss=int(o[1]), solver=abi.SOLVER_DENSE)


def test_radial500_full_fp64_follows_oracle(radial500_golden):
    p, z = radial500_golden
    assert p.reduced_dim() == int(z["reduced_dim"]) == 4994
    g = native.bundle_adjust_arrays(p, **_radial500_kw(z))
    idx = z["point_index"]
    R.record("radial500_full_fp64", R.errors(p, g, z["out_poses"], z["out_points"], z["out_camera_params"],
                                             float(z["final_cost"]), float(z["rms_px"]), point_index=idx))
    _fp64_follows(g, float(z["initial_cost"]), float(z["final_cost"]), int(z["iterations_run"]), z["out_poses"],
                  z["out_points"], z["out_camera_params"], points=idx)
    assert np.allclose(np.sum(g.points, axis=0), z["points_sum"], rtol=1e-7)
    assert np.allclose(np.sum(g.points ** 2, axis=0), z["points_sumsq"], rtol=1e-7)


def test_radial500_full_mixed_errors(radial500_golden):
    p, z = radial500_golden
    g = native.bundle_adjust_arrays(p, precision=abi.PRECISION_MIXED, **_radial500_kw(z))
    e = R.errors(p, g, z["out_poses"], z["out_points"], z["out_camera_params"], float(z["final_cost"]),
                 float(z["rms_px"]), point_index=z["point_index"])
    try:
        _mixed_bars(e, float(z["last_step_raw"]))
    finally:
        R.record("radial500_full_mixed", e)
