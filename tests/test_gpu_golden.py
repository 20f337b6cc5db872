"""GPU path against the committed golden fixtures (through the C ABI).

Bars: FP64 dense - initial cost 1e-12, final cost and parameters 1e-6
relative, same iteration count; FP32 (mixed) - final cost 1e-6 relative;
FP64 PCG with a tight tolerance - final cost 1e-6 relative; Jacobians FP64
1e-9 relative.
"""
import numpy as np
import pytest

import golden_util as G
from sfmtory_gb300 import abi, native, scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", G.CASES)
def test_fp64_dense_matches_golden(name):
    p, kw, exp = G.load(name)
    r = native.bundle_adjust_arrays(p, solver=abi.SOLVER_DENSE, **kw)
    assert abs(r.initial_cost - exp["initial_cost"]) <= 1e-12 * abs(exp["initial_cost"])
    assert r.iterations_run == exp["iterations_run"]
    if exp["final_cost"] > 1e-12:
        assert abs(r.final_cost - exp["final_cost"]) <= 1e-6 * exp["final_cost"]
        assert G.rel_err(r.points, exp["points"]) < 1e-6
        assert G.rel_err(r.poses, exp["poses"]) < 1e-6
        assert G.rel_err(r.camera_params, exp["camera_params"]) < 1e-6
    else:  # noiseless fixture: compare the converged geometry
        assert r.final_cost < 1e-12
        assert np.allclose(r.points, exp["points"], atol=1e-8)


# The reference's Huber cost sum w |r|^2 (w = s/|r| outside the scale) has a
# derivative kink at |r| = s, and its IRLS step is not the gradient of that
# cost for outliers, so LM can stall at points the FP64 path also cannot
# leave. On this fixture the mixed trajectory reaches such a point 1.2e-6
# above the oracle's minimum; the bar there is 2e-6 plus the stall check.
HUBER_STALL = {"shared_focal_fixed": 2e-6}


@pytest.mark.parametrize("name", [n for n in G.CASES if n != "recovers_ground_truth"])
@pytest.mark.parametrize("polish", [0, 1])
def test_mixed_reaches_golden_cost(name, polish):
    """The mixed path (FP32 linearisation and Schur with FP64 residuals, FP64
    cost, Cholesky and refinement; optionally the FP64 polish) reaches the
    FP64 oracle's final cost to 1e-6 relative."""
    p, kw, exp = G.load(name)
    r = native.bundle_adjust_arrays(p, precision=abi.PRECISION_MIXED, solver=abi.SOLVER_DENSE,
                                    fp64_polish=polish, **kw)
    bar = HUBER_STALL.get(name, 1e-6)
    assert r.final_cost <= exp["final_cost"] * (1 + bar), (r.final_cost, exp["final_cost"], r.polish_iteration)
    if name in HUBER_STALL:
        # the FP64 path started from the mixed result cannot lower it by 1e-6
        q = p.copy(poses=r.poses, points=r.points, camera_params=r.camera_params)
        s = native.bundle_adjust_arrays(q, solver=abi.SOLVER_DENSE, **kw)
        assert s.final_cost >= r.final_cost * (1 - 1e-6)


@pytest.mark.parametrize("name", ["ring16_s005", "radial2000_s0005", "window_mixed_models"])
def test_pcg_reaches_golden_cost(name):
    """PCG solved tightly: FP64 to a relative residual of 1e-10 reaches the
    oracle's final cost to 1e-6; so does the mixed path (FP32 PCG to 1e-6,
    the most its FP32 vectors resolve) with the FP64 polish. The mixed path
    alone ends within 1e-4: the LM loop stops at the first accepted step
    that lowers the cost by < 1e-6 relative (lib.rs:1215-1221), and on
    ring16 the oracle's own iteration 8 lowers it by just over that, so a
    step computed in FP32 can end the loop there."""
    p, kw, exp = G.load(name)
    runs = ((abi.PRECISION_FP64, 1e-10, 0, 1e-6), (abi.PRECISION_MIXED, 1e-6, 1, 1e-6),
            (abi.PRECISION_MIXED, 1e-6, 0, 1e-4))
    for prec, tol, polish, bar in runs:
        r = native.bundle_adjust_arrays(p, precision=prec, solver=abi.SOLVER_PCG, pcg_tolerance=tol,
                                        pcg_max_iterations=2000, fp64_polish=polish, **kw)
        assert r.final_cost <= exp["final_cost"] * (1 + bar), (prec, polish, r.final_cost, exp["final_cost"])


def test_gpu_jacobians_match_golden():
    z = G.jacobians()
    from sfmtory_gb300.problem import Problem

    for m, params in scenes.JACOBIAN_TEST_CAMERAS.items():
        cp = np.zeros((1, 8))
        cp[0, : len(params)] = params
        p = Problem(camera_of_image=np.array([0], np.int32), camera_model=np.array([m], np.int32),
                    camera_params=cp, poses=z["pose"][None], points=z["point"][None],
                    obs_image=np.array([0], np.int32), obs_point=np.array([0], np.int32),
                    obs_xy=np.array(z["obs"], np.float64)[None])
        r, jp, jx, jc, valid = native.residuals_jacobians(p)
        assert valid[0]
        for got, key in ((r[0], "r"), (jp[0], "jp"), (jx[0], "jx"), (jc[0], "jc")):
            assert G.rel_err(got, z[f"m{m}_{key}"]) < 1e-9


def test_pcg_coarse_polish_reaches_golden_cost():
    """PCG with the coarse correction and the FP64 polish: the chunk graphs
    captured for the FP32 loop are dropped when the loop continues in FP64,
    and the polished result reaches the FP64 oracle's final cost to 1e-6."""
    p, kw, exp = G.load("radial2000_s0005")
    r = native.bundle_adjust_arrays(p, precision=abi.PRECISION_MIXED, solver=abi.SOLVER_PCG, fp64_polish=1,
                                    pcg_tolerance=1e-10, pcg_max_iterations=2000, **kw)
    assert r.polish_iteration >= 0
    assert r.final_cost <= exp["final_cost"] * (1 + 1e-6), (r.final_cost, exp["final_cost"])
