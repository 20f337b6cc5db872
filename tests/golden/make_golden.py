"""Generate the golden fixtures in this folder from the CPU FP64 oracle.

Each fixture stores a seeded problem (inputs) and the oracle's outputs for
it: final poses, points and camera parameters, initial/final cost, the
iteration count, and (for the Jacobian fixture) the analytic Jacobians of
the reference's test observation for all six camera models. The oracle is
pinned by the reference's own tests (tests/test_oracle.py); these files pin
the oracle and the GPU path against regressions.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from sfmtory_gb300 import abi, scenes  # noqa: E402

# name -> (problem factory, bundle_adjust keyword arguments)
CASES = {
    "recovers_ground_truth": (scenes.recovers_ground_truth_fixture, dict(max_iterations=30)),
    "shared_focal_fixed": (scenes.shared_focal_fixture, dict(max_iterations=50)),
    "ring16_s005": (lambda: scenes.ring16(seed=101, scale=0.05),
                    dict(robust_loss=abi.LOSS_NONE, max_iterations=50)),
    "opencv47_s002_huber": (lambda: scenes.opencv47(seed=102, scale=0.02),
                            dict(robust_loss=abi.LOSS_HUBER, loss_scale_px=1.0, max_iterations=30)),
    "radial2000_s0005": (lambda: scenes.radial2000(seed=103, scale=0.0005),
                         dict(robust_loss=abi.LOSS_NONE, max_iterations=50)),
    "window_mixed_models": (lambda: scenes.local_window(np.random.default_rng(104), 12, 300),
                            dict(robust_loss=abi.LOSS_CAUCHY, loss_scale_px=1.5, max_iterations=40)),
}

KW_KEYS = ("max_iterations", "robust_loss", "loss_scale_px")


def problem_arrays(p):
    d = dict(camera_of_image=p.camera_of_image, camera_model=p.camera_model, camera_params=p.camera_params,
             poses=p.poses, points=p.points, obs_image=p.obs_image, obs_point=p.obs_point, obs_xy=p.obs_xy)
    for k in ("fixed_poses", "fixed_cameras", "fixed_camera_params"):
        v = getattr(p, k)
        if v is not None:
            d[k] = np.asarray(v)
    return d


def main():
    oracle.set_threads(1)  # fixed summation order
    for name, (make, kw) in CASES.items():
        p = make()
        r = oracle.bundle_adjust(p, **kw)
        opts = np.array([kw.get("max_iterations", 50), kw.get("robust_loss", abi.LOSS_HUBER),
                         kw.get("loss_scale_px", 2.0)], dtype=np.float64)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **problem_arrays(p), options=opts,
                            out_poses=r.poses, out_points=r.points, out_camera_params=r.camera_params,
                            initial_cost=r.initial_cost, final_cost=r.final_cost,
                            iterations_run=r.iterations_run)
        print(f"{name}: {p.num_observations} obs, cost {r.initial_cost:.6g} -> {r.final_cost:.9g}, "
              f"{r.iterations_run} iterations")
    pose, X, obs = scenes.jacobian_test_fixture()
    jac = {}
    for m, params in scenes.JACOBIAN_TEST_CAMERAS.items():
        rr, jp, jx, jc = oracle.analytic_jacobians(pose, m, params, X, obs)
        jac[f"m{m}_r"], jac[f"m{m}_jp"], jac[f"m{m}_jx"], jac[f"m{m}_jc"] = rr, jp, jx, jc
    np.savez_compressed(os.path.join(HERE, "jacobians.npz"), pose=pose, point=X, obs=np.array(obs), **jac)
    print("jacobians: 6 models")


if __name__ == "__main__":
    main()
