"""Loading of the golden fixtures in tests/golden (made by make_golden.py)."""
import os

import numpy as np

from sfmtory_gb300.problem import Problem

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ("recovers_ground_truth", "shared_focal_fixed", "ring16_s005", "opencv47_s002_huber",
         "radial2000_s0005", "window_mixed_models")


def load(name):
    """(problem, bundle_adjust keyword arguments, expected outputs)."""
    z = np.load(os.path.join(HERE, f"{name}.npz"))
    p = Problem(camera_of_image=z["camera_of_image"], camera_model=z["camera_model"],
                camera_params=z["camera_params"], poses=z["poses"], points=z["points"],
                obs_image=z["obs_image"], obs_point=z["obs_point"], obs_xy=z["obs_xy"],
                fixed_poses=z["fixed_poses"] if "fixed_poses" in z else None,
                fixed_cameras=z["fixed_cameras"] if "fixed_cameras" in z else None,
                fixed_camera_params=z["fixed_camera_params"] if "fixed_camera_params" in z else None)
    o = z["options"]
    kw = dict(max_iterations=int(o[0]), robust_loss=int(o[1]), loss_scale_px=float(o[2]))
    out = dict(poses=z["out_poses"], points=z["out_points"], camera_params=z["out_camera_params"],
               initial_cost=float(z["initial_cost"]), final_cost=float(z["final_cost"]),
               iterations_run=int(z["iterations_run"]))
    return p, kw, out


def jacobians():
    return np.load(os.path.join(HERE, "jacobians.npz"))


def rel_err(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b)) / np.maximum(np.abs(np.asarray(b)), 1.0)))
