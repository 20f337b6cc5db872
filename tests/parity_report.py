"""Parity figures of the full-size configuration tests.

``errors`` states a solution's error against the FP64 oracle's on the three
quantities the specification bounds: final cost (relative), RMS reprojection
error (px) and parameters (relative; raw and after removing the free scale).
``record`` prints them and, when SFMBA_PARITY_REPORT names a file, appends
them there as one JSON line, so a test run leaves the measured errors beside
its pass/fail result.
"""
import json
import os

from sfmtory_gb300.problem import parameter_errors, rms_of

# The bars of the specification.
COST_RTOL = 1e-6
RMS_PX = 1e-4
PARAM_RTOL = 1e-6


def errors(problem, sol, ref_poses, ref_points, ref_cams, ref_cost, ref_rms=None, point_index=None):
    """Errors of ``sol`` (an object with poses/points/camera_params/final_cost)
    against a reference solution. point_index: compare only these points
    (the reference holds a subset)."""
    pts = sol.points if point_index is None else sol.points[point_index]
    pe = parameter_errors(sol.poses, pts, sol.camera_params, ref_poses, ref_points, ref_cams)
    rms = rms_of(problem, sol.poses, sol.points, sol.camera_params)
    out = {
        "cost_rel": abs(sol.final_cost - ref_cost) / abs(ref_cost) if ref_cost else abs(sol.final_cost),
        "cost_signed_rel": (sol.final_cost - ref_cost) / abs(ref_cost) if ref_cost else sol.final_cost,
        "rms_px": rms,
        "param_raw": pe["raw"], "param_normalized": pe["normalized"],
        "param_raw_max": pe["raw_max"], "param_normalized_max": pe["normalized_max"],
        "scale_ratio": pe["scale_ratio"],
    }
    if ref_rms is not None:
        out["rms_ref_px"] = ref_rms
        out["rms_diff_px"] = abs(rms - ref_rms)
    out["meets"] = {
        "cost": out["cost_rel"] <= COST_RTOL,
        "rms": ref_rms is None or out["rms_diff_px"] <= RMS_PX,
        "param_raw": pe["raw_max"] <= PARAM_RTOL,
        "param_normalized": pe["normalized_max"] <= PARAM_RTOL,
    }
    return out


def record(name: str, data: dict) -> None:
    line = json.dumps({"case": name, **data}, default=float, sort_keys=True)
    print(line)
    path = os.environ.get("SFMBA_PARITY_REPORT")
    if path:
        with open(path, "a") as f:
            f.write(line + "\n")
