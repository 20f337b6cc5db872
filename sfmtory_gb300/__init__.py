"""GB300-native drop-in for sfmtory's ``sfm-ba`` bundle adjuster.

The solver is the CUDA library ``libsfmba_gb300.so`` (C ABI in
``include/sfmba.h``); :mod:`sfmtory_gb300.sfm_ba` mirrors the Rust crate's
interface over it and :mod:`sfmtory_gb300.native` exposes the array-level
calls. Importing this package does not load the library; the first solve
does, and raises if it is missing.
"""
from . import abi, problem, scenes  # noqa: F401
from .sfm_ba import (  # noqa: F401
    BaInput,
    BaOutput,
    BaParams,
    CameraModel,
    IntrinsicsRefineParams,
    Observation,
    Pose,
    RobustLoss,
    bundle_adjust,
    default_fixed_params_mask,
    mean_reprojection_error,
    refine_intrinsics,
)

__all__ = [
    "BaInput", "BaOutput", "BaParams", "CameraModel", "IntrinsicsRefineParams", "Observation", "Pose",
    "RobustLoss", "bundle_adjust", "default_fixed_params_mask", "mean_reprojection_error",
    "refine_intrinsics",
]
