"""Failure handling, injected on the host (no GPU fault is ever provoked):
non-finite observations, a singular reduced system (Cholesky fails, the LU
fallback fails, the damping grows until the retries run out), bad indices
given to the device entry point. The GPU must behave as the oracle."""
import ctypes as C

import numpy as np
import pytest

from sfmtory_gb300 import abi, native, scenes

pytestmark = pytest.mark.gpu


def test_nan_observation_is_rejected_like_the_reference(oracle_lib):
    p = scenes.ring16(seed=31, scale=0.05)
    xy = p.obs_xy.copy()
    xy[7, 0] = np.nan
    p = p.copy(obs_xy=xy)
    kw = dict(robust_loss=abi.LOSS_HUBER, max_iterations=10)
    r = oracle_lib.bundle_adjust(p, **kw)
    for prec in (abi.PRECISION_FP64, abi.PRECISION_MIXED):
        g = native.bundle_adjust_arrays(p, precision=prec, **kw)
        assert np.isnan(g.initial_cost) and np.isnan(r.initial_cost)
        assert g.iterations_run == r.iterations_run == 1
        assert np.array_equal(g.points, p.points)


def test_singular_system_exercises_lu_fallback(oracle_lib):
    """A free camera that no image uses: its diagonal block is 0 + lambda*0,
    Cholesky fails on the zero pivot, LU finds a zero column and fails, the
    damping grows through all 8 retries and the solve stops unchanged."""
    p = scenes.ring16(seed=32, scale=0.05)
    cams = np.vstack([p.camera_params, p.camera_params[:1]])
    p = p.copy(camera_model=np.append(p.camera_model, p.camera_model[0]).astype(np.int32), camera_params=cams,
               fixed_cameras=np.zeros(len(cams), bool),
               fixed_camera_params=np.vstack([p.fixed_camera_params, p.fixed_camera_params[:1]]))
    kw = dict(robust_loss=abi.LOSS_NONE, max_iterations=5)
    r = oracle_lib.bundle_adjust(p, **kw)
    g = native.bundle_adjust_arrays(p, solver=abi.SOLVER_DENSE, **kw)
    assert r.iterations_run == 1 and g.iterations_run == 1
    assert g.damping_retries == 8
    assert g.final_cost == g.initial_cost
    assert abs(g.initial_cost - r.initial_cost) <= 1e-12 * r.initial_cost


def test_device_entry_rejects_bad_indices():
    import torch

    p = scenes.ring16(seed=33, scale=0.05)
    obs_point = p.obs_point.copy()
    obs_point[3] = p.num_points + 5
    pk = abi.PackedProblem(p.copy(obs_point=obs_point))
    keep = []

    def dev(a):
        t = torch.from_numpy(np.ascontiguousarray(a)).cuda()
        keep.append(t)
        return t.data_ptr()

    s = abi.SfmbaProblem()
    for f in ("num_images", "num_cameras", "num_points", "num_observations"):
        setattr(s, f, getattr(pk.struct, f))
    for f in ("camera_of_image", "camera_model", "camera_params", "poses", "points", "obs_image", "obs_point",
              "obs_xy", "fixed_poses", "fixed_cameras", "fixed_camera_params"):
        a = getattr(pk, f)
        setattr(s, f, dev(a) if a is not None else None)
    out_pts = torch.zeros((p.num_points, 3), dtype=torch.float64, device="cuda")
    res = abi.SfmbaResult()
    res.points = out_pts.data_ptr()
    L = native.load()
    st = L.sfmba_bundle_adjust_device(C.byref(s), C.byref(abi.default_options()), C.byref(res), None)
    assert st == 1
    assert b"out of range" in L.sfmba_last_error()
    # The library stays usable after the rejected call.
    g = native.bundle_adjust_arrays(p, robust_loss=abi.LOSS_NONE, max_iterations=2)
    assert g.iterations_run >= 1
