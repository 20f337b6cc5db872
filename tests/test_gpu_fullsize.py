"""Size-independent properties at the full benchmark size (2000 RADIAL
cameras, 1M points, 5.96M observations), where the dense CPU oracle cannot
run a whole solve:

* the final cost each path reports equals the cost the GPU and the CPU
  oracle compute for the returned parameters (1e-9 relative) - a checksum
  of the whole returned state;
* both paths decrease the cost and finish within 1e-6 relative of each other;
* observation order does not change the result.
"""
import numpy as np
import pytest

from sfmtory_gb300 import abi, native, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def big():
    return scenes.radial2000(seed=0, scale=1.0)


def test_fullsize_fp32_and_fp64_agree_and_costs_check_out(oracle_lib, big):
    kw = dict(robust_loss=abi.LOSS_NONE, solver=abi.SOLVER_PCG, max_iterations=50)
    r32 = native.bundle_adjust_arrays(big, precision=abi.PRECISION_MIXED, **kw)
    r64 = native.bundle_adjust_arrays(big, precision=abi.PRECISION_FP64, **kw)
    for r in (r32, r64):
        assert r.final_cost < 1e-2 * r.initial_cost
        out = big.copy(poses=r.poses, points=r.points, camera_params=r.camera_params)
        gpu_cost = native.total_cost(out, robust_loss=abi.LOSS_NONE)
        cpu_cost = oracle_lib.total_cost(out, robust_loss=abi.LOSS_NONE)
        assert abs(gpu_cost - r.final_cost) <= 1e-9 * r.final_cost
        assert abs(cpu_cost - r.final_cost) <= 1e-9 * r.final_cost
    assert abs(r32.final_cost - r64.final_cost) <= 1e-6 * r64.final_cost
    assert abs(r32.initial_cost - r64.initial_cost) <= 1e-12 * r64.initial_cost


def test_fullsize_observation_order_invariance(big):
    """FP64: three iterations agree to 1e-9 whatever the input order (only
    summation order changes). FP32: an unconverged trajectory is sensitive
    to summation order at ~1e-6, so the FP32 runs are compared converged."""
    rng = np.random.default_rng(5)
    perm = rng.permutation(big.num_observations)
    shuffled = big.copy(obs_image=big.obs_image[perm], obs_point=big.obs_point[perm], obs_xy=big.obs_xy[perm])
    kw = dict(robust_loss=abi.LOSS_NONE, solver=abi.SOLVER_PCG)
    a = native.bundle_adjust_arrays(big, precision=abi.PRECISION_FP64, max_iterations=3, **kw)
    b = native.bundle_adjust_arrays(shuffled, precision=abi.PRECISION_FP64, max_iterations=3, **kw)
    assert a.iterations_run == b.iterations_run == 3
    assert abs(a.final_cost - b.final_cost) <= 1e-9 * a.final_cost
    a = native.bundle_adjust_arrays(big, precision=abi.PRECISION_MIXED, max_iterations=50, **kw)
    b = native.bundle_adjust_arrays(shuffled, precision=abi.PRECISION_MIXED, max_iterations=50, **kw)
    assert abs(a.final_cost - b.final_cost) <= 1e-6 * a.final_cost
