"""The autotuner picks among launch variants of the two PCG observation
passes; every variant must give bit-identical solves, so the choice (which
depends on timing) never changes a result."""
import numpy as np
import pytest

from sfmtory_gb300 import abi, native, scenes

pytestmark = pytest.mark.gpu


def test_pass_variants_are_bit_identical():
    p = scenes.radial2000(seed=3, scale=0.05)
    kw = dict(precision=abi.PRECISION_MIXED, solver=abi.SOLVER_PCG, robust_loss=abi.LOSS_NONE, max_iterations=8)
    ref = native.bundle_adjust_arrays(p, kernel_variant=1, **kw)
    for v in (2, 3, 4, 5, 6, 0):
        r = native.bundle_adjust_arrays(p, kernel_variant=v, **kw)
        assert r.final_cost == ref.final_cost, v
        assert r.iterations_run == ref.iterations_run and r.linear_iterations == ref.linear_iterations
        assert np.array_equal(r.points, ref.points) and np.array_equal(r.poses, ref.poses)
        assert np.array_equal(r.camera_params, ref.camera_params)


def test_autotune_report_lists_choices():
    p = scenes.radial2000(seed=4, scale=0.05)
    native.bundle_adjust_arrays(p, precision=abi.PRECISION_MIXED, solver=abi.SOLVER_PCG, max_iterations=2)
    rep = native.profile_report()["autotune"]
    assert {e["pass"] for e in rep} >= {"points", "images"}
    for e in rep:
        n = 6
        assert 0 <= e["variant"] < n and len(e["us"]) == n and min(e["us"]) > 0
        assert e["us"][e["variant"]] == min(e["us"])
