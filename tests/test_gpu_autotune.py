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
    for v in (2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 0):
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
        # launch variants per kernel (kernels.cuh: kPointPassVariants, kImagePassVariants, kWbSchurVariants)
        n = {"points": 11, "images": 10}.get(e["pass"], 3)
        assert 0 <= e["variant"] < n and len(e["us"]) == n and min(e["us"]) > 0
        assert e["us"][e["variant"]] == min(e["us"])


@pytest.mark.parametrize("precision", [abi.PRECISION_MIXED, abi.PRECISION_FP64])
def test_batched_schur_shapes_are_bit_identical(precision):
    """Every launch shape of the batched windows' Schur reduction (warps per
    block, register budget) gives the same batch, bit for bit; the tuner's
    report then lists its choice for the batch."""
    rng = np.random.default_rng(21)
    wins = [scenes.local_window(rng, int(rng.integers(8, 24)), int(rng.integers(150, 600))) for _ in range(12)]
    kw = dict(precision=precision, robust_loss=abi.LOSS_HUBER, loss_scale_px=2.0, max_iterations=6)
    ref = native.bundle_adjust_batched_arrays(wins, kernel_variant=1, **kw)
    for v in (2, 3):
        res = native.bundle_adjust_batched_arrays(wins, kernel_variant=v, **kw)
        for a, b in zip(res, ref):
            assert a.final_cost == b.final_cost and a.iterations_run == b.iterations_run, v
            assert np.array_equal(a.points, b.points) and np.array_equal(a.poses, b.poses)
            assert np.array_equal(a.camera_params, b.camera_params)
    tuned = native.bundle_adjust_batched_arrays(wins, **kw)
    for a, b in zip(tuned, ref):
        assert a.final_cost == b.final_cost
    assert any(e["pass"].startswith("wb_schur") for e in native.profile_report()["autotune"])


@pytest.mark.parametrize("scene, loss", [
    ("ring16", abi.LOSS_HUBER),        # PINHOLE, robust weight from the FP32 residual
    ("radial500", abi.LOSS_NONE),      # SIMPLE_RADIAL
    ("shared_radial", abi.LOSS_CAUCHY),  # one RADIAL camera shared by every image
])
def test_tma_point_pass_is_bit_identical(scene, loss):
    """The point pass that streams its records by bulk copies (variant 11)
    against the register-prefetch pass it mirrors (variant 9) on other
    camera models, losses and a shared camera: the same solve, bit for bit."""
    p = {"ring16": lambda: scenes.ring16(seed=5, scale=0.25),
         "radial500": lambda: scenes.radial500(seed=5, scale=0.05),
         "shared_radial": lambda: scenes.shared_radial(seed=5, scale=0.02)}[scene]()
    kw = dict(precision=abi.PRECISION_MIXED, solver=abi.SOLVER_PCG, robust_loss=loss, loss_scale_px=1.0,
              max_iterations=6)
    ref = native.bundle_adjust_arrays(p, kernel_variant=9, **kw)
    for v in (11,):
        r = native.bundle_adjust_arrays(p, kernel_variant=v, **kw)
        assert r.final_cost == ref.final_cost and r.linear_iterations == ref.linear_iterations, v
        assert np.array_equal(r.points, ref.points) and np.array_equal(r.poses, ref.poses)
        assert np.array_equal(r.camera_params, ref.camera_params)
