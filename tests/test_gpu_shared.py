"""Free cameras shared by many images on the matrix-free PCG solver.

The reference's bundle_adjust takes every camera-sharing pattern: a camera
is one slot block however many images use it (crates/sfm-ba/src/lib.rs:
753-787, cross blocks :946-956), and its production caller runs the global
pass with intrinsics shared across a sequence (crates/sfm-reconstruction/
src/lib.rs:1489-1520, :1567-1708). These tests hold the PCG solver's
shared-camera path to the FP64 oracle on small scenes and check the full
2000-image, one-camera scene on the FP32 and FP64 paths against each other.

Bars: FP64 PCG solved tightly follows the oracle's trajectory (same
iterations, final cost and parameters 1e-6 relative); the mixed path
reaches the oracle's final cost to 1e-6 relative; at full size the FP32 and
FP64 final costs agree to 1e-6 relative.
"""
import numpy as np
import pytest

from sfmtory_gb300 import abi, native, scenes

pytestmark = pytest.mark.gpu

TIGHT = dict(pcg_tolerance=1e-12, pcg_max_iterations=3000)


def _rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b)) / np.maximum(np.abs(np.asarray(b)), 1.0)))


SCENES = {
    "ring_two_pinhole": lambda: scenes.shared_ring(seed=31, scale=0.1, images_per_camera=(8, 8)),
    "ring_uneven_radial": lambda: scenes.shared_ring(seed=32, scale=0.1, images_per_camera=(3, 5, 8),
                                                     model=abi.SIMPLE_RADIAL, k=0.02),
    "radial_one_camera": lambda: scenes.shared_radial(seed=33, scale=0.002, n_cameras=1),
    "radial_three_cameras": lambda: scenes.shared_radial(seed=34, scale=0.002, n_cameras=3),
}


@pytest.mark.parametrize("name", list(SCENES))
def test_shared_camera_pcg_fp64_follows_oracle(oracle_lib, name):
    p = SCENES[name]()
    kw = dict(robust_loss=abi.LOSS_NONE, max_iterations=50)
    r = oracle_lib.bundle_adjust(p, **kw)
    g = native.bundle_adjust_arrays(p, solver=abi.SOLVER_PCG, **TIGHT, **kw)
    assert g.solver_used == abi.SOLVER_PCG and g.linear_iterations > 0
    assert abs(g.initial_cost - r.initial_cost) <= 1e-12 * r.initial_cost
    assert g.iterations_run == r.iterations_run, (g.iterations_run, r.iterations_run)
    assert abs(g.final_cost - r.final_cost) <= 1e-6 * r.final_cost, (g.final_cost, r.final_cost)
    assert _rel(g.camera_params, r.camera_params) <= 1e-6
    assert _rel(g.poses, r.poses) <= 1e-6
    assert _rel(g.points, r.points) <= 1e-6


@pytest.mark.parametrize("name", list(SCENES))
@pytest.mark.parametrize("coarse", [0, -1], ids=["coarse", "block_jacobi"])
def test_shared_camera_pcg_mixed_reaches_oracle_cost(oracle_lib, name, coarse):
    """FP32 PCG, with and without the coarse correction (which covers the
    linked images' pose columns only), reaches the oracle's cost to 1e-6 with
    the FP64 polish and to 1e-5 alone (the FP32 loop's stopping point)."""
    p = SCENES[name]()
    kw = dict(robust_loss=abi.LOSS_NONE, max_iterations=50)
    r = oracle_lib.bundle_adjust(p, **kw)
    for polish, bar in ((1, 1e-6), (0, 1e-5)):
        g = native.bundle_adjust_arrays(p, solver=abi.SOLVER_PCG, precision=abi.PRECISION_MIXED, pcg_tolerance=1e-6,
                                        pcg_max_iterations=500, pcg_coarse_clusters=coarse, fp64_polish=polish, **kw)
        assert g.solver_used == abi.SOLVER_PCG
        assert g.final_cost <= r.final_cost * (1 + bar), (polish, g.final_cost, r.final_cost)


def test_shared_camera_pcg_matches_dense_gpu():
    """Same problem, same path otherwise: PCG solved tightly against the
    dense solver on the GPU (FP64), a camera shared by all 283 images."""
    p = scenes.shared_radial(seed=35, scale=0.02, n_cameras=1)
    kw = dict(robust_loss=abi.LOSS_NONE, max_iterations=8)
    d = native.bundle_adjust_arrays(p, solver=abi.SOLVER_DENSE, **kw)
    g = native.bundle_adjust_arrays(p, solver=abi.SOLVER_PCG, **TIGHT, **kw)
    assert d.solver_used == abi.SOLVER_DENSE and g.solver_used == abi.SOLVER_PCG
    assert g.iterations_run == d.iterations_run
    assert abs(g.final_cost - d.final_cost) <= 1e-6 * d.final_cost, (g.final_cost, d.final_cost)
    assert _rel(g.camera_params, d.camera_params) <= 1e-6


@pytest.fixture(scope="module")
def shared_radial_full():
    p = scenes.shared_radial(seed=0, scale=1.0, n_cameras=1)
    assert p.num_images == 2000 and p.num_cameras == 1 and p.num_observations > 5_000_000
    return p


@pytest.mark.parametrize("solver", [abi.SOLVER_AUTO, abi.SOLVER_PCG])
def test_shared_radial_full_fp32_and_fp64_stop_together(shared_radial_full, solver):
    """2000 images, one shared RADIAL camera, 1M points, ~6M observations
    (reduced dimension 11 999, above the dense default): both precisions
    solve it and end within 1e-5 of each other: each stops by the
    reference's rule (an iteration lowering the cost by < 1e-6 relative,
    lib.rs:1215-1221), and on this flat problem two trajectories that differ
    by rounding (FP32 against FP64 operators) stop at points up to a few
    1e-6 apart (the FP64 path itself lands 1e-5 lower without the coarse
    correction); with the FP64 polish the mixed path's stop is an FP64
    iteration's."""
    p = shared_radial_full
    kw = dict(robust_loss=abi.LOSS_NONE, max_iterations=50, solver=solver)
    g64 = native.bundle_adjust_arrays(p, precision=abi.PRECISION_FP64, **kw)
    g32 = native.bundle_adjust_arrays(p, precision=abi.PRECISION_MIXED, fp64_polish=1, **kw)
    for g in (g64, g32):
        assert g.solver_used == abi.SOLVER_PCG
        assert g.final_cost < 2e-3 * g.initial_cost  # converged: ~1e-3 of the initial cost
    assert abs(g32.final_cost - g64.final_cost) <= 1e-5 * g64.final_cost, (g32.final_cost, g64.final_cost)


def test_dense_request_above_its_limit_runs_pcg():
    """A dense request for a reduced system above 16384 unknowns (here
    18 397) is solved by the PCG solver instead of being refused."""
    p = scenes.radial2000(seed=36, scale=0.7)
    assert p.reduced_dim() > 16384
    kw = dict(robust_loss=abi.LOSS_NONE, max_iterations=3, precision=abi.PRECISION_MIXED)
    d = native.bundle_adjust_arrays(p, solver=abi.SOLVER_DENSE, **kw)
    g = native.bundle_adjust_arrays(p, solver=abi.SOLVER_PCG, **kw)
    assert d.solver_used == abi.SOLVER_PCG
    assert d.final_cost == g.final_cost and d.iterations_run == g.iterations_run
