"""Expected FP64 oracle outputs of the dense 500-camera scene at full size.

radial500(seed=0, scale=1): 500 SIMPLE_RADIAL cameras, 200k points, ~1.2M
observations, reduced dimension 4994, squared loss, 50 LM iterations. The
oracle's unblocked single-thread Cholesky makes this solve take minutes, so
it runs once here and the test compares the GPU against the stored result.
The file holds the seed, checksums of the regenerated inputs (the test
checks it rebuilt the same scene), the costs, iteration count and RMS, every
pose and camera, and every 100th point with checksums of all points; not the
inputs themselves. It also holds how far the oracle's own parameters moved
in its last iteration (the same solve stopped one iteration earlier, against
the final one): the resolution of the reference's stopping rule, beside
which the mixed path's parameter error is stated.

    python tests/golden/make_config_golden.py
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from sfmtory_gb300 import abi, scenes  # noqa: E402
from sfmtory_gb300.problem import parameter_errors, rms_of  # noqa: E402

SEED = 0
POINT_STRIDE = 100
OPTIONS = dict(robust_loss=abi.LOSS_NONE, max_iterations=50)
THREADS = 8  # fixed thread count: fixed Schur summation order


def input_checksums(p):
    return np.array([p.num_images, p.num_points, p.num_observations, float(np.sum(p.obs_xy)),
                     float(np.sum(p.poses)), float(np.sum(p.points)), float(np.sum(p.camera_params)),
                     float(np.sum(p.obs_point.astype(np.float64) * (1.0 + p.obs_image)))])


def main():
    p = scenes.radial500(seed=SEED, scale=1.0)
    oracle.set_threads(THREADS)
    t = time.time()
    r = oracle.bundle_adjust(p, **OPTIONS)
    secs = time.time() - t
    prev = oracle.bundle_adjust(p, **dict(OPTIONS, max_iterations=r.iterations_run - 1))
    last = parameter_errors(prev.poses, prev.points, prev.camera_params, r.poses, r.points, r.camera_params)
    idx = np.arange(0, p.num_points, POINT_STRIDE)
    np.savez_compressed(
        os.path.join(HERE, "radial500_full.npz"),
        seed=SEED, scale=1.0, options=np.array([OPTIONS["max_iterations"], OPTIONS["robust_loss"], 2.0]),
        input_checksums=input_checksums(p), reduced_dim=r.reduced_dim,
        initial_cost=r.initial_cost, final_cost=r.final_cost, iterations_run=r.iterations_run,
        damping_retries=r.damping_retries, rms_px=rms_of(p, r.poses, r.points, r.camera_params),
        out_poses=r.poses, out_camera_params=r.camera_params, point_index=idx, out_points=r.points[idx],
        points_sum=np.sum(r.points, axis=0), points_sumsq=np.sum(r.points ** 2, axis=0),
        oracle_seconds=secs, oracle_threads=THREADS,
        last_step_raw=last["raw_max"], last_step_normalized=last["normalized_max"],
        last_step_cost_rel=(prev.final_cost - r.final_cost) / r.final_cost)
    print(f"radial500: n={r.reduced_dim}, cost {r.initial_cost:.9g} -> {r.final_cost:.9g}, "
          f"{r.iterations_run} iterations, {r.damping_retries} retries, {secs:.1f} s; last step moved the "
          f"parameters by {last['raw_max']:.3g} (raw)")


if __name__ == "__main__":
    main()
