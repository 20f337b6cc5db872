"""Batched PnP registration and Gauss-Newton pose refinement
(crates/sfm-geometry/src/pnp.rs, ransac.rs) on the GPU against the oracle's
restatement and the reference's own known-answer test.

Bars: the same images registered (found), the same RANSAC iteration count,
the same inlier masks, poses within 1e-9 (quaternion up to sign,
translation absolute; FP64 throughout, the sums differ only in order).
Gauss-Newton refinement: poses within 1e-10 of the oracle's."""
import numpy as np
import pytest

from sfmtory_gb300 import native, scenes
from sfmtory_gb300.problem import quat_to_matrix

pytestmark = pytest.mark.gpu


def _pose_close(a, b, tol):
    q = min(np.abs(a[:4] - b[:4]).max(), np.abs(a[:4] + b[:4]).max())
    return q <= tol and np.abs(a[4:] - b[4:]).max() <= tol * max(1.0, np.abs(b[4:]).max())


def test_pnp_recovers_known_pose():
    """pnp.rs:311-339 on the GPU: every point an inlier, rotation and
    translation errors below 1e-4."""
    pose, X, uv = scenes.pnp_known_pose_fixture()
    (r,) = native.pnp_ransac_batched([X], [uv], 0.01, 500)
    assert r is not None
    p, inl, _ = r
    assert inl.all()
    Rt, Re = quat_to_matrix(pose[:4]), quat_to_matrix(p[:4])
    assert np.arccos(np.clip((np.trace(Rt.T @ Re) - 1) / 2, -1, 1)) < 1e-4
    assert np.linalg.norm(p[4:] - pose[4:]) < 1e-4


@pytest.mark.parametrize("seed,outliers", [(0, 0.3), (1, 0.6), (2, 0.0)])
def test_pnp_batch_matches_oracle(oracle_lib, seed, outliers):
    P, Xs, uvs, thr = scenes.pnp_batch(seed, num_images=24, n_min=30, n_max=600, outlier_frac=outliers)
    got = native.pnp_ransac_batched(Xs, uvs, thr, 2000)
    for k in range(len(Xs)):
        ref = oracle_lib.pnp_ransac(Xs[k], uvs[k], thr, 2000)
        g = got[k]
        assert (g is None) == (ref is None), k
        if ref is None:
            continue
        assert g[2] == ref[2], (k, g[2], ref[2])
        assert np.array_equal(g[1], ref[1]), (k, int((g[1] != ref[1]).sum()))
        assert _pose_close(g[0], ref[0], 1e-9), (k, g[0], ref[0])


def test_pnp_none_cases(oracle_lib):
    """Fewer than 6 correspondences, no iterations, coplanar points: None,
    alongside an image that registers, in one batch."""
    pose, X, uv = scenes.pnp_known_pose_fixture()
    flat = X.copy()
    flat[:, 2] = 5.0
    res = native.pnp_ransac_batched([X[:5], X, flat], [uv[:5], uv, uv], 0.01, 50)
    assert res[0] is None and res[2] is None and res[1] is not None
    assert native.pnp_ransac_batched([X], [uv], 0.01, 0) == [None]


def test_refine_pose_gauss_newton_matches_oracle(oracle_lib):
    P, Xs, uvs, _ = scenes.pnp_batch(3, num_images=16, n_min=6, n_max=400, outlier_frac=0.0)
    rng = np.random.default_rng(5)
    init = P.copy()
    init[:, 4:] += rng.normal(0.0, 0.05, (len(P), 3))
    g = native.refine_pose_gauss_newton_batched(init, Xs, uvs, 10)
    r = oracle_lib.refine_pose_gauss_newton(init, Xs, uvs, 10)
    for k in range(len(P)):
        assert _pose_close(g[k], r[k], 1e-10), k
        assert _pose_close(g[k], P[k], 1e-2), k  # near the truth (0.5 px noise, as few as 6 points)
