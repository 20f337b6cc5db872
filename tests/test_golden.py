"""The oracle against its committed golden fixtures (regression pin).

Fixtures: tests/golden/*.npz, generated by tests/golden/make_golden.py with
one oracle thread. Bars: initial cost 1e-12 relative, final cost and
parameters 1e-9 relative (OpenMP summation order may differ), same
iteration count; Jacobians 1e-12 relative.
"""
import numpy as np
import pytest

import golden_util as G
from sfmtory_gb300 import scenes


@pytest.mark.parametrize("name", G.CASES)
def test_oracle_reproduces_golden(oracle_lib, name):
    p, kw, exp = G.load(name)
    r = oracle_lib.bundle_adjust(p, **kw)
    assert abs(r.initial_cost - exp["initial_cost"]) <= 1e-12 * abs(exp["initial_cost"])
    assert r.iterations_run == exp["iterations_run"]
    assert abs(r.final_cost - exp["final_cost"]) <= 1e-9 * abs(exp["final_cost"]) + 1e-20
    assert G.rel_err(r.points, exp["points"]) < 1e-9
    assert G.rel_err(r.poses, exp["poses"]) < 1e-9
    assert G.rel_err(r.camera_params, exp["camera_params"]) < 1e-9


def test_oracle_jacobians_match_golden(oracle_lib):
    z = G.jacobians()
    for m, params in scenes.JACOBIAN_TEST_CAMERAS.items():
        rr, jp, jx, jc = oracle_lib.analytic_jacobians(z["pose"], m, params, z["point"], z["obs"])
        for got, key in ((rr, "r"), (jp, "jp"), (jx, "jx"), (jc, "jc")):
            assert G.rel_err(got, z[f"m{m}_{key}"]) < 1e-12
