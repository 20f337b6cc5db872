"""sfmba_total_cost_noalloc: the robust cost computed without allocating.

Callers that cannot let a library allocate GPU memory (a service that hands
each component a fixed slice of the device, or a thread that must not pay
for cudaFree's device-wide synchronisation) use this entry point with their
own device arrays. It must give the same cost as sfmba_total_cost, call
after call, even though every call reuses one fixed scratch array inside the
library that still holds the previous call's partial sums.

The expected values come from the CPU FP64 oracle (and, for the same
problem, from sfmba_total_cost). This file is collected last so that a run
stopping at its first failure has already run every other test; it also
passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from sfmtory_gb300 import abi, native, scenes

pytestmark = pytest.mark.gpu


class _DeviceProblem:
    """The problem's arrays copied to the GPU by the test (the entry point
    under test allocates nothing itself)."""

    def __init__(self, p):
        import torch

        pk = abi.PackedProblem(p)
        self.keep = []

        def dev(a):
            t = torch.from_numpy(np.ascontiguousarray(a)).cuda()
            self.keep.append(t)
            return t.data_ptr()

        s = abi.SfmbaProblem()
        s.num_images, s.num_cameras = pk.struct.num_images, pk.struct.num_cameras
        s.num_points, s.num_observations = pk.struct.num_points, pk.struct.num_observations
        s.camera_of_image, s.camera_model = dev(pk.camera_of_image), dev(pk.camera_model)
        s.camera_params, s.poses, s.points = dev(pk.camera_params), dev(pk.poses), dev(pk.points)
        s.obs_image, s.obs_point, s.obs_xy = dev(pk.obs_image), dev(pk.obs_point), dev(pk.obs_xy)
        self.struct = s


def _noalloc_call(L, dp, opts):
    import torch

    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    st = L.sfmba_total_cost_noalloc(C.byref(dp.struct), C.byref(opts), C.c_void_p(out.data_ptr()), None)
    return st, float(out.item())


def _noalloc_cost(L, p, opts):
    st, v = _noalloc_call(L, _DeviceProblem(p), opts)
    assert st == 0, L.sfmba_last_error()
    return v


def test_noalloc_cost_matches_oracle_on_two_calls_in_a_row(oracle_lib):
    L = native.load()
    opts = abi.default_options(robust_loss=abi.LOSS_HUBER, loss_scale_px=1.0)
    # A larger problem first, then a smaller one: the second call must not
    # pick up partial sums the first call left in the shared scratch array.
    first = scenes.opencv47(seed=21, scale=0.3)
    second = scenes.ring16(seed=22, scale=0.05)
    for p in (first, second):
        expected = oracle_lib.total_cost(p, opts)
        got = _noalloc_cost(L, p, opts)
        assert abs(got - expected) <= 1e-12 * abs(expected), (got, expected)
        assert abs(got - native.total_cost(p, opts)) <= 1e-12 * abs(expected)


def test_noalloc_allocates_no_device_memory():
    """The property the entry point exists for: after a first call (which
    looks up the scratch array's address), further calls leave the device's
    free memory unchanged."""
    import torch

    L = native.load()
    opts = abi.default_options(robust_loss=abi.LOSS_CAUCHY, loss_scale_px=2.0)
    dp = _DeviceProblem(scenes.opencv47(seed=23, scale=0.1))
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    assert L.sfmba_total_cost_noalloc(C.byref(dp.struct), C.byref(opts), C.c_void_p(out.data_ptr()), None) == 0
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        assert L.sfmba_total_cost_noalloc(C.byref(dp.struct), C.byref(opts), C.c_void_p(out.data_ptr()),
                                          None) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before


def test_noalloc_bad_index_is_reported_and_cleared(oracle_lib):
    """An observation whose point index equals num_points: the kernel checks
    every index before loading through it, flags the call as invalid
    (status 1, NaN written) and the next valid call is unaffected."""
    L = native.load()
    opts = abi.default_options(robust_loss=abi.LOSS_HUBER, loss_scale_px=1.0)
    p = scenes.ring16(seed=24, scale=0.05)
    bad = p.copy()
    bad.obs_point[len(bad.obs_point) // 2] = bad.num_points
    st, v = _noalloc_call(L, _DeviceProblem(bad), opts)
    assert st == 1 and np.isnan(v)
    assert b"out of range" in L.sfmba_last_error()
    bad_cam = p.copy()
    bad_cam.camera_of_image[0] = bad_cam.num_cameras  # an image index check, not an observation one
    st, v = _noalloc_call(L, _DeviceProblem(bad_cam), opts)
    assert st == 1 and np.isnan(v)
    got = _noalloc_cost(L, p, opts)
    expected = oracle_lib.total_cost(p, opts)
    assert abs(got - expected) <= 1e-12 * abs(expected), (got, expected)


def test_noalloc_rejects_problems_above_its_limit():
    L = native.load()
    s = abi.SfmbaProblem()
    s.num_images = s.num_cameras = s.num_points = 1
    s.num_observations = 16777216 + 1
    out = C.c_double(0.0)
    st = L.sfmba_total_cost_noalloc(C.byref(s), None, C.byref(out), None)
    assert st == 1
    assert b"16777216" in L.sfmba_last_error()
