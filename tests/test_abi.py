"""C ABI checks that need no GPU: the library loads, exports every entry
point include/sfmba.h declares, and rejects invalid input before any device
work (return codes, never aborts)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from sfmtory_gb300 import abi, native, scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    text = open(os.path.join(ROOT, "include", "sfmba.h")).read()
    return sorted(set(re.findall(r"^(?:int|void|const char \*)\s*(sfmba_[a-z_]+)\s*\(", text, re.M)))


def test_header_and_binding_agree():
    assert sorted(native.EXPORTED_SYMBOLS) == _declared_symbols()


def test_library_exports_every_declared_symbol():
    L = native.load()
    for name in _declared_symbols():
        assert hasattr(L, name), name


def test_struct_sizes_match_header_layout():
    # int64 x4 + 11 pointers
    assert C.sizeof(abi.SfmbaProblem) == 4 * 8 + 11 * 8
    L = native.load()
    o = abi.SfmbaOptions()
    L.sfmba_default_options(C.byref(o))
    assert o.max_iterations == 50 and o.initial_lambda == 1e-3
    assert o.robust_loss == abi.LOSS_HUBER and o.loss_scale_px == 2.0


def test_default_fixed_params_mask_matches_oracle(oracle_lib):
    models = [0, 1, 2, 3, 4, 5, 3, 0]
    assert np.array_equal(native.default_fixed_params_mask_arrays(models),
                          oracle_lib.default_fixed_params_mask(models))
    with pytest.raises(native.SfmbaError):
        native.default_fixed_params_mask_arrays([9])


@pytest.mark.parametrize("field,value", [
    ("obs_point", 10**6), ("obs_image", -1), ("camera_of_image", 5), ("camera_model", 7)])
def test_invalid_indices_rejected_before_device(field, value):
    p = scenes.recovers_ground_truth_fixture()
    arr = getattr(p, field).copy()
    arr[0] = value
    setattr(p, field, arr)
    with pytest.raises(native.SfmbaError) as e:
        native.bundle_adjust_arrays(p)
    assert e.value.status == 1  # INVALID_ARGUMENT


def test_invalid_options_rejected():
    p = scenes.recovers_ground_truth_fixture()
    for kw in (dict(robust_loss=5), dict(max_iterations=-1), dict(precision=3), dict(initial_lambda=-1.0)):
        with pytest.raises(native.SfmbaError) as e:
            native.bundle_adjust_arrays(p, **kw)
        assert e.value.status == 1


def test_null_result_is_an_error():
    L = native.load()
    packed = abi.PackedProblem(scenes.recovers_ground_truth_fixture())
    o = abi.default_options()
    st = L.sfmba_bundle_adjust(C.byref(packed.struct), C.byref(o), None)
    assert st == 1
    assert b"NULL" in L.sfmba_last_error()


def test_batched_rejects_invalid_input_before_device():
    """The batched entry validates every window on the host first: a bad
    index in any window, a negative count or NULL arrays are errors, and the
    failing status is written into every window's result."""
    good = scenes.recovers_ground_truth_fixture()
    bad = scenes.recovers_ground_truth_fixture()
    arr = bad.obs_point.copy()
    arr[0] = 10**6
    bad.obs_point = arr
    with pytest.raises(native.SfmbaError) as e:
        native.bundle_adjust_batched_arrays([good, bad])
    assert e.value.status == 1
    L = native.load()
    o = abi.default_options()
    assert L.sfmba_bundle_adjust_batched(-1, None, C.byref(o), None) == 1
    assert L.sfmba_bundle_adjust_batched(2, None, C.byref(o), None) == 1
    packed = abi.PackedProblem(good)
    res = (abi.SfmbaResult * 1)()
    bad_opts = abi.default_options(robust_loss=9)
    assert L.sfmba_bundle_adjust_batched(1, C.byref(packed.struct), C.byref(bad_opts), res) == 1
    assert res[0].status == 1
    assert L.sfmba_bundle_adjust_batched(0, None, C.byref(o), None) == 0


def test_pnp_entries_reject_invalid_input_before_device():
    """Batch offsets must start at 0 and not decrease; counts and iteration
    limits must be non-negative; an empty batch is a no-op."""
    L = native.load()
    off_bad = np.array([0, 10, 5], np.int64)
    off_start = np.array([3, 10], np.int64)
    X = np.zeros((10, 3))
    uv = np.zeros((10, 2))
    poses = np.zeros((2, 7))
    found = np.zeros(2, np.int32)
    for off, n in ((off_bad, 2), (off_start, 1)):
        assert L.sfmba_pnp_ransac_batched(n, off.ctypes.data, X.ctypes.data, uv.ctypes.data, C.c_double(0.01),
                                          100, poses.ctypes.data, None, found.ctypes.data, None) == 1
        assert L.sfmba_refine_pose_gauss_newton_batched(n, off.ctypes.data, X.ctypes.data, uv.ctypes.data, 5,
                                                        poses.ctypes.data) == 1
    ok = np.array([0, 10], np.int64)
    assert L.sfmba_pnp_ransac_batched(1, ok.ctypes.data, X.ctypes.data, uv.ctypes.data, C.c_double(0.01), -1,
                                      poses.ctypes.data, None, found.ctypes.data, None) == 1
    assert L.sfmba_pnp_ransac_batched(1, ok.ctypes.data, X.ctypes.data, uv.ctypes.data, C.c_double(float("nan")),
                                      10, poses.ctypes.data, None, found.ctypes.data, None) == 1
    assert L.sfmba_refine_pose_gauss_newton_batched(1, ok.ctypes.data, X.ctypes.data, uv.ctypes.data, -2,
                                                    poses.ctypes.data) == 1
    assert L.sfmba_pnp_ransac_batched(-1, None, None, None, C.c_double(0.01), 10, None, None, None, None) == 1
    assert L.sfmba_pnp_ransac_batched(0, None, None, None, C.c_double(0.01), 10, None, None, None, None) == 0
    assert L.sfmba_refine_pose_gauss_newton_batched(0, None, None, None, 10, None) == 0


def test_adjust_global_rejects_unknown_mode_before_device():
    p = scenes.shared_ring(0, 0.05)
    with pytest.raises(native.SfmbaError) as e:
        native.adjust_global_arrays(p, 7, 4.0)
    assert e.value.status == 1
