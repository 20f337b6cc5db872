"""The double-float arithmetic of the FP32 path's cost (dfloat.cuh), built
for the host and checked against exact rational arithmetic on seeded random
pairs, including near-cancelling sums. Bars: every result normalised
(|lo| <= 2^-24 |hi|); relative error of a split <= 2^-47, of a sum or
product <= 2^-45, of a reciprocal <= 2^-44 (the published bounds for these
algorithms are a few 2^-48)."""
import ctypes as C
import os
import shutil
import subprocess
from fractions import Fraction

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "sfmtory_gb300", "csrc")


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    out = str(tmp_path_factory.mktemp("dfloat") / "libdfhost.so")
    cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I", CSRC,
           "-I", os.path.join(cuda, "include"), os.path.join(HERE, "dfloat_host.cpp"), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    L = C.CDLL(out)
    f2 = C.POINTER(C.c_float)
    L.h_df_from.argtypes = [C.c_double, f2]
    for name in ("h_df_add", "h_df_mul"):
        getattr(L, name).argtypes = [C.c_float] * 4 + [f2]
    L.h_df_recip.argtypes = [C.c_float, C.c_float, f2]
    return L


def _call(fn, *args):
    out = (C.c_float * 2)()
    fn(*args, out)
    return float(out[0]), float(out[1])


def _exact(hi, lo):
    return Fraction(hi) + Fraction(lo)


def _normalised(hi, lo):
    return abs(lo) <= abs(hi) * 2.0 ** -24


def _pairs(lib, rng, n):
    mags = 2.0 ** rng.integers(-20, 20, n)
    xs = rng.uniform(-1.0, 1.0, n) * mags
    return [_call(lib.h_df_from, float(x)) for x in xs], xs


def test_split(lib):
    rng = np.random.default_rng(1)
    pairs, xs = _pairs(lib, rng, 2000)
    for (h, l), x in zip(pairs, xs):
        assert _normalised(h, l)
        assert abs(_exact(h, l) - Fraction(float(x))) <= abs(Fraction(float(x))) * Fraction(2) ** -47


@pytest.mark.parametrize("op", ["add", "mul"])
def test_add_mul(lib, op):
    rng = np.random.default_rng(2 if op == "add" else 3)
    a, _ = _pairs(lib, rng, 2000)
    b, _ = _pairs(lib, rng, 2000)
    if op == "add":  # near-cancelling sums: b = -(a + a tiny relative change)
        for k in range(0, 2000, 4):
            h, l = a[k]
            b[k] = _call(lib.h_df_from, -float(np.float64(h) + np.float64(l)) * (1.0 + 1e-9 * (k + 1)))
    fn = lib.h_df_add if op == "add" else lib.h_df_mul
    for (ah, al), (bh, bl) in zip(a, b):
        rh, rl = _call(fn, ah, al, bh, bl)
        exact = _exact(ah, al) + _exact(bh, bl) if op == "add" else _exact(ah, al) * _exact(bh, bl)
        assert _normalised(rh, rl), (ah, al, bh, bl, rh, rl)
        assert abs(_exact(rh, rl) - exact) <= abs(exact) * Fraction(2) ** -45, (ah, al, bh, bl)


def test_reciprocal(lib):
    rng = np.random.default_rng(4)
    a, _ = _pairs(lib, rng, 2000)
    for ah, al in a:
        if ah == 0.0:
            continue
        rh, rl = _call(lib.h_df_recip, ah, al)
        exact = 1 / _exact(ah, al)
        assert _normalised(rh, rl)
        assert abs(_exact(rh, rl) - exact) <= abs(exact) * Fraction(2) ** -44, (ah, al)
