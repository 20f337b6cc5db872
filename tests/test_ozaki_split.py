"""The arithmetic of the tensor-core Cholesky update (ozaki.cuh) restated in
numpy: per-row power-of-two scaling, seven 8-bit slices, the 28 slice
products with i + j <= 8 accumulated in FP32 per weight, the exact 64-bit
integer combination of the weights up to 6 and the FP32 fold of the two
smallest. Checked against exact rational arithmetic: the update
P_R P_C^T is reproduced to FP64 accuracy (error below 2^-49 of
max|P_r| max|P_c| times the panel width, and below 8 ulp of the FP64
product in the typical entry).

The slices are exact integers below 256 (BF16 values) and every group
sum of weight <= 5 stays below 2^24, which is what makes the FP32
accumulation of the tensor cores exact; both are asserted here."""
from fractions import Fraction

import numpy as np


def split(P, slices=7):
    m = np.abs(P).max(axis=1)
    e = np.where(m > 0, np.frexp(m)[1], 0)
    x = np.ldexp(P, -e[:, None])
    out = []
    for _ in range(slices):
        y = x * 256.0
        s = np.trunc(y)
        x = y - s
        out.append(s)
    return out, e


def update(PR, PC):
    SR, eR = split(PR)
    SC, eC = split(PC)
    for s in SR + SC:
        assert np.all(np.abs(s) <= 255) and np.all(s == np.round(s))
    G = {}
    for d in range(8, 1, -1):
        g = np.zeros((len(PR), len(PC)), np.float32)
        for i in range(max(1, d - 7), min(7, d - 1) + 1):
            g = (g + SR[i - 1].astype(np.float32) @ SC[d - i - 1].T.astype(np.float32)).astype(np.float32)
        if d <= 5:
            assert np.all(np.abs(g) < 2 ** 24)
        G[d] = g
    L = G[2].astype(np.int64)
    for d in (3, 4, 5, 6):
        L = L * 256 + G[d].astype(np.int64)
    assert np.all(np.abs(L) < 2 ** 55)
    T = (G[8] * np.float32(1 / 256) + G[7]).astype(np.float32)
    v = T.astype(np.float64) / 256.0 + L.astype(np.float64)
    return v * np.ldexp(1.0, eR[:, None] - 48) * np.ldexp(1.0, eC[None, :])


def test_update_matches_exact_products():
    rng = np.random.default_rng(7)
    for scale_decades in (0.0, 4.0):
        PR = rng.standard_normal((24, 64)) * 10.0 ** rng.uniform(-scale_decades, scale_decades, (24, 1))
        PC = rng.standard_normal((20, 64)) * 10.0 ** rng.uniform(-scale_decades, scale_decades, (20, 1))
        got = update(PR, PC)
        ref64 = PR @ PC.T
        for r in range(0, 24, 5):
            for c in range(0, 20, 3):
                exact = sum(Fraction(PR[r, t]) * Fraction(PC[c, t]) for t in range(64))
                scale = float(np.abs(PR[r]).max() * np.abs(PC[c]).max()) * 64
                assert abs(float(Fraction(got[r, c]) - exact)) <= 2.0 ** -49 * scale
                # FP64's own rounding of the same product is of the same order
                assert abs(float(Fraction(ref64[r, c]) - exact)) <= 2.0 ** -49 * scale
        typical = np.median(np.abs(got - ref64) / np.abs(ref64).clip(1e-300))
        assert typical < 8 * 2.0 ** -52


def test_zero_rows_give_zero_update():
    PR = np.zeros((3, 64))
    PR[1, 5] = 3.0
    PC = np.ones((2, 64))
    got = update(PR, PC)
    assert got[0].tolist() == [0.0, 0.0] and got[2].tolist() == [0.0, 0.0]
    assert got[1].tolist() == [3.0, 3.0]
