"""The lean interior update drops Etalon's `+ 0` CPML terms; checked exhaustively on the CPU.

Inside the unit rectangle c = 0, b = 1 and 1/kappa = 1, so Etalon's Hz update
(``numpy_backend.py:41-49``) computes hz + db·((d_y·1 + (1·psi + 0·d_y)) − (d_x·1 + (1·psi +
0·d_x))) with psi = +0, and its E updates (``numpy_backend.py:51-61``) ex + cb·(d·1 + (1·psi +
0·d)) and ey − cb·(d·1 + ...). The interior tiles compute hz + db·(d_y − d_x), ex + cb·d and
ey − cb·d instead, whenever no field value they load is −0. Over every combination of a value
set (zeros, equal neighbours, signs, subnormals) both forms give the same bits when the set has
no −0, in float32 and float64; with −0 in the set some combination differs, which is why a tile
that loads a −0 keeps Etalon's form.
"""

import itertools
from types import SimpleNamespace

import numpy as np
import pytest

from oracle.te_numpy import update_e, update_h


def values(dtype, with_negative_zero):
    tiny = np.finfo(dtype).smallest_subnormal
    v = [0.0, 1.0, -1.0, 0.5, 3.0, tiny, -tiny, 1.0 + np.finfo(dtype).eps]
    if with_negative_zero:
        v.append(-0.0)
    return np.array(v, dtype=dtype)


def combos(v, n):
    return [np.array(c, dtype=v.dtype) for c in zip(*itertools.product(v, repeat=n))]


def etalon_hz(hz, ex0, ex1, ey0, ey1, db, inv):
    """Etalon's Hz update of one interior cell, operation for operation (psi = +0, b = 1, c = 0)."""
    t = hz.dtype.type
    one, zero, psi = t(1), t(0), t(0)
    dy = (ex1 - ex0) * inv
    dx = (ey1 - ey0) * inv
    py = one * psi + zero * dy
    px = one * psi + zero * dx
    return hz + db * ((dy * one + py) - (dx * one + px))


def etalon_e(f, h0, h1, cb, inv, sign):
    t = f.dtype.type
    one, zero, psi = t(1), t(0), t(0)
    d = (h1 - h0) * inv
    p = one * psi + zero * d
    return f + cb * (d * one + p) if sign > 0 else f - cb * (d * one + p)


def same_bits(a, b):
    a, b = np.atleast_1d(a), np.atleast_1d(b)
    return a.dtype == b.dtype and np.array_equal(a.view(np.uint8), b.view(np.uint8))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_the_restated_expressions_are_the_oracles(dtype):
    """The one-cell expressions above equal the oracle's whole-array updates on an interior cell."""
    rng = np.random.default_rng(3)
    t = np.dtype(dtype).type
    s = SimpleNamespace(db=t(0.37), inv_dx=t(1.7), inv_dy=t(1.7))
    s.hz = rng.standard_normal((3, 3)).astype(dtype)
    s.ex = rng.standard_normal((3, 4)).astype(dtype)
    s.ey = rng.standard_normal((4, 3)).astype(dtype)
    s.cb_ex, s.cb_ey = (rng.uniform(0.2, 0.5, a.shape).astype(dtype) for a in (s.ex, s.ey))
    for name, like in (("psi_hz_x", s.hz), ("psi_hz_y", s.hz), ("psi_ex_y", s.ex), ("psi_ey_x", s.ey)):
        setattr(s, name, np.zeros_like(like))
    for axis, n in (("x", 3), ("y", 3)):
        for pos, m in (("h", n), ("e", n + 1)):
            setattr(s, f"b{axis}_{pos}", np.ones(m, dtype))
            setattr(s, f"c{axis}_{pos}", np.zeros(m, dtype))
            setattr(s, f"ik{axis}_{pos}", np.ones(m, dtype))
    hz = etalon_hz(s.hz[1, 1], s.ex[1, 1], s.ex[1, 2], s.ey[1, 1], s.ey[2, 1], s.db, s.inv_dx)
    update_h(s)
    assert same_bits(np.asarray(hz), np.asarray(s.hz[1, 1]))
    ex = etalon_e(s.ex[1, 1], s.hz[1, 0], s.hz[1, 1], s.cb_ex[1, 1], s.inv_dy, +1)
    ey = etalon_e(s.ey[1, 1], s.hz[0, 1], s.hz[1, 1], s.cb_ey[1, 1], s.inv_dx, -1)
    update_e(s)
    assert same_bits(np.asarray(ex), np.asarray(s.ex[1, 1]))
    assert same_bits(np.asarray(ey), np.asarray(s.ey[1, 1]))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_dropping_the_zero_terms_is_exact_without_negative_zero(dtype):
    t = np.dtype(dtype).type
    db, cb, inv = t(0.37), t(0.29), t(1.7)
    hz, ex0, ex1, ey0, ey1 = combos(values(dtype, False), 5)
    assert same_bits(etalon_hz(hz, ex0, ex1, ey0, ey1, db, inv), hz + db * ((ex1 - ex0) * inv - (ey1 - ey0) * inv))
    f, h0, h1 = combos(values(dtype, False), 3)
    assert same_bits(etalon_e(f, h0, h1, cb, inv, +1), f + cb * ((h1 - h0) * inv))
    assert same_bits(etalon_e(f, h0, h1, cb, inv, -1), f - cb * ((h1 - h0) * inv))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_a_negative_zero_can_change_the_bits(dtype):
    t = np.dtype(dtype).type
    db, inv = t(0.37), t(1.7)
    hz, ex0, ex1, ey0, ey1 = combos(values(dtype, True), 5)
    full = etalon_hz(hz, ex0, ex1, ey0, ey1, db, inv)
    lean = hz + db * ((ex1 - ex0) * inv - (ey1 - ey0) * inv)
    assert not same_bits(full, lean)
    assert np.array_equal(full, lean)  # equal as numbers: only the sign of a zero differs
