"""Monitor values pinned to Etalon's own ``monitor_dataarray`` (etalon/io/result.py:54-91).

The fixtures hold, per monitor component, the accumulator Etalon's NumPy run produced and
the value Etalon's ``monitor_dataarray`` reported for it (tests/golden/make_golden.py). Both
the result path (``solver.interpolate_monitor``) and the objective path
(``adjoint.point_value`` / ``point_power``, in torch) must give that value bit for bit, with
this package's own samplings (weights and node order). No GPU needed.
"""

import numpy as np
import pytest
import torch

from etalon_gb300.adjoint import point_power, point_value
from etalon_gb300.solver import interpolate_monitor
from tests import cases
from tests.golden_io import GOLDEN, count, load, sha

CASES = ["config1", "g4_full", "small", "config2"]
BUILDERS = {"config1": cases.config1, "g4_full": cases.g4_full, "small": cases.small,
            "config2": lambda precision: cases.config2(precision, n_steps=0)}  # fmt: skip


def _fixture(name, precision):
    if not (GOLDEN / f"{name}_{precision}.npz").exists():
        pytest.skip(f"no fixture {name}_{precision}")
    g = load(name, precision)
    if "out_value0_sha" not in g:
        pytest.skip("fixture without monitor values")
    return g


@pytest.mark.parametrize("precision", ["single", "double"])
@pytest.mark.parametrize("name", CASES)
def test_interpolate_monitor_equals_etalon(name, precision):
    g = _fixture(name, precision)
    p = BUILDERS[name](precision)
    checked = 0
    for k, s in enumerate(p.samplings):
        for axis, a in (("x", s.x), ("y", s.y)):
            key = f"mon{k}_{axis}w"
            assert (a.weights is None) == (key not in g), f"monitor {k}: {axis} interpolated on one side only"
            if a.weights is not None:
                np.testing.assert_array_equal(a.weights, g[key])
        if f"out_acc{k}" not in g:
            continue  # a large plane monitor: only hashes are kept (compared on the GPU)
        v = interpolate_monitor(s, g[f"out_acc{k}"])
        assert v.dtype == g[f"out_acc{k}"].dtype
        assert sha(v) == str(g[f"out_value{k}_sha"]), f"monitor {k} ({s.monitor}/{s.component})"
        dims = [d for d, a in (("x", s.x), ("y", s.y)) if a.weights is None] + ["wavelength"]
        assert ",".join(dims) == str(g[f"out_value{k}_dims"])
        checked += 1
    assert checked == sum(f"out_acc{k}" in g for k in range(count(g, "mon"))) >= 1


@pytest.mark.parametrize("precision", ["single", "double"])
@pytest.mark.parametrize("name", CASES)
def test_point_value_equals_etalon(name, precision):
    """The objective sees Etalon's monitor value: the torch contraction gives its bits."""
    g = _fixture(name, precision)
    p = BUILDERS[name](precision)
    checked = 0
    for k, s in enumerate(p.samplings):
        if f"out_acc{k}" not in g or f"out_value{k}" not in g:
            continue
        acc = g[f"out_acc{k}"]
        t = torch.as_tensor(np.stack([acc.real, acc.imag], -1).astype(np.float64))
        re, im = point_value(t, s)
        v = (re.numpy() + 1j * im.numpy())
        v = np.moveaxis(v, 0, -1).astype(acc.dtype)
        want = g[f"out_value{k}"]
        assert v.shape == want.shape
        assert np.array_equal(np.ascontiguousarray(v).view(np.uint8), np.ascontiguousarray(want).view(np.uint8)), (
            f"monitor {k}")
        j = float(point_power(t, s))
        w64 = (re.numpy() + 1j * im.numpy())
        assert j == pytest.approx(float((np.abs(w64) ** 2).sum()), rel=1e-14)  # Σ_f |F|², any order
        checked += 1
    assert checked >= 1
