"""The oracle is pinned to Etalon: on the fixture inputs it reproduces Etalon's outputs bit for bit.

The fixtures were written by tests/golden/make_golden.py, which runs Etalon's own
NumpyBackend / FDTDSolver. The oracle is then trusted as the checker of the CUDA path.
"""

import numpy as np
import pytest

from tests import cases
from tests.golden_io import FIELDS, compare_outputs, load, oracle_from_golden, sha

PRECISIONS = ["single", "double"]


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("name", ["config1", "g4_full", "small"])
def test_oracle_reproduces_reference_run(name, precision):
    g = load(name, precision)
    o = oracle_from_golden(g, precision)
    o.run(int(g["n_steps"]))
    assert np.abs(o.hz).max() > 0
    assert compare_outputs(g, o.fields(), o.acc) == []


@pytest.mark.parametrize("precision", PRECISIONS)
def test_oracle_own_tables_equal_reference_tables(precision):
    """Per-step deltas and phasors evaluated by the oracle equal Etalon's, bit for bit."""
    g = load("g4_full", precision)
    o = oracle_from_golden(g, precision)
    for s in o.sources:
        table, s.table = s.table, None
        own = np.stack([o.delta(s, n) for n in range(table.shape[0])])
        np.testing.assert_array_equal(own, table)
    for m in o.monitors:
        table, m.table = m.table, None
        own = np.stack([o.phasor(m, n) for n in range(0, table.shape[0], 37)])
        np.testing.assert_array_equal(own, table[::37])


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("update", ["update_h_te", "update_e_te"])
def test_oracle_kernels_on_random_state(precision, update):
    """Etalon's random 67×53 state with live CPML everywhere (its GPU tests G1/G2)."""
    from oracle import te_numpy

    dtype = np.float32 if precision == "single" else np.float64
    g = load("kernels", precision)
    grid, c, fields = cases.random_state_inputs(dtype)
    for f in FIELDS:
        assert sha(fields[f]) == str(g[f"{update}_in_{f}_sha"]), f"regenerated input {f} differs"
    s = _state(grid, c, fields)
    {"update_h_te": te_numpy.update_h, "update_e_te": te_numpy.update_e}[update](s)
    for f in FIELDS:
        assert sha(getattr(s, f)) == str(g[f"{update}_out_{f}_sha"]), f


@pytest.mark.parametrize("precision", PRECISIONS)
def test_oracle_dft_kernel(precision):
    from oracle import te_numpy

    dtype = np.float32 if precision == "single" else np.float64
    g = load("kernels", precision)
    field, index, phasors, acc = cases.dft_inputs(dtype)
    te_numpy.accumulate_dft(acc, field, index, phasors)
    assert sha(acc) == str(g["dft_out_acc_sha"])


def test_oracle_row_bands_equal_whole_arrays():
    """The threaded CPU baseline updates row bands; values equal the whole-array update."""
    from concurrent.futures import ThreadPoolExecutor

    g = load("g4_full", "single")
    a, b = oracle_from_golden(g, "single"), oracle_from_golden(g, "single")
    with ThreadPoolExecutor(4) as pool:
        for _ in range(50):
            a.step()
            b.step(pool=pool, bands=7)
    for f in FIELDS:
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f))
    for x, y in zip(a.acc, b.acc):
        np.testing.assert_array_equal(x, y)


class _State:
    pass


def _state(grid, c, fields):
    s = _State()
    s.nx, s.ny = grid.nx, grid.ny
    for k, v in vars(c).items():
        setattr(s, k, v)
    for k, v in fields.items():
        setattr(s, k, v.copy())
    return s
