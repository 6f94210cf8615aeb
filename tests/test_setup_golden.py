"""The float64 host setup of etalon_gb300.physics equals Etalon's, bit for bit.

Grid, ε maps, CPML profiles, injections, monitor samplings, the cast coefficient
arrays and the source/phasor tables of every fixture case are compared with the values
Etalon itself computed (tests/golden/make_golden.py).
"""

import numpy as np
import pytest

from etalon_gb300 import physics as ph
from tests import cases
from tests.golden_io import COEFFS, GOLDEN, count, load, sha

CASES = ["config1", "g4_full", "small"] + (["config2"] if (GOLDEN / "config2_single.npz").exists() else [])


def _check_setup(g, p, tables=True):
    grid = p.grid
    assert [grid.nx, grid.ny, grid.pml_layers] == list(g["grid"])
    np.testing.assert_array_equal(
        [grid.dx, grid.dy, grid.dt, grid.x_min, grid.y_min, grid.z, grid.courant], g["grid_f"]
    )
    for axis, c in (("x", p.cpml_x), ("y", p.cpml_y)):
        for name in ("b_e", "c_e", "inv_kappa_e", "b_h", "c_h", "inv_kappa_h"):
            np.testing.assert_array_equal(getattr(c, name), g[f"cpml_{axis}_{name}"], err_msg=f"{axis}.{name}")
    for comp in ("Ex", "Ey"):
        assert sha(p.eps[comp]) == str(g[f"eps_{comp}_sha"]), comp
    assert len(p.injections) == count(g, "src")
    for k, inj in enumerate(p.injections):
        assert inj.component == str(g[f"src{k}_component"])
        np.testing.assert_array_equal(inj.i, g[f"src{k}_i"])
        np.testing.assert_array_equal(inj.j, g[f"src{k}_j"])
        np.testing.assert_array_equal(inj.weights, g[f"src{k}_weights"])
        np.testing.assert_array_equal(inj.coefficient, g[f"src{k}_coef"])
    assert len(p.samplings) == count(g, "mon")
    for k, s in enumerate(p.samplings):
        assert s.component == str(g[f"mon{k}_component"])
        np.testing.assert_array_equal(s.flat_index, g[f"mon{k}_flat"])
        np.testing.assert_array_equal(s.frequencies, g[f"mon{k}_freq"])
    c = ph.cast_coefficients(p)
    for name in COEFFS:
        key = f"in_{name}"
        if key in g:
            np.testing.assert_array_equal(getattr(c, name), g[key], err_msg=name)
        else:
            assert sha(getattr(c, name)) == str(g[f"{key}_sha"]), name
    np.testing.assert_array_equal([c.db, c.inv_dx, c.inv_dy], g["in_scalars"])
    if not tables:
        return
    n = int(g["n_steps"])
    for k, inj in enumerate(p.injections):
        table = inj.delta_table(0, n, grid.dt, p.real)
        assert sha(table) == str(g[f"src{k}_table_sha"]), f"source {k} deltas"
    for k, s in enumerate(p.samplings):
        table = ph.phasor_table(s, 0, n, grid.dt, p.complex)
        assert sha(table) == str(g[f"mon{k}_table_sha"]), f"monitor {k} phasors"


@pytest.mark.parametrize("precision", ["single", "double"])
@pytest.mark.parametrize("name", CASES)
def test_setup_matches_reference(name, precision):
    g = load(name, precision)
    p = cases.CASES[name](precision=precision, n_steps=int(g["n_steps"]))
    _check_setup(g, p, tables=(name != "config2" or precision == "double"))


def test_config2_tables_match_reference_single():
    """The 10 000-step fp32 tables of the headline case (hash of every delta and phasor)."""
    if not (GOLDEN / "config2_single.npz").exists():
        pytest.skip("config2 fixture not generated")
    g = load("config2", "single")
    p = cases.config2("single")
    n = int(g["n_steps"])
    assert n == 10000
    for k, inj in enumerate(p.injections):
        assert sha(inj.delta_table(0, n, p.grid.dt, p.real)) == str(g[f"src{k}_table_sha"])
    for k, s in enumerate(p.samplings):
        assert sha(ph.phasor_table(s, 0, n, p.grid.dt, p.complex)) == str(g[f"mon{k}_table_sha"])


def test_monitor_nodes_are_rectangles():
    """Every sampling is a rectangle of consecutive nodes, which the fused kernels rely on."""
    for name in ("config1", "g4_full", "small"):
        for s in cases.CASES[name]().samplings:
            assert np.all(np.diff(s.x.index) == 1) and np.all(np.diff(s.y.index) == 1)
            flat = (s.x.index[:, None] * 0 + s.y.index[None, :]).ravel()
            assert flat.size == s.flat_index.size
