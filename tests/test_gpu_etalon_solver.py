"""Etalon's solver-level entry points on the GPU (needs a GPU).

* Etalon's own ``FDTDSolver`` driving ``Gb300Backend``: the recorded protocol traces of
  Etalon's unchanged solver (tests/etalon_trace.py) replayed call for call — Etalon's G4
  (600 steps of its GPU parity simulation) and G4b (``run()`` of a run shorter than a
  phasor chunk, to its end) — must end with Etalon's arrays, bit for bit. Etalon itself
  (pydantic, its source tree) is not importable on the GPU machine, so its calls are replayed.
* ``GB300Solver`` (Etalon's FDTDSolver interface over the resident engine): ``run()``,
  ``fields()`` and ``result()`` on Etalon's inputs give Etalon's fields and accumulators bit
  for bit, and the monitor values of Etalon's ``monitor_dataarray`` (etalon/io/result.py:54-91):
  bit for bit against its float64 interpolation of Etalon's accumulators on the same machine
  (NumPy's einsum and matmul round their two-term sums differently on x86 and Arm), within a
  few ulp of the values Etalon reported on the machine that made the fixtures.
* Etalon's G5 (``auto`` picks the GPU; the result's metadata names "cuda" and ``cuda:0``),
  its result layout per monitor type and its point-versus-plane interpolation check
  (tests/unit/test_solver.py:34-79), on the GPU solver.
"""

from __future__ import annotations

import numpy as np
import pytest

from etalon_gb300 import physics as ph
from etalon_gb300.solver import GB300Solver, interpolate_monitor
from tests import cases
from tests import etalon_trace as tr
from tests.golden_io import FIELDS, compare_outputs, count, load, sha
from tests.test_gpu_parity import golden_coeffs

pytestmark = pytest.mark.gpu
PRECISIONS = ["single", "double"]


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("name", ["g4_full", "small"])
def test_etalon_solver_trace_on_gb300_backend(gpu, name, precision):
    """Every call Etalon's FDTDSolver made (g4_full: 600 × step() then fields(); small: run()
    to its end), replayed on Gb300Backend, ends with Etalon's arrays bit for bit."""
    from etalon_gb300.backend import Gb300Backend

    t = tr.load_trace(name, precision)
    r = tr.Replay(Gb300Backend(precision), t).run()
    assert r.mismatches() == []
    assert r.calls[tr.OP_UPDATE_H] == int(t["n_steps"])


def _solver_on_reference_inputs(name, precision, g, **kw):
    n = int(g["n_steps"])
    s = GB300Solver(cases.CASES[name](precision=precision, n_steps=n), **kw)
    s.engine.set_coefficients(golden_coeffs(g))
    for k in range(count(g, "src")):
        s.engine.set_source_table(k, 0, g[f"src{k}_table"])
    for k in range(count(g, "mon")):
        s.engine.set_phasor_table(k, 0, g[f"mon{k}_table"])
    return s, n


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("name", ["config1", "g4_full", "small"])
def test_gb300_solver_run_result_matches_etalon(gpu, name, precision):
    g = load(name, precision)
    s, n = _solver_on_reference_inputs(name, precision, g)
    res = s.run()
    assert s.n == n and res.metadata["n_steps"] == n
    fields = {f: s.engine.field(f) for f in FIELDS}
    accs = [m.acc for m in s.monitors]
    assert compare_outputs(g, fields, accs) == []
    host = s.fields()
    for comp, f in (("Ex", "ex"), ("Ey", "ey"), ("Hz", "hz")):
        assert np.array_equal(host[comp], fields[f])
    for k, m in enumerate(s.monitors):
        v = res[m.sampling.monitor][m.sampling.component]
        label = f"monitor value {k} ({m.sampling.monitor}/{m.sampling.component})"
        if f"out_acc{k}" in g:
            # Etalon's float64 interpolation is NumPy einsum and matmul, whose last bits depend on
            # the machine's BLAS: bit for bit against Etalon's accumulators interpolated here,
            # and within a few ulp of the value Etalon reported on the machine that ran it
            assert np.array_equal(v, interpolate_monitor(m.sampling, g[f"out_acc{k}"])), label
            want = g[f"out_value{k}"]
            tol = 4 * np.finfo(want.real.dtype).eps * np.abs(want).max()
            assert np.abs(v - want).max() <= tol, label
        else:  # large plane monitors: no interpolation, so the bits are the platform's too
            assert sha(v) == str(g[f"out_value{k}_sha"]), label
    assert res.metadata["backend"] == "cuda"
    assert res.metadata["device"].startswith("cuda:0")
    assert res.metadata["precision"] == precision
    s.close()


@pytest.mark.parametrize("precision", PRECISIONS)
def test_gb300_solver_short_run_own_setup_vs_live_oracle(gpu, precision):
    """G4b on the resident solver: Etalon's short case run() to its end with this package's own
    host setup, against the oracle run here on the same problem; the result values are the
    interpolation of the oracle's accumulators."""
    from oracle.te_numpy import OracleMonitor, OracleSource, OracleTE

    p = cases.small(precision)
    s = GB300Solver(p)
    res = s.run()
    assert s.n == p.n_steps
    c = vars(ph.cast_coefficients(p))
    o = OracleTE(p.grid.nx, p.grid.ny, p.grid.dt, c, p.real,
                 [OracleSource(i.component, i.i, i.j, i.coefficient,
                               (i.pulse.wavelength, i.pulse.bandwidth, i.pulse.amplitude))
                  for i in p.injections],
                 [OracleMonitor(m.component, m.flat_index, m.frequencies) for m in p.samplings])  # fmt: skip
    o.run(p.n_steps)
    for k, m in enumerate(s.monitors):
        assert np.array_equal(m.acc, o.acc[k])
        want = interpolate_monitor(m.sampling, o.acc[k])
        assert np.array_equal(res[m.sampling.monitor][m.sampling.component], want)
        assert np.abs(want).max() > 0
    s.close()


def test_g5_auto_picks_the_gpu(gpu):
    """Etalon's G5: "auto" selects the GPU backend, named "cuda", and a run's metadata says so."""
    from etalon_gb300 import compat

    class NumpyStandIn:
        name = "numpy"

    assert compat.uses_gpu("auto") and compat.uses_gpu("cuda") and not compat.uses_gpu("numpy")
    b = compat.select_backend("auto", "single", NumpyStandIn)
    assert b.name == "cuda" and b.device.startswith("cuda:0")
    assert isinstance(compat.select_backend("numpy", "single", NumpyStandIn), NumpyStandIn)
    with pytest.raises(ValueError, match="unknown backend"):
        compat.select_backend("metal", "single", NumpyStandIn)
    p = cases.small("single")
    p.n_steps = p.grid.n_steps(5e-15)
    res = GB300Solver(p).run()
    assert res.metadata["backend"] == "cuda"
    assert res.metadata["device"].startswith("cuda:0")
    assert res.metadata["n_steps"] == p.n_steps > 0


def _small_with(monitors, precision="single"):
    """Etalon's small_sim (tests/sims.py:12-24) with other monitors."""
    return ph.te_problem(size=(2.0, 1.5), dl=0.05, pml=ph.PMLSpec(layers=8),
                         sources=[ph.PointSource((-0.5, 0.1, 0.0), "Hz", ph.GaussianPulse(1.55, 0.5))],
                         monitors=monitors, run_time=20e-15, precision=precision)  # fmt: skip


def test_result_layout_per_monitor_type(gpu):
    """Etalon's tests/unit/test_solver.py:34-66 on the GPU solver: point → (n_f,), line along x →
    (nodes, n_f), plane → (x nodes, y nodes, n_f) over the region inside the CPML; complex64."""
    wls = [1.5, 1.55, 1.6]
    p = _small_with([
        ph.DFTMonitor("point", wls, center=(0.31, 0.12, 0.0)),
        ph.DFTMonitor("line", wls, center=(0.0, 0.1, 0.0), size=(0.6, 0.0, 0.0)),
        ph.DFTMonitor("plane", wls, size=(2.0, 1.5, 0.0), components=("Hz",)),
    ])  # fmt: skip
    res = GB300Solver(p).run()
    assert res.monitors == ["point", "line", "plane"]
    point = res["point"]["Ey"]
    assert point.shape == (3,) and point.dtype == np.complex64
    line = res["line"]["Hz"]
    xs = [s for s in p.samplings if s.monitor == "line" and s.component == "Hz"][0].x.coords
    assert line.shape == (xs.size, 3) and np.all(np.abs(xs) <= 0.3 + 1e-9)
    assert set(res["plane"]) == {"Hz"}
    region = p.grid.pml_layers
    assert res["plane"]["Hz"].shape == (p.grid.nx - 2 * region, p.grid.ny - 2 * region, 3)
    with pytest.raises(KeyError, match="no monitor named 'nope'"):
        res["nope"]
    assert res.metadata["backend"] == "cuda"
    assert res.metadata["n_steps"] == p.grid.n_steps(20e-15)


def test_point_monitor_interpolation_matches_plane_nodes(gpu):
    """Etalon's tests/unit/test_solver.py:69-79 on the GPU solver: the point monitor equals
    bilinear interpolation of the same run's plane monitor (float64, rel 1e-12)."""
    p = _small_with([
        ph.DFTMonitor("point", [1.55], center=(0.31, 0.12, 0.0), components=("Hz",)),
        ph.DFTMonitor("plane", [1.55], size=(2.0, 1.5, 0.0), components=("Hz",)),
    ], precision="double")  # fmt: skip
    res = GB300Solver(p).run()
    plane = res["plane"]["Hz"][..., 0]
    ps = [s for s in p.samplings if s.monitor == "plane"][0]
    x, y = ps.x.coords, ps.y.coords
    i = int(np.searchsorted(x, 0.31)) - 1
    j = int(np.searchsorted(y, 0.12)) - 1
    tx = (0.31 - x[i]) / (x[i + 1] - x[i])
    ty = (0.12 - y[j]) / (y[j + 1] - y[j])
    expected = ((1 - tx) * (1 - ty) * plane[i, j] + tx * (1 - ty) * plane[i + 1, j]
                + (1 - tx) * ty * plane[i, j + 1] + tx * ty * plane[i + 1, j + 1])  # fmt: skip
    got = complex(res["point"]["Hz"][0])
    assert abs(expected) > 0
    assert got == pytest.approx(complex(expected), rel=1e-12)
