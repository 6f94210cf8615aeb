"""Drop-in wiring into Etalon: the problem Etalon's own setup builds equals this package's.

Runs where Etalon's source tree can be imported (it needs pydantic and a stub xarray);
skipped elsewhere. No GPU needed: only host setup and backend selection are checked.
"""

import math
import os
import sys
import types

import numpy as np
import pytest

from etalon_gb300 import physics as ph
from tests import cases

def _etalon_tree() -> str:
    """Etalon's source tree: $ETALON_SRC, else the checkout the oracle's build recipe reads."""
    from oracle import build_ref

    return os.environ.get("ETALON_SRC") or str(build_ref.DEFAULT_TREE)


REF = _etalon_tree()


@pytest.fixture(scope="module")
def et():
    if not os.path.isdir(os.path.join(REF, "etalon")):
        pytest.skip("Etalon source tree not available")
    pytest.importorskip("pydantic")
    if REF not in sys.path:
        sys.path.insert(0, REF)
    if "xarray" not in sys.modules:
        stub = types.ModuleType("xarray")
        stub.DataArray = object
        sys.modules["xarray"] = stub
    import etalon

    return etalon


def _sims(et):
    g = et.GaussianPulse
    config1 = et.Simulation(
        size=(8.0, 8.0, 0.0), grid=et.UniformGrid(dl=0.05), boundary=et.PML(layers=12),
        sources=[et.PointSource(center=(-3.0, 0.0, 0.0), component="Hz", pulse=g(wavelength=1.55, bandwidth=0.5))],
        monitors=[et.DFTMonitor(name="probe", center=(3.0, 0.0, 0.0), wavelengths=list(np.linspace(1.3, 1.8, 5)))],
        run_time=1.0, backend="numpy")  # fmt: skip
    config2 = et.Simulation(
        size=(40.0, 40.0, 0.0), grid=et.UniformGrid(dl=0.02), medium=et.Medium(n=math.sqrt(2.085)),
        structures=[et.Box(center=(0, 0, 0), size=(42.0, 0.5, 0.22), medium=et.Medium(n=math.sqrt(12.11)))],
        sources=[et.PointSource(center=(-15.0, 0.0, 0.0), component="Hz", pulse=g(wavelength=1.55, bandwidth=0.5))],
        monitors=[et.DFTMonitor(name=f"m{k}", center=(x, 0.0, 0.0), wavelengths=list(np.linspace(1.5, 1.6, 16)))
                  for k, x in enumerate((-5.0, 5.0, 15.0))],
        run_time=1.0, backend="numpy")  # fmt: skip
    return {"config1": config1, "config2": config2}


@pytest.mark.parametrize("name", ["config1", "config2"])
def test_problem_from_simulation_equals_own_setup(et, name):
    from etalon_gb300.compat import problem_from_simulation

    a = problem_from_simulation(_sims(et)[name])
    b = cases.CASES[name]()
    assert a.grid == b.grid
    for c in ("Ex", "Ey"):
        np.testing.assert_array_equal(a.eps[c], b.eps[c])
    ca, cb = ph.cast_coefficients(a), ph.cast_coefficients(b)
    for k, v in vars(ca).items():
        np.testing.assert_array_equal(v, getattr(cb, k), err_msg=k)
    for x, y in zip(a.injections, b.injections, strict=True):
        np.testing.assert_array_equal(x.coefficient, y.coefficient)
        np.testing.assert_array_equal(x.delta_table(0, 50, a.grid.dt, a.real), y.delta_table(0, 50, b.grid.dt, b.real))
    for x, y in zip(a.samplings, b.samplings, strict=True):
        assert (x.monitor, x.component) == (y.monitor, y.component)
        np.testing.assert_array_equal(x.flat_index, y.flat_index)
        np.testing.assert_array_equal(ph.phasor_table(x, 0, 20, a.grid.dt, a.complex),
                                      ph.phasor_table(y, 0, 20, b.grid.dt, b.complex))  # fmt: skip


def test_install_routes_backends(et, monkeypatch):
    """After install(): numpy stays NumPy; cuda never falls back silently; auto falls back without a GPU."""
    import etalon.fdtd.backends as backends
    import etalon.fdtd.solver as solver_module
    from etalon.fdtd.backends.numpy_backend import NumpyBackend

    from etalon_gb300 import compat

    monkeypatch.setattr(backends, "get_backend", backends.get_backend)
    monkeypatch.setattr(solver_module, "get_backend", solver_module.get_backend)
    monkeypatch.setattr(solver_module, "run", solver_module.run)
    monkeypatch.setattr(compat, "gpu_available", lambda: False)
    compat.install()
    assert isinstance(backends.get_backend("numpy", "single"), NumpyBackend)
    assert isinstance(backends.get_backend("auto", "single"), NumpyBackend)
    with pytest.raises(RuntimeError, match="cuda"):
        backends.get_backend("cuda", "single")
    with pytest.raises(ValueError, match="unknown backend"):
        backends.get_backend("metal", "single")


def test_install_fused_solver_routes_stepped_solvers(et, monkeypatch):
    """install(fused_solver=True): FDTDSolver(sim) — what Studio's runner builds — is the fused
    engine's solver for GPU backends and Etalon's own for NumPy."""
    import etalon.fdtd.backends as backends
    import etalon.fdtd.solver as solver_module

    from etalon_gb300 import compat

    for name in ("get_backend", "run", "FDTDSolver"):
        monkeypatch.setattr(solver_module, name, getattr(solver_module, name))
    monkeypatch.setattr(backends, "get_backend", backends.get_backend)
    plain = solver_module.FDTDSolver
    built = []

    class FakeFused:
        def __init__(self, sim):
            built.append(sim.backend)

    monkeypatch.setattr(compat, "GB300FDTDSolver", FakeFused)
    monkeypatch.setattr(compat, "gpu_available", lambda: True)
    compat.install(fused_solver=True)
    compat.install(fused_solver=True)  # twice: still wraps Etalon's own class
    sims = _sims(et)
    assert isinstance(solver_module.FDTDSolver(sims["config1"].model_copy(update={"backend": "cuda"})), FakeFused)
    assert isinstance(solver_module.FDTDSolver(sims["config1"].model_copy(update={"backend": "auto"})), FakeFused)
    assert built == ["cuda", "auto"]
    assert isinstance(solver_module.FDTDSolver(sims["config1"]), plain)
