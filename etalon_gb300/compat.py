"""Drop-in wiring into an installed Etalon (``import etalon``).

* ``problem_from_simulation(sim)`` resolves an ``etalon.Simulation`` with Etalon's own
  host setup — build_yee_grid, permittivity_on_nodes, cpml_axis, point_injection,
  monitor_samplings (etalon/fdtd/solver.py:55-81) — so the GPU consumes exactly the
  float64 arrays Etalon's NumPy backend would.
* ``GB300FDTDSolver(sim)`` is Etalon's FDTDSolver interface (step, run, fields, result,
  n, n_steps, grid, monitors, backend) over the fused resident engine.
* ``install()`` makes ``backend="cuda"`` (and ``"auto"`` on a GPU machine) use this
  backend: ``get_backend`` returns ``Gb300Backend`` for the per-step protocol, and
  ``Simulation.run`` goes through ``GB300FDTDSolver``. ``Simulation.backend`` is a
  ``Literal["auto", "numpy", "cuda"]`` (etalon/core/simulation.py:63), so the backend
  takes over the "cuda" name rather than adding one.
"""

from __future__ import annotations

import time
from typing import Any

from . import physics as ph
from .solver import GB300Solver, __version__


def _pulse(p) -> ph.GaussianPulse:
    return ph.GaussianPulse(p.wavelength, p.bandwidth, p.amplitude)


def problem_from_simulation(sim) -> ph.TEProblem:
    """A TEProblem built by Etalon's own setup functions (bit-identical float64 inputs)."""
    from etalon.fdtd.capabilities import check_supported
    from etalon.fdtd.cpml import cpml_axis
    from etalon.fdtd.dft import monitor_samplings
    from etalon.fdtd.sources import point_injection
    from etalon.grid.materials import permittivity_on_nodes
    from etalon.grid.yee import build_yee_grid

    check_supported(sim)
    g = build_yee_grid(sim)
    grid = ph.YeeGrid2D(g.nx, g.ny, g.dx, g.dy, g.dt, g.pml_layers, g.x_min, g.y_min, g.z, g.courant)
    eps = permittivity_on_nodes(sim, g)
    bg = sim.medium.permittivity
    cx = cpml_axis(g.nx, g.dx, g.dt, sim.boundary, bg)
    cy = cpml_axis(g.ny, g.dy, g.dt, sim.boundary, bg)
    axis = lambda c: ph.CPMLAxis(c.b_e, c.c_e, c.inv_kappa_e, c.b_h, c.c_h, c.inv_kappa_h)  # noqa: E731
    injections = []
    for source in sim.sources:
        inj = point_injection(source, g, eps)
        injections.append(ph.PointInjection(inj.component, inj.i, inj.j, inj.weights, inj.coefficient,
                                            _pulse(inj.pulse)))  # fmt: skip
    samplings = []
    for monitor in sim.monitors:
        for s in monitor_samplings(monitor, g):
            ax = lambda a: ph.AxisSampling(a.index, a.coords, a.weights, a.point)  # noqa: E731
            samplings.append(ph.ComponentSampling(s.monitor, s.component, s.wavelengths, ax(s.x), ax(s.y),
                                                  s.flat_index))  # fmt: skip
    monitors = [ph.DFTMonitor(m.name, tuple(m.wavelengths), m.center, m.size, m.components) for m in sim.monitors]
    return ph.TEProblem(grid, eps, axis(cx), axis(cy), injections, samplings, sim.precision,
                        g.n_steps(sim.run_time), bg, monitors)  # fmt: skip


class GB300FDTDSolver:
    """Etalon's FDTDSolver (etalon/fdtd/solver.py:49-165) on the fused GB300 engine."""

    def __init__(self, sim, **engine_options) -> None:
        self.sim = sim
        problem = problem_from_simulation(sim)
        self._solver = GB300Solver(problem, **engine_options)
        self.grid = self._solver.grid
        self.n_steps = problem.n_steps
        self.backend = self._solver.backend
        self.real, self.complex = problem.real, problem.complex
        self.injections = problem.injections
        self.monitors = self._solver.monitors

    @property
    def n(self) -> int:
        return self._solver.n

    @property
    def state(self):
        """Device views of the fields and coefficients (what Etalon Studio's live view reads)."""
        return self._solver.state

    def step(self) -> None:
        self._solver.step()

    def fields(self):
        return self._solver.fields()

    def result(self, wall_time: float = float("nan")):
        from etalon.io.result import SimulationResult, monitor_dataarray

        data: dict[str, dict[str, Any]] = {m.name: {} for m in self.sim.monitors}
        for mon in self.monitors:
            s = mon.sampling
            data[s.monitor][s.component] = monitor_dataarray(s, mon.acc, self.grid.z)
        n = self.n
        metadata = {
            "etalon_version": _etalon_version(),
            "etalon_gb300_version": __version__,
            "backend": self.backend.name,
            "device": self.backend.device,
            "precision": self.sim.precision,
            "n_steps": n,
            "dt_s": self.grid.dt,
            "grid_cells": (self.grid.nx, self.grid.ny),
            "wall_time_s": wall_time,
            "cell_updates_per_s": self.grid.n_cells * n / wall_time if wall_time > 0 else None,
        }
        return SimulationResult(self.sim, self.grid, data, metadata)

    def run(self):
        start = time.perf_counter()
        left = self.n_steps - self.n
        if left > 0:
            self._solver.advance(left)
        self._solver.engine.synchronize()
        return self.result(time.perf_counter() - start)


def _etalon_version() -> str:
    try:
        from etalon import __version__ as v

        return v
    except Exception:
        return "unknown"


def gpu_available() -> bool:
    """Whether this backend can run here: the library loads and reports a CUDA device."""
    from . import _lib

    try:
        _lib.device_info()
        return True
    except Exception:
        return False


def select_backend(name: str, precision: str, numpy_backend):
    """Etalon's backend selection (etalon/fdtd/backends/__init__.py:16-43) with "cuda" meaning
    this backend: "numpy" → ``numpy_backend()``; "cuda" → ``Gb300Backend`` or a RuntimeError
    (never a silent fallback); "auto" → ``Gb300Backend`` when a GPU is usable, else NumPy, with
    a warning when a device is present but the backend fails to start."""
    import warnings

    from .backend import Gb300Backend

    if name == "numpy":
        return numpy_backend()
    if name == "cuda":
        return Gb300Backend(precision)
    if name == "auto":
        if not gpu_available():
            return numpy_backend()
        try:
            return Gb300Backend(precision)
        except RuntimeError as error:
            warnings.warn(f"{error}\nFalling back to the NumPy backend.", stacklevel=3)
            return numpy_backend()
    raise ValueError(f"unknown backend {name!r}; use 'auto', 'numpy' or 'cuda'")


def uses_gpu(backend_name: str) -> bool:
    """Whether ``Simulation.run`` goes to the fused engine for this ``Simulation.backend``."""
    return backend_name == "cuda" or (backend_name == "auto" and gpu_available())


def install(fused_solver: bool = False) -> None:
    """Route Etalon's "cuda" backend (and "auto" on a GPU machine) to this backend.

    Explicit "cuda" without a usable GPU raises (never a silent fallback); "auto" falls
    back to NumPy with a warning, as etalon/fdtd/backends/__init__.py:16-43 does.
    ``Simulation.run`` goes through the fused engine (``GB300FDTDSolver``). Code that builds
    ``FDTDSolver(sim)`` itself and steps it — Etalon Studio's runner
    (etalon/studio/runner.py:463) — gets Etalon's own solver on the per-step protocol, or, with
    ``fused_solver=True``, ``GB300FDTDSolver`` for GPU backends: the same ``step``, ``n``,
    ``n_steps``, ``grid``, ``backend``, ``state`` (device views), ``fields`` and ``result``,
    on the fused engine.
    """
    import etalon.fdtd.backends as backends
    import etalon.fdtd.solver as solver_module
    from etalon.fdtd.backends.numpy_backend import NumpyBackend

    def get_backend(name: str, precision: str):
        return select_backend(name, precision, NumpyBackend)

    plain_run = solver_module.run

    def run(sim):
        if uses_gpu(sim.backend):
            return GB300FDTDSolver(sim).run()
        return plain_run(sim)

    backends.get_backend = get_backend
    solver_module.get_backend = get_backend
    solver_module.run = run
    if fused_solver:
        plain_solver = getattr(solver_module.FDTDSolver, "etalon_solver", solver_module.FDTDSolver)

        def FDTDSolver(sim):  # noqa: N802 - stands in for Etalon's class
            return GB300FDTDSolver(sim) if uses_gpu(sim.backend) else plain_solver(sim)

        FDTDSolver.etalon_solver = plain_solver
        solver_module.FDTDSolver = FDTDSolver
