"""``GB300Solver``: Etalon's FDTDSolver interface over a resident ``TEEngine``.

Mirrors etalon/fdtd/solver.py:49-160 — ``n``, ``n_steps``, ``grid``, ``monitors``
(with ``sampling`` and ``acc``), ``backend``, ``step()``, ``run()``, ``fields()`` and
``result()`` — but each ``run()`` is one device-resident advance instead of a Python
loop of kernel launches and per-step host copies.
"""

from __future__ import annotations

import time
from dataclasses import dataclass, field
from typing import Any

import numpy as np

from .backend import Gb300Backend
from .engine import TEEngine
from .physics import ComponentSampling, TEProblem

__version__ = "1.0.0"


class _MonitorView:
    """FDTDSolver's per-monitor record: the sampling and its (host copy of the) accumulator."""

    def __init__(self, engine: TEEngine, k: int):
        self._engine, self._k = engine, k
        self.sampling: ComponentSampling = engine.monitors[k].sampling

    @property
    def acc(self) -> np.ndarray:
        return self._engine.dft(self._k)


@dataclass
class RunResult:
    """Monitor accumulators and run metadata (Etalon wraps these in xarray; io/result.py)."""

    problem: TEProblem
    data: dict[str, dict[str, np.ndarray]]
    metadata: dict[str, Any] = field(default_factory=dict)

    @property
    def monitors(self) -> list[str]:
        return list(self.data)

    def __getitem__(self, name: str) -> dict[str, np.ndarray]:
        try:
            return self.data[name]
        except KeyError:
            raise KeyError(f"no monitor named {name!r}; monitors: {self.monitors}") from None


def interpolate_monitor(sampling: ComponentSampling, acc: np.ndarray) -> np.ndarray:
    """Bilinear reduction of interpolated axes in float64, as etalon/io/result.py:54-91.

    Returns an array with the raw axes first (x, then y) and wavelength last.
    """
    n_f = sampling.wavelengths.size
    data = acc.reshape(n_f, sampling.x.index.size, sampling.y.index.size).astype(np.complex128)
    if sampling.x.weights is not None:
        data = np.einsum("fab,a->fb", data, sampling.x.weights)
    if sampling.y.weights is not None:
        data = data @ sampling.y.weights
    return np.moveaxis(data, 0, -1).astype(acc.dtype)


class EngineState:
    """Etalon's ``TEState`` (etalon/fdtd/state.py:15-49) as device views of a resident engine.

    ``ex``, ``ey``, ``hz``, the four ψ arrays, ``cb_ex`` and ``cb_ey`` are ``DeviceArray`` views
    of the engine's own pitched arrays (no copy); reading an attribute first waits for the
    engine's queued steps. ``db``, ``inv_dx``, ``inv_dy`` are the cast scalars and ``nx``, ``ny``
    the grid. This is what Etalon Studio's live view reads (etalon/studio/runner.py:258-310:
    ``field_energy`` and ``snapshot_frame``), through ``Gb300Backend.xp``."""

    _ARRAYS = {"ex": 0, "ey": 1, "hz": 2, "psi_ex_y": 3, "psi_ey_x": 4, "psi_hz_x": 5, "psi_hz_y": 6,
               "cb_ex": 7, "cb_ey": 8}  # fmt: skip

    def __init__(self, engine: TEEngine):
        self._engine = engine
        c = engine._coeffs
        real = engine.real
        self.db, self.inv_dx, self.inv_dy = real(c.db), real(c.inv_dx), real(c.inv_dy)
        self.nx, self.ny = engine.nx, engine.ny

    def __getattr__(self, name: str):
        if name not in EngineState._ARRAYS:
            raise AttributeError(name)
        import ctypes as C

        from . import _lib
        from .backend import DeviceArray

        e = self._engine
        e.synchronize()
        ptr, pitch = C.c_void_p(), C.c_int64()
        _lib.call("etg_sim_device_array", e._h, EngineState._ARRAYS[name], C.byref(ptr), C.byref(pitch))
        shape = e.field_shape(name) if not name.startswith("cb") else e.field_shape("ex" if name == "cb_ex" else "ey")
        return DeviceArray(shape, e.real, ptr.value, base=e, pitch=pitch.value)


class GB300Solver:
    """Builds the device state of a problem and advances it."""

    def __init__(self, problem: TEProblem, **engine_options) -> None:
        self.problem = problem
        self.grid = problem.grid
        self.n_steps = problem.n_steps
        self.backend = Gb300Backend(problem.precision)
        self.real, self.complex = problem.real, problem.complex
        self.engine = TEEngine(problem, **engine_options)
        self.injections = problem.injections
        self.monitors = [_MonitorView(self.engine, k) for k in range(len(self.engine.monitors))]

    @property
    def n(self) -> int:
        return self.engine.n

    @property
    def state(self) -> EngineState:
        """Device views of the fields and coefficients, as Etalon's ``FDTDSolver.state``."""
        return EngineState(self.engine)

    def step(self) -> None:
        """One time step (H, inject M, DFT H, E, inject J, DFT E)."""
        self.engine.advance(1)

    def advance(self, k: int) -> None:
        self.engine.advance(k)

    def fields(self) -> dict[str, np.ndarray]:
        return self.engine.fields()

    def result(self, wall_time: float = float("nan")) -> RunResult:
        data: dict[str, dict[str, np.ndarray]] = {m.name: {} for m in self.problem.monitors}
        for mon in self.monitors:
            s = mon.sampling
            data.setdefault(s.monitor, {})[s.component] = interpolate_monitor(s, mon.acc)
        n = self.n
        meta = {
            "etalon_gb300_version": __version__,
            "backend": self.backend.name,
            "device": self.backend.device,
            "precision": self.problem.precision,
            "n_steps": n,
            "dt_s": self.grid.dt,
            "grid_cells": (self.grid.nx, self.grid.ny),
            "wall_time_s": wall_time,
            "cell_updates_per_s": self.grid.n_cells * n / wall_time if wall_time > 0 else None,
        }
        return RunResult(self.problem, data, meta)

    def run(self) -> RunResult:
        start = time.perf_counter()
        left = self.n_steps - self.n
        if left > 0:
            self.engine.advance(left)
        self.engine.synchronize()
        return self.result(time.perf_counter() - start)

    def close(self) -> None:
        self.engine.close()
