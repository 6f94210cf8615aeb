"""Resident 2D TE run on the GPU: the Python side of ``etg_sim`` (include/etalon_gb300.h).

``TEEngine(problem)`` uploads the cast coefficients (etalon/fdtd/state.py:52-99), one
table of per-step source deltas per source (etalon/fdtd/sources.py:54-56) and one
table of phasor rows per monitor component (etalon/fdtd/solver.py:91-110), then
``advance(k)`` runs k whole steps on the device. The per-step host work of Etalon's
FDTDSolver — a float64 pulse evaluation, a cast and a host-to-device copy per source
per step — becomes one upload of rows computed with the same float64 operations.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import call
from .physics import (_BOX_TOL, EPSILON_0, ComponentSampling, PointInjection, TEProblem, cast_coefficients,
                      phasor_table)

# Etalon's phasor-table bound (etalon/fdtd/solver.py:32): rows × frequencies per upload.
PHASOR_TABLE_ENTRIES = 1 << 22


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def _rect(s: ComponentSampling) -> tuple[int, int, int, int]:
    """The node rectangle of a sampling; its indices are consecutive by construction."""
    xi, yi = s.x.index, s.y.index
    if not (np.all(np.diff(xi) == 1) and np.all(np.diff(yi) == 1)):
        raise ValueError(f"monitor {s.monitor!r} ({s.component}) is not a rectangle of nodes")
    return int(xi[0]), int(xi.size), int(yi[0]), int(yi.size)


@dataclass
class EngineMonitor:
    sampling: ComponentSampling
    id: int
    n0: int = 0
    rows: int = 0


@dataclass
class EngineSource:
    injection: PointInjection
    id: int
    n0: int = 0
    rows: int = 0


class TEEngine:
    """One resident simulation. Not thread-safe; one engine per host thread."""

    def __init__(self, problem: TEProblem, *, table_steps: int | None = None,
                 kernel: str = "auto", graph_steps: int = 32) -> None:  # fmt: skip
        self.problem = problem
        g = problem.grid
        self.nx, self.ny, self.dt = g.nx, g.ny, g.dt
        self.real, self.complex = problem.real, problem.complex
        self.n_steps = problem.n_steps
        lib = _lib.lib()
        handle = C.c_void_p()
        call("etg_sim_create", C.byref(handle), _lib.dtype_code(self.real), g.nx, g.ny)
        self._h = handle
        self._lib = lib
        try:
            self._upload_coefficients()
            self.set_option(_lib.OPT_GRAPH_STEPS, graph_steps)
            self.set_kernel(kernel)
            rows = table_steps if table_steps is not None else (self.n_steps or 0)
            self.sources = []
            for k, inj in enumerate(problem.injections):
                self.sources.append(self._add_source(inj, k, rows))
            self.monitors = [self._add_monitor(s, rows) for s in problem.samplings]
        except Exception:
            self.close()
            raise

    # ------------------------------------------------------------------ setup
    def _upload_coefficients(self) -> None:
        self.set_coefficients(cast_coefficients(self.problem))

    def set_coefficients(self, c) -> None:
        """Upload cast coefficients (a ``CastCoefficients`` or an object with its fields)."""
        self._coeffs = c  # keep host copies alive for the duration of the copy
        arrays = [np.ascontiguousarray(getattr(c, k), dtype=self.real) for k in
                  ("cb_ex", "cb_ey", "bx_e", "cx_e", "ikx_e", "bx_h", "cx_h", "ikx_h",
                   "by_e", "cy_e", "iky_e", "by_h", "cy_h", "iky_h")]  # fmt: skip
        self._coeff_arrays = arrays
        call("etg_sim_set_coefficients", self._h, *[_ptr(a) for a in arrays],
             float(c.db), float(c.inv_dx), float(c.inv_dy))  # fmt: skip

    def rasterize(self, boxes, background_eps: float) -> None:
        """Replace cb_ex and cb_ey by the staircase of ``boxes`` rasterised on the device.

        Same result, bit for bit, as ``permittivity_on_nodes`` then ``cast_coefficients`` on
        the host (etalon/grid/materials.py:12-35, etalon/fdtd/state.py:80-81): boxes that miss
        the plane z = grid.z are left out here with the host's test, the rest become rows of
        (cx, cy, sx/2 + tol, sy/2 + tol, eps) in their order (the last box wins).
        """
        g = self.problem.grid
        rows = [(b.center[0], b.center[1], b.size[0] / 2.0 + _BOX_TOL, b.size[1] / 2.0 + _BOX_TOL, b.eps)
                for b in boxes if not abs(g.z - b.center[2]) > b.size[2] / 2.0 + _BOX_TOL]  # fmt: skip
        table = np.ascontiguousarray(np.asarray(rows, dtype=np.float64).reshape(-1, 5))
        call("etg_sim_rasterize_cb", self._h, float(g.x_min), float(g.y_min), float(g.dx), float(g.dy),
             float(g.dt), float(EPSILON_0), float(background_eps), len(rows), _ptr(table))  # fmt: skip

    def cb(self, which: str) -> np.ndarray:
        """The device copy of cb_ex (``"ex"``) or cb_ey (``"ey"``)."""
        k = {"ex": 0, "ey": 1}[which]
        out = np.empty((self.nx, self.ny + 1) if k == 0 else (self.nx + 1, self.ny), self.real)
        call("etg_sim_get_cb", self._h, k, _ptr(out))
        return out

    def _delta_rows(self, inj: PointInjection, n0: int, rows: int) -> np.ndarray:
        return np.ascontiguousarray(inj.delta_table(n0, rows, self.dt, self.real))

    def _add_source(self, inj: PointInjection, k: int, rows: int) -> EngineSource:
        table = self._delta_rows(inj, 0, rows) if rows else np.zeros((1, inj.i.size), self.real)
        i = np.ascontiguousarray(inj.i, dtype=np.int64)
        j = np.ascontiguousarray(inj.j, dtype=np.int64)
        call("etg_sim_add_source", self._h, _lib.COMPONENT_IDS[inj.component], i.size,
             _ptr(i), _ptr(j), 0, rows, _ptr(table))  # fmt: skip
        return EngineSource(inj, k, 0, rows)

    def _add_monitor(self, s: ComponentSampling, rows: int) -> EngineMonitor:
        ix0, nxm, jy0, nym = _rect(s)
        table = (phasor_table(s, 0, rows, self.dt, self.complex) if rows
                 else np.zeros((1, s.wavelengths.size), self.complex))  # fmt: skip
        table = np.ascontiguousarray(table)
        mid = C.c_int()
        call("etg_sim_add_monitor", self._h, _lib.COMPONENT_IDS[s.component], ix0, nxm, jy0, nym,
             s.wavelengths.size, 0, rows, _ptr(table), C.byref(mid))  # fmt: skip
        return EngineMonitor(s, mid.value, 0, rows)

    def set_source_table(self, k: int, n0: int, table: np.ndarray) -> None:
        """Replace the deltas of source k by rows for steps n0 … n0+len(table)−1."""
        t = np.ascontiguousarray(table, dtype=self.real)
        call("etg_sim_set_deltas", self._h, self.sources[k].id, n0, t.shape[0], _ptr(t))
        self.sources[k].n0, self.sources[k].rows = n0, t.shape[0]

    def set_phasor_table(self, k: int, n0: int, table: np.ndarray) -> None:
        """Replace the phasor rows of monitor component k for steps n0 … n0+len(table)−1."""
        t = np.ascontiguousarray(table, dtype=self.complex)
        call("etg_sim_set_phasors", self._h, self.monitors[k].id, n0, t.shape[0], _ptr(t))
        self.monitors[k].n0, self.monitors[k].rows = n0, t.shape[0]

    def _ensure_tables(self, n: int, k: int) -> None:
        """Refill tables that do not cover steps [n, n+k), Etalon-style in bounded chunks."""
        for src in self.sources:
            if not (src.n0 <= n and n + k <= src.n0 + src.rows):
                rows = max(k, 4096)
                table = self._delta_rows(src.injection, n, rows)
                call("etg_sim_set_deltas", self._h, src.id, n, rows, _ptr(table))
                src.n0, src.rows = n, rows
        for mon in self.monitors:
            if not (mon.n0 <= n and n + k <= mon.n0 + mon.rows):
                n_f = mon.sampling.wavelengths.size
                rows = max(k, PHASOR_TABLE_ENTRIES // n_f)
                table = np.ascontiguousarray(phasor_table(mon.sampling, n, rows, self.dt, self.complex))
                call("etg_sim_set_phasors", self._h, mon.id, n, rows, _ptr(table))
                mon.n0, mon.rows = n, rows

    # ------------------------------------------------------------------ run
    @property
    def n(self) -> int:
        v = C.c_int64()
        call("etg_sim_step_index", self._h, C.byref(v))
        return v.value

    def advance(self, k: int, *, max_block: int = 1 << 20) -> None:
        """Run k whole steps (H, inject M, DFT H, E, inject J, DFT E per step)."""
        n = self.n
        done = 0
        while done < k:
            block = min(k - done, max_block)
            self._ensure_tables(n + done, block)
            call("etg_sim_advance", self._h, block)
            done += block

    def synchronize(self) -> None:
        call("etg_sim_synchronize", self._h)

    def reset(self) -> None:
        call("etg_sim_reset", self._h)

    # ------------------------------------------------------------------ io
    def field(self, name: str) -> np.ndarray:
        fid = _lib.FIELD_IDS[name]
        shape = {"ex": (self.nx, self.ny + 1), "ey": (self.nx + 1, self.ny), "hz": (self.nx, self.ny),
                 "psi_ex_y": (self.nx, self.ny + 1), "psi_ey_x": (self.nx + 1, self.ny),
                 "psi_hz_x": (self.nx, self.ny), "psi_hz_y": (self.nx, self.ny)}[name]  # fmt: skip
        out = np.empty(shape, self.real)
        call("etg_sim_get_field", self._h, fid, _ptr(out))
        return out

    def set_field(self, name: str, value: np.ndarray) -> None:
        a = np.ascontiguousarray(value, dtype=self.real)
        expect = self.field_shape(name)
        if a.shape != expect:
            raise ValueError(f"{name}: shape {a.shape}, expected {expect}")
        call("etg_sim_set_field", self._h, _lib.FIELD_IDS[name], _ptr(a))

    def field_shape(self, name: str) -> tuple[int, int]:
        rows = self.nx + 1 if name in ("ey", "psi_ey_x") else self.nx
        cols = self.ny + 1 if name in ("ex", "psi_ex_y") else self.ny
        return rows, cols

    def fields(self) -> dict[str, np.ndarray]:
        """Host copies of Ex, Ey, Hz (E at nΔt, H at (n−½)Δt), as FDTDSolver.fields()."""
        return {"Ex": self.field("ex"), "Ey": self.field("ey"), "Hz": self.field("hz")}

    def dft(self, k: int) -> np.ndarray:
        """Accumulator of monitor component k: (n_f, n_nodes) complex, x-major nodes."""
        m = self.monitors[k].sampling
        out = np.empty((m.wavelengths.size, m.flat_index.size), self.complex)
        call("etg_sim_get_dft", self._h, self.monitors[k].id, _ptr(out))
        return out

    def set_dft(self, k: int, value: np.ndarray) -> None:
        m = self.monitors[k].sampling
        a = np.ascontiguousarray(value, dtype=self.complex)
        if a.shape != (m.wavelengths.size, m.flat_index.size):
            raise ValueError(f"monitor {k}: shape {a.shape}, expected {(m.wavelengths.size, m.flat_index.size)}")
        call("etg_sim_set_dft", self._h, self.monitors[k].id, _ptr(a))

    # ------------------------------------------------------------------ checkpoint / resume
    STATE_FIELDS = ("ex", "ey", "hz", "psi_ex_y", "psi_ey_x", "psi_hz_x", "psi_hz_y")

    def save_state(self, path=None) -> dict[str, np.ndarray]:
        """Everything a run needs to continue: the seven field and ψ arrays, every DFT
        accumulator and the step index (host copies; also written to ``path`` as .npz)."""
        state = {f: self.field(f) for f in self.STATE_FIELDS}
        for k in range(len(self.monitors)):
            state[f"dft{k}"] = self.dft(k)
        state["step"] = np.array(self.n, dtype=np.int64)
        if path is not None:
            np.savez(path, **state)
        return state

    def load_state(self, state) -> None:
        """Resume from ``save_state`` output (a dict or an .npz path) of a run of the same
        problem; the continued run gives the uninterrupted run's bits."""
        if not isinstance(state, dict):
            with np.load(state, allow_pickle=False) as z:
                state = {k: z[k] for k in z.files}
        n_mon = sum(1 for k in state if k.startswith("dft"))
        if n_mon != len(self.monitors):
            raise ValueError(f"state holds {n_mon} monitor accumulators, the engine has {len(self.monitors)}")
        for f in self.STATE_FIELDS:
            self.set_field(f, state[f])
        for k in range(len(self.monitors)):
            self.set_dft(k, state[f"dft{k}"])
        call("etg_sim_set_step_index", self._h, int(state["step"]))

    def set_option(self, option: int, value: int) -> None:
        call("etg_sim_set_option", self._h, option, int(value))

    def set_kernel(self, kernel: str) -> None:
        self.set_option(_lib.OPT_KERNEL, {"auto": 0, "plain": 1, "tb": 2, "tma": 3, "pipe": 4}[kernel])

    def last_timing(self) -> tuple[float, int]:
        ms, launches = C.c_double(), C.c_int64()
        call("etg_sim_last_timing", self._h, C.byref(ms), C.byref(launches))
        return ms.value, launches.value

    def kernel_timing(self) -> dict[str, tuple[float, int, int]]:
        """{"interior"|"cpml"|"cpml_x"|"cpml_y"|"cpml_xy": (total ms, launches, output cells per
        launch)} of the last advance run with option TIMING = 2 (temporally blocked kernels
        timed one by one; each CPML kind also alone)."""
        ms, launches, cells = (C.c_double * 5)(), (C.c_int64 * 5)(), (C.c_int64 * 5)()
        call("etg_sim_kernel_timing", self._h, ms, launches, cells)
        names = ("interior", "cpml", "cpml_x", "cpml_y", "cpml_xy")
        return {k: (ms[i], launches[i], cells[i]) for i, k in enumerate(names)}

    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.etg_sim_destroy(h)
            self._h = C.c_void_p()

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self) -> "TEEngine":
        return self

    def __exit__(self, *exc) -> None:
        self.close()
