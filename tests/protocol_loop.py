"""Etalon's FDTDSolver step loop (etalon/fdtd/solver.py:83-128), written against any backend.

Used by the GPU tests to drive ``Gb300Backend`` the way Etalon's unchanged solver does:
``to_device`` for every array, ``field[i, j] -= delta`` with a per-step device delta,
and ``accumulate_dft`` with a row view of a device phasor table.
"""

from __future__ import annotations

from types import SimpleNamespace

import numpy as np

from tests.golden_io import COEFFS, count


class ProtocolRun:
    def __init__(self, backend, g: dict, precision: str):
        self.backend = backend
        real = np.float32 if precision == "single" else np.float64
        nx, ny, _ = (int(v) for v in g["grid"])
        s = SimpleNamespace(nx=nx, ny=ny)
        for c in COEFFS:
            setattr(s, c, backend.to_device(g[f"in_{c}"]))
        s.db, s.inv_dx, s.inv_dy = (real(v) for v in g["in_scalars"])
        shapes = {"ex": (nx, ny + 1), "ey": (nx + 1, ny), "hz": (nx, ny), "psi_ex_y": (nx, ny + 1),
                  "psi_ey_x": (nx + 1, ny), "psi_hz_x": (nx, ny), "psi_hz_y": (nx, ny)}  # fmt: skip
        for k, shape in shapes.items():
            setattr(s, k, backend.to_device(np.zeros(shape, real)))
        self.state = s
        self.sources = [
            (str(g[f"src{k}_component"]), backend.to_device(g[f"src{k}_i"]),
             backend.to_device(g[f"src{k}_j"]), g[f"src{k}_table"])
            for k in range(count(g, "src"))
        ]  # fmt: skip
        self.monitors = []
        for k in range(count(g, "mon")):
            table = g[f"mon{k}_table"]
            acc = backend.to_device(np.zeros((table.shape[1], g[f"mon{k}_flat"].size), table.dtype))
            self.monitors.append((str(g[f"mon{k}_component"]), backend.to_device(g[f"mon{k}_flat"]),
                                  acc, backend.to_device(table)))  # fmt: skip
        self.n = 0

    def _inject(self, magnetic: bool) -> None:
        for comp, i, j, table in self.sources:
            if comp.startswith("H") == magnetic:
                field = getattr(self.state, comp.lower())
                field[i, j] -= self.backend.to_device(table[self.n])

    def _accumulate(self, magnetic: bool) -> None:
        for comp, index, acc, table in self.monitors:
            if comp.startswith("H") == magnetic:
                self.backend.accumulate_dft(acc, getattr(self.state, comp.lower()), index, table[self.n])

    def step(self) -> None:
        self.backend.update_h_te(self.state)
        self._inject(True)
        self._accumulate(True)
        self.backend.update_e_te(self.state)
        self._inject(False)
        self._accumulate(False)
        self.n += 1

    def fields(self) -> dict:
        return {k: self.backend.to_host(getattr(self.state, k))
                for k in ("ex", "ey", "hz", "psi_ex_y", "psi_ey_x", "psi_hz_x", "psi_hz_y")}  # fmt: skip

    def accs(self) -> list:
        return [self.backend.to_host(acc) for _, _, acc, _ in self.monitors]
