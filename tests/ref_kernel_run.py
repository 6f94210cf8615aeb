"""A run of Etalon's own CUDA kernels (oracle/ref_kernels.py) over a TEProblem, step by step.

Test and bench infrastructure. It does what Etalon's FDTDSolver.step does on its CuPy backend
(etalon/fdtd/solver.py:120-128): update_h_te, injection of the H sources, the H monitors'
accumulate_dft, update_e_te, injection of the E sources, the E monitors' accumulate_dft — with
the reference's kernels for the updates and the DFT, in the reference's array layout. The
injection (CuPy's ``field[i, j] -= delta`` in Etalon) is one ``etg_scatter_sub`` of this
package, which has NumPy's fancy-index semantics. Source deltas and phasor rows are the
whole-run tables of ``physics`` (Etalon's float64 values, cast once), uploaded before the run.
"""

from __future__ import annotations

import ctypes as C
from types import SimpleNamespace

import numpy as np

from etalon_gb300 import _lib
from etalon_gb300 import physics as ph

COEFFS = ("cb_ex", "cb_ey", "bx_e", "cx_e", "ikx_e", "bx_h", "cx_h", "ikx_h",
          "by_e", "cy_e", "iky_e", "by_h", "cy_h", "iky_h")  # fmt: skip


class RefRun:
    def __init__(self, kernels, p: ph.TEProblem, n_steps: int):
        self.k, self.p, self.real = kernels, p, np.dtype(p.real)
        self.code = _lib.dtype_code(p.real)
        self.ptrs: list[int] = []
        nx, ny = p.grid.nx, p.grid.ny
        self.shapes = {"ex": (nx, ny + 1), "ey": (nx + 1, ny), "hz": (nx, ny), "psi_ex_y": (nx, ny + 1),
                       "psi_ey_x": (nx + 1, ny), "psi_hz_x": (nx, ny), "psi_hz_y": (nx, ny)}  # fmt: skip
        c = ph.cast_coefficients(p)
        s = SimpleNamespace(nx=nx, ny=ny, db=float(c.db), inv_dx=float(c.inv_dx), inv_dy=float(c.inv_dy))
        for f, shape in self.shapes.items():
            setattr(s, f, self._zeros(int(np.prod(shape)) * self.real.itemsize))
        for name in COEFFS:
            setattr(s, name, self._upload(np.ascontiguousarray(getattr(c, name), dtype=self.real)))
        self.s = s
        self.sources = []
        for inj in p.injections:
            table = np.ascontiguousarray(inj.delta_table(0, n_steps, p.grid.dt, p.real))
            self.sources.append((inj.component, inj.i.size, self._upload(np.ascontiguousarray(inj.i, np.int64)),
                                 self._upload(np.ascontiguousarray(inj.j, np.int64)), self._upload(table)))  # fmt: skip
        self.monitors = []
        for sm in p.samplings:
            n_f, nodes = sm.wavelengths.size, sm.flat_index.size
            table = np.ascontiguousarray(ph.phasor_table(sm, 0, n_steps, p.grid.dt, p.complex))
            acc = self._zeros(n_f * nodes * 2 * self.real.itemsize)
            self.monitors.append((sm, n_f, nodes, acc, self._upload(np.ascontiguousarray(sm.flat_index, np.int64)),
                                  self._upload(table)))  # fmt: skip
        self.n = 0
        self.n_steps = n_steps

    def _zeros(self, nbytes: int) -> int:
        q = C.c_void_p()
        _lib.call("etg_malloc", C.byref(q), max(nbytes, 16))
        _lib.call("etg_memset", q.value, 0, max(nbytes, 16))
        self.ptrs.append(q.value)
        return q.value

    def _upload(self, a: np.ndarray) -> int:
        q = self._zeros(a.nbytes)
        _lib.call("etg_memcpy_h2d", q, a.ctypes.data, a.nbytes)
        return q

    def _inject(self, magnetic: bool) -> None:
        s, n, item = self.s, self.n, self.real.itemsize
        for comp, nodes, i, j, table in self.sources:
            if comp.startswith("H") != magnetic:
                continue
            field = getattr(s, comp.lower())
            cols = self.shapes[comp.lower()][1]
            _lib.call("etg_scatter_sub", self.code, cols, nodes, field, i, j, table + n * nodes * item)

    def _accumulate(self, magnetic: bool) -> None:
        n, item = self.n, self.real.itemsize
        for sm, n_f, nodes, acc, index, table in self.monitors:
            if sm.is_magnetic != magnetic:
                continue
            field = getattr(self.s, sm.component.lower())
            self.k.accumulate(acc, field, index, table + n * n_f * 2 * item, n_f, nodes)

    def step(self) -> None:
        if self.n >= self.n_steps:
            raise ValueError("the uploaded tables end here")
        self.k.update_h(self.s)
        self._inject(True)
        self._accumulate(True)
        self.k.update_e(self.s)
        self._inject(False)
        self._accumulate(False)
        self.n += 1

    def field(self, name: str) -> np.ndarray:
        out = np.empty(self.shapes[name], self.real)
        _lib.call("etg_synchronize")
        _lib.call("etg_memcpy_d2h", out.ctypes.data, getattr(self.s, name), out.nbytes)
        return out

    def acc(self, k: int) -> np.ndarray:
        sm, n_f, nodes, acc, _, _ = self.monitors[k]
        out = np.empty((n_f, nodes), self.p.complex)
        _lib.call("etg_synchronize")
        _lib.call("etg_memcpy_d2h", out.ctypes.data, acc, out.nbytes)
        return out

    def close(self) -> None:
        _lib.call("etg_synchronize")
        for q in self.ptrs:
            _lib.call("etg_free", q)
        self.ptrs = []
