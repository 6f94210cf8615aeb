"""CPU oracle for the 2D TM mode (Ez, Hx, Hy): the TM Yee update written out directly.

TEST INFRASTRUCTURE ONLY: the checker of the GPU's TM mode; the product never imports it.

Etalon has no TM solver (it refuses TM sources and monitors, etalon/fdtd/capabilities.py:7-24),
so there is no reference behaviour to restate. This oracle writes the TM equations in the form
and operation order of Etalon's TE update (etalon/fdtd/backends/numpy_backend.py:41-61), one
field at a time, on this grid:

    Ez (nx, ny)     at the cell centres (x_i+1/2, y_j+1/2), time (n+1/2) dt
    Hx (nx, ny+1)   at (x_i+1/2, y_j), time (n+1) dt; Hx at j = 0 and j = ny stays 0
    Hy (nx+1, ny)   at (x_i, y_j+1/2), time (n+1) dt; Hy at i = 0 and i = nx stays 0

    Ez += ce * ((dHy/dx * ikx_h + psi_ez_x) - (dHx/dy * iky_h + psi_ez_y)),  ce = dt/(eps0 eps_r)
    Hx -= ch * (dEz/dy * iky_e + psi_hx_y)                                     ch = dt/mu0
    Hy += ch * (dEz/dx * ikx_e + psi_hy_x)

with the CPML recursions psi <- b psi + c d of the same profiles (h at half nodes, e at integer
nodes). A step is: Ez update, Ez sources (current J sampled at n dt: Ez -= ce w/(dx dy) g(n dt),
cast), DFT of Ez at (n+1/2) dt, H update, DFT of Hx, Hy at (n+1) dt. It shares no code with the
GPU path, which runs the TM mode through the dual TE update. tests/test_tm_oracle.py pins it to
the TE oracle (oracle/te_numpy.py, itself pinned to Etalon) in uniform media, where the
duality maps one onto the other exactly.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from oracle.te_numpy import accumulate_dft, dft_phasors, pulse_signal


def update_ez(s) -> None:
    """Ez^(n-1/2) -> Ez^(n+1/2) from Hx^n, Hy^n, with the CPML psi of Ez."""
    dhx_dy = (s.hx[:, 1:] - s.hx[:, :-1]) * s.inv_dy
    dhy_dx = (s.hy[1:, :] - s.hy[:-1, :]) * s.inv_dx
    s.psi_ez_y[...] = s.by_h[None, :] * s.psi_ez_y + s.cy_h[None, :] * dhx_dy
    s.psi_ez_x[...] = s.bx_h[:, None] * s.psi_ez_x + s.cx_h[:, None] * dhy_dx
    s.ez += s.ce * ((dhy_dx * s.ikx_h[:, None] + s.psi_ez_x) - (dhx_dy * s.iky_h[None, :] + s.psi_ez_y))


def update_hxy(s) -> None:
    """Hx^n, Hy^n -> n+1 from Ez^(n+1/2); the outer tangential H stays 0."""
    dez_dy = (s.ez[:, 1:] - s.ez[:, :-1]) * s.inv_dy
    psi = s.psi_hx_y[:, 1:-1]
    psi[...] = s.by_e[None, 1:-1] * psi + s.cy_e[None, 1:-1] * dez_dy
    s.hx[:, 1:-1] -= s.ch * (dez_dy * s.iky_e[None, 1:-1] + psi)

    dez_dx = (s.ez[1:, :] - s.ez[:-1, :]) * s.inv_dx
    psi = s.psi_hy_x[1:-1, :]
    psi[...] = s.bx_e[1:-1, None] * psi + s.cx_e[1:-1, None] * dez_dx
    s.hy[1:-1, :] += s.ch * (dez_dx * s.ikx_e[1:-1, None] + psi)


@dataclass
class TMSource:
    """A point current on Ez: nodes, float64 coefficients ce w/(dx dy), pulse parameters."""

    i: np.ndarray
    j: np.ndarray
    coefficient: np.ndarray
    pulse: tuple[float, float, float]


@dataclass
class TMMonitor:
    component: str  # "Ez", "Hx" or "Hy"
    flat_index: np.ndarray
    frequencies: np.ndarray


class OracleTM:
    """One 2D TM run. ``coeffs``: ce (nx, ny), ch (scalar), the twelve 1D CPML profiles named as
    in etalon/fdtd/state.py (bx_e … iky_h), inv_dx, inv_dy, all cast to ``dtype``."""

    FIELDS = ("ez", "hx", "hy", "psi_ez_x", "psi_ez_y", "psi_hx_y", "psi_hy_x")

    def __init__(self, nx, ny, dt, coeffs, dtype, sources=(), monitors=()):
        self.nx, self.ny, self.dt = nx, ny, dt
        self.real = np.dtype(dtype).type
        self.complex = np.complex64 if self.real == np.float32 else np.complex128
        for k, v in coeffs.items():
            setattr(self, k, v)
        shapes = {"ez": (nx, ny), "hx": (nx, ny + 1), "hy": (nx + 1, ny), "psi_ez_x": (nx, ny),
                  "psi_ez_y": (nx, ny), "psi_hx_y": (nx, ny + 1), "psi_hy_x": (nx + 1, ny)}  # fmt: skip
        for k, shape in shapes.items():
            setattr(self, k, np.zeros(shape, self.real))
        self.sources = list(sources)
        self.monitors = list(monitors)
        self.acc = [np.zeros((m.frequencies.size, m.flat_index.size), self.complex) for m in self.monitors]
        self.n = 0

    def _accumulate(self, electric: bool) -> None:
        t = np.array([self.n + (0.5 if electric else 1.0)], dtype=np.float64) * self.dt
        for mon, acc in zip(self.monitors, self.acc):
            if (mon.component == "Ez") == electric:
                ph = dft_phasors(mon.frequencies, t, self.dt).astype(self.complex)[0]
                accumulate_dft(acc, getattr(self, mon.component.lower()), mon.flat_index, ph)

    def step(self) -> None:
        update_ez(self)
        for src in self.sources:
            delta = (src.coefficient * pulse_signal(*src.pulse, self.n * self.dt)).astype(self.real)
            self.ez[src.i, src.j] -= delta
        self._accumulate(True)
        update_hxy(self)
        self._accumulate(False)
        self.n += 1

    def run(self, steps: int) -> None:
        for _ in range(steps):
            self.step()
