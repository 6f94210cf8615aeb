"""CPU oracle for the 2D TE hot path: a NumPy restatement of Etalon's reference backend.

TEST INFRASTRUCTURE ONLY. This module is the checker the parity tests, the smoke
check and the bench's CPU-baseline leg compare the CUDA path with; the product never
imports it. It is pinned against vectors generated by running Etalon itself
(tests/golden/make_golden.py → tests/golden/*.npz, checked by tests/test_oracle_golden.py).

Restated from Etalon (paths within the Etalon project):
  update_h            etalon/fdtd/backends/numpy_backend.py:41-49
  update_e            etalon/fdtd/backends/numpy_backend.py:51-61
  accumulate_dft      etalon/fdtd/backends/numpy_backend.py:63-67
  pulse_signal        etalon/fdtd/sources.py:26-30 (+ PointInjection.delta 50-56)
  dft_phasors         etalon/fdtd/dft.py:110-119 (+ FDTDSolver._phasor_rows 91-110)
  OracleTE.step       etalon/fdtd/solver.py:83-128 (H, inject M, DFT H, E, inject J, DFT E)

Every expression performs the same NumPy operations in the same order as Etalon's,
so on the same inputs the results are the reference's, bit for bit. It does not import
the ``etalon_gb300`` package: sources and monitors arrive as plain arrays.
"""

from __future__ import annotations

import math
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass

import numpy as np

C_0 = 299_792_458.0 * 1e6  # µm/s, etalon/constants.py:16


def update_h(s) -> None:
    """Hz^(n−½) → Hz^(n+½) with the CPML ψ of Hz (numpy_backend.py:41-49)."""
    dex_dy = (s.ex[:, 1:] - s.ex[:, :-1]) * s.inv_dy
    dey_dx = (s.ey[1:, :] - s.ey[:-1, :]) * s.inv_dx
    s.psi_hz_y[...] = s.by_h[None, :] * s.psi_hz_y + s.cy_h[None, :] * dex_dy
    s.psi_hz_x[...] = s.bx_h[:, None] * s.psi_hz_x + s.cx_h[:, None] * dey_dx
    s.hz += s.db * (
        (dex_dy * s.iky_h[None, :] + s.psi_hz_y) - (dey_dx * s.ikx_h[:, None] + s.psi_hz_x)
    )


def update_e(s) -> None:
    """Ex^n, Ey^n → Ex^(n+1), Ey^(n+1); tangential E on the outer edge stays 0 (51-61)."""
    dhz_dy = (s.hz[:, 1:] - s.hz[:, :-1]) * s.inv_dy
    psi = s.psi_ex_y[:, 1:-1]
    psi[...] = s.by_e[None, 1:-1] * psi + s.cy_e[None, 1:-1] * dhz_dy
    s.ex[:, 1:-1] += s.cb_ex[:, 1:-1] * (dhz_dy * s.iky_e[None, 1:-1] + psi)

    dhz_dx = (s.hz[1:, :] - s.hz[:-1, :]) * s.inv_dx
    psi = s.psi_ey_x[1:-1, :]
    psi[...] = s.bx_e[1:-1, None] * psi + s.cx_e[1:-1, None] * dhz_dx
    s.ey[1:-1, :] -= s.cb_ey[1:-1, :] * (dhz_dx * s.ikx_e[1:-1, None] + psi)


def update_h_rows(s, r0: int, r1: int) -> None:
    """``update_h`` restricted to Hz rows [r0, r1); identical values element by element."""
    dex_dy = (s.ex[r0:r1, 1:] - s.ex[r0:r1, :-1]) * s.inv_dy
    dey_dx = (s.ey[r0 + 1 : r1 + 1, :] - s.ey[r0:r1, :]) * s.inv_dx
    py = s.psi_hz_y[r0:r1]
    px = s.psi_hz_x[r0:r1]
    py[...] = s.by_h[None, :] * py + s.cy_h[None, :] * dex_dy
    px[...] = s.bx_h[r0:r1, None] * px + s.cx_h[r0:r1, None] * dey_dx
    s.hz[r0:r1] += s.db * ((dex_dy * s.iky_h[None, :] + py) - (dey_dx * s.ikx_h[r0:r1, None] + px))


def update_e_rows(s, r0: int, r1: int) -> None:
    """``update_e`` restricted to Ex rows [r0, r1) and Ey rows [max(r0,1), min(r1, nx))."""
    dhz_dy = (s.hz[r0:r1, 1:] - s.hz[r0:r1, :-1]) * s.inv_dy
    psi = s.psi_ex_y[r0:r1, 1:-1]
    psi[...] = s.by_e[None, 1:-1] * psi + s.cy_e[None, 1:-1] * dhz_dy
    s.ex[r0:r1, 1:-1] += s.cb_ex[r0:r1, 1:-1] * (dhz_dy * s.iky_e[None, 1:-1] + psi)
    a, b = max(r0, 1), min(r1, s.nx)
    if a >= b:
        return
    dhz_dx = (s.hz[a:b, :] - s.hz[a - 1 : b - 1, :]) * s.inv_dx
    psi = s.psi_ey_x[a:b, :]
    psi[...] = s.bx_e[a:b, None] * psi + s.cx_e[a:b, None] * dhz_dx
    s.ey[a:b, :] -= s.cb_ey[a:b, :] * (dhz_dx * s.ikx_e[a:b, None] + psi)


def accumulate_dft(acc, field, index, phasors) -> None:
    """acc[f, k] += field.flat[index[k]] · phasors[f] (numpy_backend.py:63-67)."""
    acc += field.ravel()[index][None, :] * phasors[:, None]


def pulse_signal(wavelength: float, bandwidth: float, amplitude: float, t) -> np.ndarray:
    """Gaussian pulse g(t) (etalon/fdtd/sources.py:26-30, etalon/core/source.py:50-68)."""
    frequency = C_0 / wavelength
    f_hi = C_0 / (wavelength - bandwidth / 2.0)
    f_lo = C_0 / (wavelength + bandwidth / 2.0)
    width = 1.0 / (2.0 * math.pi * ((f_hi - f_lo) / 2.0))
    delay = 5.0 * width
    s = np.asarray(t, dtype=np.float64) - delay
    envelope = np.exp(-(s**2) / (2.0 * width**2))
    return amplitude * envelope * np.sin(2.0 * np.pi * frequency * s)


def dft_phasors(frequencies, times, dt) -> np.ndarray:
    """exp(+i2πft)·Δt, float64 (etalon/fdtd/dft.py:110-119)."""
    phase = 2.0 * np.pi * times[:, None] * frequencies[None, :]
    return np.asarray(np.exp(1j * phase) * dt, dtype=np.complex128)


@dataclass
class OracleSource:
    """A resolved point source: nodes (i, j), float64 coefficients, pulse parameters.

    ``table`` (optional, shape (n_steps, n_nodes), already cast) replaces the per-step
    evaluation of the pulse, for fixtures that carry the reference's own host values.
    """

    component: str
    i: np.ndarray
    j: np.ndarray
    coefficient: np.ndarray
    pulse: tuple[float, float, float]
    table: np.ndarray | None = None

    @property
    def magnetic(self) -> bool:
        return self.component.startswith("H")


@dataclass
class OracleMonitor:
    """One monitor component: flat node indices and frequencies (Hz).

    ``table`` (optional, shape (n_steps, n_f), complex, already cast) replaces the
    phasor evaluation, as for ``OracleSource.table``.
    """

    component: str
    flat_index: np.ndarray
    frequencies: np.ndarray
    table: np.ndarray | None = None

    @property
    def magnetic(self) -> bool:
        return self.component.startswith("H")


class OracleTE:
    """Fields, ψ and coefficients of one 2D TE run, stepped like Etalon's FDTDSolver.

    ``coeffs`` maps the names of etalon/fdtd/state.py:15-49 (cb_ex … iky_h, db, inv_dx,
    inv_dy) to arrays already cast to ``dtype``.
    """

    FIELDS = ("ex", "ey", "hz", "psi_ex_y", "psi_ey_x", "psi_hz_x", "psi_hz_y")

    def __init__(self, nx, ny, dt, coeffs, dtype, sources=(), monitors=()):
        self.nx, self.ny, self.dt = nx, ny, dt
        self.real = np.dtype(dtype).type
        self.complex = np.complex64 if self.real == np.float32 else np.complex128
        for k, v in coeffs.items():
            setattr(self, k, v)
        shapes = {"ex": (nx, ny + 1), "ey": (nx + 1, ny), "hz": (nx, ny),
                  "psi_ex_y": (nx, ny + 1), "psi_ey_x": (nx + 1, ny),
                  "psi_hz_x": (nx, ny), "psi_hz_y": (nx, ny)}  # fmt: skip
        for k, shape in shapes.items():
            setattr(self, k, np.zeros(shape, self.real))
        self.sources = list(sources)
        self.monitors = list(monitors)
        self.acc = [np.zeros((m.frequencies.size, m.flat_index.size), self.complex) for m in self.monitors]
        self.n = 0

    # -- per-step host values, as FDTDSolver computes them
    def delta(self, src: OracleSource, n: int) -> np.ndarray:
        if src.table is not None:
            return src.table[n]
        t = n * self.dt if src.magnetic else (n + 0.5) * self.dt
        return (src.coefficient * pulse_signal(*src.pulse, t)).astype(self.real)

    def phasor(self, mon: OracleMonitor, n: int) -> np.ndarray:
        if mon.table is not None:
            return mon.table[n]
        t = np.array([n + (0.5 if mon.magnetic else 1.0)], dtype=np.float64) * self.dt
        return dft_phasors(mon.frequencies, t, self.dt).astype(self.complex)[0]

    def _inject(self, magnetic: bool) -> None:
        for src in self.sources:
            if src.magnetic == magnetic:
                field = getattr(self, src.component.lower())
                field[src.i, src.j] -= self.delta(src, self.n)

    def _accumulate(self, magnetic: bool) -> None:
        for mon, acc in zip(self.monitors, self.acc):
            if mon.magnetic == magnetic:
                accumulate_dft(acc, getattr(self, mon.component.lower()), mon.flat_index,
                               self.phasor(mon, self.n))

    def step(self, pool: ThreadPoolExecutor | None = None, bands: int = 1) -> None:
        """One leapfrog step in Etalon's order; with ``pool`` the updates run in row bands."""
        if pool is None:
            update_h(self)
        else:
            _bands(pool, bands, self.nx, lambda a, b: update_h_rows(self, a, b))
        self._inject(True)
        self._accumulate(True)
        if pool is None:
            update_e(self)
        else:
            _bands(pool, bands, self.nx, lambda a, b: update_e_rows(self, a, b))
        self._inject(False)
        self._accumulate(False)
        self.n += 1

    def run(self, steps: int, **kw) -> None:
        for _ in range(steps):
            self.step(**kw)

    def fields(self) -> dict[str, np.ndarray]:
        return {k: getattr(self, k) for k in self.FIELDS}


def _bands(pool: ThreadPoolExecutor, bands: int, n: int, fn) -> None:
    edges = np.linspace(0, n, bands + 1).astype(int)
    list(pool.map(lambda k: fn(int(edges[k]), int(edges[k + 1])), range(bands)))
