"""CPU oracle for the 3D Yee update: a NumPy statement of Maxwell's curl equations.

TEST INFRASTRUCTURE ONLY. The 3D CUDA path is compared with this module; the product never
imports it. Etalon has no 3D solver (etalon/fdtd/capabilities.py:7-24 refuses it), so the
oracle is written from the equations, in Etalon's own discretisation and style:

* the layout extends etalon/grid/yee.py:27-79 by one axis: E components sit on cell edges,
  H components on cell faces, and along a PEC axis the integer positions include both
  walls (n + 1 of them) while half positions number n; along a periodic axis both number n;
* every update has the operation order of the 2D TE update it generalises
  (etalon/fdtd/backends/numpy_backend.py:41-61): forward differences times 1/Δ, the CPML
  ψ update b·ψ + c·∂, then F ± coef·((∂·1/κ + ψ) − (∂'·1/κ' + ψ')); tangential E on a PEC
  wall stays 0;
* sources and DFT monitors behave as in etalon/fdtd/solver.py:83-128 (H, inject M, DFT H,
  E, inject J, DFT E) with flat node indices into the C-ordered component arrays.

Pinning (tests/test_yee3d_oracle.py): a run that is invariant along one periodic axis of one
cell is three 2D TE runs in disguise. z-invariant: (Ex, Ey, Hz) in the (x, y) plane;
x-invariant: (Ey, Ez, Hx) in the (y, z) plane; y-invariant: (Ez, Ex, Hy) in the (z, x) plane.
Each reproduces oracle/te_numpy.py bit for bit (with CPML on the two other axes), and that
oracle is pinned to Etalon's own outputs; together the three fix all six update formulas.
The one freedom left is the sign of a zero increment where a 2D update subtracts a term
that the 3D one adds through a difference (Ey, Ex, Ez in the x-, y- and z-invariant cases):
it changes a -0 field, which a run started from zero fields never holds.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from oracle.te_numpy import accumulate_dft, dft_phasors, pulse_signal

COMPONENTS = ("ex", "ey", "ez", "hx", "hy", "hz")
# half position (True) or integer position (False) along x, y, z
HALF = {"ex": (True, False, False), "ey": (False, True, False), "ez": (False, False, True),
        "hx": (False, True, True), "hy": (True, False, True), "hz": (True, True, False)}  # fmt: skip
# ψ of each component, one per derivative axis (0 = x, 1 = y, 2 = z)
PSI = (("hx", 1), ("hx", 2), ("hy", 2), ("hy", 0), ("hz", 0), ("hz", 1),
       ("ex", 1), ("ex", 2), ("ey", 2), ("ey", 0), ("ez", 0), ("ez", 1))  # fmt: skip
AXES = "xyz"


def psi_name(comp: str, axis: int) -> str:
    return f"psi_{comp}_{AXES[axis]}"


def shape_of(comp: str, n: tuple[int, int, int], periodic: tuple[bool, bool, bool]) -> tuple[int, int, int]:
    """Array shape of a component: n_a at half positions, n_a + 1 at integer ones (PEC axis)."""
    return tuple(n[a] + (0 if HALF[comp][a] or periodic[a] else 1) for a in range(3))  # type: ignore[return-value]


def _sl(axis: int, s: slice) -> tuple:
    out = [slice(None)] * 3
    out[axis] = s
    return tuple(out)


def _bcast(v: np.ndarray, axis: int) -> np.ndarray:
    shape = [1, 1, 1]
    shape[axis] = v.size
    return v.reshape(shape)


class Oracle3D:
    """Fields, ψ and coefficients of one 3D run.

    ``coeffs``: cb_ex, cb_ey, cb_ez (component shapes), db, inv_dx, inv_dy, inv_dz (scalars)
    and per axis a in "xyz" the CPML profiles b{a}_e, c{a}_e, ik{a}_e (integer positions)
    and b{a}_h, c{a}_h, ik{a}_h (half positions), all cast to ``dtype``. Sources and monitors
    are oracle/te_numpy.py's OracleSource / OracleMonitor with ``i`` the flat index of each
    node (``j`` unused) and ``flat_index`` into the component arrays.
    """

    FIELDS = COMPONENTS + tuple(psi_name(c, a) for c, a in PSI)

    def __init__(self, n, periodic, dt, coeffs, dtype, sources=(), monitors=()):
        self.n = tuple(int(v) for v in n)
        self.periodic = tuple(bool(p) for p in periodic)
        self.dt = dt
        self.real = np.dtype(dtype).type
        self.complex = np.complex64 if self.real == np.float32 else np.complex128
        for k, v in coeffs.items():
            setattr(self, k, v)
        for c in COMPONENTS:
            setattr(self, c, np.zeros(shape_of(c, self.n, self.periodic), self.real))
        for c, a in PSI:
            setattr(self, psi_name(c, a), np.zeros(shape_of(c, self.n, self.periodic), self.real))
        self.sources = list(sources)
        self.monitors = list(monitors)
        self.acc = [np.zeros((m.frequencies.size, m.flat_index.size), self.complex) for m in self.monitors]
        self.step_index = 0

    # -- differences: forward (H update, at half positions) and backward (E update, at the
    # integer positions off the walls: 1 … n-1 on a PEC axis, all n on a periodic one)
    def _fwd(self, f, axis):
        if self.periodic[axis]:
            return np.roll(f, -1, axis) - f
        return f[_sl(axis, slice(1, None))] - f[_sl(axis, slice(None, -1))]

    def _bwd(self, f, axis):
        if self.periodic[axis]:
            return f - np.roll(f, 1, axis)
        return f[_sl(axis, slice(1, None))] - f[_sl(axis, slice(None, -1))]

    def _inner(self, axis):
        return slice(None) if self.periodic[axis] else slice(1, -1)

    def _prof(self, name, axis, kind, inner=False):
        v = getattr(self, f"{name}{AXES[axis]}_{kind}")
        return _bcast(v[self._inner(axis)] if inner else v, axis)

    def _h_term(self, comp, axis, d):
        """ψ ← b·ψ + c·∂ (half positions along ``axis``), then ∂·1/κ + ψ."""
        psi = getattr(self, psi_name(comp, axis))
        psi[...] = self._prof("b", axis, "h") * psi + self._prof("c", axis, "h") * d
        return d * self._prof("ik", axis, "h") + psi

    def _e_term(self, comp, axis, d, region):
        psi = getattr(self, psi_name(comp, axis))[region]
        psi[...] = self._prof("b", axis, "e", True) * psi + self._prof("c", axis, "e", True) * d
        return d * self._prof("ik", axis, "e", True) + psi

    def update_h(self) -> None:
        dey_dz = self._fwd(self.ey, 2) * self.inv_dz
        dez_dy = self._fwd(self.ez, 1) * self.inv_dy
        self.hx += self.db * (self._h_term("hx", 2, dey_dz) - self._h_term("hx", 1, dez_dy))
        dez_dx = self._fwd(self.ez, 0) * self.inv_dx
        dex_dz = self._fwd(self.ex, 2) * self.inv_dz
        self.hy += self.db * (self._h_term("hy", 0, dez_dx) - self._h_term("hy", 2, dex_dz))
        dex_dy = self._fwd(self.ex, 1) * self.inv_dy
        dey_dx = self._fwd(self.ey, 0) * self.inv_dx
        self.hz += self.db * (self._h_term("hz", 1, dex_dy) - self._h_term("hz", 0, dey_dx))

    def update_e(self) -> None:
        ix, iy, iz = self._inner(0), self._inner(1), self._inner(2)
        r = (slice(None), iy, iz)  # Ex: every x cell, y and z positions off the walls
        dhz_dy = self._bwd(self.hz, 1)[:, :, iz] * self.inv_dy
        dhy_dz = self._bwd(self.hy, 2)[:, iy, :] * self.inv_dz
        self.ex[r] += self.cb_ex[r] * (self._e_term("ex", 1, dhz_dy, r) - self._e_term("ex", 2, dhy_dz, r))
        r = (ix, slice(None), iz)
        dhz_dx = self._bwd(self.hz, 0)[:, :, iz] * self.inv_dx
        dhx_dz = self._bwd(self.hx, 2)[ix, :, :] * self.inv_dz
        self.ey[r] -= self.cb_ey[r] * (self._e_term("ey", 0, dhz_dx, r) - self._e_term("ey", 2, dhx_dz, r))
        r = (ix, iy, slice(None))
        dhy_dx = self._bwd(self.hy, 0)[:, iy, :] * self.inv_dx
        dhx_dy = self._bwd(self.hx, 1)[ix, :, :] * self.inv_dy
        self.ez[r] += self.cb_ez[r] * (self._e_term("ez", 0, dhy_dx, r) - self._e_term("ez", 1, dhx_dy, r))

    # -- per-step host values, as etalon/fdtd/solver.py:83-110 computes them
    def delta(self, src, n: int) -> np.ndarray:
        if src.table is not None:
            return src.table[n]
        t = n * self.dt if src.magnetic else (n + 0.5) * self.dt
        return (src.coefficient * pulse_signal(*src.pulse, t)).astype(self.real)

    def phasor(self, mon, n: int) -> np.ndarray:
        if mon.table is not None:
            return mon.table[n]
        t = np.array([n + (0.5 if mon.magnetic else 1.0)], dtype=np.float64) * self.dt
        return dft_phasors(mon.frequencies, t, self.dt).astype(self.complex)[0]

    def _inject(self, magnetic: bool) -> None:
        for src in self.sources:
            if src.magnetic == magnetic:
                flat = getattr(self, src.component.lower()).reshape(-1)
                flat[src.i] -= self.delta(src, self.step_index)

    def _accumulate(self, magnetic: bool) -> None:
        for mon, acc in zip(self.monitors, self.acc):
            if mon.magnetic == magnetic:
                accumulate_dft(acc, getattr(self, mon.component.lower()), mon.flat_index,
                               self.phasor(mon, self.step_index))

    def step(self) -> None:
        self.update_h()
        self._inject(True)
        self._accumulate(True)
        self.update_e()
        self._inject(False)
        self._accumulate(False)
        self.step_index += 1

    def run(self, steps: int) -> None:
        for _ in range(steps):
            self.step()

    def energy(self) -> float:
        """Σ ε E² + μ H² over the grid in float64 (units of the cast coefficients: 1/cb and 1/db)."""
        e = sum(np.sum(getattr(self, c).astype(np.float64) ** 2 / getattr(self, "cb_" + c).astype(np.float64))
                for c in ("ex", "ey", "ez"))
        h = sum(np.sum(getattr(self, c).astype(np.float64) ** 2) for c in ("hx", "hy", "hz"))
        return float(e + h / float(self.db))


@dataclass
class Reduction:
    """How a one-cell periodic axis turns a 3D run into a 2D TE run.

    ``axes``: the 3D axes playing the 2D x and y; ``e2d``: the 3D components playing the 2D
    ex and ey; ``h2d``: the one playing hz.
    """

    invariant: int
    axes: tuple[int, int]
    e2d: tuple[str, str]
    h2d: str


REDUCTIONS = (
    Reduction(2, (0, 1), ("ex", "ey"), "hz"),
    Reduction(0, (1, 2), ("ey", "ez"), "hx"),
    Reduction(1, (2, 0), ("ez", "ex"), "hy"),
)


def to_2d(red: Reduction, a: np.ndarray) -> np.ndarray:
    """A 3D component array of an invariant run as the 2D array of its role (axes reordered)."""
    a = np.take(a, 0, axis=red.invariant)
    keep = [ax for ax in range(3) if ax != red.invariant]
    order = [keep.index(red.axes[0]), keep.index(red.axes[1])]
    return np.transpose(a, order)


def from_2d(red: Reduction, a: np.ndarray) -> np.ndarray:
    """Inverse of ``to_2d``: a 2D array placed in the 3D layout (one cell along the invariant axis)."""
    keep = [ax for ax in range(3) if ax != red.invariant]
    order = [red.axes.index(keep[0]), red.axes.index(keep[1])]
    return np.expand_dims(np.transpose(a, order), red.invariant)
