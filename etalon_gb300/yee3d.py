"""3D Yee runs on the GPU: float64 setup on the host, one cast, then the resident engine.

Etalon has no 3D solver (etalon/fdtd/capabilities.py:7-24 refuses it); its mvp-spec plans 3D
FDTD as milestone M1 (docs/mvp-spec.md:77). This module carries Etalon's 2D TE setup to three
axes, function by function, so a 3D run shares every convention of the 2D path:

* ``YeeGrid3D`` / ``yee_grid_3d``: etalon/grid/yee.py:82-116 per axis (N = ceil(size/dl),
  Δ = size/N, PML layers outside the region) with the 3D CFL step; node convention of
  etalon/grid/yee.py:27-79: E on cell edges, H on cell faces; along a PEC axis the integer
  positions include both walls. An axis may instead be periodic (no walls, no CPML).
* ``permittivity_3d``: the staircase of etalon/grid/materials.py:12-35 at the Ex, Ey and Ez
  nodes (a node inside a box within the tolerance takes its ε; the last box wins).
* ``cpml_profile_3d``: etalon/fdtd/cpml.py:74-92 along each axis with CPML.
* ``point_injection_3d``: etalon/fdtd/sources.py:59-83 with a third axis (trilinear weights
  over the bracketing nodes, coefficient Δt/μ0 or Δt/(ε0 ε_r) times weight over the cell
  volume); the per-step values are the same float64 expression cast once.
* ``monitor_samplings_3d``: etalon/fdtd/dft.py:39-107 per axis; phasors as
  etalon/fdtd/solver.py:91-110 (H at (n+½)Δt, E at (n+1)Δt).

``Yee3DEngine`` steps the run on the device (etalon_gb300/csrc/etg_yee3d.cu, entry points
``etg_yee3d_*`` of include/etalon_gb300.h).
"""

from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np
from numpy.typing import NDArray

from . import _lib
from ._lib import call
from .physics import (_BOX_TOL, C_0, EPSILON_0, MU_0, UM, AxisSampling, Box, CPMLAxis, DFTMonitor, GaussianPulse,
                      PMLSpec, PointSource, axis_sampling, cells_along, cpml_axis, phasor_table, pulse_signal)

COMPONENTS_3D = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")
# half position (True) or integer position (False) along x, y, z
HALF_3D = {"Ex": (True, False, False), "Ey": (False, True, False), "Ez": (False, False, True),
           "Hx": (False, True, True), "Hy": (True, False, True), "Hz": (True, True, False)}  # fmt: skip
PSI_3D = (("hx", "y"), ("hx", "z"), ("hy", "z"), ("hy", "x"), ("hz", "x"), ("hz", "y"),
          ("ex", "y"), ("ex", "z"), ("ey", "z"), ("ey", "x"), ("ez", "x"), ("ez", "y"))  # fmt: skip
ARRAY_IDS_3D = {c.lower(): k for k, c in enumerate(COMPONENTS_3D)}
ARRAY_IDS_3D.update({f"psi_{c}_{a}": 6 + k for k, (c, a) in enumerate(PSI_3D)})
ARRAY_IDS_3D.update({"cb_ex": 18, "cb_ey": 19, "cb_ez": 20})


def _triple(v) -> tuple:
    return tuple(v) if isinstance(v, (tuple, list)) else (v, v, v)


@dataclass(frozen=True)
class YeeGrid3D:
    """Cells per axis (PML included), spacings (µm), Δt (s), CPML layers and periodic axes."""

    nx: int
    ny: int
    nz: int
    dx: float
    dy: float
    dz: float
    dt: float
    pml_layers: tuple[int, int, int]
    periodic: tuple[bool, bool, bool]
    origin: tuple[float, float, float]  # coordinates (µm) of integer position (0, 0, 0)
    courant: float = 0.99

    @property
    def n(self) -> tuple[int, int, int]:
        return self.nx, self.ny, self.nz

    @property
    def d(self) -> tuple[float, float, float]:
        return self.dx, self.dy, self.dz

    @property
    def n_cells(self) -> int:
        return self.nx * self.ny * self.nz

    def shape(self, component: str) -> tuple[int, int, int]:
        half = HALF_3D[component]
        return tuple(self.n[a] + (0 if half[a] or self.periodic[a] else 1) for a in range(3))  # type: ignore[return-value]

    def coords(self, component: str) -> tuple[NDArray[np.float64], ...]:
        half = HALF_3D[component]
        shape = self.shape(component)
        return tuple(np.asarray(self.origin[a] + (np.arange(shape[a]) + (0.5 if half[a] else 0.0)) * self.d[a],
                                dtype=np.float64) for a in range(3))  # fmt: skip

    def n_steps(self, run_time: float) -> int:
        return math.ceil(round(run_time / self.dt, 9))


def courant_time_step_3d(courant: float, dx: float, dy: float, dz: float) -> float:
    """3D CFL step scaled by ``courant`` (the 2D rule of etalon/grid/yee.py:87-93 with dz)."""
    return courant / (C_0 * math.sqrt(1.0 / dx**2 + 1.0 / dy**2 + 1.0 / dz**2))


def yee_grid_3d(
    size: tuple[float, float, float],
    dl,
    layers=12,
    *,
    periodic=(False, False, False),
    courant: float = 0.99,
    center: tuple[float, float, float] = (0.0, 0.0, 0.0),
    dt: float | None = None,
) -> YeeGrid3D:
    """The grid of a region ``size`` (µm, PML excluded); ``dl`` and ``layers`` per axis or one
    for all. Periodic axes take no layers. ``dt`` overrides the CFL step (a run reduced to 2D
    uses the 2D run's step)."""
    dl, layers, periodic = _triple(dl), list(_triple(layers)), tuple(bool(p) for p in _triple(periodic))
    cells, spacing, origin = [], [], []
    for a in range(3):
        if periodic[a]:
            layers[a] = 0
        n = cells_along(size[a], dl[a])
        d = size[a] / n
        cells.append(n + 2 * layers[a])
        spacing.append(d)
        origin.append(center[a] - size[a] / 2.0 - layers[a] * d)
    step = courant_time_step_3d(courant, *spacing) if dt is None else float(dt)
    return YeeGrid3D(cells[0], cells[1], cells[2], spacing[0], spacing[1], spacing[2], step, tuple(layers),
                     periodic, tuple(origin), courant)  # type: ignore[arg-type]


def _unit_axis(n_e: int, n_h: int) -> CPMLAxis:
    return CPMLAxis(np.ones(n_e), np.zeros(n_e), np.ones(n_e), np.ones(n_h), np.zeros(n_h), np.ones(n_h))


def cpml_profile_3d(grid: YeeGrid3D, axis: int, pml: PMLSpec, background_eps: float) -> CPMLAxis:
    """b, c, 1/κ along one axis (etalon/fdtd/cpml.py:74-92); unit profiles without CPML."""
    n, layers = grid.n[axis], grid.pml_layers[axis]
    if grid.periodic[axis]:
        return _unit_axis(n, n)
    if layers == 0:
        return _unit_axis(n + 1, n)
    spec = PMLSpec(layers=layers, grading_order=pml.grading_order, sigma_scale=pml.sigma_scale,
                   kappa_max=pml.kappa_max)  # fmt: skip
    return cpml_axis(n, grid.d[axis], grid.dt, spec, background_eps)


def permittivity_3d(grid: YeeGrid3D, background_eps: float, boxes: Sequence[Box] = ()) -> dict[str, NDArray]:
    """Staircase ε_r at the Ex, Ey and Ez nodes, the last box winning (materials.py:12-35)."""
    eps = {}
    for component in ("Ex", "Ey", "Ez"):
        x, y, z = grid.coords(component)
        values = np.full(grid.shape(component), background_eps)
        for box in boxes:
            (cx, cy, cz), (sx, sy, sz) = box.center, box.size
            inside = ((np.abs(x - cx) <= sx / 2.0 + _BOX_TOL)[:, None, None]
                      & (np.abs(y - cy) <= sy / 2.0 + _BOX_TOL)[None, :, None]
                      & (np.abs(z - cz) <= sz / 2.0 + _BOX_TOL)[None, None, :])  # fmt: skip
            values[inside] = box.eps
        eps[component] = values
    return eps


@dataclass(frozen=True)
class PointInjection3D:
    """A point source resolved onto nodes: flat C-order indices into its component."""

    component: str
    flat: NDArray[np.int64]
    weights: NDArray[np.float64]
    coefficient: NDArray[np.float64]
    pulse: GaussianPulse

    @property
    def is_magnetic(self) -> bool:
        return self.component.startswith("H")

    def sample_time(self, n: int, dt: float) -> float:
        return n * dt if self.is_magnetic else (n + 0.5) * dt

    def delta(self, n: int, dt: float) -> NDArray[np.float64]:
        return self.coefficient * pulse_signal(self.pulse, self.sample_time(n, dt))

    def delta_table(self, n0: int, rows: int, dt: float, dtype) -> NDArray:
        out = np.empty((rows, self.coefficient.size), dtype=dtype)
        for r in range(rows):
            out[r] = self.delta(n0 + r, dt).astype(dtype)
        return out


def _sampling(nodes: NDArray[np.float64], center: float, size: float, what: str) -> AxisSampling:
    """``axis_sampling`` (etalon/fdtd/dft.py:39-66), or the one position of an axis that has
    a single one (a one-cell periodic axis: the run does not vary along it)."""
    if nodes.size == 1:
        return AxisSampling(np.zeros(1, np.int64), nodes.copy(), None if size > 0.0 else np.ones(1),
                            None if size > 0.0 else center)  # fmt: skip
    return axis_sampling(nodes, center, size, what)


def point_injection_3d(source: PointSource, grid: YeeGrid3D, eps: dict[str, NDArray]) -> PointInjection3D:
    """Trilinear weights and coefficients of a point source (sources.py:59-83 with z)."""
    what = f"source at {source.center}"
    s = [_sampling(c, source.center[a], 0.0, what) for a, c in enumerate(grid.coords(source.component))]
    ii, jj, kk = np.meshgrid(s[0].index, s[1].index, s[2].index, indexing="ij")
    weights = (np.outer(s[0].weights, s[1].weights)[:, :, None] * s[2].weights[None, None, :]).ravel()
    volume = (grid.dx * UM) * (grid.dy * UM) * (grid.dz * UM)
    i, j, k = ii.ravel(), jj.ravel(), kk.ravel()
    if source.component.startswith("H"):
        update = np.full(weights.shape, grid.dt / MU_0)
    else:
        update = grid.dt / (EPSILON_0 * eps[source.component][i, j, k])
    flat = np.ravel_multi_index((i, j, k), grid.shape(source.component)).astype(np.int64)
    return PointInjection3D(source.component, flat, weights, update * weights / volume, source.pulse)


@dataclass(frozen=True)
class ComponentSampling3D:
    """The nodes one monitor records for one component: a box of consecutive indices."""

    monitor: str
    component: str
    wavelengths: NDArray[np.float64]
    axes: tuple[AxisSampling, AxisSampling, AxisSampling]
    flat_index: NDArray[np.int64]

    @property
    def frequencies(self) -> NDArray[np.float64]:
        return C_0 / self.wavelengths

    @property
    def is_magnetic(self) -> bool:
        return self.component.startswith("H")

    def interpolate(self, acc: NDArray) -> NDArray:
        """Point value of a point sampling: Σ w_x w_y w_z acc (float64), one per frequency."""
        w = [a.weights if a.weights is not None else np.ones(a.index.size) for a in self.axes]
        weights = (np.outer(w[0], w[1])[:, :, None] * w[2][None, None, :]).ravel()
        return np.asarray(acc, dtype=np.complex128) @ weights


def monitor_samplings_3d(monitor: DFTMonitor, grid: YeeGrid3D) -> list[ComponentSampling3D]:
    """One sampling per recorded component (etalon/fdtd/dft.py:92-107 with z)."""
    components = monitor.components or COMPONENTS_3D
    wavelengths = np.asarray(monitor.wavelengths, dtype=np.float64)
    out = []
    for component in components:
        what = f"monitor {monitor.name!r} ({component})"
        axes = tuple(_sampling(c, monitor.center[a], monitor.size[a], what)
                     for a, c in enumerate(grid.coords(component)))  # fmt: skip
        ii, jj, kk = np.meshgrid(axes[0].index, axes[1].index, axes[2].index, indexing="ij")
        flat = np.ravel_multi_index((ii.ravel(), jj.ravel(), kk.ravel()), grid.shape(component))
        out.append(ComponentSampling3D(monitor.name, component, wavelengths, axes, flat.astype(np.int64)))  # type: ignore[arg-type]
    return out


@dataclass
class Yee3DProblem:
    """Everything a 3D run consumes, in float64, before the cast to its precision."""

    grid: YeeGrid3D
    eps: dict[str, NDArray[np.float64]]
    cpml: tuple[CPMLAxis, CPMLAxis, CPMLAxis]
    injections: list[PointInjection3D]
    samplings: list[ComponentSampling3D]
    precision: str = "single"
    n_steps: int = 0
    background_eps: float = 1.0
    monitors: list[DFTMonitor] = field(default_factory=list)

    @property
    def real(self):
        return np.float32 if self.precision == "single" else np.float64

    @property
    def complex(self):
        return np.complex64 if self.precision == "single" else np.complex128


def yee3d_problem(
    size: tuple[float, float, float],
    dl,
    sources: Sequence[PointSource] = (),
    monitors: Sequence[DFTMonitor] = (),
    *,
    background_eps: float = 1.0,
    boxes: Sequence[Box] = (),
    eps: dict[str, NDArray] | None = None,
    pml: PMLSpec = PMLSpec(),
    layers=None,
    periodic=(False, False, False),
    courant: float = 0.99,
    center: tuple[float, float, float] = (0.0, 0.0, 0.0),
    dt: float | None = None,
    n_steps: int = 0,
    run_time: float | None = None,
    precision: str = "single",
) -> Yee3DProblem:
    """Resolve a 3D run the way etalon/fdtd/solver.py:55-81 resolves a 2D one."""
    if precision not in ("single", "double"):
        raise ValueError(f"precision must be 'single' or 'double', not {precision!r}")
    grid = yee_grid_3d(size, dl, pml.layers if layers is None else layers, periodic=periodic, courant=courant,
                       center=center, dt=dt)  # fmt: skip
    if eps is None:
        eps = permittivity_3d(grid, background_eps, boxes)
    else:
        for c in ("Ex", "Ey", "Ez"):
            if eps[c].shape != grid.shape(c):
                raise ValueError(f"eps[{c!r}] has shape {eps[c].shape}, grid needs {grid.shape(c)}")
        eps = {c: np.asarray(eps[c], dtype=np.float64) for c in ("Ex", "Ey", "Ez")}
    cpml = tuple(cpml_profile_3d(grid, a, pml, background_eps) for a in range(3))
    injections = [point_injection_3d(s, grid, eps) for s in sources]
    samplings = [s for m in monitors for s in monitor_samplings_3d(m, grid)]
    if run_time is not None:
        n_steps = grid.n_steps(run_time)
    return Yee3DProblem(grid, eps, cpml, injections, samplings, precision, n_steps, background_eps,  # type: ignore[arg-type]
                        list(monitors))


def cast_coefficients_3d(problem: Yee3DProblem) -> dict[str, np.ndarray]:
    """cb = Δt/(ε0 ε_r) per E component, db = Δt/μ0, 1/Δ in 1/m and the CPML profiles, each
    computed in float64 and cast once (etalon/fdtd/state.py:75-97 with z)."""
    g, dtype = problem.grid, problem.real
    out = {f"cb_{c.lower()}": np.ascontiguousarray(g.dt / (EPSILON_0 * problem.eps[c]), dtype=dtype)
           for c in ("Ex", "Ey", "Ez")}  # fmt: skip
    out["db"] = dtype(g.dt / MU_0)
    for a, name in enumerate("xyz"):
        out[f"inv_d{name}"] = dtype(1.0 / (g.d[a] * UM))
        p = problem.cpml[a]
        for k, v in (("b", p.b_e), ("c", p.c_e), ("ik", p.inv_kappa_e)):
            out[f"{k}{name}_e"] = np.ascontiguousarray(v, dtype=dtype)
        for k, v in (("b", p.b_h), ("c", p.c_h), ("ik", p.inv_kappa_h)):
            out[f"{k}{name}_h"] = np.ascontiguousarray(v, dtype=dtype)
    return out


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


class Yee3DEngine:
    """One resident 3D run. ``table_steps``: steps the source and phasor tables cover (the
    problem's n_steps by default). ``fused``: an H and an E kernel per step in place (False,
    the default and the faster), or one kernel per step over two buffer sets; both give the
    same bits. Not thread-safe; one engine per host thread."""

    def __init__(self, problem: Yee3DProblem, *, table_steps: int | None = None, fused: bool = False) -> None:
        self.problem = problem
        g = problem.grid
        self.real, self.complex = problem.real, problem.complex
        self._lib = _lib.lib()
        handle = C.c_void_p()
        mask = sum(1 << a for a in range(3) if g.periodic[a])
        call("etg_yee3d_create", C.byref(handle), _lib.dtype_code(self.real), g.nx, g.ny, g.nz, mask)
        self._h = handle
        try:
            call("etg_yee3d_set_option", self._h, 0, int(bool(fused)))
            c = cast_coefficients_3d(problem)
            self._coeffs = c
            scal = np.array([c["db"], c["inv_dx"], c["inv_dy"], c["inv_dz"]], dtype=self.real)
            call("etg_yee3d_set_scalars", self._h, _ptr(scal))
            for a, name in enumerate("xyz"):
                arrays = [c[f"{k}{name}_{w}"] for w in ("e", "h") for k in ("b", "c", "ik")]
                call("etg_yee3d_set_profile", self._h, a, *[_ptr(v) for v in arrays])
            for comp in ("ex", "ey", "ez"):
                self.set_field("cb_" + comp, c["cb_" + comp])
            rows = table_steps if table_steps is not None else (problem.n_steps or 0)
            for inj in problem.injections:
                table = np.ascontiguousarray(inj.delta_table(0, max(rows, 1), g.dt, self.real))
                flat = np.ascontiguousarray(inj.flat, dtype=np.int64)
                call("etg_yee3d_add_source", self._h, COMPONENTS_3D.index(inj.component), flat.size, _ptr(flat), 0,
                     table.shape[0], _ptr(table))  # fmt: skip
            for s in problem.samplings:
                table = np.ascontiguousarray(phasor_table(s, 0, max(rows, 1), g.dt, self.complex))  # type: ignore[arg-type]
                flat = np.ascontiguousarray(s.flat_index, dtype=np.int64)
                call("etg_yee3d_add_monitor", self._h, COMPONENTS_3D.index(s.component), flat.size, _ptr(flat),
                     s.wavelengths.size, 0, table.shape[0], _ptr(table))  # fmt: skip
        except Exception:
            self.close()
            raise

    @property
    def n(self) -> int:
        v = C.c_int64()
        call("etg_yee3d_step_index", self._h, C.byref(v))
        return v.value

    def advance(self, k: int) -> None:
        call("etg_yee3d_advance", self._h, int(k))

    def set_fused(self, fused: bool) -> None:
        """Switch between the fused step and the two-kernel step (the state carries over)."""
        call("etg_yee3d_set_option", self._h, 0, int(bool(fused)))

    def synchronize(self) -> None:
        call("etg_yee3d_synchronize", self._h)

    def shape(self, name: str) -> tuple[int, int, int]:
        comp = name[4:6] if name.startswith("psi_") else name[3:5] if name.startswith("cb_") else name
        return self.problem.grid.shape(comp[0].upper() + comp[1])

    def field(self, name: str) -> np.ndarray:
        out = np.empty(self.shape(name), self.real)
        call("etg_yee3d_get_field", self._h, ARRAY_IDS_3D[name], _ptr(out))
        return out

    def set_field(self, name: str, value: np.ndarray) -> None:
        a = np.ascontiguousarray(value, dtype=self.real)
        if a.shape != self.shape(name):
            raise ValueError(f"{name}: shape {a.shape}, expected {self.shape(name)}")
        call("etg_yee3d_set_field", self._h, ARRAY_IDS_3D[name], _ptr(a))

    def fields(self) -> dict[str, np.ndarray]:
        return {c: self.field(c.lower()) for c in COMPONENTS_3D}

    def dft(self, k: int) -> np.ndarray:
        s = self.problem.samplings[k]
        out = np.empty((s.wavelengths.size, s.flat_index.size), self.complex)
        call("etg_yee3d_get_dft", self._h, k, _ptr(out))
        return out

    def last_timing(self) -> tuple[float, int]:
        ms, launches = C.c_double(), C.c_int64()
        call("etg_yee3d_last_timing", self._h, C.byref(ms), C.byref(launches))
        return ms.value, launches.value

    def kernel_timing(self, steps: int) -> tuple[float, float]:
        """Run ``steps`` more steps, timing each stencil launch alone: mean ms of the fused
        step's kernel and 0, or of the H and the E kernel."""
        h, e = C.c_double(), C.c_double()
        call("etg_yee3d_kernel_timing", self._h, int(steps), C.byref(h), C.byref(e))
        return h.value, e.value

    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.etg_yee3d_destroy(h)
            self._h = C.c_void_p()

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self) -> "Yee3DEngine":
        return self

    def __exit__(self, *exc) -> None:
        self.close()
