"""Float64 host-side setup of a 2D TE run: grid, CPML profiles, pulses, sampling, phasors.

Everything the kernels consume is computed here in float64 on the host and cast once
to the run's precision, exactly as Etalon does, so that the GPU starts from
bit-identical inputs. Each function performs the same IEEE operations, in the same
order and with the same NumPy call shapes, as the Etalon function it stands in for
(cited per function); only then are the casts bit-identical. The module has no
dependency on the Etalon package, so the backend also runs where Etalon's pydantic
models are not installed.

Units: lengths in µm, times in s, frequencies in Hz (the API units of Etalon);
coefficients in SI.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np
from numpy.typing import NDArray

# CODATA 2018, as etalon/constants.py:13-28.
C_0_SI: float = 299_792_458.0
C_0: float = C_0_SI * 1e6  # µm/s
MU_0: float = 1.25663706212e-6
EPSILON_0: float = 1.0 / (MU_0 * C_0_SI**2)
ETA_0: float = MU_0 * C_0_SI
UM: float = 1e-6

TE_COMPONENTS = ("Ex", "Ey", "Hz")
# half-node (True) or integer-node (False) along x, y — etalon/grid/yee.py:27
_HALF_NODES = {"Hz": (True, True), "Ex": (True, False), "Ey": (False, True)}
_ON_NODE = 1e-9  # etalon/fdtd/dft.py:25
_BOX_TOL = 1e-9  # etalon/grid/materials.py:9


# ----------------------------------------------------------------------------- grid


@dataclass(frozen=True)
class YeeGrid2D:
    """Cell counts (PML included), spacings (µm), Δt (s) and node origin of a TE grid.

    Same fields and node convention as etalon/grid/yee.py:30-79: Hz (nx, ny),
    Ex (nx, ny+1), Ey (nx+1, ny), C-ordered with y fastest.
    """

    nx: int
    ny: int
    dx: float
    dy: float
    dt: float
    pml_layers: int
    x_min: float
    y_min: float
    z: float = 0.0
    courant: float = 0.99

    @property
    def n_cells(self) -> int:
        return self.nx * self.ny

    @property
    def region_cells(self) -> tuple[int, int]:
        return self.nx - 2 * self.pml_layers, self.ny - 2 * self.pml_layers

    def shape(self, component: str) -> tuple[int, int]:
        half_x, half_y = _HALF_NODES[component]
        return (self.nx if half_x else self.nx + 1, self.ny if half_y else self.ny + 1)

    def coords(self, component: str) -> tuple[NDArray[np.float64], NDArray[np.float64]]:
        """Node coordinates along both axes (etalon/grid/yee.py:69-75)."""
        half_x, half_y = _HALF_NODES[component]
        n_x, n_y = self.shape(component)
        x = self.x_min + (np.arange(n_x) + (0.5 if half_x else 0.0)) * self.dx
        y = self.y_min + (np.arange(n_y) + (0.5 if half_y else 0.0)) * self.dy
        return np.asarray(x, dtype=np.float64), np.asarray(y, dtype=np.float64)

    def n_steps(self, run_time: float) -> int:
        """etalon/grid/yee.py:77-79."""
        return math.ceil(round(run_time / self.dt, 9))


def cells_along(size: float, dl: float) -> int:
    """N = ceil(size/dl) without float noise (etalon/grid/yee.py:82-84)."""
    return math.ceil(round(size / dl, 9))


def courant_time_step(courant: float, dx: float, dy: float) -> float:
    """2D CFL step scaled by ``courant`` (etalon/grid/yee.py:87-93)."""
    return courant / (C_0 * math.sqrt(1.0 / dx**2 + 1.0 / dy**2))


def yee_grid(
    size: tuple[float, float],
    dl: float,
    layers: int = 12,
    courant: float = 0.99,
    center: tuple[float, float, float] = (0.0, 0.0, 0.0),
) -> YeeGrid2D:
    """The grid of a region ``size`` (µm, PML excluded) — etalon/grid/yee.py:96-116."""
    n_x = cells_along(size[0], dl)
    n_y = cells_along(size[1], dl)
    dx = size[0] / n_x
    dy = size[1] / n_y
    return YeeGrid2D(
        nx=n_x + 2 * layers,
        ny=n_y + 2 * layers,
        dx=dx,
        dy=dy,
        dt=courant_time_step(courant, dx, dy),
        pml_layers=layers,
        x_min=center[0] - size[0] / 2.0 - layers * dx,
        y_min=center[1] - size[1] / 2.0 - layers * dy,
        z=center[2],
        courant=courant,
    )


# ----------------------------------------------------------------------------- materials


@dataclass(frozen=True)
class Box:
    """Axis-aligned block of relative permittivity ``eps`` (etalon/geometry/box.py:11-32)."""

    center: tuple[float, float, float]
    size: tuple[float, float, float]
    eps: float


def permittivity_on_nodes(
    grid: YeeGrid2D, background_eps: float, boxes: Sequence[Box] = ()
) -> dict[str, NDArray[np.float64]]:
    """Staircase ε_r at the Ex and Ey nodes, last box wins (etalon/grid/materials.py:12-35)."""
    eps: dict[str, NDArray[np.float64]] = {}
    for component in ("Ex", "Ey"):
        x, y = grid.coords(component)
        x_nodes, y_nodes = np.meshgrid(x, y, indexing="ij")
        values = np.full(x_nodes.shape, background_eps)
        for box in boxes:
            (cx, cy, cz), (sx, sy, sz) = box.center, box.size
            if abs(grid.z - cz) > sz / 2.0 + _BOX_TOL:
                continue
            inside = (np.abs(x_nodes - cx) <= sx / 2.0 + _BOX_TOL) & (
                np.abs(y_nodes - cy) <= sy / 2.0 + _BOX_TOL
            )
            values[inside] = box.eps
        eps[component] = values
    return eps


# ----------------------------------------------------------------------------- CPML


@dataclass(frozen=True)
class PMLSpec:
    """CPML settings (etalon/core/boundary.py:34-42)."""

    layers: int = 12
    grading_order: float = 3.0
    sigma_scale: float = 1.0
    kappa_max: float = 1.0


@dataclass(frozen=True)
class CPMLAxis:
    """b, c, 1/κ at integer nodes (``_e``, n+1) and half nodes (``_h``, n)."""

    b_e: NDArray[np.float64]
    c_e: NDArray[np.float64]
    inv_kappa_e: NDArray[np.float64]
    b_h: NDArray[np.float64]
    c_h: NDArray[np.float64]
    inv_kappa_h: NDArray[np.float64]


def pml_depth(n_cells: int, layers: int) -> tuple[NDArray[np.float64], NDArray[np.float64]]:
    """Normalised depth ρ on integer and half nodes (etalon/fdtd/cpml.py:43-51)."""
    rho_e = np.zeros(n_cells + 1)
    rho_h = np.zeros(n_cells)
    k = np.arange(layers + 1)
    rho_e[: layers + 1] = (layers - k) / layers
    k = np.arange(layers)
    rho_h[:layers] = (layers - k - 0.5) / layers
    return np.maximum(rho_e, rho_e[::-1]), np.maximum(rho_h, rho_h[::-1])


def _cpml_profile(rho, sigma_max, kappa_max, alpha_max, order, dt):
    """b, c, 1/κ from ρ (etalon/fdtd/cpml.py:54-71), same operation order."""
    sigma = sigma_max * rho**order
    kappa = 1.0 + (kappa_max - 1.0) * rho**order
    alpha = alpha_max * (1.0 - rho)
    b = np.exp(-(sigma / kappa + alpha) * dt / EPSILON_0)
    c = np.zeros_like(rho)
    inside = rho > 0.0
    s, k, a = sigma[inside], kappa[inside], alpha[inside]
    c[inside] = s * (b[inside] - 1.0) / (s * k + k**2 * a)
    b[~inside] = 1.0
    return b, c, 1.0 / kappa


def cpml_axis(
    n_cells: int, spacing: float, dt: float, pml: PMLSpec, eps_r: float, alpha_max: float = 0.0
) -> CPMLAxis:
    """CPML coefficients along one axis (etalon/fdtd/cpml.py:74-92)."""
    order = pml.grading_order
    sigma_max = pml.sigma_scale * 0.8 * (order + 1.0) / (ETA_0 * spacing * UM * math.sqrt(eps_r))
    rho_e, rho_h = pml_depth(n_cells, pml.layers)
    b_e, c_e, ik_e = _cpml_profile(rho_e, sigma_max, pml.kappa_max, alpha_max, order, dt)
    b_h, c_h, ik_h = _cpml_profile(rho_h, sigma_max, pml.kappa_max, alpha_max, order, dt)
    return CPMLAxis(b_e, c_e, ik_e, b_h, c_h, ik_h)


# ----------------------------------------------------------------------------- sources


@dataclass(frozen=True)
class GaussianPulse:
    """Sine-modulated Gaussian (etalon/core/source.py:12-68); wavelengths in µm."""

    wavelength: float
    bandwidth: float
    amplitude: float = 1.0

    @property
    def frequency(self) -> float:
        return C_0 / self.wavelength

    @property
    def frequency_width(self) -> float:
        f_hi = C_0 / (self.wavelength - self.bandwidth / 2.0)
        f_lo = C_0 / (self.wavelength + self.bandwidth / 2.0)
        return (f_hi - f_lo) / 2.0

    @property
    def width(self) -> float:
        return 1.0 / (2.0 * math.pi * self.frequency_width)

    @property
    def delay(self) -> float:
        return 5.0 * self.width


def pulse_signal(pulse: GaussianPulse, t) -> NDArray[np.float64]:
    """g(t) (etalon/fdtd/sources.py:26-30); same NumPy calls, so scalar ``t`` stays 0-d."""
    s = np.asarray(t, dtype=np.float64) - pulse.delay
    envelope = np.exp(-(s**2) / (2.0 * pulse.width**2))
    return pulse.amplitude * envelope * np.sin(2.0 * np.pi * pulse.frequency * s)


@dataclass(frozen=True)
class PointSource:
    """A point current on one TE component (etalon/core/source.py:71-97)."""

    center: tuple[float, float, float]
    component: str
    pulse: GaussianPulse


@dataclass(frozen=True)
class PointInjection:
    """A point source resolved onto nodes (etalon/fdtd/sources.py:33-56)."""

    component: str
    i: NDArray[np.int64]
    j: NDArray[np.int64]
    weights: NDArray[np.float64]
    coefficient: NDArray[np.float64]
    pulse: GaussianPulse

    @property
    def is_magnetic(self) -> bool:
        return self.component.startswith("H")

    def sample_time(self, n: int, dt: float) -> float:
        """nΔt for M, (n+½)Δt for J (etalon/fdtd/sources.py:50-52)."""
        return n * dt if self.is_magnetic else (n + 0.5) * dt

    def delta(self, n: int, dt: float) -> NDArray[np.float64]:
        """Float64 amount subtracted at the nodes during step n (sources.py:54-56)."""
        return self.coefficient * pulse_signal(self.pulse, self.sample_time(n, dt))

    def delta_table(self, n0: int, rows: int, dt: float, dtype) -> NDArray:
        """Rows n0 … n0+rows−1 of ``delta(n).astype(dtype)``, one scalar evaluation per step.

        Each step is evaluated exactly as Etalon's solver evaluates it (a 0-d g(t)
        times the coefficient vector, then the cast), so every row is bit-identical
        to the per-step host value the NumPy backend subtracts.
        """
        out = np.empty((rows, self.coefficient.size), dtype=dtype)
        for r in range(rows):
            out[r] = self.delta(n0 + r, dt).astype(dtype)
        return out


def point_injection(
    source: PointSource, grid: YeeGrid2D, eps_r: dict[str, NDArray[np.float64]]
) -> PointInjection:
    """Bilinear weights and coefficients of a point source (etalon/fdtd/sources.py:59-83)."""
    x_nodes, y_nodes = grid.coords(source.component)
    what = f"source at {source.center}"
    sx = axis_sampling(x_nodes, source.center[0], 0.0, what)
    sy = axis_sampling(y_nodes, source.center[1], 0.0, what)
    i = np.repeat(sx.index, sy.index.size)
    j = np.tile(sy.index, sx.index.size)
    weights = np.outer(sx.weights, sy.weights).ravel()
    area = (grid.dx * UM) * (grid.dy * UM)
    if source.component.startswith("H"):
        update = np.full(weights.shape, grid.dt / MU_0)
    else:
        update = grid.dt / (EPSILON_0 * eps_r[source.component][i, j])
    return PointInjection(source.component, i, j, weights, update * weights / area, source.pulse)


# ----------------------------------------------------------------------------- monitors


@dataclass(frozen=True)
class AxisSampling:
    """Nodes taken along one axis (etalon/fdtd/dft.py:28-36)."""

    index: NDArray[np.int64]
    coords: NDArray[np.float64]
    weights: NDArray[np.float64] | None
    point: float | None


def axis_sampling(nodes: NDArray[np.float64], center: float, size: float, what: str) -> AxisSampling:
    """Raw nodes inside the span (size > 0) or the bracketing pair (size = 0) — dft.py:39-66."""
    spacing = nodes[1] - nodes[0]
    if size > 0.0:
        tol = _ON_NODE * spacing
        lo, hi = center - size / 2.0, center + size / 2.0
        index = np.nonzero((nodes >= lo - tol) & (nodes <= hi + tol))[0].astype(np.int64)
        if index.size == 0:
            raise ValueError(
                f"{what} contains no grid node along this axis (thinner than one cell, "
                f"{spacing} µm); give it size 0 to interpolate instead"
            )
        return AxisSampling(index, nodes[index], None, None)
    position = (center - nodes[0]) / spacing
    i0 = math.floor(position)
    frac = position - i0
    if frac < _ON_NODE:
        index, weights = np.array([i0]), np.array([1.0])
    elif frac > 1.0 - _ON_NODE:
        index, weights = np.array([i0 + 1]), np.array([1.0])
    else:
        index, weights = np.array([i0, i0 + 1]), np.array([1.0 - frac, frac])
    if index[0] < 0 or index[-1] >= nodes.size:
        raise ValueError(f"{what} at {center} µm is outside the grid")
    index = index.astype(np.int64)
    return AxisSampling(index, nodes[index], weights, center)


@dataclass(frozen=True)
class DFTMonitor:
    """Running-DFT monitor (etalon/core/monitor.py:10-52)."""

    name: str
    wavelengths: Sequence[float]
    center: tuple[float, float, float] = (0.0, 0.0, 0.0)
    size: tuple[float, float, float] = (0.0, 0.0, 0.0)
    components: tuple[str, ...] | None = None


@dataclass(frozen=True)
class ComponentSampling:
    """The nodes one monitor records for one component (etalon/fdtd/dft.py:69-89).

    The nodes always form a rectangle [x.index] × [y.index] of consecutive indices,
    which is what lets the fused kernels test membership with two comparisons.
    """

    monitor: str
    component: str
    wavelengths: NDArray[np.float64]
    x: AxisSampling
    y: AxisSampling
    flat_index: NDArray[np.int64]

    @property
    def frequencies(self) -> NDArray[np.float64]:
        return C_0 / self.wavelengths

    @property
    def is_magnetic(self) -> bool:
        return self.component.startswith("H")


def monitor_samplings(monitor: DFTMonitor, grid: YeeGrid2D) -> list[ComponentSampling]:
    """One sampling per recorded component (etalon/fdtd/dft.py:92-107)."""
    components = monitor.components or TE_COMPONENTS
    wavelengths = np.asarray(monitor.wavelengths, dtype=np.float64)
    out = []
    for component in components:
        x_nodes, y_nodes = grid.coords(component)
        what = f"monitor {monitor.name!r} ({component})"
        sx = axis_sampling(x_nodes, monitor.center[0], monitor.size[0], what)
        sy = axis_sampling(y_nodes, monitor.center[1], monitor.size[1], what)
        n_y = grid.shape(component)[1]
        flat = (sx.index[:, None] * n_y + sy.index[None, :]).ravel()
        out.append(ComponentSampling(monitor.name, component, wavelengths, sx, sy, flat.astype(np.int64)))
    return out


def dft_phasors(frequencies: NDArray[np.float64], times: NDArray[np.float64], dt: float) -> NDArray[np.complex128]:
    """exp(+i2πft)·Δt in float64, shape (n_t, n_f) (etalon/fdtd/dft.py:110-119)."""
    phase = 2.0 * np.pi * times[:, None] * frequencies[None, :]
    return np.asarray(np.exp(1j * phase) * dt, dtype=np.complex128)


def phasor_table(
    sampling: ComponentSampling, n0: int, rows: int, dt: float, complex_dtype
) -> NDArray:
    """Phasor rows for steps n0 … n0+rows−1 at the sampling's own DFT time.

    H is sampled at (n+½)Δt and E at (n+1)Δt (etalon/fdtd/solver.py:91-110). Every
    entry depends only on its own step, so one table for the whole run equals
    Etalon's chunked tables bit for bit (tests/unit/test_sources_cpml_dft.py:189-221).
    """
    steps = np.arange(n0, n0 + rows, dtype=np.float64)
    offset = 0.5 if sampling.is_magnetic else 1.0
    return dft_phasors(sampling.frequencies, (steps + offset) * dt, dt).astype(complex_dtype)


# ----------------------------------------------------------------------------- problem


@dataclass
class TEProblem:
    """Everything a 2D TE run consumes, in float64, before the cast to its precision."""

    grid: YeeGrid2D
    eps: dict[str, NDArray[np.float64]]
    cpml_x: CPMLAxis
    cpml_y: CPMLAxis
    injections: list[PointInjection]
    samplings: list[ComponentSampling]
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


def te_problem(
    size: tuple[float, float],
    dl: float,
    sources: Sequence[PointSource],
    monitors: Sequence[DFTMonitor] = (),
    *,
    background_eps: float = 1.0,
    boxes: Sequence[Box] = (),
    eps: dict[str, NDArray[np.float64]] | None = None,
    pml: PMLSpec = PMLSpec(),
    courant: float = 0.99,
    center: tuple[float, float, float] = (0.0, 0.0, 0.0),
    n_steps: int = 0,
    run_time: float | None = None,
    precision: str = "single",
) -> TEProblem:
    """Resolve a TE simulation description the way etalon/fdtd/solver.py:55-81 does.

    ``eps`` overrides the staircase of ``boxes`` with explicit maps at the Ex and Ey
    nodes (shapes grid.shape("Ex"), grid.shape("Ey")), for seeded synthetic devices.
    """
    if precision not in ("single", "double"):
        raise ValueError(f"precision must be 'single' or 'double', not {precision!r}")
    grid = yee_grid(size, dl, pml.layers, courant, center)
    if eps is None:
        eps = permittivity_on_nodes(grid, background_eps, boxes)
    else:
        for c in ("Ex", "Ey"):
            if eps[c].shape != grid.shape(c):
                raise ValueError(f"eps[{c!r}] has shape {eps[c].shape}, grid needs {grid.shape(c)}")
        eps = {c: np.asarray(eps[c], dtype=np.float64) for c in ("Ex", "Ey")}
    cpml_x = cpml_axis(grid.nx, grid.dx, grid.dt, pml, background_eps)
    cpml_y = cpml_axis(grid.ny, grid.dy, grid.dt, pml, background_eps)
    injections = [point_injection(s, grid, eps) for s in sources]
    samplings = [s for m in monitors for s in monitor_samplings(m, grid)]
    if run_time is not None:
        n_steps = grid.n_steps(run_time)
    return TEProblem(grid, eps, cpml_x, cpml_y, injections, samplings, precision, n_steps,
                     background_eps, list(monitors))


@dataclass
class CastCoefficients:
    """The coefficient arrays of etalon/fdtd/state.py:52-99, cast once to the run's dtype."""

    cb_ex: NDArray
    cb_ey: NDArray
    bx_e: NDArray
    cx_e: NDArray
    ikx_e: NDArray
    bx_h: NDArray
    cx_h: NDArray
    ikx_h: NDArray
    by_e: NDArray
    cy_e: NDArray
    iky_e: NDArray
    by_h: NDArray
    cy_h: NDArray
    iky_h: NDArray
    db: np.floating
    inv_dx: np.floating
    inv_dy: np.floating


def cast_coefficients(problem: TEProblem) -> CastCoefficients:
    """cb = Δt/(ε0 ε_r), db = Δt/μ0, 1/Δ in 1/m, then one cast (etalon/fdtd/state.py:75-97)."""
    g, dtype = problem.grid, problem.real

    def put(a):
        return np.ascontiguousarray(a, dtype=dtype)

    cx, cy = problem.cpml_x, problem.cpml_y
    return CastCoefficients(
        cb_ex=put(g.dt / (EPSILON_0 * problem.eps["Ex"])),
        cb_ey=put(g.dt / (EPSILON_0 * problem.eps["Ey"])),
        bx_e=put(cx.b_e), cx_e=put(cx.c_e), ikx_e=put(cx.inv_kappa_e),
        bx_h=put(cx.b_h), cx_h=put(cx.c_h), ikx_h=put(cx.inv_kappa_h),
        by_e=put(cy.b_e), cy_e=put(cy.c_e), iky_e=put(cy.inv_kappa_e),
        by_h=put(cy.b_h), cy_h=put(cy.c_h), iky_h=put(cy.inv_kappa_h),
        db=dtype(g.dt / MU_0),
        inv_dx=dtype(1.0 / (g.dx * UM)),
        inv_dy=dtype(1.0 / (g.dy * UM)),
    )  # fmt: skip
