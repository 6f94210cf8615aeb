"""2D TM runs (Ez, Hx, Hy) on the TE kernels, through the TE/TM duality (no counterpart in Etalon).

Etalon solves 2D TE only and refuses TM sources and monitors (etalon/fdtd/capabilities.py:7-24).
The TM equations are the TE equations of etalon/fdtd/backends/numpy_backend.py:41-61 with the
roles of E and H exchanged:

    TE   Hz += db (dEx/dy - dEy/dx)   Ex += cb dHz/dy        Ey -= cb dHz/dx
    TM   Ez += ce (dHy/dx - dHx/dy)   Hx -= ch dEz/dy        Hy += ch dEz/dx

(each derivative with its CPML term). With Ez held in the Hz array, -Hx in Ex and -Hy in Ey,
ch = dt/mu0 as cb and ce = dt/(eps0 eps_r) per Ez node in place of the scalar db, the TE
update computes the TM one; IEEE rounding is symmetric, so the negated operands give the
negated results exactly, and the engine's TE arithmetic yields the TM values bit for bit.
The grid follows: Ez at the cell centres (TE's Hz nodes, the staircase eps_r taken there), Hx
at (x_i+1/2, y_j), Hy at (x_i, y_j+1/2); Hx on the outer rows j = 0, ny and Hy on the outer
columns i = 0, nx stay zero (a magnetic wall behind the CPML, the dual of Etalon's PEC). Ez
lives at (n+1/2) dt and H at (n+1) dt; an Ez point current is sampled at n dt and subtracted
right after the Ez update, with Etalon's bilinear weights (etalon/fdtd/sources.py:59-83) and
coefficient dt/(eps0 eps_r) w/(dx dy). Monitors of Ez are Fourier sums at (n+1/2) dt, of Hx, Hy
at (n+1) dt, as Etalon's H and E monitors of the dual run.

The dual run takes the temporally blocked kernels (in their tiles the cb_ey plane, which in
TM mode would only repeat dt/mu0, carries the per-node Ez coefficient) or the one-step ones;
batches and the adjoint are for TE.
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Sequence

import numpy as np
from numpy.typing import NDArray

from ._lib import call
from .physics import (_BOX_TOL, EPSILON_0, MU_0, UM, Box, CastCoefficients, ComponentSampling, DFTMonitor,
                      GaussianPulse, PMLSpec, PointInjection, TEProblem, axis_sampling, cpml_axis, monitor_samplings,
                      yee_grid)
from .solver import interpolate_monitor

TM_COMPONENTS = ("Ez", "Hx", "Hy")
DUAL = {"Ez": "Hz", "Hx": "Ex", "Hy": "Ey"}  # the TE array that holds each TM component
NEGATED = {"Ez": False, "Hx": True, "Hy": True}  # held with the opposite sign


@dataclass(frozen=True)
class TMPointSource:
    """A point current on Ez."""

    center: tuple[float, float, float]
    pulse: GaussianPulse
    component: str = "Ez"


@dataclass
class TMProblem:
    """A TM run and the dual TE problem the engine steps."""

    te: TEProblem                    # grid, CPML, Ez injections (on "Hz"), samplings on the dual components
    eps_ez: NDArray[np.float64]      # eps_r at the Ez nodes (nx, ny)
    components: list[str] = field(default_factory=list)  # the TM component of each sampling of te
    monitors: list[DFTMonitor] = field(default_factory=list)

    @property
    def grid(self):
        return self.te.grid

    @property
    def n_steps(self) -> int:
        return self.te.n_steps

    @property
    def precision(self) -> str:
        return self.te.precision

    @property
    def real(self):
        return self.te.real

    @property
    def complex(self):
        return self.te.complex


def permittivity_at_ez(grid, background_eps: float, boxes: Sequence[Box] = ()) -> NDArray[np.float64]:
    """Staircase eps_r at the Ez nodes (the cell centres), with the box test and order of
    etalon/grid/materials.py:12-35 (last box wins)."""
    x, y = grid.coords("Hz")
    x_nodes, y_nodes = np.meshgrid(x, y, indexing="ij")
    values = np.full(x_nodes.shape, background_eps)
    for box in boxes:
        (cx, cy, cz), (sx, sy, sz) = box.center, box.size
        if abs(grid.z - cz) > sz / 2.0 + _BOX_TOL:
            continue
        inside = (np.abs(x_nodes - cx) <= sx / 2.0 + _BOX_TOL) & (np.abs(y_nodes - cy) <= sy / 2.0 + _BOX_TOL)
        values[inside] = box.eps
    return values


def tm_injection(source: TMPointSource, grid, eps_ez: NDArray[np.float64]) -> PointInjection:
    """An Ez point current on the Ez nodes, as the dual run's Hz injection (sampled at n dt)."""
    if source.component != "Ez":
        raise NotImplementedError(f"TM point sources drive Ez, not {source.component}")
    x_nodes, y_nodes = grid.coords("Hz")
    what = f"source at {source.center}"
    sx = axis_sampling(x_nodes, source.center[0], 0.0, what)
    sy = axis_sampling(y_nodes, source.center[1], 0.0, what)
    i = np.repeat(sx.index, sy.index.size)
    j = np.tile(sy.index, sx.index.size)
    weights = np.outer(sx.weights, sy.weights).ravel()
    area = (grid.dx * UM) * (grid.dy * UM)
    update = grid.dt / (EPSILON_0 * eps_ez[i, j])
    return PointInjection("Hz", i, j, weights, update * weights / area, source.pulse)


def tm_problem(
    size: tuple[float, float],
    dl: float,
    sources: Sequence[TMPointSource],
    monitors: Sequence[DFTMonitor] = (),
    *,
    background_eps: float = 1.0,
    boxes: Sequence[Box] = (),
    pml: PMLSpec = PMLSpec(),
    courant: float = 0.99,
    center: tuple[float, float, float] = (0.0, 0.0, 0.0),
    n_steps: int = 0,
    run_time: float | None = None,
    precision: str = "single",
) -> TMProblem:
    """Resolve a TM simulation onto its dual TE problem (grid and CPML as for TE)."""
    if precision not in ("single", "double"):
        raise ValueError(f"precision must be 'single' or 'double', not {precision!r}")
    grid = yee_grid(size, dl, pml.layers, courant, center)
    eps_ez = permittivity_at_ez(grid, background_eps, boxes)
    cpml_x = cpml_axis(grid.nx, grid.dx, grid.dt, pml, background_eps)
    cpml_y = cpml_axis(grid.ny, grid.dy, grid.dt, pml, background_eps)
    injections = [tm_injection(s, grid, eps_ez) for s in sources]
    samplings, components = [], []
    for m in monitors:
        comps = tuple(m.components or TM_COMPONENTS)
        bad = [c for c in comps if c not in TM_COMPONENTS]
        if bad:
            raise NotImplementedError(f"monitor {m.name!r} asks for {bad}; TM runs record Ez, Hx, Hy")
        dual = DFTMonitor(m.name, m.wavelengths, m.center, m.size, tuple(DUAL[c] for c in comps))
        samplings.extend(monitor_samplings(dual, grid))
        components.extend(comps)
    if run_time is not None:
        n_steps = grid.n_steps(run_time)
    ones = {c: np.ones(grid.shape(c)) for c in ("Ex", "Ey")}  # TE eps: unused, cb is set below
    te = TEProblem(grid, ones, cpml_x, cpml_y, injections, samplings, precision, n_steps, background_eps,
                   [DFTMonitor(m.name, m.wavelengths, m.center, m.size, m.components) for m in monitors])  # fmt: skip
    return TMProblem(te, eps_ez, components, list(monitors))


def tm_cast_coefficients(problem: TMProblem) -> tuple[CastCoefficients, NDArray]:
    """The dual run's coefficients, cast once: cb = dt/mu0 everywhere, the CPML profiles of TE,
    and the per-Ez-node dt/(eps0 eps_r) that replaces db."""
    g, dtype = problem.grid, problem.real

    def put(a):
        return np.ascontiguousarray(a, dtype=dtype)

    ch = g.dt / MU_0
    cx, cy = problem.te.cpml_x, problem.te.cpml_y
    c = CastCoefficients(
        cb_ex=put(np.full(g.shape("Ex"), ch)), cb_ey=put(np.full(g.shape("Ey"), ch)),
        bx_e=put(cx.b_e), cx_e=put(cx.c_e), ikx_e=put(cx.inv_kappa_e),
        bx_h=put(cx.b_h), cx_h=put(cx.c_h), ikx_h=put(cx.inv_kappa_h),
        by_e=put(cy.b_e), cy_e=put(cy.c_e), iky_e=put(cy.inv_kappa_e),
        by_h=put(cy.b_h), cy_h=put(cy.c_h), iky_h=put(cy.inv_kappa_h),
        db=dtype(g.dt / EPSILON_0),  # not read: the per-node coefficients replace it
        inv_dx=dtype(1.0 / (g.dx * UM)),
        inv_dy=dtype(1.0 / (g.dy * UM)),
    )  # fmt: skip
    return c, put(g.dt / (EPSILON_0 * problem.eps_ez))


def _flip(a: np.ndarray) -> np.ndarray:
    """-a for a held negated: 0 - a is -a exactly, and +0 where a is zero of either sign."""
    return np.zeros_like(a) - a


class TMEngine:
    """A resident TM run: the dual TE run on the one-step kernels."""

    def __init__(self, problem: TMProblem, **engine_options) -> None:
        from .engine import TEEngine

        self.problem = problem
        self.te = TEEngine(problem.te, **engine_options)
        try:
            c, ce = tm_cast_coefficients(problem)
            self.te.set_coefficients(c)
            self._ce = ce
            call("etg_sim_set_db_nodes", self.te._h, ce.ctypes.data)
        except Exception:
            self.te.close()
            raise

    @property
    def n(self) -> int:
        return self.te.n

    def advance(self, k: int) -> None:
        self.te.advance(k)

    def synchronize(self) -> None:
        self.te.synchronize()

    def reset(self) -> None:
        self.te.reset()

    def field(self, name: str) -> np.ndarray:
        """"ez", "hx" or "hy" (and the CPML "psi_ez_x", "psi_ez_y", "psi_hx_y", "psi_hy_x")."""
        te = {"ez": ("hz", False), "hx": ("ex", True), "hy": ("ey", True), "psi_ez_x": ("psi_hz_x", True),
              "psi_ez_y": ("psi_hz_y", True), "psi_hx_y": ("psi_ex_y", False), "psi_hy_x": ("psi_ey_x", False)}
        if name not in te:
            raise KeyError(f"no TM field {name!r}")
        src, flip = te[name]
        a = self.te.field(src)
        return _flip(a) if flip else a

    def dft(self, k: int) -> np.ndarray:
        """Accumulator (n_f, nodes) of sampling k, in the TM component's sign."""
        a = self.te.dft(k)
        return _flip(a) if NEGATED[self.problem.components[k]] else a

    def result(self) -> dict[str, dict[str, np.ndarray]]:
        """Monitor values as ``GB300Solver.result`` gives them, keyed by TM component."""
        out: dict[str, dict[str, np.ndarray]] = {m.name: {} for m in self.problem.monitors}
        for k, (s, comp) in enumerate(zip(self.problem.te.samplings, self.problem.components)):
            out[s.monitor][comp] = interpolate_monitor(s, self.dft(k))
        return out

    def close(self) -> None:
        self.te.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def samplings(problem: TMProblem) -> list[tuple[str, ComponentSampling]]:
    """(TM component, node sampling) of every monitor component, in order."""
    return list(zip(problem.components, problem.te.samplings))
