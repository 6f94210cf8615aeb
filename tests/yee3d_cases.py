"""3D test cases and their oracles (no GPU needed to build them).

``case3d``: a small CPML-bounded run with a dielectric block, an E and an H point source, a
point monitor on all six components and a plane monitor. ``oracle_3d`` turns a
``Yee3DProblem`` into oracle/yee3d_numpy.py's ``Oracle3D``. ``te_case`` / ``reduced_oracle``:
a 2D TE run and the 3D oracle of the same run laid along one of the three planes (one
periodic cell along the third axis), with the maps between their arrays.
"""

from __future__ import annotations

import numpy as np

from etalon_gb300 import physics as ph
from etalon_gb300 import yee3d
from oracle.te_numpy import OracleMonitor, OracleSource, OracleTE
from oracle.yee3d_numpy import AXES, Oracle3D, Reduction, from_2d, shape_of

PULSE = ph.GaussianPulse(1.55, 0.5)


def case3d(precision="single", n_steps=60, *, periodic=(False, False, False), layers=6, size=(1.2, 1.0, 0.8),
           dl=0.05, boxes=None, background_eps=2.085):  # fmt: skip
    if boxes is None:
        boxes = [ph.Box((0.05, 0.0, 0.0), (0.5, 0.2, 0.22), 12.11)]
    c = [0.0 if periodic[a] else v for a, v in enumerate((0.11, -0.07, 0.031))]
    h = [0.0 if periodic[a] else v for a, v in enumerate((-0.2, 0.15, -0.1))]
    m = [0.0 if periodic[a] else v for a, v in enumerate((0.3, 0.2, 0.1))]
    return yee3d.yee3d_problem(
        size, dl,
        sources=[ph.PointSource(tuple(c), "Ez", PULSE), ph.PointSource(tuple(h), "Hy", PULSE)],
        monitors=[ph.DFTMonitor("p", [1.5, 1.6], center=tuple(m)),
                  ph.DFTMonitor("plane", [1.55], center=(0.0, 0.0, 0.0),
                                size=tuple(0.0 if periodic[a] else s for a, s in enumerate((0.6, 0.4, 0.0))),
                                components=("Ex", "Hz"))],
        background_eps=background_eps, boxes=boxes, layers=layers, periodic=periodic, n_steps=n_steps,
        precision=precision,
    )  # fmt: skip


def _pulse(p: ph.GaussianPulse) -> tuple[float, float, float]:
    return p.wavelength, p.bandwidth, p.amplitude


def oracle_3d(p: yee3d.Yee3DProblem) -> Oracle3D:
    c = yee3d.cast_coefficients_3d(p)
    srcs = [OracleSource(inj.component, inj.flat, None, inj.coefficient, _pulse(inj.pulse)) for inj in p.injections]
    mons = [OracleMonitor(s.component, s.flat_index, s.frequencies) for s in p.samplings]
    return Oracle3D(p.grid.n, p.grid.periodic, p.grid.dt, c, p.real, srcs, mons)


# ----------------------------------------------------------------------------- 2D reductions


def te_case(precision="single", n_steps=80):
    """A 2D TE run with CPML, a dielectric box, an Hz and an Ex source and two monitors."""
    return ph.te_problem(
        size=(2.0, 1.5), dl=0.05, background_eps=2.085, boxes=[ph.Box((0.1, -0.05, 0.0), (0.7, 0.35, 0.22), 11.7)],
        pml=ph.PMLSpec(layers=8),
        sources=[ph.PointSource((-0.63, 0.071, 0.0), "Hz", PULSE), ph.PointSource((0.41, -0.23, 0.0), "Ex", PULSE)],
        monitors=[ph.DFTMonitor("point", [1.5, 1.6], center=(0.52, -0.13, 0.0)),
                  ph.DFTMonitor("plane", [1.55], size=(0.8, 0.5, 0.0), components=("Hz", "Ey"))],
        n_steps=n_steps, precision=precision,
    )  # fmt: skip


def oracle_te(p) -> OracleTE:
    c = vars(ph.cast_coefficients(p))
    srcs = [OracleSource(inj.component, inj.i, inj.j, inj.coefficient, _pulse(inj.pulse)) for inj in p.injections]
    mons = [OracleMonitor(s.component, s.flat_index, s.frequencies) for s in p.samplings]
    return OracleTE(p.grid.nx, p.grid.ny, p.grid.dt, c, p.real, srcs, mons)


def roles(red: Reduction) -> dict[str, str]:
    """2D TE array name -> the 3D array playing it."""
    ax, ay = AXES[red.axes[0]], AXES[red.axes[1]]
    (e0, e1), h = red.e2d, red.h2d
    return {"ex": e0, "ey": e1, "hz": h, "psi_hz_y": f"psi_{h}_{ay}", "psi_hz_x": f"psi_{h}_{ax}",
            "psi_ex_y": f"psi_{e0}_{ay}", "psi_ey_x": f"psi_{e1}_{ax}"}  # fmt: skip


def reduced_shape(p, red: Reduction) -> tuple[int, int, int]:
    n = [1, 1, 1]
    n[red.axes[0]], n[red.axes[1]] = p.grid.nx, p.grid.ny
    return tuple(n)  # type: ignore[return-value]


def flat_map(red: Reduction, shape2d) -> np.ndarray:
    """2D flat index -> 3D flat index of the role's array."""
    ids = from_2d(red, np.arange(int(np.prod(shape2d))).reshape(shape2d))
    out = np.empty(ids.size, np.int64)
    out[ids.ravel()] = np.arange(ids.size)
    return out


def reduced_oracle(p, red: Reduction, inv_d_third: float = 1.0 / (0.05e-6)) -> Oracle3D:
    """The 3D oracle of the 2D run ``p`` laid along ``red``'s plane."""
    c = ph.cast_coefficients(p)
    dtype = p.real
    n3 = reduced_shape(p, red)
    periodic = tuple(a == red.invariant for a in range(3))
    coeffs: dict = {"db": c.db}
    roles_e = {red.e2d[0]: c.cb_ex, red.e2d[1]: c.cb_ey}
    for comp in ("ex", "ey", "ez"):
        if comp in roles_e:
            coeffs["cb_" + comp] = from_2d(red, roles_e[comp])
        else:  # the component stays zero; any coefficient
            coeffs["cb_" + comp] = np.full(shape_of(comp, n3, periodic), c.cb_ex.flat[0], dtype)
    for a, (name2d, inv) in zip(red.axes, (("x", c.inv_dx), ("y", c.inv_dy))):
        coeffs[f"inv_d{AXES[a]}"] = inv
        for k in ("b", "c", "ik"):
            for w in ("e", "h"):
                coeffs[f"{k}{AXES[a]}_{w}"] = getattr(c, f"{k}{name2d}_{w}")
    t = AXES[red.invariant]
    coeffs[f"inv_d{t}"] = dtype(inv_d_third)
    for k, v in (("b", 1.0), ("c", 0.0), ("ik", 1.0)):
        for w in ("e", "h"):
            coeffs[f"{k}{t}_{w}"] = np.full(1, v, dtype)
    r = roles(red)
    srcs = []
    for inj in p.injections:
        name = inj.component.lower()
        shape2d = p.grid.shape(inj.component)
        flat2d = np.ravel_multi_index((inj.i, inj.j), shape2d)
        srcs.append(OracleSource(r[name].capitalize(), flat_map(red, shape2d)[flat2d], None, inj.coefficient,
                                 _pulse(inj.pulse)))  # fmt: skip
    mons = []
    for s in p.samplings:
        name = s.component.lower()
        mons.append(OracleMonitor(r[name].capitalize(), flat_map(red, p.grid.shape(s.component))[s.flat_index],
                                  s.frequencies))  # fmt: skip
    return Oracle3D(n3, periodic, p.grid.dt, coeffs, dtype, srcs, mons)
