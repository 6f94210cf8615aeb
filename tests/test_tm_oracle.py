"""The 2D TM oracle against the TE oracle through the TE/TM duality (no GPU).

oracle/tm_numpy.py writes the TM update directly. Run on the dual problem (Ez in Hz, -Hx in
Ex, -Hy in Ey, dt/mu0 as cb, dt/(eps0 eps_r) per Ez node as db), the TE oracle — Etalon's
update restated (oracle/te_numpy.py, pinned to Etalon's fixtures) — must give the TM fields,
psi and accumulators bit for bit: uniform media and a dielectric box, float32 and float64.
"""

import numpy as np
import pytest

from etalon_gb300 import physics as ph
from etalon_gb300 import tm
from oracle.te_numpy import OracleMonitor, OracleSource, OracleTE
from oracle.tm_numpy import OracleTM, TMMonitor, TMSource


def tm_case(precision, boxes=(), background_eps=1.0, n_steps=160):
    return tm.tm_problem(
        size=(2.4, 1.8), dl=0.05, background_eps=background_eps, boxes=boxes, pml=ph.PMLSpec(layers=8),
        sources=[tm.TMPointSource((-0.63, 0.071, 0.0), ph.GaussianPulse(1.55, 0.4))],
        monitors=[ph.DFTMonitor("point", [1.5, 1.6], center=(0.52, -0.13, 0.0)),
                  ph.DFTMonitor("plane", [1.55], size=(1.0, 0.6, 0.0), components=("Ez", "Hy"))],
        n_steps=n_steps, precision=precision,
    )  # fmt: skip


def oracle_tm(p):
    c, ce = tm.tm_cast_coefficients(p)
    coeffs = {k: getattr(c, k) for k in ("bx_e", "cx_e", "ikx_e", "bx_h", "cx_h", "ikx_h",
                                          "by_e", "cy_e", "iky_e", "by_h", "cy_h", "iky_h")}  # fmt: skip
    coeffs.update(ce=ce, ch=c.cb_ex.flat[0], inv_dx=c.inv_dx, inv_dy=c.inv_dy)
    g = p.grid
    srcs = [TMSource(inj.i, inj.j, inj.coefficient, (inj.pulse.wavelength, inj.pulse.bandwidth, inj.pulse.amplitude))
            for inj in p.te.injections]  # fmt: skip
    mons = [TMMonitor(comp, s.flat_index, s.frequencies) for comp, s in tm.samplings(p)]
    return OracleTM(g.nx, g.ny, g.dt, coeffs, p.real, srcs, mons)


def oracle_te_dual(p):
    c, ce = tm.tm_cast_coefficients(p)
    coeffs = dict(vars(c))
    coeffs["db"] = ce  # a per-node coefficient broadcasts through Etalon's own expression
    g = p.grid
    srcs = [OracleSource("Hz", inj.i, inj.j, inj.coefficient,
                         (inj.pulse.wavelength, inj.pulse.bandwidth, inj.pulse.amplitude))
            for inj in p.te.injections]  # fmt: skip
    mons = [OracleMonitor(s.component, s.flat_index, s.frequencies) for s in p.te.samplings]
    return OracleTE(g.nx, g.ny, g.dt, coeffs, p.real, srcs, mons)


def raw(a):
    return np.ascontiguousarray(a).view(np.uint8)


@pytest.mark.parametrize("precision", ["single", "double"])
@pytest.mark.parametrize("medium", ["uniform", "box"])
def test_tm_oracle_is_the_dual_te_oracle(precision, medium):
    boxes = [ph.Box((0.1, -0.05, 0.0), (0.7, 0.35, 0.22), 11.7)] if medium == "box" else []
    p = tm_case(precision, boxes=boxes, background_eps=2.085)
    a, b = oracle_tm(p), oracle_te_dual(p)
    a.run(p.n_steps)
    b.run(p.n_steps)
    flip = lambda x: np.zeros_like(x) - x  # noqa: E731
    pairs = {"ez": b.hz, "hx": flip(b.ex), "hy": flip(b.ey), "psi_ez_x": flip(b.psi_hz_x),
             "psi_ez_y": flip(b.psi_hz_y), "psi_hx_y": b.psi_ex_y, "psi_hy_x": b.psi_ey_x}  # fmt: skip
    for name, want in pairs.items():
        assert np.array_equal(raw(getattr(a, name)), raw(want)), name
    for k, comp in enumerate(p.components):
        want = flip(b.acc[k]) if tm.NEGATED[comp] else b.acc[k]
        assert np.array_equal(raw(a.acc[k]), raw(want)), f"accumulator {k} ({comp})"
    assert np.abs(a.ez).max() > 0 and np.abs(a.hy).max() > 0
    assert all(np.abs(x).max() > 0 for x in a.acc)


def test_tm_problem_layout_and_refusals():
    p = tm_case("single", boxes=[ph.Box((0.0, 0.0, 0.0), (0.4, 0.4, 0.22), 12.11)], background_eps=2.085)
    g = p.grid
    assert p.eps_ez.shape == (g.nx, g.ny)
    assert p.eps_ez.max() == 12.11 and p.eps_ez.min() == 2.085
    assert p.components == ["Ez", "Hx", "Hy", "Ez", "Hy"]
    assert [s.component for s in p.te.samplings] == ["Hz", "Ex", "Ey", "Hz", "Ey"]
    assert all(inj.component == "Hz" for inj in p.te.injections)
    inj = p.te.injections[0]
    np.testing.assert_allclose(inj.coefficient.sum() * g.dx * g.dy * 1e-12,
                               np.sum(inj.weights * g.dt / (ph.EPSILON_0 * p.eps_ez[inj.i, inj.j])), rtol=1e-12)
    with pytest.raises(NotImplementedError, match="drive Ez"):
        tm.tm_injection(tm.TMPointSource((0, 0, 0), ph.GaussianPulse(1.55, 0.5), "Hx"), g, p.eps_ez)
    with pytest.raises(NotImplementedError, match="TM runs record"):
        tm.tm_problem((1.0, 1.0), 0.05, [], [ph.DFTMonitor("m", [1.55], components=("Hz",))])
