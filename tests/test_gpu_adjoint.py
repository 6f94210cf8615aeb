"""GPU discrete adjoint vs the float64 torch gradient oracle and finite differences (needs a GPU).

J = Σ_f |F(f)|², F the bilinearly interpolated DFT of Hz at an output point; the parameters
are cb_ex/cb_ey on a design window and, through DesignRegion, the design cells' ε.
Tolerances: float64 adjoint within 1e-8 of the oracle (same derivative, other rounding);
float32 adjoint within 1e-3 of the float64 oracle, relative to the largest component.
"""

import numpy as np
import pytest
import torch

from etalon_gb300 import physics as ph
from etalon_gb300.adjoint import AdjointRunner, DesignRegion, point_power, simulate
from oracle.adjoint_torch import TorchTE

pytestmark = pytest.mark.gpu


def _problem(precision, n_steps=360):
    return ph.te_problem(
        size=(3.0, 2.4), dl=0.05, background_eps=2.085,
        boxes=[ph.Box((0.0, 0.0, 0.0), (4.0, 0.5, 1.0), 12.11)],
        pml=ph.PMLSpec(layers=8),
        sources=[ph.PointSource((-1.0, 0.0, 0.0), "Hz", ph.GaussianPulse(1.55, 0.5))],
        monitors=[ph.DFTMonitor("out", [1.50, 1.55, 1.60], center=(1.03, 0.02, 0.0), components=("Hz",))],
        n_steps=n_steps, precision=precision,
    )  # fmt: skip


def _design(p):
    return DesignRegion.from_box(p, (0.0, 0.0), (0.6, 0.6))


def _oracle_grad(p, design):
    """dJ/dcb on the window from the float64 torch transcription of Etalon's update."""
    c = ph.cast_coefficients(ph.TEProblem(p.grid, p.eps, p.cpml_x, p.cpml_y, [], [], "double"))
    n = p.n_steps
    sources = [(i.component, i.i, i.j, i.delta_table(0, n, p.grid.dt, np.float64)) for i in p.injections]
    monitors = [(s.component, s.flat_index, ph.phasor_table(s, 0, n, p.grid.dt, np.complex128)) for s in p.samplings]
    te = TorchTE(p.grid.nx, p.grid.ny, vars(c), sources, monitors, n)
    cbx = torch.as_tensor(c.cb_ex).clone().requires_grad_(True)
    cby = torch.as_tensor(c.cb_ey).clone().requires_grad_(True)
    _, accs = te.run(cbx, cby)
    j = point_power(accs[0], p.samplings[0])
    j.backward()
    sx, sy = design.node_windows()
    return float(j.detach()), cbx.grad.numpy()[sx], cby.grad.numpy()[sy]


def _gpu_grad(p, design, **kw):
    r = AdjointRunner(p, design, **kw)
    r.set_eps(p.eps["Ex"][design.node_windows()[0]], p.eps["Ey"][design.node_windows()[1]])
    accs = r.forward()
    acc = torch.as_tensor(np.stack([accs[0].real, accs[0].imag], -1).astype(np.float64)).requires_grad_(True)
    j = point_power(acc, p.samplings[0])
    j.backward()
    g = acc.grad[..., 0].numpy() + 1j * acc.grad[..., 1].numpy()
    gx, gy = r.backward([g])
    r.close()
    return float(j.detach()), gx, gy


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.fixture(scope="module")
def oracle64():
    p = _problem("double")
    return p, _oracle_grad(p, _design(p))


def test_adjoint_float64_equals_oracle(gpu, oracle64):
    p, (j_ref, gx_ref, gy_ref) = oracle64
    j, gx, gy = _gpu_grad(p, _design(p), kernel="plain")
    assert j == pytest.approx(j_ref, rel=1e-12)
    assert np.abs(gx_ref).max() > 0
    assert _rel(gx, gx_ref) < 1e-8 and _rel(gy, gy_ref) < 1e-8


def test_adjoint_float32_within_1e3_of_float64_oracle(gpu, oracle64):
    _, (j_ref, gx_ref, gy_ref) = oracle64
    p = _problem("single")
    j, gx, gy = _gpu_grad(p, _design(p))
    assert j == pytest.approx(j_ref, rel=1e-4)
    assert _rel(gx, gx_ref) < 1e-3 and _rel(gy, gy_ref) < 1e-3


@pytest.mark.parametrize("precision", ["single", "double"])
def test_checkpointing_and_trace_give_the_same_bits(gpu, precision):
    p = _problem(precision)
    d = _design(p)
    a = _gpu_grad(p, d, stride=0)
    b = _gpu_grad(p, d, stride=AdjointRunner.sqrt_stride(p.n_steps))
    c = _gpu_grad(p, d, stride=7, kernel="plain")
    for x, y in zip(a[1:], b[1:]):
        np.testing.assert_array_equal(x, y)
    for x, y in zip(a[1:], c[1:]):
        np.testing.assert_array_equal(x, y)


def test_eps_gradient_matches_central_differences(gpu):
    """dJ/dε of design cells through simulate() vs central differences of the float64 forward."""
    p = _problem("double")
    d = _design(p)
    r = AdjointRunner(p, d)
    rng = np.random.default_rng(3)
    eps0 = torch.as_tensor(rng.uniform(2.085, 12.11, (d.nx, d.ny)))
    eps = eps0.clone().requires_grad_(True)
    j = point_power(simulate(eps, r)[0], p.samplings[0])
    j.backward()
    grad = eps.grad.numpy()
    for _ in range(5):
        a, b = int(rng.integers(0, d.nx)), int(rng.integers(0, d.ny))
        h = 1e-3 * float(eps0[a, b])
        vals = []
        for sign in (1, -1):
            e = eps0.clone()
            e[a, b] += sign * h
            with torch.no_grad():
                vals.append(float(point_power(simulate(e, r)[0], p.samplings[0])))
        fd = (vals[0] - vals[1]) / (2 * h)
        assert grad[a, b] == pytest.approx(fd, rel=1e-3, abs=1e-6 * np.abs(grad).max())
    r.close()
