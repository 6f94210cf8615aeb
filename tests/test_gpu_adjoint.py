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


def _large_problem(precision, n_steps=400):
    """216×166 cells (a strip through a 1.2×1.0 µm design window): interior and CPML tiles."""
    return ph.te_problem(
        size=(8.0, 6.0), dl=0.04, background_eps=2.085,
        boxes=[ph.Box((0.0, 0.0, 0.0), (9.0, 0.5, 1.0), 12.11)],
        pml=ph.PMLSpec(layers=10),
        sources=[ph.PointSource((-3.0, 0.0, 0.0), "Hz", ph.GaussianPulse(1.55, 0.5))],
        monitors=[ph.DFTMonitor("out", [1.50, 1.55, 1.60], center=(3.03, 0.02, 0.0), components=("Hz",)),
                  ph.DFTMonitor("e", [1.55], center=(2.51, 0.33, 0.0), components=("Ex", "Ey"))],
        n_steps=n_steps, precision=precision,
    )  # fmt: skip


def _gpu_grad_all(p, design, **kw):
    """J = Σ over every monitor component of Σ_f |F|² (H and E adjoint sources)."""
    r = AdjointRunner(p, design, **kw)
    sx, sy = design.node_windows()
    r.set_eps(p.eps["Ex"][sx], p.eps["Ey"][sy])
    accs = r.forward()
    grads = []
    for acc_np, sampling in zip(accs, p.samplings):
        acc = torch.as_tensor(np.stack([acc_np.real, acc_np.imag], -1).astype(np.float64)).requires_grad_(True)
        point_power(acc, sampling).backward()
        grads.append(acc.grad[..., 0].numpy() + 1j * acc.grad[..., 1].numpy())
    gx, gy = r.backward(grads)
    r.close()
    return gx, gy


@pytest.mark.parametrize("precision", ["single", "double"])
def test_blocked_adjoint_sweep_equals_one_step_sweep_bitwise(gpu, precision):
    """The temporally blocked reverse sweep gives the one-step kernels' bits, H and E sources."""
    p = _large_problem(precision)
    d = DesignRegion.from_box(p, (0.0, 0.0), (1.2, 1.0))
    for stride in (0, 37):
        a = _gpu_grad_all(p, d, stride=stride)
        b = _gpu_grad_all(p, d, stride=stride, kernel="plain")
        assert np.abs(a[0]).max() > 0 and np.abs(a[1]).max() > 0
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[1], b[1])


def test_blocked_adjoint_float32_within_1e3_of_float64(gpu):
    p64, p32 = _large_problem("double"), _large_problem("single")
    d = DesignRegion.from_box(p64, (0.0, 0.0), (1.2, 1.0))
    ref = _gpu_grad_all(p64, d, kernel="plain")
    got = _gpu_grad_all(p32, d)
    assert _rel(got[0], ref[0]) < 1e-3 and _rel(got[1], ref[1]) < 1e-3


def _variant(seed, precision, n_steps=900):
    """A small seeded design variant: uneven region, design window of uneven size; the pulse
    reaches the output monitor well within the run."""
    from tests import cases

    rng = np.random.default_rng(seed)
    region, design = int(rng.integers(70, 130)), int(rng.integers(12, 30))
    p, win = cases.adjoint_device(precision, n_steps=n_steps, region=region, design=design, n_wavelengths=4)
    d = DesignRegion.from_box(p, win[:2], win[2:])
    return p, d, torch.as_tensor(cases.smooth_design(d.nx, d.ny, seed))


@pytest.mark.parametrize("precision", ["single", "double"])
@pytest.mark.parametrize("stride", [0, 23])
def test_batched_gradients_equal_single_design_gradients(gpu, precision, stride):
    from etalon_gb300.adjoint import AdjointBatch, simulate_batch

    variants = [_variant(s, precision) for s in range(4)]
    singles = []
    for p, d, eps0 in variants:
        r = AdjointRunner(p, d, stride=stride)
        eps = eps0.clone().requires_grad_(True)
        point_power(simulate(eps, r)[0], p.samplings[0]).backward()
        singles.append(eps.grad.numpy().copy())
        r.close()
    runners = [AdjointRunner(p, d, stride=stride) for p, d, _ in variants]
    batch = AdjointBatch(runners)
    eps = [e.clone().requires_grad_(True) for _, _, e in variants]
    outs = simulate_batch(eps, batch)
    sum(point_power(o[0], v[0].samplings[0]) for o, v in zip(outs, variants)).backward()
    for e, ref in zip(eps, singles):
        assert np.abs(ref).max() > 0
        np.testing.assert_array_equal(e.grad.numpy(), ref)
    batch.close()
    for r in runners:
        r.close()


def _workload_fd_check(n):
    """The 1224² single-design workload (100×100 cells of smoothed random ε, 3 λ) run for n
    steps: float64 dJ/dε of 20 random design cells against central differences (h = 1e-3
    relative), and the float32 blocked gradient against the float64 one. Returns the largest
    relative FD error, |g − fd| / |fd|, and the float32 error."""
    from tests import cases

    p64, win = cases.adjoint_device("double", n_steps=n)
    d = DesignRegion.from_box(p64, win[:2], win[2:])
    eps0 = torch.as_tensor(cases.smooth_design(d.nx, d.ny, 0))
    r = AdjointRunner(p64, d, stride=AdjointRunner.sqrt_stride(n))
    eps = eps0.clone().requires_grad_(True)
    point_power(simulate(eps, r)[0], p64.samplings[0]).backward()
    g64 = eps.grad.numpy().copy()
    assert np.abs(g64).max() > 0
    rng = np.random.default_rng(11)
    cells = rng.choice(d.nx * d.ny, 20, replace=False)
    scale = np.abs(g64).max()
    worst = 0.0
    for q in cells:
        a, b = divmod(int(q), d.ny)
        h = 1e-3 * float(eps0[a, b])
        vals = []
        for sign in (1, -1):
            e = eps0.clone()
            e[a, b] += sign * h
            with torch.no_grad():
                vals.append(float(point_power(simulate(e, r)[0], p64.samplings[0])))
        fd = (vals[0] - vals[1]) / (2 * h)
        assert g64[a, b] == pytest.approx(fd, rel=1e-3, abs=1e-4 * scale)
        if abs(fd) > 1e-2 * scale:
            worst = max(worst, abs(g64[a, b] - fd) / abs(fd))
    r.close()
    p32, _ = cases.adjoint_device("single", n_steps=n)
    r32 = AdjointRunner(p32, d, stride=AdjointRunner.sqrt_stride(n))
    eps = eps0.clone().requires_grad_(True)
    point_power(simulate(eps, r32)[0], p32.samplings[0]).backward()
    r32.close()
    err32 = _rel(eps.grad.numpy(), g64)
    assert err32 < 1e-3
    return worst, err32


def test_single_design_workload_gradient_vs_central_differences(gpu):
    """The single-design workload shortened to 3000 steps (see _workload_fd_check)."""
    _workload_fd_check(3000)


def test_single_design_workload_full_length_vs_central_differences(gpu):
    """The single-design workload at its full 20 000 steps: 40 float64 forward runs of the
    1224² grid for the differences (about a minute)."""
    worst, err32 = _workload_fd_check(20000)
    print(f"\n20 000 steps: max relative FD error {worst:.3e}, float32 vs float64 {err32:.3e}")
    assert worst <= 1e-3


@pytest.mark.parametrize("precision", ["single", "double"])
def test_segment_recompute_in_the_window_light_cone_keeps_the_bits(gpu, precision):
    """On a grid much larger than the window's light cone over one segment, the checkpointed
    gradient (segments recomputed only within the cone) equals the full-trace gradient bit for
    bit, for one design and inside a batch."""
    from etalon_gb300.adjoint import AdjointBatch, simulate_batch
    from tests import cases

    n = 1500
    p, win = cases.adjoint_device(precision, n_steps=n, region=500, design=40, n_wavelengths=2)
    d = DesignRegion.from_box(p, win[:2], win[2:])
    stride = AdjointRunner.sqrt_stride(n)
    assert d.nx + 2 * (stride + 18) < p.grid.nx // 2  # the cone is a small part of the grid
    eps0 = torch.as_tensor(cases.smooth_design(d.nx, d.ny, 3))
    grads = []
    for s in (0, stride):
        r = AdjointRunner(p, d, stride=s)
        eps = eps0.clone().requires_grad_(True)
        point_power(simulate(eps, r)[0], p.samplings[0]).backward()
        grads.append(eps.grad.numpy().copy())
        r.close()
    assert np.abs(grads[0]).max() > 0
    np.testing.assert_array_equal(grads[1], grads[0])
    runners = [AdjointRunner(p, d, stride=stride), AdjointRunner(p, d, stride=stride)]
    batch = AdjointBatch(runners)
    eps = [eps0.clone().requires_grad_(True), (eps0 + 0.5).requires_grad_(True)]
    outs = simulate_batch(eps, batch)
    point_power(outs[0][0], p.samplings[0]).backward()
    np.testing.assert_array_equal(eps[0].grad.numpy(), grads[0])
    batch.close()
    for r in runners:
        r.close()
