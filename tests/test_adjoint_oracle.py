"""The float64 gradient oracle is pinned: its forward pass is the reference's, bit for bit."""

import numpy as np
import pytest
import torch

from etalon_gb300 import physics as ph
from oracle.adjoint_torch import TorchTE
from tests import cases


def torch_oracle_for(p, n_steps):
    c = ph.cast_coefficients(p)
    coeffs = vars(c)
    sources = [(i.component, i.i, i.j, i.delta_table(0, n_steps, p.grid.dt, np.float64)) for i in p.injections]
    monitors = [(s.component, s.flat_index, ph.phasor_table(s, 0, n_steps, p.grid.dt, np.complex128))
                for s in p.samplings]  # fmt: skip
    te = TorchTE(p.grid.nx, p.grid.ny, coeffs, sources, monitors, n_steps)
    return te, torch.as_tensor(c.cb_ex), torch.as_tensor(c.cb_ey)


def test_torch_forward_equals_reference_float64():
    from tests.golden_io import FIELDS, compare_outputs, load

    g = load("small", "double")
    p = cases.small("double")
    n = int(g["n_steps"])
    te, cbx, cby = torch_oracle_for(p, n)
    with torch.no_grad():
        fields, accs = te.run(cbx, cby)
    out = dict(zip(FIELDS, (f.numpy() for f in fields)))
    acc = [a[..., 0].numpy() + 1j * a[..., 1].numpy() for a in accs]
    assert compare_outputs(g, out, acc) == []


def test_torch_gradient_matches_central_differences():
    """d|A|²/d cb at a few interior nodes vs central differences of the same float64 code."""
    p = cases.small("double", n_steps=60)
    te, cbx, cby = torch_oracle_for(p, 60)
    cbx = cbx.clone().requires_grad_(True)
    _, accs = te.run(cbx, cby)
    j = (accs[2] ** 2).sum()  # |DFT Hz|² of the probe, all frequencies
    j.backward()
    rng = np.random.default_rng(0)
    for _ in range(3):
        i, k = int(rng.integers(10, 30)), int(rng.integers(10, 20))
        h = 1e-3 * float(cbx.detach()[i, k])
        vals = []
        for sign in (1, -1):
            x = cbx.detach().clone()
            x[i, k] += sign * h
            with torch.no_grad():
                vals.append(float((te.run(x, cby)[1][2] ** 2).sum()))
        fd = (vals[0] - vals[1]) / (2 * h)
        assert float(cbx.grad[i, k]) == pytest.approx(fd, rel=1e-5, abs=1e-12 * abs(float(j.detach())) / abs(h))


@pytest.mark.parametrize("n_steps", [1, 15, 16, 255, 256, 2000, 20000, 10**6])
def test_checkpoint_stride_is_root_n_rounded_up_to_whole_launch_pairs(n_steps):
    """√N checkpoint segments are whole launch pairs of the 8- and 4-step tiles: multiples of 16,
    never shorter than √N rounded (144 at the 20 000-step single-design workload)."""
    from etalon_gb300.adjoint import AdjointRunner

    s = AdjointRunner.sqrt_stride(n_steps)
    assert s % 16 == 0 and s >= round(np.sqrt(n_steps)) and s - round(np.sqrt(n_steps)) < 16
    if n_steps == 20000:
        assert s == 144
