"""Float64 gradient oracle: Etalon's TE update transcribed to PyTorch, differentiated by autograd.

TEST INFRASTRUCTURE ONLY. Etalon has no adjoint, so the gradients of the GPU adjoint
are checked against this: a plain torch restatement of
etalon/fdtd/backends/numpy_backend.py:41-67 stepped in the order of
etalon/fdtd/solver.py:83-128, in float64, with the cb coefficients of a window of
nodes as leaf tensors. Its forward pass equals the NumPy oracle (oracle/te_numpy.py)
bit for bit in float64 (tests/test_adjoint_oracle.py), so its gradient is the exact
derivative of the reference computation. Memory is bounded by recomputing segments of
steps in the backward pass (torch.utils.checkpoint).
"""

from __future__ import annotations

import numpy as np
import torch
from torch.utils.checkpoint import checkpoint


class TorchTE:
    """One float64 TE run; sources and monitor phasors are precomputed host tables."""

    def __init__(self, nx, ny, coeffs: dict, sources, monitors, n_steps: int):
        self.nx, self.ny, self.n_steps = nx, ny, n_steps
        t = lambda a: torch.as_tensor(np.asarray(a, dtype=np.float64))  # noqa: E731
        self.c = {k: t(v) for k, v in coeffs.items() if k not in ("cb_ex", "cb_ey")}
        # sources: (component, i, j, table (n_steps, n_nodes) float64 values subtracted)
        self.sources = [(comp, torch.as_tensor(i), torch.as_tensor(j), t(table)) for comp, i, j, table in sources]
        # monitors: (component, flat_index, phasor table (n_steps, n_f) complex128)
        self.monitors = [(comp, torch.as_tensor(flat), torch.as_tensor(np.asarray(ph, np.complex128)))
                         for comp, flat, ph in monitors]  # fmt: skip

    def _step(self, n, cb_ex, cb_ey, ex, ey, hz, pexy, peyx, phzx, phzy, *accs):
        c = self.c
        dex_dy = (ex[:, 1:] - ex[:, :-1]) * c["inv_dy"]
        dey_dx = (ey[1:, :] - ey[:-1, :]) * c["inv_dx"]
        phzy = c["by_h"][None, :] * phzy + c["cy_h"][None, :] * dex_dy
        phzx = c["bx_h"][:, None] * phzx + c["cx_h"][:, None] * dey_dx
        hz = hz + c["db"] * ((dex_dy * c["iky_h"][None, :] + phzy) - (dey_dx * c["ikx_h"][:, None] + phzx))
        hz = self._inject(hz, "Hz", n)
        accs = list(accs)
        self._accumulate(accs, {"Hz": hz}, n, magnetic=True)
        dhz_dy = (hz[:, 1:] - hz[:, :-1]) * c["inv_dy"]
        p = c["by_e"][None, 1:-1] * pexy[:, 1:-1] + c["cy_e"][None, 1:-1] * dhz_dy
        pexy = torch.cat([pexy[:, :1], p, pexy[:, -1:]], dim=1)
        ex_in = ex[:, 1:-1] + cb_ex[:, 1:-1] * (dhz_dy * c["iky_e"][None, 1:-1] + p)
        ex = torch.cat([ex[:, :1], ex_in, ex[:, -1:]], dim=1)
        dhz_dx = (hz[1:, :] - hz[:-1, :]) * c["inv_dx"]
        p = c["bx_e"][1:-1, None] * peyx[1:-1, :] + c["cx_e"][1:-1, None] * dhz_dx
        peyx = torch.cat([peyx[:1], p, peyx[-1:]], dim=0)
        ey_in = ey[1:-1, :] - cb_ey[1:-1, :] * (dhz_dx * c["ikx_e"][1:-1, None] + p)
        ey = torch.cat([ey[:1], ey_in, ey[-1:]], dim=0)
        ex = self._inject(ex, "Ex", n)
        ey = self._inject(ey, "Ey", n)
        self._accumulate(accs, {"Ex": ex, "Ey": ey}, n, magnetic=False)
        return (ex, ey, hz, pexy, peyx, phzx, phzy, *accs)

    def _inject(self, field, comp, n):
        for c, i, j, table in self.sources:
            if c == comp:
                field = field.index_put((i, j), field[i, j] - table[n])
        return field

    def _accumulate(self, accs, fields, n, magnetic):
        for k, (comp, flat, ph) in enumerate(self.monitors):
            if comp.startswith("H") == magnetic and comp in fields:
                v = fields[comp].reshape(-1)[flat]
                accs[k] = accs[k] + torch.stack([v[None, :] * ph[n].real[:, None], v[None, :] * ph[n].imag[:, None]], -1)

    def run(self, cb_ex, cb_ey, segment: int = 50):
        """DFT accumulators (n_f, nodes, 2) per monitor after n_steps, differentiable in cb."""
        nx, ny = self.nx, self.ny
        z = lambda *s: torch.zeros(s, dtype=torch.float64)  # noqa: E731
        state = (z(nx, ny + 1), z(nx + 1, ny), z(nx, ny), z(nx, ny + 1), z(nx + 1, ny), z(nx, ny), z(nx, ny))
        accs = tuple(z(ph.shape[1], flat.numel(), 2) for _, flat, ph in self.monitors)
        state = state + accs

        def segment_fn(n0, n1):
            def f(cbx, cby, *st):
                for n in range(n0, n1):
                    st = self._step(n, cbx, cby, *st)
                return st
            return f

        for n0 in range(0, self.n_steps, segment):
            n1 = min(n0 + segment, self.n_steps)
            state = checkpoint(segment_fn(n0, n1), cb_ex, cb_ey, *state, use_reentrant=False)
        return state[:7], state[7:]
