"""Gradients of DFT-monitor objectives with respect to per-cell permittivity (no counterpart in Etalon).

``DesignRegion`` is a rectangle of cells [i0, i0+nx) x [j0, j0+ny) (Hz-cell indices) whose
permittivity is a free parameter. The reference stores ε only at the Ex and Ey nodes
(etalon/grid/materials.py:12-35), each node sitting on the face between two cells, so a
node's ε is the mean of the two cells sharing its face; a cell outside the region counts
with the node's static ε. The map is affine, so torch differentiates it exactly.

``simulate(eps, design, runner)`` is a ``torch.autograd.Function``: ε of the design cells
(float64) → the DFT accumulators of every monitor, as float64 tensors (n_f, nodes, 2). Its
backward pass runs the GPU adjoint (etg_adj_*) and maps dJ/dcb to dJ/dε with
dcb/dε = −cb/ε (cb = Δt/(ε0 ε), etalon/fdtd/state.py:80-81). Any objective written in torch
on the accumulators — e.g. ``point_power`` — then has an exact gradient.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from ._lib import call
from .engine import TEEngine
from .physics import EPSILON_0, ComponentSampling, TEProblem


# Steps per launch of the temporally blocked forward passes (a precision missing here keeps the
# engine's default): 40 x 128 tiles of 8 steps, the autotuner's choice for float32 grids of
# 512² to 2024², also shorten the gradients (config-5 batch 2.04 s to 1.90 s, bit-identical).
FORWARD_DEPTH = {"single": 8}


@dataclass(frozen=True)
class DesignRegion:
    """Cells [i0, i0+nx) x [j0, j0+ny) of free permittivity."""

    i0: int
    nx: int
    j0: int
    ny: int

    @classmethod
    def from_box(cls, problem: TEProblem, center: tuple[float, float], size: tuple[float, float]) -> "DesignRegion":
        """The cells whose centres lie in center ± size/2 (µm)."""
        x, y = problem.grid.coords("Hz")
        xi = np.nonzero(np.abs(x - center[0]) <= size[0] / 2 + 1e-9)[0]
        yj = np.nonzero(np.abs(y - center[1]) <= size[1] / 2 + 1e-9)[0]
        return cls(int(xi[0]), int(xi.size), int(yj[0]), int(yj.size))

    def node_windows(self):
        """Slices of the Ex window (nx, ny+1) and Ey window (nx+1, ny) in the node arrays."""
        ex = (slice(self.i0, self.i0 + self.nx), slice(self.j0, self.j0 + self.ny + 1))
        ey = (slice(self.i0, self.i0 + self.nx + 1), slice(self.j0, self.j0 + self.ny))
        return ex, ey

    def node_eps(self, eps_cells: torch.Tensor, static: dict[str, np.ndarray]):
        """Affine map cell ε (nx, ny) → ε at the Ex and Ey nodes of the window (float64)."""
        sx, sy = self.node_windows()
        st_ex = torch.as_tensor(static["Ex"][sx], dtype=torch.float64)
        st_ey = torch.as_tensor(static["Ey"][sy], dtype=torch.float64)
        # Ex(i, j) lies between cells (i, j-1) and (i, j); outside cells count as the node's value
        left = torch.cat([st_ex[:, :1], eps_cells], dim=1)
        right = torch.cat([eps_cells, st_ex[:, -1:]], dim=1)
        eps_ex = 0.5 * (left + right)
        # Ey(i, j) lies between cells (i-1, j) and (i, j)
        up = torch.cat([st_ey[:1, :], eps_cells], dim=0)
        down = torch.cat([eps_cells, st_ey[-1:, :]], dim=0)
        eps_ey = 0.5 * (up + down)
        return eps_ex, eps_ey


class AdjointRunner:
    """A resident engine plus its adjoint context for one design region."""

    def __init__(self, problem: TEProblem, design: DesignRegion, *, stride: int = 0, depth: int | None = None,
                 **engine_options):  # fmt: skip
        """``depth``: steps per launch of the forward passes (None: 8 in float32, the temporally
        blocked shape the tuner takes at these sizes; the default 2 in float64)."""
        self.problem, self.design = problem, design
        self.engine = TEEngine(problem, **engine_options)
        if depth is None:
            depth = FORWARD_DEPTH.get(problem.precision, 0)
        if depth:
            self.engine.set_option(_lib.OPT_TB_DEPTH, depth)
        self.static = {c: np.array(problem.eps[c], dtype=np.float64) for c in ("Ex", "Ey")}
        self.stride = stride
        h = C.c_void_p()
        call("etg_adj_create", C.byref(h), self.engine._h, design.i0, design.nx, design.j0, design.ny)
        self._h = h
        self.dt = problem.grid.dt

    @staticmethod
    def sqrt_stride(n_steps: int) -> int:
        """√N rounded up to a multiple of 16: a segment is then whole launch pairs of the 8-step
        tiles (and of the 4-step ones), with no one-step remainder."""
        s = max(1, int(round(np.sqrt(n_steps))))
        return (s + 15) // 16 * 16

    def set_eps(self, eps_ex: np.ndarray, eps_ey: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        """Upload cb = Δt/(ε0 ε) of the window nodes (float64, then one cast); returns cb64."""
        cbx = self.dt / (EPSILON_0 * eps_ex)
        cby = self.dt / (EPSILON_0 * eps_ey)
        real = self.problem.real
        d = self.design
        for which, cb, (i0, j0) in ((0, cbx, (d.i0, d.j0)), (1, cby, (d.i0, d.j0))):
            host = np.ascontiguousarray(cb, dtype=real)
            call("etg_sim_set_cb_window", self.engine._h, which, i0, host.shape[0], j0, host.shape[1],
                 host.ctypes.data)  # fmt: skip
        return cbx, cby

    def forward(self) -> list[np.ndarray]:
        call("etg_adj_forward", self._h, self.problem.n_steps, self.stride)
        return [self.engine.dft(k) for k in range(len(self.engine.monitors))]

    def backward(self, grad_accs: list[np.ndarray | None]) -> tuple[np.ndarray, np.ndarray]:
        """dJ/dcb on the window's Ex and Ey nodes (float64) from dJ/dacc per monitor."""
        keep, ptrs = self._objective_pointers(grad_accs)
        gx, gy = self._gradient_buffers()
        call("etg_adj_backward", self._h, ptrs, gx.ctypes.data_as(C.POINTER(C.c_double)),
             gy.ctypes.data_as(C.POINTER(C.c_double)))  # fmt: skip
        return gx, gy

    def _objective_pointers(self, grad_accs):
        keep = [None if g is None else np.ascontiguousarray(g, dtype=self.problem.complex) for g in grad_accs]
        return keep, (C.c_void_p * len(keep))(*[None if g is None else g.ctypes.data for g in keep])

    def _gradient_buffers(self):
        d = self.design
        return np.zeros((d.nx, d.ny + 1)), np.zeros((d.nx + 1, d.ny))

    def set_objective(self, grad_accs: list[np.ndarray | None]) -> None:
        _, ptrs = self._objective_pointers(grad_accs)
        call("etg_adj_set_objective", self._h, ptrs)

    def gradient(self) -> tuple[np.ndarray, np.ndarray]:
        gx, gy = self._gradient_buffers()
        call("etg_adj_gradient", self._h, gx.ctypes.data_as(C.POINTER(C.c_double)),
             gy.ctypes.data_as(C.POINTER(C.c_double)))  # fmt: skip
        return gx, gy

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.lib().etg_adj_destroy(self._h)
            self._h = C.c_void_p()
        self.engine.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class AdjointBatch:
    """Forward and reverse passes of many designs at once (etg_adj_batch_*).

    The runners (one precision, one step count and stride, any grid sizes) step together as
    a batch in the forward pass and share each K-step launch of the reverse sweep; every
    gradient is bit-identical to the runner's own ``backward``.
    """

    def __init__(self, runners: list[AdjointRunner]) -> None:
        if len({(r.problem.n_steps, r.stride, r.problem.precision) for r in runners}) != 1:
            raise ValueError("the designs of a batch need one step count, one stride and one precision")
        self.runners = runners
        handles = (C.c_void_p * len(runners))(*[r._h.value for r in runners])
        h = C.c_void_p()
        call("etg_adj_batch_create", C.byref(h), len(runners), handles)
        self._h = h
        depth = FORWARD_DEPTH.get(runners[0].problem.precision, 0)
        if depth:  # the forward passes of the batch, as each runner's own
            call("etg_adj_batch_set_option", h, _lib.OPT_TB_DEPTH, depth)
            call("etg_adj_batch_set_option", h, _lib.OPT_TILE_ROWS, 40)

    def forward(self) -> list[list[np.ndarray]]:
        """DFT accumulators of every monitor of every design."""
        r0 = self.runners[0]
        call("etg_adj_batch_forward", self._h, r0.problem.n_steps, r0.stride)
        return [[r.engine.dft(k) for k in range(len(r.engine.monitors))] for r in self.runners]

    def backward(self, grad_accs: list[list[np.ndarray | None]]) -> list[tuple[np.ndarray, np.ndarray]]:
        """dJ/dcb of every design from its dJ/dacc per monitor."""
        for r, g in zip(self.runners, grad_accs):
            r.set_objective(g)
        call("etg_adj_batch_backward", self._h)
        return [r.gradient() for r in self.runners]

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.lib().etg_adj_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _SimulateBatch(torch.autograd.Function):
    @staticmethod
    def forward(ctx, batch: AdjointBatch, *eps):
        cbs = []
        for r, k in zip(batch.runners, range(0, len(eps), 2)):
            cbs.append(r.set_eps(eps[k].detach().cpu().numpy(), eps[k + 1].detach().cpu().numpy()))
        accs = batch.forward()
        ctx.batch, ctx.cbs = batch, cbs
        ctx.save_for_backward(*eps)
        ctx.counts = [len(a) for a in accs]
        return tuple(torch.as_tensor(np.stack([a.real, a.imag], -1).astype(np.float64)) for per in accs for a in per)

    @staticmethod
    def backward(ctx, *grads):
        eps = ctx.saved_tensors
        per, k = [], 0
        for c in ctx.counts:
            per.append([None if t is None else (t[..., 0].numpy() + 1j * t[..., 1].numpy()) for t in grads[k:k + c]])
            k += c
        out = []
        for (gx, gy), (cbx, cby), q in zip(ctx.batch.backward(per), ctx.cbs, range(0, len(eps), 2)):
            out.append(torch.as_tensor(gx * (-cbx / eps[q].detach().numpy())))
            out.append(torch.as_tensor(gy * (-cby / eps[q + 1].detach().numpy())))
        return (None, *out)


def simulate_batch(eps_cells: list[torch.Tensor], batch: AdjointBatch) -> list[tuple[torch.Tensor, ...]]:
    """``simulate`` for every design of a batch: per design, the accumulators of its monitors."""
    node_eps = []
    for e, r in zip(eps_cells, batch.runners):
        node_eps.extend(r.design.node_eps(e, r.static))
    flat = _SimulateBatch.apply(batch, *node_eps)
    out, k = [], 0
    for r in batch.runners:
        c = len(r.engine.monitors)
        out.append(tuple(flat[k:k + c]))
        k += c
    return out


class _Simulate(torch.autograd.Function):
    @staticmethod
    def forward(ctx, eps_ex, eps_ey, runner: AdjointRunner):
        cbx, cby = runner.set_eps(eps_ex.detach().cpu().numpy(), eps_ey.detach().cpu().numpy())
        accs = runner.forward()
        ctx.runner, ctx.cb = runner, (cbx, cby)
        ctx.save_for_backward(eps_ex, eps_ey)
        return tuple(torch.as_tensor(np.stack([a.real, a.imag], -1).astype(np.float64)) for a in accs)

    @staticmethod
    def backward(ctx, *grads):
        eps_ex, eps_ey = ctx.saved_tensors
        g = [None if t is None else (t[..., 0].numpy() + 1j * t[..., 1].numpy()) for t in grads]
        gx, gy = ctx.runner.backward(g)
        cbx, cby = ctx.cb
        dx = torch.as_tensor(gx * (-cbx / eps_ex.detach().numpy()))
        dy = torch.as_tensor(gy * (-cby / eps_ey.detach().numpy()))
        return dx, dy, None


def simulate(eps_cells: torch.Tensor, runner: AdjointRunner) -> tuple[torch.Tensor, ...]:
    """DFT accumulators (n_f, nodes, 2) of every monitor, differentiable in the design cells' ε."""
    eps_ex, eps_ey = runner.design.node_eps(eps_cells, runner.static)
    return _Simulate.apply(eps_ex, eps_ey, runner)


def point_value(acc: torch.Tensor, sampling: ComponentSampling) -> tuple[torch.Tensor, torch.Tensor]:
    """The monitor value F as (real, imaginary) float64 tensors of shape (n_f, raw axes...).

    ``acc`` is an accumulator as ``simulate`` returns it, (n_f, nodes, 2). The nodes are
    contracted with the bilinear weights of each interpolated axis, x first and then y, as
    etalon/io/result.py:60-79 does in float64 (an interpolated axis holds at most two nodes).
    F equals Etalon's value bit for bit where torch and NumPy round these two-term sums alike
    (tested against Etalon's own values on the machine that made the fixtures); elsewhere it
    can differ in the last bit, as Etalon's own value does between x86 and Arm."""
    n_f = sampling.wavelengths.size
    shape = (n_f, sampling.x.index.size, sampling.y.index.size)
    re, im = acc[..., 0].reshape(shape), acc[..., 1].reshape(shape)
    if sampling.x.weights is not None:
        wx = torch.as_tensor(sampling.x.weights, dtype=torch.float64)
        re, im = torch.einsum("fab,a->fb", re, wx), torch.einsum("fab,a->fb", im, wx)
    if sampling.y.weights is not None:
        wy = torch.as_tensor(sampling.y.weights, dtype=torch.float64)
        re, im = re @ wy, im @ wy
    return re, im


def point_power(acc: torch.Tensor, sampling: ComponentSampling) -> torch.Tensor:
    """Σ_f |F(f)|² of a monitor component, F its interpolated value (``point_value``)."""
    re, im = point_value(acc, sampling)
    return (re**2 + im**2).sum()
