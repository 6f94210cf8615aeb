"""Etalon Studio's live-view arithmetic on this backend's device arrays (needs a GPU).

The expressions below are the ones of etalon/studio/runner.py:258-291 (field_energy and
downsample), written against the backend's ``xp``; they must run on the device and agree
with NumPy on the same host arrays (sums in float64, so only the summation order differs).
"""

import math

import numpy as np
import pytest

from etalon_gb300.backend import Gb300Backend

pytestmark = pytest.mark.gpu


def _energy(state, xp, dt, db, cell_area):
    """runner.py:258-281, on any array module."""

    def weighted(field, coefficient):
        values = field.astype(xp.float64)
        return float(xp.sum(values * values / coefficient))

    hz = state["hz"].astype(xp.float64)
    electric = dt * (weighted(state["ex"], state["cb_ex"]) + weighted(state["ey"], state["cb_ey"]))
    magnetic = dt / float(db) * float(xp.sum(hz * hz))
    return float(0.5 * cell_area * (electric + magnetic))


def _downsample(field, xp, max_nodes):
    """runner.py:284-291."""
    n_x, n_y = field.shape
    sx = max(1, math.ceil(n_x / max_nodes))
    sy = max(1, math.ceil(n_y / max_nodes))
    mx, my = n_x // sx, n_y // sy
    blocks = field[: mx * sx, : my * sy].reshape(mx, sx, my, sy).mean(axis=(1, 3))
    return blocks.astype(xp.float32), sx, sy


@pytest.mark.parametrize("precision", ["single", "double"])
def test_field_energy_on_device_matches_numpy(gpu, precision):
    dtype = np.float32 if precision == "single" else np.float64
    rng = np.random.default_rng(4)
    nx, ny = 301, 257
    host = {"ex": rng.standard_normal((nx, ny + 1)), "ey": rng.standard_normal((nx + 1, ny)),
            "hz": rng.standard_normal((nx, ny)) / 377.0,
            "cb_ex": rng.uniform(1e-4, 1e-3, (nx, ny + 1)), "cb_ey": rng.uniform(1e-4, 1e-3, (nx + 1, ny))}  # fmt: skip
    host = {k: v.astype(dtype) for k, v in host.items()}
    backend = Gb300Backend(precision)
    dev = {k: backend.to_device(v) for k, v in host.items()}
    args = (1.1e-16, dtype(2.3e-7), 4e-16)
    got = _energy(dev, backend.xp, *args)
    want = _energy(host, np, *args)
    assert got == pytest.approx(want, rel=1e-12)


@pytest.mark.parametrize("precision", ["single", "double"])
@pytest.mark.parametrize("shape", [(1000, 700), (255, 256), (48, 31)])
def test_snapshot_downsample_on_device_matches_numpy(gpu, precision, shape):
    dtype = np.float32 if precision == "single" else np.float64
    field = np.random.default_rng(5).standard_normal(shape).astype(dtype)
    backend = Gb300Backend(precision)
    blocks, sx, sy = _downsample(backend.to_device(field), backend.xp, 256)
    ref, rx, ry = _downsample(field, np, 256)
    assert (sx, sy) == (rx, ry)
    got = np.asarray(backend.to_host(blocks), dtype=np.float32)
    assert got.shape == ref.shape
    np.testing.assert_allclose(got, ref, rtol=2e-6, atol=1e-7)


def test_unsupported_device_expressions_fail_loudly(gpu):
    backend = Gb300Backend("single")
    a = backend.to_device(np.ones((4, 4), np.float32))
    with pytest.raises(TypeError):
        backend.xp.sum(a)
    with pytest.raises(TypeError):
        a[1:, :]


def _studio_progress_loop(solver, every, frames, cell_area):
    """Studio's stepping loop (etalon/studio/runner.py:525-545): step(), then every few steps a
    progress frame (field_energy, runner.py:258-281) and a snapshot (snapshot_frame's
    downsample, runner.py:284-297), read from ``solver.state`` through ``solver.backend.xp``."""
    out = []
    xp = solver.backend.xp
    for _ in range(frames):
        for _ in range(every):
            solver.step()
        state = solver.state
        s = {k: getattr(state, k) for k in ("ex", "ey", "hz", "cb_ex", "cb_ey")}
        energy = _energy(s, xp, solver.grid.dt, state.db, cell_area)
        blocks, sx, sy = _downsample(state.hz, xp, 64)
        out.append((solver.n, energy, np.asarray(solver.backend.to_host(blocks), dtype=np.float32), sx, sy))
    return out


@pytest.mark.parametrize("precision", ["single", "double"])
def test_studio_loop_on_the_resident_solver(gpu, precision):
    """Studio's live view on the fused engine: GB300Solver.state exposes the engine's own
    (pitched) arrays to the same expressions; each frame equals NumPy on host copies of the
    same fields (energy to float64 summation order, snapshot to float32 rounding)."""
    from etalon_gb300 import physics as ph
    from etalon_gb300.solver import GB300Solver
    from tests import cases

    p = cases.config1(precision, n_steps=600)
    solver = GB300Solver(p)
    c = ph.cast_coefficients(p)
    cell_area = p.grid.dx * 1e-6 * p.grid.dy * 1e-6
    frames = _studio_progress_loop(solver, every=97, frames=6, cell_area=cell_area)
    ref = GB300Solver(p)
    for n, energy, snap, sx, sy in frames:
        ref.advance(n - ref.n)
        host = {k: ref.engine.field(k) for k in ("ex", "ey", "hz")}
        host.update(cb_ex=c.cb_ex, cb_ey=c.cb_ey)
        want = _energy(host, np, p.grid.dt, c.db, cell_area)
        assert energy == pytest.approx(want, rel=1e-12) and want > 0
        blocks, rx, ry = _downsample(host["hz"], np, 64)
        assert (sx, sy) == (rx, ry) and snap.shape == blocks.shape
        np.testing.assert_allclose(snap, blocks, rtol=2e-6, atol=1e-7 * np.abs(blocks).max())
    assert frames[-1][0] == 6 * 97
    solver.close()
    ref.close()
