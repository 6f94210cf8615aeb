"""Permittivity rasterised on the device (etg_sim_rasterize_cb) against the host path.

The host path is Etalon's staircase (etalon/grid/materials.py:12-35: last box wins, faces
included within 1e-9 µm, boxes off the plane z = grid.z skipped) followed by the cast of
etalon/fdtd/state.py:80-81; the device copy of cb_ex and cb_ey must equal it bit for bit.
"""

import numpy as np
import pytest

from etalon_gb300 import physics as ph
from etalon_gb300.engine import TEEngine
from etalon_gb300.physics import Box, PMLSpec
from tests import cases

pytestmark = pytest.mark.gpu


def _boxes(grid, seed, n=24):
    """Random boxes over the grid (into the CPML too), boxes whose faces sit exactly on nodes,
    one box off the simulated plane and one of zero thickness on it."""
    rng = np.random.default_rng(seed)
    lx, ly = grid.nx * grid.dx, grid.ny * grid.dy
    x0, y0 = grid.x_min, grid.y_min
    out = []
    for _ in range(n):
        c = (x0 + rng.uniform(0, lx), y0 + rng.uniform(0, ly), 0.0)
        s = (rng.uniform(0.02, 0.6) * lx, rng.uniform(0.02, 0.6) * ly, 0.22)
        out.append(Box(c, s, float(rng.choice([1.0, 2.085, 12.11, float(rng.uniform(1, 13))]))))
    for _ in range(6):  # faces on Ey x-nodes / Ex y-nodes and on half nodes
        kx, ky = (int(v) for v in rng.integers(4, min(grid.nx, grid.ny) - 4, 2))
        mx, my = (int(v) for v in rng.integers(1, 12, 2))
        half = float(rng.integers(0, 2)) * 0.5
        c = (x0 + (kx + half) * grid.dx, y0 + (ky + half) * grid.dy, 0.0)
        out.append(Box(c, (2 * mx * grid.dx, 2 * my * grid.dy, 0.22), 7.5))
    out.append(Box((x0 + lx / 2, y0 + ly / 2, 1.0), (lx, ly, 0.22), 99.0))  # off the plane: skipped
    out.append(Box((x0 + lx / 3, y0 + ly / 3, 0.0), (0.2 * lx, 0.2 * ly, 0.0), 5.0))  # zero thickness
    return out


@pytest.mark.parametrize("precision", ["single", "double"])
@pytest.mark.parametrize("size,dl,seed", [((131 * 0.03, 97 * 0.03), 0.03, 1), ((40.48, 40.48), 0.02, 2)])
def test_rasterized_cb_bit_identical_to_host(gpu, precision, size, dl, seed):
    grid = ph.yee_grid(size, dl, 12, 0.99, (0.0, 0.0, 0.0))
    boxes = _boxes(grid, seed)
    src = [ph.PointSource((0.0, 0.0, 0.0), "Hz", ph.GaussianPulse(1.55, 0.5))]
    host = ph.te_problem(size=size, dl=dl, sources=src, background_eps=2.085, boxes=boxes,
                         pml=PMLSpec(layers=12), precision=precision)  # fmt: skip
    blank = ph.te_problem(size=size, dl=dl, sources=src, background_eps=2.085, pml=PMLSpec(layers=12),
                          precision=precision)  # fmt: skip
    want = ph.cast_coefficients(host)
    e = TEEngine(blank, table_steps=0)
    try:
        e.rasterize(boxes, 2.085)
        for which, ref in (("ex", want.cb_ex), ("ey", want.cb_ey)):
            got = e.cb(which)
            assert got.dtype == ref.dtype and got.shape == ref.shape
            assert np.array_equal(got.view(np.uint8), ref.view(np.uint8)), (which, np.argwhere(got != ref)[:5])
        e.rasterize([], 2.085)  # no boxes: the background everywhere
        assert np.array_equal(e.cb("ex"), ph.cast_coefficients(blank).cb_ex)
    finally:
        e.close()


@pytest.mark.parametrize("precision", ["single", "double"])
def test_rasterized_run_matches_host_run(gpu, precision):
    """A run on rasterised coefficients equals the run on host-cast ones, after a restart."""
    host = cases.g4_full(precision, n_steps=300)
    box = Box((0.3, -0.2, 0.0), (1.5, 0.5, 0.22), 3.476**2)
    a = TEEngine(host)
    b = TEEngine(host)
    try:
        a.advance(300)
        b.advance(50)  # resident work queued first, then the coefficients change under it
        b.rasterize([Box((0.0, 0.0, 0.0), (1.0, 1.0, 0.22), 1.0)], 1.444**2)
        b.rasterize([box], 1.444**2)
        b.reset()
        b.advance(300)
        for name in ("ex", "ey", "hz"):
            assert np.array_equal(a.field(name), b.field(name)), name
        for k in range(len(a.monitors)):
            assert np.array_equal(a.dft(k), b.dft(k))
    finally:
        a.close()
        b.close()
