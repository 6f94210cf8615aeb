"""Named 2D TE cases shared by the tests, the golden generator and the bench.

Each builder returns an ``etalon_gb300.physics.TEProblem``. tests/golden/make_golden.py
builds the same cases through Etalon's own API, so the fixtures it writes pin both the
host setup and the time stepping of these exact problems.
"""

from __future__ import annotations

import math

import numpy as np

from etalon_gb300 import physics as ph
from etalon_gb300.physics import Box, DFTMonitor, GaussianPulse, PMLSpec, PointSource

N_OXIDE = math.sqrt(2.085)
N_SILICON = math.sqrt(12.11)


def config1(precision="single", n_steps=2000):
    """8×8 µm vacuum at dl 0.05 (160² + 12-layer CPML), Hz source at (−3, 0), probe at (3, 0)."""
    return ph.te_problem(
        size=(8.0, 8.0),
        dl=0.05,
        sources=[PointSource((-3.0, 0.0, 0.0), "Hz", GaussianPulse(1.55, 0.5))],
        monitors=[DFTMonitor("probe", list(np.linspace(1.3, 1.8, 5)), center=(3.0, 0.0, 0.0))],
        pml=PMLSpec(layers=12),
        n_steps=n_steps,
        precision=precision,
    )


def g4_full(precision="single", n_steps=600):
    """Etalon's GPU parity run: Si box in oxide, off-grid Ey + Hz sources, point + plane monitors.

    The same simulation as tests/gpu/test_cupy_equality.py:113-147 of Etalon.
    """
    return ph.te_problem(
        size=(131 * 0.03, 97 * 0.03),
        dl=0.03,
        background_eps=1.444**2,
        boxes=[Box((0.3, -0.2, 0.0), (1.5, 0.5, 0.22), 3.476**2)],
        pml=PMLSpec(layers=10, kappa_max=2.0),
        sources=[
            PointSource((-1.234, 0.071, 0.0), "Ey", GaussianPulse(1.55, 0.3)),
            PointSource((0.517, 0.633, 0.0), "Hz", GaussianPulse(1.31, 0.2, amplitude=0.5)),
        ],
        monitors=[
            DFTMonitor("point", list(np.linspace(1.3, 1.7, 9)), center=(1.11, -0.37, 0.0)),
            DFTMonitor("plane", [1.31, 1.55], size=(3.0, 2.0, 0.0)),
        ],
        n_steps=n_steps,
        precision=precision,
    )


def small(precision="single", n_steps=None):
    """2 × 1.5 µm vacuum, dl 0.05, 8-layer CPML (Etalon tests/sims.py:12-24) + a plane monitor."""
    p = ph.te_problem(
        size=(2.0, 1.5),
        dl=0.05,
        pml=PMLSpec(layers=8),
        sources=[PointSource((-0.5, 0.1, 0.0), "Hz", GaussianPulse(1.55, 0.5))],
        monitors=[
            DFTMonitor("probe", [1.5, 1.6], center=(0.5, 0.0, 0.0)),
            DFTMonitor("plane", [1.31, 1.55], size=(1.0, 0.6, 0.0), components=("Hz",)),
        ],
        run_time=20e-15,
        precision=precision,
    )
    if n_steps is not None:
        p.n_steps = n_steps
    return p


def config2(precision="single", n_steps=10000, region=2000):
    """40 × 40 µm at dl 0.02 (2000² + 12-layer CPML): Si strip (w 0.5 µm, along x) in oxide.

    Hz source in the core at x = −15 µm; three point monitors on the axis at x = −5, 5, 15 µm,
    each at 16 wavelengths in 1.5–1.6 µm. ``region`` scales the square region (cells per side)
    for smaller replicas of the same device.
    """
    dl = 0.02
    side = region * dl
    scale = side / 40.0
    wl = list(np.linspace(1.5, 1.6, 16))
    return ph.te_problem(
        size=(side, side),
        dl=dl,
        background_eps=N_OXIDE**2,
        boxes=[Box((0.0, 0.0, 0.0), (side + 2.0, 0.5, 0.22), N_SILICON**2)],
        pml=PMLSpec(layers=12),
        sources=[PointSource((-15.0 * scale, 0.0, 0.0), "Hz", GaussianPulse(1.55, 0.5))],
        monitors=[
            DFTMonitor(f"m{k}", wl, center=(x * scale, 0.0, 0.0)) for k, x in enumerate((-5.0, 5.0, 15.0))
        ],
        n_steps=n_steps,
        precision=precision,
    )


def centred(precision="double", n_steps=300):
    """Odd 41×41 region with a centred Hz source: fields are exactly mirror-symmetric.

    Etalon tests/unit/test_numpy_backend.py:61-85.
    """
    return ph.te_problem(
        size=(41 * 0.05, 41 * 0.05),
        dl=0.05,
        pml=PMLSpec(layers=8),
        sources=[PointSource((0.0, 0.0, 0.0), "Hz", GaussianPulse(1.55, 0.5))],
        n_steps=n_steps,
        precision=precision,
    )


CASES = {"config1": config1, "g4_full": g4_full, "small": small, "config2": config2, "centred": centred}


def random_state_inputs(dtype, seed=1):
    """Etalon's random 67×53 TE state (tests/gpu/test_cupy_equality.py:36-79), as plain arrays.

    Returns (grid, coeffs, fields): coefficients cast to ``dtype`` and the seven initial
    field/ψ arrays. The random CPML profiles are non-zero everywhere, so ψ is live on
    every node.
    """
    rng = np.random.default_rng(seed)
    nx, ny, dx, dy = 67, 53, 0.05, 0.04
    grid = ph.YeeGrid2D(nx=nx, ny=ny, dx=dx, dy=dy, dt=ph.courant_time_step(0.99, dx, dy),
                        pml_layers=0, x_min=0.0, y_min=0.0)  # fmt: skip
    eps = {c: rng.uniform(1.0, 12.0, grid.shape(c)) for c in ("Ex", "Ey")}

    def axis(n):
        return ph.CPMLAxis(
            rng.uniform(0.2, 1.0, n + 1), -rng.uniform(0, 0.8, n + 1), rng.uniform(0.3, 1.0, n + 1),
            rng.uniform(0.2, 1.0, n), -rng.uniform(0, 0.8, n), rng.uniform(0.3, 1.0, n),
        )  # fmt: skip

    cx, cy = axis(nx), axis(ny)
    shapes = [("ex", grid.shape("Ex")), ("ey", grid.shape("Ey")), ("hz", grid.shape("Hz")),
              ("psi_ex_y", grid.shape("Ex")), ("psi_ey_x", grid.shape("Ey")),
              ("psi_hz_x", grid.shape("Hz")), ("psi_hz_y", grid.shape("Hz"))]  # fmt: skip
    fields = {name: rng.standard_normal(shape).astype(dtype) for name, shape in shapes}
    fields["hz"] *= 1 / 377.0
    problem = ph.TEProblem(grid, eps, cx, cy, [], [], "single" if dtype == np.float32 else "double")
    return grid, ph.cast_coefficients(problem), fields


def dft_inputs(dtype, seed=2):
    """Etalon's random DFT-kernel case (tests/gpu/test_cupy_equality.py:95-110)."""
    rng = np.random.default_rng(seed)
    complex_dtype = np.complex64 if dtype == np.float32 else np.complex128
    field = rng.standard_normal((67, 54)).astype(dtype)
    index = rng.choice(field.size, size=301, replace=False).astype(np.int64)
    phasors = np.exp(1j * rng.uniform(0, 2 * np.pi, 13)).astype(complex_dtype) * 1e-16
    acc = (rng.standard_normal((13, 301)) + 1j * rng.standard_normal((13, 301))) * 1e-15
    return field, index, phasors, acc.astype(complex_dtype)


# ----------------------------------------------------------------- seeded synthetic devices

EPS_OXIDE = 2.085
EPS_SILICON = 12.11
WIDTH = 0.5  # strip width (µm)
DEVICE_KINDS = ("bend", "ring", "mmi")


def _device_core(kind, X, Y, lx, ly, rng_params):
    """Boolean silicon mask of a device at node coordinates X, Y (µm, region centred on 0)."""
    w = WIDTH
    if kind == "bend":
        r = min(rng_params["radius"], 0.35 * min(lx, ly))
        x0, y0 = -r / 2, -r / 2  # input strip along x at y0 up to x0, quarter circle, output along +y
        rr = np.hypot(X - x0, Y - (y0 + r))
        arc = (np.abs(rr - r) <= w / 2) & (X >= x0) & (Y <= y0 + r)
        return arc | ((np.abs(Y - y0) <= w / 2) & (X <= x0)) | ((np.abs(X - (x0 + r)) <= w / 2) & (Y >= y0 + r))
    if kind == "ring":
        r = min(rng_params["radius"], 0.4 * min(lx, ly) - w)
        g = rng_params["gap"]
        yb = -(r + g + w) / 2  # bus strip along x; ring above it, separated by the gap
        yc = yb + w + g + r
        return (np.abs(Y - yb) <= w / 2) | (np.abs(np.hypot(X, Y - yc) - r) <= w / 2)
    if kind == "mmi":
        length = min(rng_params["length"], 0.7 * lx)
        width = min(rng_params["width"], 0.7 * ly)
        box = (np.abs(X) <= length / 2) & (np.abs(Y) <= width / 2)
        inp = (np.abs(Y) <= w / 2) & (X < 0)
        outs = (X > 0) & ((np.abs(Y - width / 4) <= w / 2) | (np.abs(Y + width / 4) <= w / 2))
        return box | inp | outs
    raise ValueError(kind)


def synthetic_device(seed, precision="single", n_steps=5000, min_cells=256, max_cells=1536, dl=0.02,
                     n_monitors=4, n_wavelengths=8):  # fmt: skip
    """One seeded random device on oxide: a waveguide bend (radius 1-5 µm), a ring resonator
    (radius 2-6 µm, gap 0.1-0.3 µm) or an MMI box (1-8 µm), ε ∈ {2.085, 12.11}.

    Interior nx, ny drawn uniformly in [min_cells, max_cells] (non-square), 12-layer CPML, one
    Gaussian Hz source in the input strip, ``n_monitors`` point monitors at ``n_wavelengths``
    wavelengths in 1.5-1.6 µm. Geometry beyond the region continues into the CPML.
    """
    rng = np.random.default_rng(seed)
    nx, ny = (int(v) for v in rng.integers(min_cells, max_cells + 1, 2))
    lx, ly = nx * dl, ny * dl
    kind = DEVICE_KINDS[int(rng.integers(0, 3))]
    params = {"radius": float(rng.uniform(1.0, 5.0) if kind == "bend" else rng.uniform(2.0, 6.0)),
              "gap": float(rng.uniform(0.1, 0.3)), "length": float(rng.uniform(1.0, 8.0)),
              "width": float(rng.uniform(1.0, 3.0))}  # fmt: skip
    grid = ph.yee_grid((lx, ly), dl, 12, 0.99, (0.0, 0.0, 0.0))
    eps = {}
    for c in ("Ex", "Ey"):
        x, y = grid.coords(c)
        X, Y = np.meshgrid(x, y, indexing="ij")
        eps[c] = np.where(_device_core(kind, X, Y, lx, ly, params), EPS_SILICON, EPS_OXIDE)
    if kind == "bend":
        r = min(params["radius"], 0.35 * min(lx, ly))
        y_in = -r / 2
    elif kind == "ring":
        r = min(params["radius"], 0.4 * min(lx, ly) - WIDTH)
        y_in = -(r + params["gap"] + WIDTH) / 2
    else:
        y_in = 0.0
    src = PointSource((-0.4 * lx, y_in, 0.0), "Hz", GaussianPulse(1.55, 0.5))
    wl = list(np.linspace(1.5, 1.6, n_wavelengths))
    pts = rng.uniform(-0.4, 0.4, (n_monitors, 2)) * np.array([lx, ly])
    monitors = [DFTMonitor(f"m{k}", wl, center=(float(px), float(py), 0.0)) for k, (px, py) in enumerate(pts)]
    return ph.te_problem(size=(lx, ly), dl=dl, sources=[src], monitors=monitors, background_eps=EPS_OXIDE,
                         eps=eps, pml=PMLSpec(layers=12), n_steps=n_steps, precision=precision)  # fmt: skip


def synthetic_batch(n=64, seed=2024, **kw):
    """``n`` seeded synthetic devices (sizes 256²-1536² unless overridden)."""
    return [synthetic_device(seed * 1000 + k, **kw) for k in range(n)]


def smooth_design(nx, ny, seed, sigma=3.0):
    """Per-cell ε in [2.085, 12.11] from a seeded uniform field smoothed with a Gaussian of
    ``sigma`` cells, rescaled to [0, 1] before mapping to ε."""
    from scipy.ndimage import gaussian_filter

    u = gaussian_filter(np.random.default_rng(seed).uniform(0.0, 1.0, (nx, ny)), sigma, mode="reflect")
    u = (u - u.min()) / max(u.max() - u.min(), 1e-30)
    return EPS_OXIDE + (EPS_SILICON - EPS_OXIDE) * u


def adjoint_device(precision="single", n_steps=20000, region=1200, design=100, dl=0.02, n_wavelengths=3):
    """Single-design adjoint workload: ``region``² cells at dl + 12-layer CPML, oxide, input and
    output Si strips (0.5 µm) along x meeting a ``design``² cell window at the centre; Hz source
    in the input strip, Hz point monitor in the output strip at 1.50/1.55/1.60 µm (3 λ) or
    ``n_wavelengths`` evenly in 1.5-1.6 µm. Returns (problem, (x0, y0, wx, wy) of the window)."""
    side = region * dl
    half = design * dl / 2
    eps_box = side / 2 + 1.0
    strips = [Box((-(eps_box + half) / 2, 0.0, 0.0), (eps_box - half, WIDTH, 0.22), EPS_SILICON),
              Box(((eps_box + half) / 2, 0.0, 0.0), (eps_box - half, WIDTH, 0.22), EPS_SILICON)]  # fmt: skip
    wl = [1.50, 1.55, 1.60] if n_wavelengths == 3 else list(np.linspace(1.5, 1.6, n_wavelengths))
    p = ph.te_problem(
        size=(side, side), dl=dl, background_eps=EPS_OXIDE, boxes=strips, pml=PMLSpec(layers=12),
        sources=[PointSource((-0.35 * side, 0.0, 0.0), "Hz", GaussianPulse(1.55, 0.5))],
        monitors=[DFTMonitor("out", wl, center=(0.35 * side + 0.011, 0.007, 0.0), components=("Hz",))],
        n_steps=n_steps, precision=precision,
    )  # fmt: skip
    return p, (0.0, 0.0, design * dl - 1e-6, design * dl - 1e-6)


def adjoint_variants(n=32, seed=5, precision="single", n_steps=10000, min_cells=512, max_cells=1024,
                     min_design=50, max_design=150):  # fmt: skip
    """``n`` seeded design variants for batched gradients: square regions of min-max cells per
    side, design windows of min-max cells per side with smoothed random ε, 8 wavelengths in
    1.5-1.6 µm. Returns [(problem, (x0, y0, wx, wy) of the window, ε cells (float64))]."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        region = int(rng.integers(min_cells, max_cells + 1))
        design = int(rng.integers(min_design, max_design + 1))
        p, win = adjoint_device(precision, n_steps=n_steps, region=region, design=design, n_wavelengths=8)
        out.append((p, win, design, seed * 1000 + k))
    return out
