"""Generate golden vectors by running Etalon's own NumPy reference (not the oracle).

Run in a checkout where Etalon's source tree is available (default /root/reference):

    python tests/golden/make_golden.py [--cases config1,g4_full,...] [--ref PATH]

Etalon's ``io/result.py`` imports xarray at module level; xarray is only needed to
label results, so a stub module stands in for it. Each case is built through Etalon's
public API (``etalon.Simulation`` …) with the same parameters as tests/cases.py and is
stepped by ``etalon.fdtd.solver.FDTDSolver`` on ``NumpyBackend``. Per case and precision
the fixture holds:

* setup pins — grid, ε maps, CPML profiles, injections and monitor samplings in float64
  (hashes only for the large config2 case);
* the host values the solver consumed — per-step source deltas and phasor rows, already
  cast — so the GPU path can be fed Etalon's exact inputs on any platform (config2 keeps
  only their hashes in float32, 10 000 steps, and the tables themselves in float64);
* outputs after the run — SHA-256, sum and max|.| of the seven field/ψ arrays, and the
  DFT accumulators in full.

Kernel-level cases (Etalon tests/gpu/test_cupy_equality.py:36-110, seeds 1 and 2) store
input and output hashes of one ``update_h_te`` / ``update_e_te`` / ``accumulate_dft`` call.
"""

from __future__ import annotations

import argparse
import hashlib
import math
import sys
import time
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
FIELDS = ("ex", "ey", "hz", "psi_ex_y", "psi_ey_x", "psi_hz_x", "psi_hz_y")
COEFFS = ("cb_ex", "cb_ey", "bx_e", "cx_e", "ikx_e", "bx_h", "cx_h", "ikx_h",
          "by_e", "cy_e", "iky_e", "by_h", "cy_h", "iky_h")  # fmt: skip


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def import_etalon(ref: str):
    sys.path.insert(0, ref)
    stub = types.ModuleType("xarray")
    stub.DataArray = object
    sys.modules.setdefault("xarray", stub)
    import etalon

    return etalon


def reference_sims(et, precision):
    """The cases of tests/cases.py, written against Etalon's API."""
    n_ox, n_si = math.sqrt(2.085), math.sqrt(12.11)
    pulse = et.GaussianPulse
    sims = {}
    sims["config1"] = (
        et.Simulation(
            size=(8.0, 8.0, 0.0), grid=et.UniformGrid(dl=0.05), boundary=et.PML(layers=12),
            sources=[et.PointSource(center=(-3.0, 0.0, 0.0), component="Hz",
                                    pulse=pulse(wavelength=1.55, bandwidth=0.5))],
            monitors=[et.DFTMonitor(name="probe", center=(3.0, 0.0, 0.0),
                                    wavelengths=list(np.linspace(1.3, 1.8, 5)))],
            run_time=1.0, precision=precision, backend="numpy"),
        2000,
    )  # fmt: skip
    sims["g4_full"] = (
        et.Simulation(
            size=(131 * 0.03, 97 * 0.03, 0.0), grid=et.UniformGrid(dl=0.03),
            medium=et.Medium(n=1.444),
            structures=[et.Box(center=(0.3, -0.2, 0.0), size=(1.5, 0.5, 0.22), medium=et.Medium(n=3.476))],
            boundary=et.PML(layers=10, kappa_max=2.0),
            sources=[
                et.PointSource(center=(-1.234, 0.071, 0.0), component="Ey",
                               pulse=pulse(wavelength=1.55, bandwidth=0.3)),
                et.PointSource(center=(0.517, 0.633, 0.0), component="Hz",
                               pulse=pulse(wavelength=1.31, bandwidth=0.2, amplitude=0.5)),
            ],
            monitors=[
                et.DFTMonitor(name="point", center=(1.11, -0.37, 0.0), wavelengths=list(np.linspace(1.3, 1.7, 9))),
                et.DFTMonitor(name="plane", size=(3.0, 2.0, 0.0), wavelengths=[1.31, 1.55]),
            ],
            run_time=1.0, precision=precision, backend="numpy"),
        600,
    )  # fmt: skip
    small = et.Simulation(
        size=(2.0, 1.5, 0.0), grid=et.UniformGrid(dl=0.05), boundary=et.PML(layers=8),
        sources=[et.PointSource(center=(-0.5, 0.1, 0.0), component="Hz",
                                pulse=pulse(wavelength=1.55, bandwidth=0.5))],
        monitors=[
            et.DFTMonitor(name="probe", center=(0.5, 0.0, 0.0), wavelengths=[1.5, 1.6]),
            et.DFTMonitor(name="plane", size=(1.0, 0.6, 0.0), wavelengths=[1.31, 1.55], components=("Hz",)),
        ],
        run_time=20e-15, precision=precision, backend="numpy")  # fmt: skip
    sims["small"] = (small, None)
    wl = list(np.linspace(1.5, 1.6, 16))
    sims["config2"] = (
        et.Simulation(
            size=(40.0, 40.0, 0.0), grid=et.UniformGrid(dl=0.02), medium=et.Medium(n=n_ox),
            structures=[et.Box(center=(0.0, 0.0, 0.0), size=(42.0, 0.5, 0.22), medium=et.Medium(n=n_si))],
            boundary=et.PML(layers=12),
            sources=[et.PointSource(center=(-15.0, 0.0, 0.0), component="Hz",
                                    pulse=pulse(wavelength=1.55, bandwidth=0.5))],
            monitors=[et.DFTMonitor(name=f"m{k}", center=(x, 0.0, 0.0), wavelengths=wl)
                      for k, x in enumerate((-5.0, 5.0, 15.0))],
            run_time=1.0, precision=precision, backend="numpy"),
        10000 if precision == "single" else 1000,
    )  # fmt: skip
    return sims


def setup_pins(solver, big: bool) -> dict:
    """Float64 host setup as Etalon computed it."""
    from etalon.fdtd.cpml import cpml_axis
    from etalon.grid.materials import permittivity_on_nodes

    g, sim = solver.grid, solver.sim
    out = {
        "grid": np.array([g.nx, g.ny, g.pml_layers], np.int64),
        "grid_f": np.array([g.dx, g.dy, g.dt, g.x_min, g.y_min, g.z, g.courant]),
    }
    eps = permittivity_on_nodes(sim, g)
    bg = sim.medium.permittivity
    for axis, (n, d) in (("x", (g.nx, g.dx)), ("y", (g.ny, g.dy))):
        c = cpml_axis(n, d, g.dt, sim.boundary, bg)
        for name in ("b_e", "c_e", "inv_kappa_e", "b_h", "c_h", "inv_kappa_h"):
            out[f"cpml_{axis}_{name}"] = getattr(c, name)
    for comp in ("Ex", "Ey"):
        out[f"eps_{comp}_sha"] = np.array(sha(eps[comp]))
        if not big:
            out[f"eps_{comp}"] = eps[comp]
    for k, inj in enumerate(solver.injections):
        out[f"src{k}_component"] = np.array(inj.component)
        out[f"src{k}_i"], out[f"src{k}_j"] = inj.i, inj.j
        out[f"src{k}_weights"], out[f"src{k}_coef"] = inj.weights, inj.coefficient
        p = inj.pulse
        out[f"src{k}_pulse"] = np.array([p.wavelength, p.bandwidth, p.amplitude])
    for k, mon in enumerate(solver.monitors):
        s = mon.sampling
        out[f"mon{k}_component"] = np.array(s.component)
        out[f"mon{k}_name"] = np.array(s.monitor)
        out[f"mon{k}_flat"] = s.flat_index
        out[f"mon{k}_freq"] = s.frequencies
        out[f"mon{k}_xi"], out[f"mon{k}_yi"] = s.x.index, s.y.index
    return out


def run_case(et, name, precision, steps_override=None):
    from etalon.fdtd.solver import FDTDSolver

    sim, n_steps = reference_sims(et, precision)[name]
    solver = FDTDSolver(sim)
    if n_steps is None:
        n_steps = solver.n_steps
    if steps_override:
        n_steps = steps_override
    solver.n_steps = n_steps
    big = name == "config2"
    out = setup_pins(solver, big)
    out["n_steps"] = np.array(n_steps)
    real = solver.real
    s = solver.state
    for c in COEFFS:
        a = getattr(s, c)
        if big and c.startswith("cb"):
            out[f"in_{c}_sha"] = np.array(sha(a))
        else:
            out[f"in_{c}"] = a
    out["in_scalars"] = np.array([s.db, s.inv_dx, s.inv_dy], dtype=real)

    # the per-step deltas the solver subtracts (solver.py:83-89); the large case keeps only
    # hashes in float32 (10 000 steps) but the tables themselves in float64 (1 000 steps), so a
    # machine whose float64 libm gives other host tables can still replay Etalon's run exactly
    keep_tables = not big or precision == "double"
    for k, inj in enumerate(solver.injections):
        table = np.stack([inj.delta(n, solver.grid.dt).astype(real) for n in range(n_steps)])
        out[f"src{k}_table_sha"] = np.array(sha(table))
        if keep_tables:
            out[f"src{k}_table"] = table
    # the phasor rows accumulate_dft receives, captured from the backend calls
    rows = {id(m.acc): [] for m in solver.monitors}
    backend = solver.backend
    plain = backend.accumulate_dft

    def capture(acc, field, index, phasors):
        rows[id(acc)].append(np.array(phasors, copy=True))
        plain(acc, field, index, phasors)

    backend.accumulate_dft = capture
    t0 = time.time()
    for n in range(n_steps):
        solver.step()
        if big and n % 500 == 0:
            print(f"  {name}/{precision}: step {n} ({time.time() - t0:.0f} s)", flush=True)
    for k, mon in enumerate(solver.monitors):
        table = np.stack(rows[id(mon.acc)])
        assert table.shape[0] == n_steps
        out[f"mon{k}_table_sha"] = np.array(sha(table))
        if keep_tables:
            out[f"mon{k}_table"] = table
        acc = np.asarray(mon.acc)
        out[f"out_acc{k}_sha"] = np.array(sha(acc))
        if acc.size <= 4096:
            out[f"out_acc{k}"] = acc
        else:  # large plane monitors: hash plus a strided sample
            out[f"out_acc{k}_sample"] = acc.ravel()[::97]
    for f in FIELDS:
        a = np.asarray(getattr(s, f))
        out[f"out_{f}_sha"] = np.array(sha(a))
        out[f"out_{f}_sum"] = np.array(float(a.astype(np.float64).sum()))
        out[f"out_{f}_absmax"] = np.array(float(np.abs(a).max()))
    path = HERE / f"{name}_{precision}.npz"
    np.savez_compressed(path, **out)
    print(f"wrote {path.name}: {n_steps} steps in {time.time() - t0:.1f} s", flush=True)


def kernel_cases(et, precision):
    """Single update_h_te / update_e_te / accumulate_dft calls on Etalon's random states."""
    from etalon.fdtd.backends.numpy_backend import NumpyBackend
    from etalon.fdtd.cpml import CPMLAxis
    from etalon.fdtd.state import build_te_state
    from etalon.grid.yee import YeeGrid2D, courant_time_step

    dtype = np.float32 if precision == "single" else np.float64
    out = {}
    for update in ("update_h_te", "update_e_te"):
        rng = np.random.default_rng(1)
        nx, ny, dx, dy = 67, 53, 0.05, 0.04
        grid = YeeGrid2D(nx=nx, ny=ny, dx=dx, dy=dy, dt=courant_time_step(0.99, dx, dy),
                         pml_layers=0, x_min=0.0, y_min=0.0, z=0.0, courant=0.99)  # fmt: skip
        eps = {c: rng.uniform(1.0, 12.0, grid.shape(c)) for c in ("Ex", "Ey")}

        def axis(n):
            return CPMLAxis(rng.uniform(0.2, 1.0, n + 1), -rng.uniform(0, 0.8, n + 1),
                            rng.uniform(0.3, 1.0, n + 1), rng.uniform(0.2, 1.0, n),
                            -rng.uniform(0, 0.8, n), rng.uniform(0.3, 1.0, n))  # fmt: skip

        cx, cy = axis(nx), axis(ny)
        shapes = [("ex", grid.shape("Ex")), ("ey", grid.shape("Ey")), ("hz", grid.shape("Hz")),
                  ("psi_ex_y", grid.shape("Ex")), ("psi_ey_x", grid.shape("Ey")),
                  ("psi_hz_x", grid.shape("Hz")), ("psi_hz_y", grid.shape("Hz"))]  # fmt: skip
        initial = {n: rng.standard_normal(sh).astype(dtype) for n, sh in shapes}
        initial["hz"] *= 1 / 377.0
        s = build_te_state(grid, eps, cx, cy, dtype, lambda a: a)
        for n, v in initial.items():
            setattr(s, n, v.copy())
        for n in FIELDS:
            out[f"{update}_in_{n}_sha"] = np.array(sha(getattr(s, n)))
        for c in COEFFS:
            out[f"{update}_in_{c}_sha"] = np.array(sha(getattr(s, c)))
        getattr(NumpyBackend(), update)(s)
        for n in FIELDS:
            out[f"{update}_out_{n}_sha"] = np.array(sha(getattr(s, n)))
    rng = np.random.default_rng(2)
    complex_dtype = np.complex64 if dtype == np.float32 else np.complex128
    field = rng.standard_normal((67, 54)).astype(dtype)
    index = rng.choice(field.size, size=301, replace=False).astype(np.int64)
    phasors = np.exp(1j * rng.uniform(0, 2 * np.pi, 13)).astype(complex_dtype) * 1e-16
    acc = ((rng.standard_normal((13, 301)) + 1j * rng.standard_normal((13, 301))) * 1e-15).astype(complex_dtype)
    for n, a in (("field", field), ("index", index), ("phasors", phasors), ("acc", acc)):
        out[f"dft_in_{n}_sha"] = np.array(sha(a))
    NumpyBackend().accumulate_dft(acc, field, index, phasors)
    out["dft_out_acc_sha"] = np.array(sha(acc))
    out["dft_out_acc"] = acc
    path = HERE / f"kernels_{precision}.npz"
    np.savez_compressed(path, **out)
    print(f"wrote {path.name}")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    ap.add_argument("--cases", default="kernels,config1,g4_full,small")
    ap.add_argument("--precisions", default="single,double")
    args = ap.parse_args()
    et = import_etalon(args.ref)
    for precision in args.precisions.split(","):
        for name in args.cases.split(","):
            if name == "kernels":
                kernel_cases(et, precision)
            else:
                run_case(et, name, precision)


if __name__ == "__main__":
    main()
