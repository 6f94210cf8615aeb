"""Generate golden vectors by running Etalon's own NumPy reference (not the oracle).

Run where Etalon's source tree is available, naming it with ``--ref`` or ``ETALON_SRC``:

    python tests/golden/make_golden.py --ref PATH [--cases config1,g4_full,...]
    python tests/golden/make_golden.py --ref PATH --augment config2   # monitor values only

Etalon's ``io/result.py`` imports xarray at module level; xarray is only needed to
label results, so a stub module stands in for it. Its ``DataArray`` keeps the data and
dimension names it is given, so the fixtures also record the monitor values Etalon's own
``monitor_dataarray`` (io/result.py:54-91) reports for each accumulator. Each case is built through Etalon's
public API (``etalon.Simulation`` …) with the same parameters as tests/cases.py and is
stepped by ``etalon.fdtd.solver.FDTDSolver`` on ``NumpyBackend``. Per case and precision
the fixture holds:

* setup pins — grid, ε maps, CPML profiles, injections and monitor samplings in float64
  (hashes only for the large config2 case);
* the host values the solver consumed — per-step source deltas and phasor rows, already
  cast — so the GPU path can be fed Etalon's exact inputs on any platform (config2 keeps
  only their hashes in float32, 10 000 steps, and the tables themselves in float64);
* outputs after the run — SHA-256, sum and max|.| of the seven field/ψ arrays, the
  DFT accumulators in full, and the interpolated monitor values ``monitor_dataarray``
  returns for them (with their dimension names).

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


class RecordedDataArray:
    """Stands in for ``xarray.DataArray``: keeps the data and dimension names."""

    def __init__(self, data, dims=(), coords=None, name=None, attrs=None):
        self.data = np.asarray(data)
        self.dims = tuple(dims)
        self.coords, self.name, self.attrs = coords, name, attrs


def import_etalon(ref: str):
    sys.path.insert(0, ref)
    stub = types.ModuleType("xarray")
    stub.DataArray = RecordedDataArray
    sys.modules.setdefault("xarray", stub)
    import etalon

    return etalon


def monitor_values(solver, accs) -> dict:
    """Etalon's own interpolated monitor values (io/result.py:54-91) for the given accumulators."""
    from etalon.io.result import monitor_dataarray

    out = {}
    for k, (mon, acc) in enumerate(zip(solver.monitors, accs)):
        s = mon.sampling
        da = monitor_dataarray(s, np.asarray(acc), solver.grid.z)
        v = np.asarray(da.data)
        out[f"out_value{k}_sha"] = np.array(sha(v))
        out[f"out_value{k}_dims"] = np.array(",".join(da.dims))
        if v.size <= 4096:
            out[f"out_value{k}"] = v
        for axis, a in (("x", s.x), ("y", s.y)):
            if a.weights is not None:
                out[f"mon{k}_{axis}w"] = a.weights
    return out


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
    out.update(monitor_values(solver, [m.acc for m in solver.monitors]))
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


# ----------------------------------------------------------------- protocol traces
# Opcodes of a recorded protocol trace (tests/test_gpu_etalon_trace.py replays them).
OP_TO_DEVICE, OP_UPDATE_H, OP_UPDATE_E, OP_ISUB, OP_ACCUMULATE, OP_TO_HOST, OP_SYNC = range(7)
STATE_ARRAYS = FIELDS + COEFFS


class _Tracked(np.ndarray):
    """A NumPy array the recording backend handed out: knows its handle, or the (handle, row)
    it is a row view of."""

    def __array_finalize__(self, obj):
        self._h = None
        self._row = None

    def __getitem__(self, key):
        if isinstance(key, (int, np.integer)) and self._h is not None:
            v = np.ndarray.__getitem__(self.view(np.ndarray), key).view(_Tracked)
            v._row = (self._h, int(key))
            return v
        if isinstance(key, tuple) and len(key) == 2 and all(isinstance(k, _Tracked) for k in key):
            return _TrackedIndexed(self, key[0], key[1])
        return np.ndarray.__getitem__(self.view(np.ndarray), key)

    def __setitem__(self, key, value):
        if isinstance(value, _TrackedIndexed) and value.target is self and value.applied:
            return
        np.ndarray.__setitem__(self.view(np.ndarray), key, value)


class _TrackedIndexed:
    """``field[i, j]`` for ``field[i, j] -= delta`` (etalon/fdtd/solver.py:89): recorded, then
    applied with NumPy's own fancy-index semantics."""

    def __init__(self, target, i, j):
        self.target, self.i, self.j, self.applied = target, i, j, False

    def __isub__(self, delta):
        rec = _TraceBackend.active
        rec.events.append((OP_ISUB, self.target._h, self.i._h, self.j._h, delta._h, 0))
        plain = self.target.view(np.ndarray)
        plain[self.i.view(np.ndarray), self.j.view(np.ndarray)] -= delta.view(np.ndarray)
        self.applied = True
        return self


class _TraceBackend:
    """Etalon's NumpyBackend, recording every protocol call Etalon's FDTDSolver makes and every
    array it moves to the device."""

    active = None

    def __init__(self, inner):
        self.inner, self.events, self.payloads = inner, [], []
        self.name, self.device, self.xp = inner.name, inner.device, inner.xp
        _TraceBackend.active = self

    def to_device(self, a):
        a = self.inner.to_device(a)
        h = len(self.payloads)
        self.payloads.append(np.array(a, copy=True))
        self.events.append((OP_TO_DEVICE, h, 0, 0, 0, 0))
        t = a.view(_Tracked)
        t._h = h
        return t

    def to_host(self, a):
        self.events.append((OP_TO_HOST, a._h, 0, 0, 0, 0))
        return np.array(a.view(np.ndarray), copy=True)

    def synchronize(self):
        self.events.append((OP_SYNC, 0, 0, 0, 0, 0))

    @staticmethod
    def _plain_state(s):
        import copy

        p = copy.copy(s)
        for k in STATE_ARRAYS:
            setattr(p, k, getattr(s, k).view(np.ndarray))
        return p

    def update_h_te(self, s):
        self.events.append((OP_UPDATE_H, 0, 0, 0, 0, 0))
        self.inner.update_h_te(self._plain_state(s))

    def update_e_te(self, s):
        self.events.append((OP_UPDATE_E, 0, 0, 0, 0, 0))
        self.inner.update_e_te(self._plain_state(s))

    def accumulate_dft(self, acc, field, index, phasors):
        table, row = phasors._row if phasors._row is not None else (phasors._h, -1)
        self.events.append((OP_ACCUMULATE, acc._h, field._h, index._h, table, row))
        self.inner.accumulate_dft(acc.view(np.ndarray), field.view(np.ndarray), index.view(np.ndarray),
                                  phasors.view(np.ndarray))  # fmt: skip


def trace_case(et, name, precision, steps=None):
    """Record the protocol calls of Etalon's FDTDSolver on a case: ``steps`` solver.step()
    calls then fields(), or solver.run() to its end when ``steps`` is None."""
    import etalon.fdtd.solver as solver_module
    from etalon.fdtd.backends.numpy_backend import NumpyBackend

    sim, _ = reference_sims(et, precision)[name]
    plain_get = solver_module.get_backend
    solver_module.get_backend = lambda n, p: _TraceBackend(NumpyBackend())
    try:
        solver = solver_module.FDTDSolver(sim)
    finally:
        solver_module.get_backend = plain_get
    if steps is not None:
        solver.n_steps = steps  # phasor tables of the steps run, not of run_time's millions
    rec = solver.backend
    s = solver.state
    state_handles = np.array([getattr(s, k)._h for k in STATE_ARRAYS], np.int64)
    scalars = np.array([s.db, s.inv_dx, s.inv_dy])
    if steps is None:
        solver.run()
    else:
        for _ in range(steps):
            solver.step()
    fields = solver.fields()
    out = {"events": np.array(rec.events, np.int64), "state_handles": state_handles,
           "state_scalars": scalars.astype(solver.real), "grid": np.array([s.nx, s.ny], np.int64),
           "n_steps": np.array(solver.n), "mon_handles": np.array([m.acc._h for m in solver.monitors], np.int64)}  # fmt: skip
    # payloads: one byte buffer, with per-handle offset, shape and dtype
    offs, shapes, dtypes, chunks, off = [], [], [], [], 0
    for a in rec.payloads:
        b = np.ascontiguousarray(a).view(np.uint8).ravel()
        offs.append(off)
        shapes.append(list(a.shape) + [-1] * (3 - a.ndim))
        dtypes.append(a.dtype.str)
        chunks.append(b)
        off += b.size
    out["payload"] = np.concatenate(chunks)
    out["p_off"], out["p_shape"], out["p_dtype"] = np.array(offs, np.int64), np.array(shapes, np.int64), np.array(dtypes)
    # what Etalon's run ended with: every state array, every accumulator, the host fields
    for k in STATE_ARRAYS:
        out[f"out_{k}_sha"] = np.array(sha(getattr(s, k).view(np.ndarray)))
    for k, m in enumerate(solver.monitors):
        out[f"out_acc{k}_sha"] = np.array(sha(m.acc.view(np.ndarray)))
    for c, a in fields.items():
        out[f"out_host_{c}_sha"] = np.array(sha(a))
    path = HERE / f"trace_{name}_{precision}.npz"
    np.savez_compressed(path, **out)
    print(f"wrote {path.name}: {len(rec.events)} protocol calls, {len(rec.payloads)} uploads, "
          f"{solver.n} steps, {path.stat().st_size} bytes")


def augment_case(et, name, precision):
    """Add Etalon's monitor values to an existing fixture from the accumulators it holds
    (for the long config2 runs, which are not stepped again)."""
    from etalon.fdtd.solver import FDTDSolver

    path = HERE / f"{name}_{precision}.npz"
    with np.load(path, allow_pickle=False) as z:
        out = {k: z[k] for k in z.files}
    sim, _ = reference_sims(et, precision)[name]
    solver = FDTDSolver(sim)  # setup only: samplings and grid
    accs = [out[f"out_acc{k}"] for k in range(len(solver.monitors))]
    out.update(monitor_values(solver, accs))
    np.savez_compressed(path, **out)
    print(f"added monitor values to {path.name}")


def main():
    import os

    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("ETALON_SRC"),
                    help="Etalon's source tree (default: $ETALON_SRC)")
    ap.add_argument("--cases", default="kernels,config1,g4_full,small")
    ap.add_argument("--augment", default="", help="cases whose existing fixtures get monitor values only")
    ap.add_argument("--trace", default="", help="cases whose protocol calls are recorded (g4_full: 600 "
                    "steps then fields(); small: run() to its end)")
    ap.add_argument("--precisions", default="single,double")
    args = ap.parse_args()
    if not args.ref:
        ap.error("name Etalon's source tree with --ref or ETALON_SRC")
    et = import_etalon(args.ref)
    for precision in args.precisions.split(","):
        if args.augment:
            for name in args.augment.split(","):
                augment_case(et, name, precision)
            continue
        if args.trace:
            for name in args.trace.split(","):
                trace_case(et, name, precision, steps=600 if name == "g4_full" else None)
            continue
        for name in args.cases.split(","):
            if name == "kernels":
                kernel_cases(et, precision)
            else:
                run_case(et, name, precision)


if __name__ == "__main__":
    main()
