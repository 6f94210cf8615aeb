"""The no-allocation advance (etg_tb_advance_static) against the resident engine (needs a GPU).

etg_tb_advance_static serves callers that cannot allocate device memory when they step
fields — an application that owns all device memory through its own arena, a process
under a hard memory budget, a loop that cannot take cudaMalloc's device-wide
synchronisation. It keeps its scratch in a static device array. Here it must give the
same fields as the existing entry point (etg_sim_advance with the temporally blocked
kernel, bit for bit as every parity test here), on two calls in a row, so that the
scratch it keeps between calls cannot leak into a result.
"""

import ctypes as C

import numpy as np
import pytest

from etalon_gb300 import _lib
from etalon_gb300 import physics as ph
from etalon_gb300.engine import TEEngine
from tests import cases

pytestmark = pytest.mark.gpu

FIELDS = ("ex", "ey", "hz", "psi_ex_y", "psi_ey_x", "psi_hz_x", "psi_hz_y")
COEFFS = ("bx_e", "cx_e", "ikx_e", "bx_h", "cx_h", "ikx_h", "by_e", "cy_e", "iky_e", "by_h", "cy_h", "iky_h")


class Pitched:
    """Device arrays in the entry point's layout, allocated by the test (not by the entry point)."""

    def __init__(self, nx, ny, dtype):
        self.nx, self.ny, self.dtype = nx, ny, np.dtype(dtype)
        self.pitch = (ny + 1 + 31) // 32 * 32
        self.bytes = (nx + 2) * self.pitch * self.dtype.itemsize
        self.ptrs = []

    def alloc(self, host=None):
        p = C.c_void_p()
        _lib.call("etg_malloc", C.byref(p), self.bytes)
        self.ptrs.append(p.value)
        pad = np.zeros((self.nx + 2, self.pitch), self.dtype)
        if host is not None:
            pad[: host.shape[0], : host.shape[1]] = host
        _lib.call("etg_memcpy_h2d", p.value, pad.ctypes.data, self.bytes)
        return p.value

    def read(self, ptr, shape):
        pad = np.empty((self.nx + 2, self.pitch), self.dtype)
        _lib.call("etg_memcpy_d2h", pad.ctypes.data, ptr, self.bytes)
        return pad[: shape[0], : shape[1]].copy()

    def free(self):
        for p in self.ptrs:
            _lib.call("etg_free", p)


def _problem(precision):
    p = cases.config1(precision)  # 184 x 184 cells with a 12-layer CPML
    p.injections, p.samplings = [], []  # the entry point steps fields only
    return p


def _other_problem(precision):
    """A larger vacuum grid (300 x 260 cells, 12-layer CPML): its scratch planes cover every
    byte the 184² grid's planes use, at another pitch."""
    return ph.te_problem(size=(13.8, 11.8), dl=0.05, sources=[], pml=ph.PMLSpec(layers=12),
                         precision=precision)  # fmt: skip


class StaticRun:
    """One grid stepped twice: by the resident engine and by etg_tb_advance_static on
    device arrays the test allocates and owns."""

    SHAPES = lambda nx, ny: {"ex": (nx, ny + 1), "ey": (nx + 1, ny), "hz": (nx, ny),  # noqa: E731
                             "psi_ex_y": (nx, ny + 1), "psi_ey_x": (nx + 1, ny),
                             "psi_hz_x": (nx, ny), "psi_hz_y": (nx, ny)}  # fmt: skip

    def __init__(self, p, seed):
        self.p = p
        nx, ny, real = p.grid.nx, p.grid.ny, p.real
        shapes = StaticRun.SHAPES(nx, ny)
        rng = np.random.default_rng(seed)
        start = {f: np.zeros(shapes[f], real) for f in FIELDS}  # psi starts at +0
        for f in ("ex", "ey", "hz"):
            start[f][...] = rng.standard_normal(shapes[f])
        start["hz"] *= 1 / 377.0
        self.engine = TEEngine(p, kernel="tb")
        for f in ("ex", "ey", "hz"):
            self.engine.set_field(f, start[f])
        self.buf = Pitched(nx, ny, real)
        c = ph.cast_coefficients(p)
        self.c = c
        self.fields = {f: self.buf.alloc(start[f]) for f in FIELDS}
        self.cb_ex, self.cb_ey = self.buf.alloc(c.cb_ex), self.buf.alloc(c.cb_ey)
        self.coef = {}
        for k in COEFFS:
            a = np.ascontiguousarray(getattr(c, k))
            q = C.c_void_p()
            _lib.call("etg_malloc", C.byref(q), a.nbytes)
            _lib.call("etg_memcpy_h2d", q.value, a.ctypes.data, a.nbytes)
            self.coef[k] = q.value
            self.buf.ptrs.append(q.value)

    def step_and_check(self, steps):
        nx, ny, c = self.p.grid.nx, self.p.grid.ny, self.c
        self.engine.advance(steps)
        self.engine.synchronize()
        _lib.call("etg_tb_advance_static", _lib.dtype_code(self.p.real), nx, ny, self.buf.pitch,
                  *[self.fields[f] for f in FIELDS], self.cb_ex, self.cb_ey,
                  *[self.coef[k] for k in COEFFS], float(c.db), float(c.inv_dx), float(c.inv_dy),
                  steps)  # fmt: skip
        for f in FIELDS:
            want = self.engine.field(f)
            got = self.buf.read(self.fields[f], want.shape)
            # raw bits, so that the sign of a zero counts too
            assert np.array_equal(got.view(np.uint8), want.view(np.uint8)), (
                f"{f} differs from the engine after {steps} more steps ({nx} x {ny}, {self.p.precision})")
        assert np.abs(self.engine.field("hz")).max() > 0

    def close(self):
        self.buf.free()
        self.engine.close()


@pytest.mark.parametrize("precision", ["single", "double"])
def test_static_advance_matches_engine_on_two_calls(gpu, precision):
    """Two calls on the 184² grid, with a call on a larger grid of the other precision (live
    psi in its strips, another pitch) in between: whatever that call leaves in the shared
    scratch must not reach the second result."""
    main = StaticRun(_problem(precision), seed=7)
    other = StaticRun(_other_problem("double" if precision == "single" else "single"), seed=11)
    try:
        main.step_and_check(21)  # TB pairs plus a one-step remainder
        other.step_and_check(40)
        assert np.abs(other.engine.field("psi_hz_x")).max() > 0  # the strips hold live psi
        main.step_and_check(30)
        main.step_and_check(16)  # whole pairs only
    finally:
        main.close()
        other.close()


def test_static_advance_rejects_grids_beyond_its_scratch(gpu):
    """A 2024² float32 grid needs ~116 MB of scratch: refused before any device access."""
    q = C.c_void_p()
    _lib.call("etg_malloc", C.byref(q), 256)  # valid, aligned, never dereferenced
    try:
        with pytest.raises(ValueError, match="bytes of scratch"):
            _lib.call("etg_tb_advance_static", _lib.F32, 2024, 2024, 2048, *([q.value] * 21),
                      1.0, 1.0, 1.0, 10)  # fmt: skip
    finally:
        _lib.call("etg_free", q.value)
