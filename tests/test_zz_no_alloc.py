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


@pytest.mark.parametrize("precision", ["single", "double"])
def test_static_advance_matches_engine_on_two_calls(gpu, precision):
    p = _problem(precision)
    nx, ny, real = p.grid.nx, p.grid.ny, p.real
    rng = np.random.default_rng(7)
    shapes = {"ex": (nx, ny + 1), "ey": (nx + 1, ny), "hz": (nx, ny), "psi_ex_y": (nx, ny + 1),
              "psi_ey_x": (nx + 1, ny), "psi_hz_x": (nx, ny), "psi_hz_y": (nx, ny)}  # fmt: skip
    start = {f: np.zeros(shapes[f], real) for f in FIELDS}  # psi starts at +0
    for f in ("ex", "ey", "hz"):
        start[f][...] = rng.standard_normal(shapes[f])
    start["hz"] *= 1 / 377.0

    engine = TEEngine(p, kernel="tb")
    for f in ("ex", "ey", "hz"):
        engine.set_field(f, start[f])

    buf = Pitched(nx, ny, real)
    c = ph.cast_coefficients(p)
    fields = {f: buf.alloc(start[f]) for f in FIELDS}
    cb_ex, cb_ey = buf.alloc(c.cb_ex), buf.alloc(c.cb_ey)
    coef = {}
    for k in COEFFS:
        a = np.ascontiguousarray(getattr(c, k))
        q = C.c_void_p()
        _lib.call("etg_malloc", C.byref(q), a.nbytes)
        _lib.call("etg_memcpy_h2d", q.value, a.ctypes.data, a.nbytes)
        coef[k] = q.value
        buf.ptrs.append(q.value)
    code = _lib.dtype_code(real)
    try:
        for steps in (21, 30):  # two calls in a row: TB pairs plus a one-step remainder each
            engine.advance(steps)
            engine.synchronize()
            _lib.call("etg_tb_advance_static", code, nx, ny, buf.pitch,
                      *[fields[f] for f in FIELDS], cb_ex, cb_ey, *[coef[k] for k in COEFFS],
                      float(c.db), float(c.inv_dx), float(c.inv_dy), steps)  # fmt: skip
            for f in FIELDS:
                want = engine.field(f)
                got = buf.read(fields[f], want.shape)
                np.testing.assert_array_equal(got, want, err_msg=f"{f} after {steps} more steps")
            assert np.abs(engine.field("hz")).max() > 0
    finally:
        buf.free()
        engine.close()


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
