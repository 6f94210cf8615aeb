"""The reference's own CUDA kernels on this GPU, launched as Etalon's CuPy backend launches them.

TEST AND BENCH INFRASTRUCTURE ONLY: the bench times these kernels beside this package's, and a
GPU test checks them against it. The product never imports this module.

The images are built by oracle/build_ref.py from Etalon's unchanged ``update_te.cu`` and
``dft.cu`` (``REAL`` = float or double, ``--fmad=false``). They are loaded with the CUDA
driver API into the device's primary context, the one the CUDA runtime (and so this package's
library) uses, so device pointers are shared. Launch shapes follow
etalon/fdtd/backends/cupy_backend.py:18-27 and 70-98: 32 × 8 thread blocks with x along y
for the two updates, over (ny, nx) for H and (ny + 1, nx + 1) for E, and 128-thread blocks
over (nodes, frequencies) for the DFT. Everything runs on the legacy default stream, as CuPy's
default does.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

from oracle import build_ref

_cu = None


def _driver() -> C.CDLL:
    global _cu
    if _cu is None:
        cu = C.CDLL("libcuda.so.1")
        _check(cu, cu.cuInit(0), "cuInit")
        _cu = cu
    return _cu


def _check(cu, rc: int, what: str) -> None:
    if rc != 0:
        msg = C.c_char_p()
        cu.cuGetErrorString(rc, C.byref(msg))
        raise RuntimeError(f"{what} failed: {rc} {msg.value.decode() if msg.value else ''}")


def available(precision: str) -> bool:
    tag = "f32" if precision == "single" else "f64"
    return all(p.exists() or p.with_suffix(".ptx").exists() for p in build_ref.images(tag).values())


class RefKernels:
    """update_h_te, update_e_te and accumulate_dft of the reference for one precision."""

    BLOCK_2D = (32, 8, 1)
    BLOCK_DFT = 128

    def __init__(self, precision: str, device: int = 0):
        cu = _driver()
        self.cu = cu
        self.real = C.c_float if precision == "single" else C.c_double
        dev = C.c_int()
        _check(cu, cu.cuDeviceGet(C.byref(dev), device), "cuDeviceGet")
        ctx = C.c_void_p()
        _check(cu, cu.cuDevicePrimaryCtxRetain(C.byref(ctx), dev), "cuDevicePrimaryCtxRetain")
        _check(cu, cu.cuCtxSetCurrent(ctx), "cuCtxSetCurrent")
        self.ctx, self.dev = ctx, dev
        tag = "f32" if precision == "single" else "f64"
        self.modules = {}
        for name, path in build_ref.images(tag).items():
            data = self._image(Path(path))
            m = C.c_void_p()
            _check(cu, cu.cuModuleLoadData(C.byref(m), data), f"cuModuleLoadData({path.name})")
            self.modules[name] = m
        self.f_h = self._function("update_te", b"update_h_te")
        self.f_e = self._function("update_te", b"update_e_te")
        self.f_dft = self._function("dft", b"accumulate_dft")
        self.launches = 0

    @staticmethod
    def _image(path: Path):
        if path.exists():
            return C.create_string_buffer(path.read_bytes())
        ptx = path.with_suffix(".ptx")
        if not ptx.exists():
            raise FileNotFoundError(f"{path.name}: build the reference kernels first (oracle/build_ref.py)")
        return C.create_string_buffer(ptx.read_bytes() + b"\0")

    def _function(self, module: str, name: bytes) -> C.c_void_p:
        f = C.c_void_p()
        _check(self.cu, self.cu.cuModuleGetFunction(C.byref(f), self.modules[module], name), name.decode())
        return f

    def _launch(self, f, grid, block, args) -> None:
        params = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        _check(self.cu, self.cu.cuLaunchKernel(f, *grid, *block, 0, None, params, None), "cuLaunchKernel")
        self.launches += 1

    @classmethod
    def _blocks(cls, n_fast: int, n_slow: int):
        bx, by, _ = cls.BLOCK_2D
        return ((n_fast + bx - 1) // bx, (n_slow + by - 1) // by, 1)

    def update_h(self, s) -> None:
        """s: device pointers hz, ex, ey, psi_hz_x, psi_hz_y, bx_h … iky_h; db, inv_dx, inv_dy; nx, ny."""
        p = C.c_uint64
        r = self.real
        args = [p(s.hz), p(s.ex), p(s.ey), p(s.psi_hz_x), p(s.psi_hz_y), p(s.bx_h), p(s.cx_h), p(s.ikx_h),
                p(s.by_h), p(s.cy_h), p(s.iky_h), r(s.db), r(s.inv_dx), r(s.inv_dy), C.c_int32(s.nx),
                C.c_int32(s.ny)]  # fmt: skip
        self._launch(self.f_h, self._blocks(s.ny, s.nx), self.BLOCK_2D, args)

    def update_e(self, s) -> None:
        p = C.c_uint64
        r = self.real
        args = [p(s.ex), p(s.ey), p(s.hz), p(s.psi_ex_y), p(s.psi_ey_x), p(s.cb_ex), p(s.cb_ey), p(s.bx_e),
                p(s.cx_e), p(s.ikx_e), p(s.by_e), p(s.cy_e), p(s.iky_e), r(s.inv_dx), r(s.inv_dy),
                C.c_int32(s.nx), C.c_int32(s.ny)]  # fmt: skip
        self._launch(self.f_e, self._blocks(s.ny + 1, s.nx + 1), self.BLOCK_2D, args)

    def accumulate(self, acc: int, field: int, index: int, phasor: int, n_f: int, n_nodes: int) -> None:
        p = C.c_uint64
        args = [p(acc), p(field), p(index), p(phasor), C.c_int32(n_f), C.c_int32(n_nodes)]
        grid = ((n_nodes + self.BLOCK_DFT - 1) // self.BLOCK_DFT, n_f, 1)
        self._launch(self.f_dft, grid, (self.BLOCK_DFT, 1, 1), args)

    # events on the legacy default stream, for timing
    def event(self) -> C.c_void_p:
        e = C.c_void_p()
        _check(self.cu, self.cu.cuEventCreate(C.byref(e), 0), "cuEventCreate")
        return e

    def record(self, e) -> None:
        _check(self.cu, self.cu.cuEventRecord(e, None), "cuEventRecord")

    def elapsed_ms(self, a, b) -> float:
        _check(self.cu, self.cu.cuEventSynchronize(b), "cuEventSynchronize")
        ms = C.c_float()
        _check(self.cu, self.cu.cuEventElapsedTime(C.byref(ms), a, b), "cuEventElapsedTime")
        return float(ms.value)

    def synchronize(self) -> None:
        _check(self.cu, self.cu.cuCtxSynchronize(), "cuCtxSynchronize")

    def close(self) -> None:
        for m in self.modules.values():
            self.cu.cuModuleUnload(m)
        self.modules = {}
        self.cu.cuDevicePrimaryCtxRelease(self.dev)
