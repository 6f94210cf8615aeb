"""Etalon's per-step backend protocol on the GB300 kernels.

``Gb300Backend`` has the methods and attributes of Etalon's backends
(etalon/fdtd/backends/__init__.py:1-53, cupy_backend.py:30-98): ``to_device``,
``to_host``, ``synchronize``, ``update_h_te``, ``update_e_te``, ``accumulate_dft``,
``name``, ``device`` and ``xp``. Etalon's unchanged ``FDTDSolver`` steps on it, one
C-ABI call per method. Device arrays are ``DeviceArray``: HBM buffers owned through
the C-ABI allocator (no CuPy, no PyTorch), supporting exactly what the solver does to
them — row views of phasor tables and ``field[i, j] -= delta`` for injection
(etalon/fdtd/solver.py:83-110) — and what Etalon Studio's live view does
(etalon/studio/runner.py:258-291): ``astype``, ``v * v / c`` and ``xp.sum`` for the field
energy, ``field[:a, :b].reshape(mx, sx, my, sy).mean(axis=(1, 3))`` for the snapshot. Those
build deferred expressions that run as one fused device reduction when summed or averaged.
"""

from __future__ import annotations

import ctypes as C
import threading
from collections import defaultdict
from typing import Any

import numpy as np

from . import _lib
from ._lib import call


class _Pool:
    """Caches freed device buffers by size, so per-step temporaries do not cudaMalloc."""

    def __init__(self) -> None:
        self.free: dict[int, list[int]] = defaultdict(list)
        self.lock = threading.Lock()

    def get(self, nbytes: int) -> int:
        key = max(256, (nbytes + 255) // 256 * 256)
        with self.lock:
            if self.free[key]:
                return self.free[key].pop()
        p = C.c_void_p()
        call("etg_malloc", C.byref(p), key)
        return p.value

    def put(self, nbytes: int, ptr: int) -> None:
        key = max(256, (nbytes + 255) // 256 * 256)
        with self.lock:
            self.free[key].append(ptr)

    def release(self) -> None:
        with self.lock:
            for ptrs in self.free.values():
                for p in ptrs:
                    _lib.lib().etg_free(p)
            self.free.clear()


POOL = _Pool()


class DeviceArray:
    """An array in device memory: C-contiguous, or (2D views of a resident simulation's arrays)
    rows of ``pitch`` elements, of which the first ``shape[1]`` belong to the array."""

    __array_priority__ = 1000

    def __init__(self, shape, dtype, ptr: int | None = None, base=None, pitch: int | None = None):
        self.shape = tuple(int(s) for s in shape)
        self.dtype = np.dtype(dtype)
        self.size = int(np.prod(self.shape, dtype=np.int64))
        self.nbytes = self.size * self.dtype.itemsize
        self.base = base
        self.pitch = self.shape[-1] if pitch is None or len(self.shape) != 2 else int(pitch)
        if self.pitch != self.shape[-1] and (ptr is None or self.pitch < self.shape[-1]):
            raise ValueError("a pitched device array is a view of memory it does not own")
        self._owner = ptr is None
        self.ptr = POOL.get(self.nbytes) if ptr is None else int(ptr)

    @property
    def contiguous(self) -> bool:
        return self.pitch == self.shape[-1] or len(self.shape) != 2

    @property
    def span(self) -> int:
        """Elements from the first to one past the last of the array (rows × pitch when pitched)."""
        return self.shape[0] * self.pitch if not self.contiguous else self.size

    @property
    def ndim(self) -> int:
        return len(self.shape)

    @classmethod
    def from_host(cls, a: np.ndarray) -> "DeviceArray":
        a = np.ascontiguousarray(a)
        out = cls(a.shape, a.dtype)
        call("etg_memcpy_h2d", out.ptr, a.ctypes.data, a.nbytes)
        return out

    def get(self) -> np.ndarray:
        if not self.contiguous:
            rows = np.empty((self.shape[0], self.pitch), self.dtype)
            call("etg_memcpy_d2h", rows.ctypes.data, self.ptr, rows.nbytes)
            return np.ascontiguousarray(rows[:, : self.shape[1]])
        out = np.empty(self.shape, self.dtype)
        call("etg_memcpy_d2h", out.ctypes.data, self.ptr, self.nbytes)
        return out

    def __array__(self, dtype=None, copy=None):
        a = self.get()
        return a if dtype is None else a.astype(dtype)

    def copy(self) -> "DeviceArray":
        if not self.contiguous:
            return DeviceArray.from_host(self.get())
        out = DeviceArray(self.shape, self.dtype)
        call("etg_memcpy_d2d", out.ptr, self.ptr, self.nbytes)
        return out

    def __len__(self) -> int:
        return self.shape[0]

    def astype(self, dtype, copy=True) -> "_Cast":
        """Deferred conversion (evaluated by the expression that uses it)."""
        return _Cast(self, np.dtype(dtype))

    def __getitem__(self, key):
        if isinstance(key, tuple) and len(key) == 2 and all(isinstance(k, slice) for k in key) and self.ndim == 2:
            return _Window(self, key)
        if isinstance(key, (int, np.integer)) and self.ndim >= 1:
            k = int(key) + (self.shape[0] if key < 0 else 0)
            if not 0 <= k < self.shape[0]:
                raise IndexError(f"index {key} out of range for axis 0 of size {self.shape[0]}")
            row = self.nbytes // self.shape[0] if self.contiguous else self.pitch * self.dtype.itemsize
            return DeviceArray(self.shape[1:], self.dtype, self.ptr + k * row, base=self)
        if isinstance(key, tuple) and len(key) == 2 and all(isinstance(k, DeviceArray) for k in key):
            if not self.contiguous:
                raise TypeError("field[i, j] -= delta needs a contiguous device array")
            return _Indexed(self, key[0], key[1])
        raise TypeError(f"DeviceArray supports a row index or two index arrays, not {key!r}")

    def __setitem__(self, key, value) -> None:
        if isinstance(value, _Indexed) and value.target is self and value.applied:
            return  # the in-place update already ran (field[i, j] -= delta)
        raise TypeError("DeviceArray only supports in-place updates through field[i, j] -= delta")

    def __repr__(self) -> str:
        return f"DeviceArray(shape={self.shape}, dtype={self.dtype})"

    def __del__(self) -> None:
        if self._owner and self.ptr:
            try:
                POOL.put(self.nbytes, self.ptr)
            except Exception:
                pass
            self.ptr = 0


class _Indexed:
    """``field[i, j]`` of a DeviceArray, for ``field[i, j] -= delta`` (solver.py:89)."""

    def __init__(self, target: DeviceArray, i: DeviceArray, j: DeviceArray):
        if target.ndim != 2 or i.shape != j.shape:
            raise ValueError("field[i, j] needs a 2D field and index arrays of one shape")
        self.target, self.i, self.j = target, i, j
        self.applied = False

    def __isub__(self, delta: DeviceArray) -> "_Indexed":
        t = self.target
        if not isinstance(delta, DeviceArray) or delta.dtype != t.dtype or delta.size != self.i.size:
            raise TypeError("field[i, j] -= delta needs a device delta of the field's dtype and size")
        if self.i.dtype != np.int64 or self.j.dtype != np.int64:
            raise TypeError("injection indices must be int64")
        call("etg_scatter_sub", _lib.dtype_code(t.dtype), t.shape[1], self.i.size, t.ptr,
             self.i.ptr, self.j.ptr, delta.ptr)  # fmt: skip
        self.applied = True
        return self


class _Cast:
    """``a.astype(dtype)``: squared, divided and summed without a converted copy; evaluated
    on the device (etg_cast) when anything else needs it."""

    def __init__(self, src: DeviceArray, dtype: np.dtype):
        self.src, self.dtype, self.shape = src, dtype, src.shape

    def __mul__(self, other):
        if isinstance(other, _Cast) and other.src is self.src:
            return _Square(self.src, self.dtype)
        raise TypeError("device arrays support v * v of one converted field")

    def value(self) -> DeviceArray:
        src = self.src
        if not src.contiguous:  # cast the pitched rows whole, then read the array's columns
            out = DeviceArray((src.shape[0] * src.pitch,), self.dtype)
            call("etg_cast", _lib.dtype_code(src.dtype), _lib.dtype_code(self.dtype), src.span, src.ptr, out.ptr)
            return DeviceArray(src.shape, self.dtype, out.ptr, base=out, pitch=src.pitch)
        out = DeviceArray(src.shape, self.dtype)
        call("etg_cast", _lib.dtype_code(src.dtype), _lib.dtype_code(self.dtype), src.size, src.ptr, out.ptr)
        return out

    def astype(self, dtype, copy=True) -> "_Cast":
        return _Cast(self.src, np.dtype(dtype))

    def get(self) -> np.ndarray:
        return self.value().get()

    def __array__(self, dtype=None, copy=None):
        a = self.get()
        return a if dtype is None else a.astype(dtype)


class _Square:
    """``v * v`` of a converted field, optionally ``/ c``; summed by ``xp.sum`` in float64."""

    def __init__(self, src: DeviceArray, dtype: np.dtype, coeff: DeviceArray | None = None):
        self.src, self.dtype, self.coeff = src, dtype, coeff

    def __truediv__(self, c):
        if (self.coeff is None and isinstance(c, DeviceArray) and c.shape == self.src.shape
                and c.dtype == self.src.dtype and c.pitch == self.src.pitch):  # fmt: skip
            return _Square(self.src, self.dtype, c)
        raise TypeError("device arrays support (v * v) / c with c a device array of the field's shape and dtype")

    def sum(self) -> np.float64:
        out = C.c_double()
        src = self.src
        rows, cols = (src.shape[0], int(np.prod(src.shape[1:]))) if src.ndim > 1 else (1, src.size)
        pitch = cols if src.contiguous else src.pitch
        call("etg_sum_sq", _lib.dtype_code(src.dtype), rows, cols, pitch, src.ptr,
             None if self.coeff is None else self.coeff.ptr, C.byref(out))  # fmt: skip
        return np.float64(out.value)


class _Window:
    """``field[:a, :b]`` of a 2D device array (a leading block of rows and columns)."""

    def __init__(self, src: DeviceArray, key: tuple[slice, slice]):
        bounds = []
        for sl, n in zip(key, src.shape):
            start, stop, step = sl.indices(n)
            if start != 0 or step != 1:
                raise TypeError("device arrays support leading windows field[:a, :b] only")
            bounds.append(stop)
        self.src, self.rows, self.cols = src, bounds[0], bounds[1]

    def reshape(self, *shape):
        shape = shape[0] if len(shape) == 1 and isinstance(shape[0], tuple) else shape
        if len(shape) != 4 or shape[0] * shape[1] != self.rows or shape[2] * shape[3] != self.cols:
            raise TypeError("device windows reshape to (mx, sx, my, sy) blocks only")
        return _Blocks(self, *(int(v) for v in shape))


class _Blocks:
    """``window.reshape(mx, sx, my, sy)``, for ``.mean(axis=(1, 3))``: block means."""

    def __init__(self, window: _Window, mx: int, sx: int, my: int, sy: int):
        self.window, self.mx, self.sx, self.my, self.sy = window, mx, sx, my, sy

    def mean(self, axis=None) -> DeviceArray:
        if tuple(axis or ()) != (1, 3):
            raise TypeError("device blocks support mean(axis=(1, 3)) only")
        src = self.window.src
        out = DeviceArray((self.mx, self.my), src.dtype)
        code = _lib.dtype_code(src.dtype)
        call("etg_block_mean", code, self.window.rows, self.window.cols, src.pitch, src.ptr, self.sx, self.sy,
             code, out.ptr)  # fmt: skip
        return out


class _ArrayModule:
    """The ``xp`` of this backend: array creation, host conversion, and the sums of the live view."""

    float32, float64, complex64, complex128 = np.float32, np.float64, np.complex64, np.complex128

    @staticmethod
    def sum(a) -> np.float64:
        if isinstance(a, _Square):
            return a.sum()
        raise TypeError(f"xp.sum of {type(a).__name__} is not supported on device arrays")

    @staticmethod
    def asarray(a, dtype=None) -> DeviceArray:
        if isinstance(a, DeviceArray) and (dtype is None or np.dtype(dtype) == a.dtype):
            return a
        return DeviceArray.from_host(np.asarray(a, dtype=dtype))

    @staticmethod
    def zeros(shape, dtype=np.float64) -> DeviceArray:
        out = DeviceArray(np.atleast_1d(shape) if np.isscalar(shape) else shape, dtype)
        call("etg_memset", out.ptr, 0, out.nbytes)
        return out

    @staticmethod
    def asnumpy(a) -> np.ndarray:
        return a.get() if isinstance(a, (DeviceArray, _Cast)) else np.asarray(a)


xp = _ArrayModule()


class Gb300Backend:
    """One GB300 GPU through libetalon_gb300; a drop-in for Etalon's "cuda" backend."""

    name = "cuda"
    xp = xp

    def __init__(self, precision: str = "single") -> None:
        if precision not in ("single", "double"):
            raise ValueError(f"precision must be 'single' or 'double', not {precision!r}")
        try:
            dev, gpu, _ = _lib.device_info()
        except _lib.BackendUnavailable as error:
            raise RuntimeError(f"backend='cuda' (GB300) is unavailable: {error}") from error
        except _lib.EtgError as error:
            raise RuntimeError(f"backend='cuda' found no usable CUDA device ({error})") from error
        self.precision = precision
        self.device = f"cuda:{dev} {gpu}"

    def to_device(self, a: np.ndarray) -> DeviceArray:
        return DeviceArray.from_host(np.asarray(a))

    def to_host(self, a: Any) -> np.ndarray:
        return a.get() if isinstance(a, (DeviceArray, _Cast)) else np.asarray(a)

    def synchronize(self) -> None:
        call("etg_synchronize")

    @staticmethod
    def _p(a: DeviceArray) -> int:
        if not isinstance(a, DeviceArray):
            raise TypeError(f"expected a device array, got {type(a).__name__}")
        return a.ptr

    def update_h_te(self, s) -> None:
        """Hz^(n−½) → Hz^(n+½) (etalon/fdtd/backends/numpy_backend.py:41-49)."""
        p = self._p
        call("etg_update_h_te", _lib.dtype_code(s.hz.dtype), s.nx, s.ny, p(s.hz), p(s.ex), p(s.ey),
             p(s.psi_hz_x), p(s.psi_hz_y), p(s.bx_h), p(s.cx_h), p(s.ikx_h), p(s.by_h), p(s.cy_h),
             p(s.iky_h), float(s.db), float(s.inv_dx), float(s.inv_dy))  # fmt: skip

    def update_e_te(self, s) -> None:
        """Ex^n, Ey^n → n+1 (etalon/fdtd/backends/numpy_backend.py:51-61)."""
        p = self._p
        call("etg_update_e_te", _lib.dtype_code(s.ex.dtype), s.nx, s.ny, p(s.ex), p(s.ey), p(s.hz),
             p(s.psi_ex_y), p(s.psi_ey_x), p(s.cb_ex), p(s.cb_ey), p(s.bx_e), p(s.cx_e), p(s.ikx_e),
             p(s.by_e), p(s.cy_e), p(s.iky_e), float(s.inv_dx), float(s.inv_dy))  # fmt: skip

    def accumulate_dft(self, acc, field, index, phasors) -> None:
        """acc[f, k] += field.flat[index[k]] · phasors[f] (numpy_backend.py:63-67)."""
        n_f, n_nodes = acc.shape
        if index.dtype != np.int64:
            raise TypeError("DFT node indices must be int64")
        call("etg_accumulate_dft", _lib.dtype_code(field.dtype), n_f, n_nodes, self._p(acc),
             self._p(field), self._p(index), self._p(phasors))  # fmt: skip
