"""ctypes binding of ``libetalon_gb300.so`` (declared in include/etalon_gb300.h).

The library is loaded once, from the package directory. There is no fallback: if the
library is missing or cannot be loaded, every entry point raises ``BackendUnavailable``.
"""

from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libetalon_gb300.so"

OK, ERR_ARGUMENT, ERR_CUDA, ERR_ALLOC, ERR_STATE, ERR_INJECTED, ERR_NONFINITE, ERR_TIMEOUT = range(8)
F32, F64 = 4, 8
EX, EY, HZ, PSI_EX_Y, PSI_EY_X, PSI_HZ_X, PSI_HZ_Y = range(7)
FIELD_IDS = {"ex": EX, "ey": EY, "hz": HZ, "psi_ex_y": PSI_EX_Y, "psi_ey_x": PSI_EY_X,
             "psi_hz_x": PSI_HZ_X, "psi_hz_y": PSI_HZ_Y}  # fmt: skip
COMPONENT_IDS = {"Ex": EX, "Ey": EY, "Hz": HZ}
OPT_KERNEL, OPT_TB_DEPTH, OPT_GRAPH_STEPS, OPT_TILE_ROWS, OPT_TILE_COLS, OPT_CHECK_FINITE, OPT_TIMING, OPT_TB_WARPS = range(8)
OPT_TB_SEGMENTS, OPT_TB_SEGMENTS_USED = 8, 9

vp, i32, i64, f64, sz = C.c_void_p, C.c_int, C.c_int64, C.c_double, C.c_size_t
pi64 = C.POINTER(C.c_int64)

# name -> argument types; every function returns int status
SIGNATURES: dict[str, list] = {
    "etg_version": [],
    "etg_device_info": [C.POINTER(i32), C.c_char_p, i32, C.POINTER(i32)],
    "etg_synchronize": [],
    "etg_set_device": [i32],
    "etg_host_alloc": [C.POINTER(vp), sz],
    "etg_host_free": [vp],
    "etg_malloc": [C.POINTER(vp), sz],
    "etg_free": [vp],
    "etg_memcpy_h2d": [vp, vp, sz],
    "etg_memcpy_d2h": [vp, vp, sz],
    "etg_memcpy_d2d": [vp, vp, sz],
    "etg_memset": [vp, i32, sz],
    "etg_update_h_te": [i32, i32, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, f64, f64, f64],
    "etg_update_e_te": [i32, i32, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, f64, f64],
    "etg_accumulate_dft": [i32, i32, i32, vp, vp, vp, vp],
    "etg_scatter_sub": [i32, i64, i32, vp, vp, vp, vp],
    "etg_sum_sq": [i32, i64, i64, i64, vp, vp, C.POINTER(f64)],
    "etg_block_mean": [i32, i64, i64, i64, vp, i32, i32, i32, vp],
    "etg_cast": [i32, i32, i64, vp, vp],
    "etg_sim_create": [C.POINTER(vp), i32, i32, i32],
    "etg_sim_destroy": [vp],
    "etg_sim_set_coefficients": [vp] + [vp] * 14 + [f64, f64, f64],
    "etg_sim_add_source": [vp, i32, i32, vp, vp, i64, i64, vp],
    "etg_sim_set_cb_window": [vp, i32, i32, i32, i32, i32, vp],
    "etg_sim_rasterize_cb": [vp, f64, f64, f64, f64, f64, f64, f64, i32, vp],
    "etg_sim_get_cb": [vp, i32, vp],
    "etg_sim_add_monitor": [vp, i32, i32, i32, i32, i32, i32, i64, i64, vp, C.POINTER(i32)],
    "etg_sim_set_phasors": [vp, i32, i64, i64, vp],
    "etg_sim_set_deltas": [vp, i32, i64, i64, vp],
    "etg_sim_set_field": [vp, i32, vp],
    "etg_sim_get_field": [vp, i32, vp],
    "etg_sim_get_dft": [vp, i32, vp],
    "etg_sim_set_dft": [vp, i32, vp],
    "etg_sim_reset": [vp],
    "etg_sim_advance": [vp, i64],
    "etg_sim_step_index": [vp, pi64],
    "etg_sim_set_step_index": [vp, i64],
    "etg_sim_synchronize": [vp],
    "etg_sim_set_option": [vp, i32, i64],
    "etg_sim_get_option": [vp, i32, pi64],
    "etg_sim_last_timing": [vp, C.POINTER(f64), pi64],
    "etg_sim_kernel_timing": [vp, C.POINTER(f64), pi64, pi64],
    "etg_batch_create": [C.POINTER(vp), i32, C.POINTER(vp)],
    "etg_batch_destroy": [vp],
    "etg_batch_advance": [vp, i64],
    "etg_batch_synchronize": [vp],
    "etg_batch_set_option": [vp, i32, i64],
    "etg_batch_last_timing": [vp, C.POINTER(f64), pi64],
    "etg_adj_create": [C.POINTER(vp), vp, i32, i32, i32, i32],
    "etg_adj_destroy": [vp],
    "etg_adj_forward": [vp, i64, i64],
    "etg_adj_backward": [vp, C.POINTER(vp), C.POINTER(C.c_double), C.POINTER(C.c_double)],
    "etg_adj_set_objective": [vp, C.POINTER(vp)],
    "etg_adj_gradient": [vp, C.POINTER(f64), C.POINTER(f64)],
    "etg_adj_batch_create": [C.POINTER(vp), i32, C.POINTER(vp)],
    "etg_adj_batch_destroy": [vp],
    "etg_adj_batch_set_option": [vp, i32, i64],
    "etg_adj_batch_forward": [vp, i64, i64],
    "etg_adj_batch_backward": [vp],
    "etg_tb_advance_static": [i32, i32, i32, i64] + [vp] * 21 + [f64, f64, f64, i64],
    "etg_yee3d_create": [C.POINTER(vp), i32, i32, i32, i32, i32],
    "etg_yee3d_destroy": [vp],
    "etg_yee3d_set_scalars": [vp, vp],
    "etg_yee3d_set_profile": [vp, i32, vp, vp, vp, vp, vp, vp],
    "etg_yee3d_set_field": [vp, i32, vp],
    "etg_yee3d_get_field": [vp, i32, vp],
    "etg_yee3d_add_source": [vp, i32, i32, vp, i64, i64, vp],
    "etg_yee3d_add_monitor": [vp, i32, i32, vp, i32, i64, i64, vp],
    "etg_yee3d_get_dft": [vp, i32, vp],
    "etg_yee3d_advance": [vp, i64],
    "etg_yee3d_synchronize": [vp],
    "etg_yee3d_step_index": [vp, pi64],
    "etg_yee3d_last_timing": [vp, C.POINTER(f64), pi64],
    "etg_yee3d_kernel_timing": [vp, i32, C.POINTER(f64), C.POINTER(f64)],
    "etg_yee3d_set_option": [vp, i32, i64],
    "etg_debug_set_wait_tries": [i64],
    "etg_sim_device_array": [vp, i32, vp, vp],
    "etg_sim_set_db_nodes": [vp, vp],
}


class BackendUnavailable(RuntimeError):
    """The CUDA library is missing, was built for another platform, or has no device."""


class EtgError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


class NonFiniteField(EtgError):
    """A field became NaN or Inf (Etalon Studio's NumericalInstability)."""


_lock = threading.Lock()
_lib: C.CDLL | None = None


def lib() -> C.CDLL:
    """The loaded library, with argument types set. Raises BackendUnavailable."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not LIB_PATH.exists():
            raise BackendUnavailable(
                f"{LIB_PATH.name} is not built; run `python -c \"import __graft_entry__ as g; g.build()\"` "
                "or `python -m etalon_gb300.build` (needs nvcc from CUDA 13)"
            )
        try:
            handle = C.CDLL(str(LIB_PATH))
        except OSError as error:
            raise BackendUnavailable(f"cannot load {LIB_PATH}: {error}") from error
        handle.etg_last_error.restype = C.c_char_p
        handle.etg_last_error.argtypes = []
        for name, args in SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = C.c_int
            fn.argtypes = args
        _lib = handle
        return handle


def last_error() -> str:
    return lib().etg_last_error().decode(errors="replace")


def check(rc: int, what: str = "") -> None:
    """Raise the exception matching a C status code."""
    if rc == OK:
        return
    msg = f"{what}: {last_error()}" if what else last_error()
    if rc == ERR_ARGUMENT:
        raise ValueError(msg)
    if rc == ERR_ALLOC:
        raise MemoryError(msg)
    if rc == ERR_NONFINITE:
        raise NonFiniteField(rc, msg)
    raise EtgError(rc, msg)


def call(name: str, *args) -> None:
    """Call ``name`` and raise on a non-zero status."""
    check(getattr(lib(), name)(*args), name)


def device_info() -> tuple[int, str, int]:
    dev, sms = C.c_int(), C.c_int()
    name = C.create_string_buffer(256)
    call("etg_device_info", C.byref(dev), name, 256, C.byref(sms))
    return dev.value, name.value.decode(), sms.value


def pinned_empty(shape, dtype):
    """A NumPy array in page-locked host memory, freed when the array is collected."""
    import weakref

    import numpy as np

    dt = np.dtype(dtype)
    nbytes = max(1, int(np.prod(shape, dtype=np.int64)) * dt.itemsize)
    p = C.c_void_p()
    call("etg_host_alloc", C.byref(p), nbytes)
    buf = (C.c_char * nbytes).from_address(p.value)
    arr = np.frombuffer(buf, dtype=dt, count=nbytes // dt.itemsize).reshape(shape)
    weakref.finalize(buf, lib().etg_host_free, p.value)
    return arr


def dtype_code(dtype) -> int:
    import numpy as np

    dt = np.dtype(dtype)
    if dt == np.float32 or dt == np.complex64:
        return F32
    if dt == np.float64 or dt == np.complex128:
        return F64
    raise ValueError(f"unsupported dtype {dt}; etalon_gb300 computes in float32 or float64")
