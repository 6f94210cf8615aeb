"""Many simulations stepped together (no counterpart in Etalon, which runs one FDTDSolver each).

``Batch(problems)`` builds one resident engine per problem (any grid sizes, one precision)
and a C-side batch over them: ``advance(k)`` moves every simulation k steps with one launch
pair per K steps for all of them, captured in CUDA graphs. Each engine keeps its own fields,
tables and monitors, and reads back exactly as if it had run alone.
"""

from __future__ import annotations

import ctypes as C

from . import _lib
from ._lib import call
from .engine import TEEngine
from .physics import TEProblem


class Batch:
    def __init__(self, problems: list[TEProblem], **engine_options) -> None:
        if not problems:
            raise ValueError("a batch needs at least one problem")
        if len({p.precision for p in problems}) != 1:
            raise ValueError("all problems of a batch must share one precision")
        self.engines = [TEEngine(p, **engine_options) for p in problems]
        handles = (C.c_void_p * len(self.engines))(*[e._h.value for e in self.engines])
        h = C.c_void_p()
        call("etg_batch_create", C.byref(h), len(self.engines), handles)
        self._h = h
        self._handles = handles

    @property
    def n_cells(self) -> int:
        return sum(e.nx * e.ny for e in self.engines)

    def set_option(self, option: int, value: int) -> None:
        call("etg_batch_set_option", self._h, option, int(value))

    def advance(self, k: int) -> None:
        for e in self.engines:
            e._ensure_tables(e.n, k)
        call("etg_batch_advance", self._h, k)

    def synchronize(self) -> None:
        call("etg_batch_synchronize", self._h)

    def reset(self) -> None:
        for e in self.engines:
            e.reset()

    def last_timing(self) -> tuple[float, int]:
        ms, launches = C.c_double(), C.c_int64()
        call("etg_batch_last_timing", self._h, C.byref(ms), C.byref(launches))
        return ms.value, launches.value

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.lib().etg_batch_destroy(self._h)
            self._h = C.c_void_p()
        for e in self.engines:
            e.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
