"""Replay of recorded protocol traces of Etalon's own FDTDSolver.

tests/golden/make_golden.py ``--trace`` runs Etalon's unchanged ``FDTDSolver``
(etalon/fdtd/solver.py:49-160) on a recording NumPy backend and stores every backend call it
makes — ``to_device`` (with the array), ``update_h_te``, ``update_e_te``,
``field[i, j] -= delta``, ``accumulate_dft`` (with the phasor-table row it passed),
``to_host``, ``synchronize`` — and the hashes of every array it ended with. ``replay`` makes
the same calls, with the same arrays, on another backend, so a backend can be driven exactly as
Etalon's solver drives it on machines where Etalon itself cannot be imported.
"""

from __future__ import annotations

from types import SimpleNamespace

import numpy as np

from tests.golden_io import COEFFS, FIELDS, GOLDEN, load, sha

OP_TO_DEVICE, OP_UPDATE_H, OP_UPDATE_E, OP_ISUB, OP_ACCUMULATE, OP_TO_HOST, OP_SYNC = range(7)
STATE_ARRAYS = FIELDS + COEFFS


def available(name: str, precision: str) -> bool:
    return (GOLDEN / f"trace_{name}_{precision}.npz").exists()


def payload(t: dict, h: int) -> np.ndarray:
    dtype = np.dtype(str(t["p_dtype"][h]))
    shape = tuple(int(d) for d in t["p_shape"][h] if d >= 0)
    n = int(np.prod(shape, dtype=np.int64)) * dtype.itemsize
    off = int(t["p_off"][h])
    return t["payload"][off:off + n].view(dtype).reshape(shape).copy()


class Replay:
    """The arrays a backend holds after replaying a trace, by the handle the trace gave them."""

    def __init__(self, backend, t: dict):
        self.backend, self.t, self.dev, self.host = backend, t, {}, {}
        self.state = None
        self.calls = {op: 0 for op in range(7)}

    def _state(self):
        if self.state is None:
            t = self.t
            nx, ny = (int(v) for v in t["grid"])
            db, inv_dx, inv_dy = t["state_scalars"]
            s = SimpleNamespace(nx=nx, ny=ny, db=db, inv_dx=inv_dx, inv_dy=inv_dy)
            for name, h in zip(STATE_ARRAYS, t["state_handles"]):
                setattr(s, name, self.dev[int(h)])
            self.state = s
        return self.state

    def run(self) -> "Replay":
        b, dev = self.backend, self.dev
        for op, a, c, d, e, f in self.t["events"]:
            self.calls[int(op)] += 1
            if op == OP_TO_DEVICE:
                dev[int(a)] = b.to_device(payload(self.t, int(a)))
            elif op == OP_UPDATE_H:
                b.update_h_te(self._state())
            elif op == OP_UPDATE_E:
                b.update_e_te(self._state())
            elif op == OP_ISUB:
                field = dev[int(a)]
                field[dev[int(c)], dev[int(d)]] -= dev[int(e)]
            elif op == OP_ACCUMULATE:
                phasors = dev[int(e)][int(f)] if f >= 0 else dev[int(e)]
                b.accumulate_dft(dev[int(a)], dev[int(c)], dev[int(d)], phasors)
            elif op == OP_TO_HOST:
                self.host.setdefault(int(a), []).append(b.to_host(dev[int(a)]))
            elif op == OP_SYNC:
                b.synchronize()
            else:
                raise ValueError(f"unknown opcode {op}")
        return self

    def mismatches(self) -> list[str]:
        """Arrays whose bits differ from what Etalon's run ended with (empty: identical)."""
        t, bad = self.t, []
        for name, h in zip(STATE_ARRAYS, t["state_handles"]):
            if sha(self.backend.to_host(self.dev[int(h)])) != str(t[f"out_{name}_sha"]):
                bad.append(name)
        for k, h in enumerate(t["mon_handles"]):
            if sha(self.backend.to_host(self.dev[int(h)])) != str(t[f"out_acc{k}_sha"]):
                bad.append(f"acc{k}")
        fields = dict(zip(("Ex", "Ey", "Hz"), (int(t["state_handles"][k]) for k in range(3))))
        for comp, h in fields.items():
            got = self.host.get(h)
            if not got or sha(got[-1]) != str(t[f"out_host_{comp}_sha"]):
                bad.append(f"host {comp}")
        return bad


def load_trace(name: str, precision: str) -> dict:
    return load(f"trace_{name}", precision)


class NumpyReplayBackend:
    """The oracle's NumPy updates (oracle/te_numpy.py) as a protocol backend, to check the
    traces and the replay on a CPU."""

    name, device, xp = "numpy", "cpu", np

    def to_device(self, a):
        return np.array(a, copy=True)

    def to_host(self, a):
        return np.array(a, copy=True)

    def synchronize(self):
        pass

    def update_h_te(self, s):
        from oracle.te_numpy import update_h

        update_h(s)

    def update_e_te(self, s):
        from oracle.te_numpy import update_e

        update_e(s)

    def accumulate_dft(self, acc, field, index, phasors):
        from oracle.te_numpy import accumulate_dft

        accumulate_dft(acc, field, index, phasors)
