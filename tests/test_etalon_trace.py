"""Recorded protocol traces of Etalon's own FDTDSolver, checked on the CPU.

The traces (tests/golden/trace_*.npz, written by make_golden.py ``--trace`` from Etalon's
unchanged solver) replayed on the NumPy oracle must end with the arrays Etalon's run ended
with, bit for bit: this pins the traces and the replay itself. The GPU test
(test_gpu_etalon_trace.py) replays the same traces on Gb300Backend.
"""

import numpy as np
import pytest

from tests import etalon_trace as tr

CASES = [("g4_full", "single"), ("g4_full", "double"), ("small", "single"), ("small", "double")]


@pytest.mark.parametrize(("name", "precision"), CASES)
def test_trace_replayed_on_the_oracle_ends_as_etalon_did(name, precision):
    if not tr.available(name, precision):
        pytest.skip("no trace fixture")
    t = tr.load_trace(name, precision)
    r = tr.Replay(tr.NumpyReplayBackend(), t).run()
    assert r.mismatches() == []
    n = int(t["n_steps"])
    assert r.calls[tr.OP_UPDATE_H] == r.calls[tr.OP_UPDATE_E] == n
    assert r.calls[tr.OP_ISUB] > 0 and r.calls[tr.OP_ACCUMULATE] > 0


def test_short_run_uploads_tables_of_its_own_length():
    """Etalon's G4b property, seen in the trace of ``run()`` on the short case: every phasor
    table the solver uploaded has exactly n_steps rows (fewer than a chunk)."""
    if not tr.available("small", "single"):
        pytest.skip("no trace fixture")
    t = tr.load_trace("small", "single")
    n = int(t["n_steps"])
    tables = {int(e[4]) for e in t["events"] if e[0] == tr.OP_ACCUMULATE and e[5] >= 0}
    assert tables
    for h in tables:
        a = tr.payload(t, h)
        assert a.shape[0] == n and np.iscomplexobj(a)
