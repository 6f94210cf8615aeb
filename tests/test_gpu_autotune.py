"""The autotuner on real engines (needs a GPU): every candidate runs or is skipped, and the
tuned engine or batch still gives the oracle's bits."""

import numpy as np
import pytest

from etalon_gb300 import autotune
from etalon_gb300.batch import Batch
from etalon_gb300.engine import TEEngine
from tests import cases
from tests.golden_io import FIELDS

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["single", "double"])
def test_tuned_engine_matches_oracle(gpu, precision, tmp_path, monkeypatch):
    from tests.test_gpu_parity import _oracle_for

    monkeypatch.setenv("ETALON_GB300_AUTOTUNE", str(tmp_path / "cache.json"))
    n = 120
    p = cases.synthetic_device(7, precision, n_steps=n, min_cells=300, max_cells=360)
    e = TEEngine(p)
    try:
        choice = autotune.tune(e, steps=32, reps=1, use_cache=False)
        assert tuple(choice) in autotune.CANDIDATES[precision]
        e.advance(n)
        o = _oracle_for(p)
        o.run(n)
        for f in FIELDS:
            np.testing.assert_array_equal(e.field(f), getattr(o, f), err_msg=f"{f} with {choice}")
        for k, acc in enumerate(o.acc):
            np.testing.assert_array_equal(e.dft(k), acc)
    finally:
        e.close()


def test_tuned_batch_matches_single_runs(gpu):
    n = 72
    problems = [cases.synthetic_device(s, "single", n_steps=n, min_cells=100, max_cells=260) for s in range(4)]
    batch = Batch(problems)
    try:
        choice = autotune.tune_batch(batch, steps=32, reps=1)
        assert tuple(choice) in autotune.BATCH_CANDIDATES["single"]
        batch.advance(n)
        batch.synchronize()
        for p, eb in zip(problems, batch.engines):
            e = TEEngine(p, kernel="plain")
            e.advance(n)
            for f in FIELDS:
                np.testing.assert_array_equal(eb.field(f), e.field(f), err_msg=f"{f} with {choice}")
            e.close()
    finally:
        batch.close()
