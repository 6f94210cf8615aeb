"""Batched stepping: every simulation of a batch ends bit-identical to its own run (needs a GPU)."""

import numpy as np
import pytest

from etalon_gb300 import _lib
from etalon_gb300.batch import Batch
from etalon_gb300.engine import TEEngine
from tests import cases
from tests.golden_io import FIELDS, compare_outputs, count, load

pytestmark = pytest.mark.gpu


def _problems(precision):
    return [cases.config1(precision, n_steps=600), cases.g4_full(precision, n_steps=600),
            cases.config2(precision, n_steps=600, region=173), cases.small(precision, n_steps=600)]  # fmt: skip


@pytest.mark.parametrize("precision", ["single", "double"])
@pytest.mark.parametrize("steps", [(600,), (1, 7, 8, 9, 63, 64, 65, 383)])
@pytest.mark.parametrize("deep", [False, True])
def test_batch_equals_individual_runs(gpu, precision, steps, deep):
    """Deep: K = 8 (float32) or 4 (float64) steps per launch instead of the default 4 or 2."""
    problems = _problems(precision)
    batch = Batch(problems)
    if deep:
        batch.set_option(_lib.OPT_TB_DEPTH, 8 if precision == "single" else 4)
        batch.set_option(_lib.OPT_TILE_ROWS, 40 if precision == "single" else 32)
    for k in steps:
        batch.advance(k)
    batch.synchronize()
    n = sum(steps)
    for p, e in zip(problems, batch.engines):
        ref = TEEngine(p, kernel="plain")
        ref.advance(n)
        for f in FIELDS:
            np.testing.assert_array_equal(e.field(f), ref.field(f), err_msg=f)
        for k in range(len(e.monitors)):
            np.testing.assert_array_equal(e.dft(k), ref.dft(k))
        assert e.n == n
    batch.close()


@pytest.mark.parametrize("precision", ["single", "double"])
def test_batch_member_matches_reference_fixture(gpu, precision):
    """The G4 member of a batch reproduces Etalon's own 600-step run bit for bit."""
    from tests.test_gpu_parity import golden_coeffs

    g = load("g4_full", precision)
    problems = _problems(precision)
    batch = Batch(problems)
    e = batch.engines[1]
    e.set_coefficients(golden_coeffs(g))
    for k in range(count(g, "src")):
        e.set_source_table(k, 0, g[f"src{k}_table"])
    for k in range(count(g, "mon")):
        e.set_phasor_table(k, 0, g[f"mon{k}_table"])
    batch.advance(600)
    batch.synchronize()
    assert compare_outputs(g, {f: e.field(f) for f in FIELDS}, [e.dft(k) for k in range(len(e.monitors))]) == []
    batch.close()


def test_batch_fault_injection_is_reported(gpu, monkeypatch):
    batch = Batch(_problems("single")[:2])
    monkeypatch.setenv("ETG_FAULT", "etg_batch_advance")
    with pytest.raises(_lib.EtgError, match="fault injected"):
        batch.advance(8)
    batch.close()


@pytest.mark.parametrize("precision", ["single", "double"])
def test_batch_of_synthetic_devices_vs_live_oracle(gpu, precision):
    """Uneven seeded devices (bend / ring / MMI) stepped as one batch vs the NumPy oracle."""
    from tests.test_gpu_parity import _oracle_for

    n = 2 * 8 * 3 + 5  # graph-captured pairs plus a one-step remainder
    problems = [cases.synthetic_device(s, precision, n_steps=n, min_cells=40, max_cells=300) for s in range(5)]
    batch = Batch(problems)
    batch.set_option(_lib.OPT_GRAPH_STEPS, 16)
    batch.advance(n)
    batch.synchronize()
    for p, e in zip(problems, batch.engines):
        o = _oracle_for(p)
        o.run(n)
        for f in FIELDS:
            np.testing.assert_array_equal(e.field(f), getattr(o, f), err_msg=f)
        for k, acc in enumerate(o.acc):
            np.testing.assert_array_equal(e.dft(k), acc)
    batch.close()


def test_config3_full_batch_equals_single_runs(gpu):
    """The 64-device, 5000-step batch of the batched throughput line, at full size: every
    device's fields, ψ and accumulators equal its own run bit for bit (the oracle cannot run
    this size; the single runs are pinned to it by the parity tests)."""
    from etalon_gb300 import autotune

    problems = cases.synthetic_batch(64, n_steps=5000)
    batch = Batch(problems)
    try:
        autotune.tune_batch(batch, steps=32, reps=1)
        batch.advance(5000)
        batch.synchronize()
        for p, eb in zip(problems, batch.engines):
            e = TEEngine(p)
            e.advance(5000)
            for f in FIELDS:
                a, b = eb.field(f), e.field(f)
                assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), f
            for k in range(len(e.monitors)):
                assert np.array_equal(eb.dft(k).view(np.uint8), e.dft(k).view(np.uint8))
            e.close()
    finally:
        batch.close()


def test_config3_every_device_vs_live_oracle(gpu):
    """All 64 devices of the batched workload (bends, rings, MMIs, 256²–1536²), 120 steps as
    one batch, each bit-identical to the oracle run on the host's cores."""
    import os
    from concurrent.futures import ThreadPoolExecutor

    from tests.test_gpu_parity import _oracle_for

    n = 120
    problems = cases.synthetic_batch(64, n_steps=n)
    batch = Batch(problems)
    try:
        batch.advance(n)
        batch.synchronize()
        workers = min(16, os.cpu_count() or 1)
        with ThreadPoolExecutor(workers) as pool:
            for p, e in zip(problems, batch.engines):
                o = _oracle_for(p)
                o.run(n, pool=pool, bands=workers)
                for f in FIELDS:
                    assert np.array_equal(e.field(f).view(np.uint8), getattr(o, f).view(np.uint8)), f
                for k, acc in enumerate(o.acc):
                    assert np.array_equal(e.dft(k).view(np.uint8), acc.view(np.uint8))
    finally:
        batch.close()


def test_config3_devices_full_length_vs_live_oracle(gpu):
    """Three devices of the batched workload — the smallest, one of middle size and the largest
    — at the full 5000 steps inside the 64-device batch (the batch tuner's shape), each
    bit-identical to the oracle run on the host's cores for all 5000 steps."""
    import os
    from concurrent.futures import ThreadPoolExecutor

    from etalon_gb300 import autotune
    from tests.test_gpu_parity import _oracle_for

    n = 5000
    problems = cases.synthetic_batch(64, n_steps=n)
    sizes = [p.grid.n_cells for p in problems]
    order = sorted(range(len(problems)), key=sizes.__getitem__)
    picked = [order[0], order[len(order) // 2], order[-1]]
    batch = Batch(problems)
    try:
        autotune.tune_batch(batch, steps=32, reps=1)
        batch.advance(n)
        batch.synchronize()
        workers = min(16, os.cpu_count() or 1)
        with ThreadPoolExecutor(workers) as pool:
            for q in picked:
                p, e = problems[q], batch.engines[q]
                o = _oracle_for(p)
                o.run(n, pool=pool, bands=workers)
                for f in FIELDS:
                    assert np.array_equal(e.field(f).view(np.uint8), getattr(o, f).view(np.uint8)), (q, f)
                for k, acc in enumerate(o.acc):
                    assert np.array_equal(e.dft(k).view(np.uint8), acc.view(np.uint8)), (q, k)
                assert np.abs(o.hz).max() > 0
    finally:
        batch.close()
