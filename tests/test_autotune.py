"""Autotuner selection and cache logic on a fake engine (no GPU): the fastest candidate wins,
candidates that fail to compile or run are skipped, the cache is reused, and a cached choice
from before warps per tile were tuned still applies (as 8 warps)."""

import json

import pytest

from etalon_gb300 import _lib, autotune


class FakeEngine:
    """Records options; 'times' a candidate by a fixed table keyed on (kernel, rows, depth, warps)."""

    def __init__(self, precision, times, fail=()):
        self.nx, self.ny = 2024, 2024
        self.problem = type("P", (), {"precision": precision})()
        self.times, self.fail = times, set(fail)
        self.opts, self.kernel, self.resets = {}, None, 0

    def set_kernel(self, kernel):
        self.kernel = kernel

    def set_option(self, option, value):
        self.opts[option] = value

    def reset(self):
        self.resets += 1

    def advance(self, steps):
        cand = (self.kernel, self.opts[_lib.OPT_TILE_ROWS], self.opts[_lib.OPT_TB_DEPTH], self.opts[_lib.OPT_TB_WARPS])
        if cand in self.fail:
            raise _lib.EtgError(1, "no compiled kernel")
        self.last = self.times.get(cand, 100.0)

    def last_timing(self):
        return self.last, 1


@pytest.fixture
def fake_device(monkeypatch, tmp_path):
    monkeypatch.setattr(_lib, "device_info", lambda: (0, "GB300", 152))
    monkeypatch.setattr(autotune, "_get", lambda engine, option: 0)
    monkeypatch.setenv("ETALON_GB300_AUTOTUNE", str(tmp_path / "cache.json"))
    return tmp_path / "cache.json"


def test_fastest_candidate_is_applied_and_cached(fake_device):
    e = FakeEngine("single", {("tb", 48, 4, 16): 5.0, ("tb", 48, 4, 8): 6.0}, fail={("pipe", 48, 4, 8)})
    choice = autotune.tune(e)
    assert choice == ("tb", 48, 4, 16)
    assert (e.kernel, e.opts[_lib.OPT_TILE_ROWS], e.opts[_lib.OPT_TB_WARPS]) == ("tb", 48, 16)
    table = json.loads(fake_device.read_text())
    entry = table["2024x2024:single:GB300:152"]
    assert entry["choice"] == ["tb", 48, 4, 16]
    assert "pipe/48/4/8" not in entry["ms"] and entry["ms"]["tb/48/4/16"] == 5.0
    e2 = FakeEngine("single", {})  # a cache hit times nothing
    assert autotune.tune(e2) == ("tb", 48, 4, 16) and e2.resets == 0


def test_cached_choice_without_warps_means_eight(fake_device):
    fake_device.write_text(json.dumps({"2024x2024:double:GB300:152": {"choice": ["tb", 40, 2], "ms": {}}}))
    e = FakeEngine("double", {})
    assert autotune.tune(e) == ("tb", 40, 2)
    assert e.opts[_lib.OPT_TB_WARPS] == 8 and e.opts[_lib.OPT_TILE_ROWS] == 40


def test_every_candidate_names_a_known_kernel():
    for precision, cands in autotune.CANDIDATES.items():
        for kernel, rows, depth, warps in cands:
            assert kernel in ("tb", "tma", "pipe", "plain") and warps in (8, 16)
            # the depths compiled: 4 and 8 steps per launch (float32), 2 and 4 (float64)
            assert kernel == "plain" or depth in ((4, 8) if precision == "single" else (2, 4))
            assert kernel != "tb" or depth == (4 if precision == "single" else 2) or rows in (40, 32)


class FakeBatch:
    """A batch of fake engines whose 'time' depends on (rows, depth, warps)."""

    def __init__(self, times, fail=()):
        self.engines = [FakeEngine("single", {})]
        self.times, self.fail = times, set(fail)
        self.opts, self.resets = {}, 0

    def set_option(self, option, value):
        self.opts[option] = value

    def reset(self):
        self.resets += 1

    def advance(self, steps):
        cand = (self.opts[_lib.OPT_TILE_ROWS], self.opts[_lib.OPT_TB_DEPTH], self.opts[_lib.OPT_TB_WARPS])
        if cand in self.fail:
            raise _lib.EtgError(1, "no compiled batched kernel")
        self.last = self.times.get(cand, 50.0)

    def last_timing(self):
        return self.last, 1


def test_batch_tuner_applies_the_fastest_shape_and_skips_missing_ones():
    b = FakeBatch({(40, 4, 8): 3.0, (48, 4, 16): 2.5}, fail={(48, 4, 16)})
    choice = autotune.tune_batch(b, steps=8, reps=1)
    assert choice == (40, 4, 8)
    assert (b.opts[_lib.OPT_TILE_ROWS], b.opts[_lib.OPT_TB_DEPTH], b.opts[_lib.OPT_TB_WARPS]) == (40, 4, 8)
    assert b.resets >= len(autotune.BATCH_CANDIDATES["single"])  # left at step 0
