"""Autotuner of the stepping kernel: kernel family, tile rows, steps per launch and warps per
tile, per grid.

The fastest choice depends on how the tiles of a grid fill the SMs: the number of tiles in
the last wave, the share of CPML tiles, and whether the grid is large enough for the
persistent TMA-fed kernel. ``tune(engine)`` times every candidate on the engine itself
(CUDA events on its stream, best of ``reps``), keeps the fastest, caches it by
(grid, precision, device) in a JSON file and leaves the engine reset to step 0. Every
candidate gives the same bits, so the choice only changes speed.

Cache file: $ETALON_GB300_AUTOTUNE or ~/.cache/etalon_gb300/autotune.json.
"""

from __future__ import annotations

import json
import os
from pathlib import Path

from . import _lib

# (kernel, tile rows, steps per launch, warps per tile); tile columns follow from the precision
CANDIDATES = {
    "single": [("tb", 48, 4, 8), ("tb", 64, 4, 8), ("tb", 40, 4, 8), ("tb", 40, 8, 8), ("tb", 48, 4, 16),
               ("tma", 40, 4, 8), ("pipe", 48, 4, 8), ("plain", 0, 0, 8)],
    "double": [("tb", 40, 2, 8), ("tb", 32, 2, 8), ("tb", 32, 4, 8), ("tma", 40, 2, 8), ("pipe", 40, 2, 8),
               ("plain", 0, 0, 8)],
}  # fmt: skip


def cache_path() -> Path:
    env = os.environ.get("ETALON_GB300_AUTOTUNE")
    return Path(env) if env else Path.home() / ".cache" / "etalon_gb300" / "autotune.json"


def _load() -> dict:
    try:
        return json.loads(cache_path().read_text())
    except (OSError, ValueError):
        return {}


def _store(table: dict) -> None:
    path = cache_path()
    try:
        path.parent.mkdir(parents=True, exist_ok=True)
        tmp = path.with_suffix(".tmp")
        tmp.write_text(json.dumps(table, indent=1, sort_keys=True))
        tmp.replace(path)
    except OSError:
        pass  # a read-only home only costs re-tuning


def apply(engine, choice: tuple) -> None:
    """Set a candidate on an engine; a cached choice without warps per tile means 8."""
    kernel, rows, depth = choice[:3]
    engine.set_kernel(kernel)
    engine.set_option(_lib.OPT_TILE_ROWS, rows)
    engine.set_option(_lib.OPT_TB_DEPTH, depth)
    engine.set_option(_lib.OPT_TB_WARPS, choice[3] if len(choice) > 3 else 8)


def key_of(engine) -> str:
    _, name, sms = _lib.device_info()
    return f"{engine.nx}x{engine.ny}:{engine.problem.precision}:{name}:{sms}"


def tune(engine, *, steps: int = 96, reps: int = 3, use_cache: bool = True) -> tuple:
    """Pick and apply the fastest candidate for this engine's grid; returns it."""
    key = key_of(engine)
    table = _load() if use_cache else {}
    if key in table:
        choice = tuple(table[key]["choice"])
        apply(engine, choice)
        return choice
    timing_was = _get(engine, _lib.OPT_TIMING)
    engine.set_option(_lib.OPT_TIMING, 1)
    results = {}
    for cand in CANDIDATES[engine.problem.precision]:
        try:
            apply(engine, cand)
            best = float("inf")
            for _ in range(reps):
                engine.reset()
                engine.advance(steps)
                best = min(best, engine.last_timing()[0])
            results[cand] = best
        except (ValueError, _lib.EtgError):
            continue  # shape not compiled, or grid too small for it
    engine.set_option(_lib.OPT_TIMING, timing_was)
    engine.reset()
    choice = min(results, key=results.get)
    apply(engine, choice)
    table[key] = {"choice": list(choice), "ms": {"/".join(map(str, c)): v for c, v in results.items()}}
    _store(table)
    return choice


def timings(engine) -> dict | None:
    """The cached time (ms) of every candidate for this engine's grid, as ``tune`` measured them."""
    entry = _load().get(key_of(engine))
    return entry.get("ms") if entry else None


def _get(engine, option: int) -> int:
    import ctypes as C

    v = C.c_int64()
    _lib.call("etg_sim_get_option", engine._h, option, C.byref(v))
    return v.value


# (tile rows, steps per launch, warps per tile)
BATCH_CANDIDATES = {
    "single": [(48, 4, 8), (40, 4, 8), (64, 4, 8), (48, 4, 16), (40, 8, 8)],
    "double": [(40, 2, 8), (32, 2, 8), (32, 4, 8)],
}  # fmt: skip


def _apply_batch(batch, choice: tuple[int, int, int]) -> None:
    batch.set_option(_lib.OPT_TILE_ROWS, choice[0])
    batch.set_option(_lib.OPT_TB_DEPTH, choice[1])
    batch.set_option(_lib.OPT_TB_WARPS, choice[2])


def tune_batch(batch, *, steps: int = 64, reps: int = 2) -> tuple[int, int, int]:
    """Pick and apply the fastest (tile rows, steps per launch, warps per tile) for a Batch;
    leaves it at step 0."""
    precision = batch.engines[0].problem.precision
    batch.set_option(_lib.OPT_TIMING, 1)
    results = {}
    for cand in BATCH_CANDIDATES[precision]:
        try:
            _apply_batch(batch, cand)
            best = float("inf")
            for _ in range(reps):
                batch.reset()
                batch.advance(steps)
                best = min(best, batch.last_timing()[0])
            results[cand] = best
        except (ValueError, _lib.EtgError):
            continue
    batch.reset()
    choice = min(results, key=results.get)
    _apply_batch(batch, choice)
    return choice
