"""``bench.py --impl reference`` on the CPU: one JSON line with the same metric and config as the
GPU arm, and under torchrun (2 ranks over gloo) only rank 0 prints (no GPU needed)."""

import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
ARGS = ["--impl", "reference", "--steps", "1", "--warmup", "0", "--cpu-seconds", "0.3"]


def _json_lines(out: str) -> list[dict]:
    return [json.loads(line) for line in out.splitlines() if line.startswith("{")]


def _env() -> dict:
    env = dict(os.environ)
    env.pop("WORLD_SIZE", None)
    env.pop("RANK", None)
    env.pop("LOCAL_RANK", None)
    return env


def test_reference_arm_prints_one_line_with_the_contract_keys():
    import bench

    res = subprocess.run([sys.executable, "bench.py", *ARGS], cwd=ROOT, env=_env(), capture_output=True,
                         text=True, timeout=600)  # fmt: skip
    assert res.returncode == 0, res.stderr[-2000:]
    lines = _json_lines(res.stdout)
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["higher_is_better"] is True and d["n_gpus"] == 1 and d["steps"] == 1
    assert d["value"] > 0 and d["cpu_baseline"]["value"] == d["value"]
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["grid"] == [2024, 2024] and d["dtype"] == "f32"


def test_reference_arm_under_torchrun_prints_from_rank_0_only():
    res = subprocess.run(
        [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
         "--master-addr", "127.0.0.1", "--master-port", "29533", "bench.py", "--gpus", "2", *ARGS],
        cwd=ROOT, env=_env(), capture_output=True, text=True, timeout=900,
    )  # fmt: skip
    assert res.returncode == 0, res.stderr[-2000:]
    lines = _json_lines(res.stdout)
    assert len(lines) == 1 and lines[0]["impl"] == "reference" and lines[0]["n_gpus"] == 2
