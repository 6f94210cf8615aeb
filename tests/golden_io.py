"""Loading the golden fixtures of tests/golden/ and comparing results with them."""

from __future__ import annotations

import hashlib
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
FIELDS = ("ex", "ey", "hz", "psi_ex_y", "psi_ey_x", "psi_hz_x", "psi_hz_y")
COEFFS = ("cb_ex", "cb_ey", "bx_e", "cx_e", "ikx_e", "bx_h", "cx_h", "ikx_h",
          "by_e", "cy_e", "iky_e", "by_h", "cy_h", "iky_h")  # fmt: skip


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def load(name: str, precision: str) -> dict:
    with np.load(GOLDEN / f"{name}_{precision}.npz", allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def count(g: dict, prefix: str) -> int:
    k = 0
    while f"{prefix}{k}_component" in g:
        k += 1
    return k


def oracle_from_golden(g: dict, precision: str):
    """An OracleTE holding the fixture's inputs, sources and phasor tables exactly."""
    from oracle.te_numpy import OracleMonitor, OracleSource, OracleTE

    dtype = np.float32 if precision == "single" else np.float64
    nx, ny, _ = (int(v) for v in g["grid"])
    dt = float(g["grid_f"][2])
    coeffs = {c: g[f"in_{c}"] for c in COEFFS}
    db, idx, idy = g["in_scalars"]
    coeffs.update(db=db, inv_dx=idx, inv_dy=idy)
    sources = [
        OracleSource(str(g[f"src{k}_component"]), g[f"src{k}_i"], g[f"src{k}_j"], g[f"src{k}_coef"],
                     tuple(g[f"src{k}_pulse"]), g.get(f"src{k}_table"))
        for k in range(count(g, "src"))
    ]  # fmt: skip
    monitors = [
        OracleMonitor(str(g[f"mon{k}_component"]), g[f"mon{k}_flat"], g[f"mon{k}_freq"], g.get(f"mon{k}_table"))
        for k in range(count(g, "mon"))
    ]
    return OracleTE(nx, ny, dt, coeffs, dtype, sources, monitors)


def compare_outputs(g: dict, fields: dict, accs: list) -> list[str]:
    """Mismatches between a run's outputs and the fixture's (empty list = bit-identical)."""
    bad = []
    for f in FIELDS:
        a = np.asarray(fields[f])
        if sha(a) != str(g[f"out_{f}_sha"]):
            diff = f"sum {a.astype(np.float64).sum():.17g} vs {float(g[f'out_{f}_sum']):.17g}"
            bad.append(f"{f}: hash differs ({diff})")
    for k, acc in enumerate(accs):
        acc = np.asarray(acc)
        if sha(acc) != str(g[f"out_acc{k}_sha"]):
            ref = g.get(f"out_acc{k}")
            err = np.abs(acc - ref).max() / np.abs(ref).max() if ref is not None else float("nan")
            bad.append(f"acc{k}: hash differs (max rel err {err:.3e})")
    return bad
