"""Throughput of the GB300 2D TE path on the 2000² Si-strip workload (one JSON line).

A bench step is one complete run of the workload: 2024 × 2024 cells (2000² region +
12-layer CPML per face), float32, Si strip (ε 12.11, 0.5 µm) in oxide (ε 2.085) at
dl 0.02 µm, one Hz Gaussian point source in the core, three point DFT monitors at 16
wavelengths each, 10 000 time steps from zero fields. The metric is Etalon's
cell-updates/s = nx·ny·time steps / time (etalon/validation/throughput.py:4-5,68).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

``value`` is device time (CUDA events on the simulation's stream) with the inputs
resident in HBM; L2 is flushed (a 512 MB write) before every timed step. ``e2e``
repeats the step through the C ABI from pinned host buffers: coefficient and table
uploads, the run, and the read-back of fields and DFT accumulators are all timed.
``--impl reference`` times the reference's CPU algorithm (the NumPy oracle, in row
bands on every host core) on a bounded prefix of the same workload. With N > 1 (one
process per GPU under torchrun) every rank runs its own replica: the workload is a
single grid, so ranks share nothing ("replicas only").
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "cell-updates/s (2000^2 fp32, bit-exact)"
UNIT = "cell-updates/s"
PEAKS = ROOT / "MEASURED_PEAKS.json"
FALLBACK_HBM_GBS = 6800.0


# ----------------------------------------------------------------------------- helpers


def workload(precision: str, time_steps: int):
    from tests import cases

    return cases.config2(precision, n_steps=time_steps)


def algorithmic_bytes_per_step(p) -> int:
    """Ex, Ey, Hz read+write, cb_ex, cb_ey read; ψ read+write in the strips; DFT acc read+write."""
    s = np.dtype(p.real).itemsize
    nx, ny, L = p.grid.nx, p.grid.ny, p.grid.pml_layers
    dft = sum(sm.flat_index.size * sm.wavelengths.size for sm in p.samplings)
    return s * (8 * nx * ny + 8 * L * (nx + ny)) + 4 * s * dft


def hbm_peak() -> tuple[float, str]:
    try:
        return float(json.loads(PEAKS.read_text())["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def profile_entry(key: str, kernel_tag: str):
    """The text of a ``key[kernel_tag]: ...`` line of a committed ncu summary, and its file."""
    for f in sorted((ROOT / "profiles").glob("*.md")):
        for line in f.read_text().splitlines():
            if line.startswith(f"{key}[{kernel_tag}]:"):
                return line.split(":", 1)[1].strip(), f.name
    return None, None


def ncu_traffic(kernel_tag: str):
    """Per-launch DRAM bytes of the dominant kernel from its committed ncu summary, if any."""
    text, src = profile_entry("traffic_bytes_per_launch", kernel_tag)
    return (float(text.split()[0]), src) if text else (None, None)


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")  # fmt: skip
    REASONS = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")

    def __init__(self, device: int):
        self.device, self.proc, self.lines = device, None, []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.device)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)  # fmt: skip
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for name, v in zip(self.REASONS, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}  # fmt: skip


def cpu_oracle_rate(precision: str, min_seconds: float, threads: int, time_steps: int = 10000):
    """The oracle (NumPy restatement of Etalon's backend) on a bounded prefix of the workload."""
    from etalon_gb300 import physics as ph
    from oracle.te_numpy import OracleMonitor, OracleSource, OracleTE

    p = workload(precision, time_steps)
    o = OracleTE(
        p.grid.nx, p.grid.ny, p.grid.dt, vars(ph.cast_coefficients(p)), p.real,
        [OracleSource(i.component, i.i, i.j, i.coefficient,
                      (i.pulse.wavelength, i.pulse.bandwidth, i.pulse.amplitude)) for i in p.injections],
        [OracleMonitor(s.component, s.flat_index, s.frequencies) for s in p.samplings],
    )  # fmt: skip
    with ThreadPoolExecutor(threads) as pool:
        kw = {"pool": pool, "bands": threads} if threads > 1 else {}
        o.run(2, **kw)  # warm-up
        t0, steps = time.perf_counter(), 0
        while time.perf_counter() - t0 < min_seconds and steps < time_steps:
            o.step(**kw)
            steps += 1
        wall = time.perf_counter() - t0
    return p.grid.n_cells * steps / wall, steps, wall, p


# ----------------------------------------------------------------------------- arms


def dist_setup(n_gpus: int):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        backend = "nccl" if os.environ.get("ETG_BENCH_IMPL", "ours") == "ours" else "gloo"
        if backend == "nccl":
            import torch

            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def reduce_max(world, x: float) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args, world, rank) -> None:
    """Reference arm: Etalon's CPU algorithm (the oracle port) on this host's cores."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    rates = []
    for k in range(args.warmup + args.steps):
        rate, steps, wall, p = cpu_oracle_rate(args.precision, args.cpu_seconds, threads)
        if k >= args.warmup:
            rates.append((rate, steps, wall))
    total_cells = sum(p.grid.n_cells * s for _, s, _ in rates)
    total_wall = sum(w for _, _, w in rates)
    value = total_cells / total_wall
    sample = (f"{p.grid.nx}x{p.grid.ny} grid of the workload, {sum(s for _, s, _ in rates)} time steps "
              f"over {args.steps} steps of ~{args.cpu_seconds:.0f} s each, NumPy oracle in {threads} row bands")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total_wall / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if args.precision == "single" else "f64", "data": "synthetic",
        "config": config_dict(p, args),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))  # fmt: skip


def config_dict(p, args) -> dict:
    return {
        "workload": "2000^2 region + 12-layer CPML (2024x2024 cells), Si strip waveguide in oxide, "
                    "dl 0.02 um, Hz Gaussian point source, 3 point DFT monitors x 16 wavelengths",
        "grid": [p.grid.nx, p.grid.ny], "time_steps_per_step": p.n_steps, "precision": args.precision,
        "l2": "flushed before each timed step (512 MB write)",
        "parallelism": f"replicas x{int(os.environ.get('WORLD_SIZE', '1'))}",
    }  # fmt: skip


def run_ours(args, world, rank, local) -> None:
    import torch

    from etalon_gb300 import _lib, autotune
    from etalon_gb300 import physics as ph
    from etalon_gb300.engine import TEEngine

    _lib.call("etg_set_device", local)
    p = workload(args.precision, args.time_steps)
    e = TEEngine(p, kernel="auto" if args.kernel == "tuned" else args.kernel)
    tuned_ms = None
    if args.kernel == "tuned":
        choice = list(autotune.tune(e))
        tuned_ms = autotune.timings(e)
    else:
        if args.tile_rows:
            e.set_option(_lib.OPT_TILE_ROWS, args.tile_rows)
        if args.warps:
            e.set_option(_lib.OPT_TB_WARPS, args.warps)
        if args.depth:
            e.set_option(_lib.OPT_TB_DEPTH, args.depth)
        choice = [args.kernel, args.tile_rows, args.depth, args.warps]
    e.set_option(_lib.OPT_TIMING, 1)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    def one(timed: bool):
        e.reset()
        flush.zero_()
        torch.cuda.synchronize()
        e.advance(p.n_steps)
        ms, launches = e.last_timing()
        return ms, launches

    for _ in range(args.warmup):
        one(False)
    barrier(world)
    torch.cuda.synchronize()
    _lib.call("etg_synchronize")
    total_ms, launches, wall0 = 0.0, 0, time.perf_counter()
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            ms, n_launch = one(True)
            total_ms += ms
            launches += n_launch
    _lib.call("etg_synchronize")
    torch.cuda.synchronize()
    barrier(world)
    wall = time.perf_counter() - wall0
    e.synchronize()
    total_ms = reduce_max(world, total_ms)
    cells = p.grid.n_cells * p.n_steps
    value = world * cells * args.steps / (total_ms / 1e3)

    # e2e through the C ABI: pinned host inputs in, fields and accumulators out, all timed
    c = ph.cast_coefficients(p)
    names = ("cb_ex", "cb_ey", "bx_e", "cx_e", "ikx_e", "bx_h", "cx_h", "ikx_h",
             "by_e", "cy_e", "iky_e", "by_h", "cy_h", "iky_h")  # fmt: skip
    pinned = {}
    for k in names:
        a = getattr(c, k)
        pinned[k] = _lib.pinned_empty(a.shape, a.dtype)
        pinned[k][...] = a
    pc = type("Pinned", (), {**pinned, "db": c.db, "inv_dx": c.inv_dx, "inv_dy": c.inv_dy})
    src_tables = [_lib.pinned_empty((p.n_steps, i.i.size), p.real) for i in p.injections]
    for t, inj in zip(src_tables, p.injections):
        t[...] = inj.delta_table(0, p.n_steps, p.grid.dt, p.real)
    mon_tables = [_lib.pinned_empty((p.n_steps, s.wavelengths.size), p.complex) for s in p.samplings]
    for t, s in zip(mon_tables, p.samplings):
        t[...] = ph.phasor_table(s, 0, p.n_steps, p.grid.dt, p.complex)
    out_fields = {f: _lib.pinned_empty(e.field_shape(f), p.real) for f in ("ex", "ey", "hz")}
    h2d = sum(a.nbytes for a in pinned.values()) + sum(t.nbytes for t in src_tables + mon_tables)
    d2h = sum(a.nbytes for a in out_fields.values()) + sum(
        2 * s.wavelengths.size * s.flat_index.size * np.dtype(p.real).itemsize for s in p.samplings)

    def e2e_step():
        e.set_coefficients(pc)
        for k, t in enumerate(src_tables):
            e.set_source_table(k, 0, t)
        for k, t in enumerate(mon_tables):
            e.set_phasor_table(k, 0, t)
        e.reset()
        e.advance(p.n_steps)
        for f, out in out_fields.items():
            _lib.call("etg_sim_get_field", e._h, _lib.FIELD_IDS[f], out.ctypes.data)
        return [e.dft(k) for k in range(len(e.monitors))]

    for _ in range(max(1, args.warmup // 2)):
        e2e_step()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_s = reduce_max(world, time.perf_counter() - t0)
    e2e_value = world * cells * args.steps / e2e_s

    # roofline of the dominant kernel: algorithmic bytes per launch / its average launch time
    roofline = kernel_roofline(e, p)
    ref_kernels = None if args.no_ref_kernels or rank != 0 else reference_kernels_line(e, p, args.ref_kernel_steps)
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if args.precision == "single" else "f64", "data": "synthetic",
        "config": config_dict(p, args),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches),
        "roofline": roofline,
        "kernel_choice": choice,
        "autotune_ms": tuned_ms,
        "clocks": clocks.summary(),
        "wall_ms_per_step": 1e3 * wall / args.steps,
    }  # fmt: skip
    if ref_kernels is not None:
        ref_kernels["ours_over_reference_kernels"] = value / world / ref_kernels["value"] if "value" in ref_kernels else None
        out["reference_kernels"] = ref_kernels
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        rate, steps, cwall, _ = cpu_oracle_rate(args.precision, args.cpu_seconds, threads)
        out["cpu_baseline"] = {
            "value": rate, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{p.grid.nx}x{p.grid.ny} workload grid, {steps} time steps in {cwall:.1f} s, "
                      f"NumPy oracle in {threads} row bands",
        }  # fmt: skip
    if not args.no_batched:
        out["batched"] = batched_line(args, local, world, rank)
    if not args.no_adjoint:
        if world == 1:  # one grid: replicas would only repeat it
            out["adjoint"] = adjoint_line(args)
        out["batched_adjoint"] = batched_adjoint_line(args, world, rank)
    if not args.no_fp64:
        out["fp64"] = fp64_line(args, local)
    if rank == 0 and not args.no_studio:
        out["tm"] = tm_line(args)
    if rank == 0 and not args.no_yee3d:
        out["yee3d"] = yee3d_line(args)
    if rank == 0 and not args.no_studio:
        out["studio"] = studio_line(e, p)
        out["rasterize"] = rasterize_line(e, p)
    if rank == 0:
        print(json.dumps(out))
    e.close()


def kernel_roofline(e, p) -> dict:
    """Roofline of the dominant kernel, timed live with CUDA events on its launching stream.

    Temporally blocked path: one more run of the workload with every kernel launch timed on
    its own (option TIMING = 2: the kernels one after the other, an event pair around each, no
    graphs). The dominant kernel is the lean interior kernel (interior tiles without a source,
    monitor or trace node; at 2024² with 40-row, K = 8 tiles the segment kernel, which steps them
    as column segments, a tile and three tiles that take the row above from it); it advances its
    output cells K steps per launch, and its algorithmic bytes are those of K single-pass steps
    over them, 8 values per cell-step (Ex, Ey, Hz read and write, cb_ex and cb_ey read).
    One-step path: the run's own time per step against the algorithmic bytes of a step.
    """
    from etalon_gb300 import _lib

    peak, peak_kind = hbm_peak()
    s = np.dtype(p.real).itemsize
    kind, rows, depth, warps = (get_option(e, o) for o in (_lib.OPT_KERNEL, _lib.OPT_TILE_ROWS, _lib.OPT_TB_DEPTH,
                                                          _lib.OPT_TB_WARPS))
    e.set_option(_lib.OPT_TIMING, 2)
    e.reset()
    e.advance(p.n_steps)
    e.synchronize()
    kt = e.kernel_timing()
    segments = get_option(e, _lib.OPT_TB_SEGMENTS_USED)  # of the tile list this run used
    e.set_option(_lib.OPT_TIMING, 1)
    ms, launches, cells = kt["interior"]
    if launches:
        dt = "float" if s == 4 else "double"
        name = f"k_tb_step<{dt},{rows // warps},{depth},false,{warps},false>"  # the lean interior kernel
        if segments:  # the lean interior tiles as column segments (the leftover tiles timed with the rest)
            name = f"k_tb_seg<{dt},{rows // warps},{depth},{warps}> ({segments} column segments of 5 tile rows)"
        launch_ms = ms / launches
        bytes_launch = 8 * s * cells * depth
        cp_ms, cp_launches, cp_cells = kt["cpml"]
        extra = {"kernel": name, "tile": [rows, 128 if s == 4 else 64], "steps_per_launch": depth,
                 "output_cells_per_launch": cells, "launch_ms": launch_ms, "launches_timed": launches,
                 "cpml_kernel": {"launch_ms": cp_ms / max(cp_launches, 1), "output_cells_per_launch": cp_cells},
                 "timing": "CUDA events around each launch, one extra run of the workload, kernels serialised"}
        tag = (f"k_tb_{'seg' if segments else 'step'}_interior_{rows}x{128 if s == 4 else 64}"
               + ("" if warps == 8 else f"_{warps}w") + ("" if depth == (4 if s == 4 else 2) else f"_k{depth}"))
    elif kind in (3, 4):  # persistent kernels: the run's device time over its launches
        e.reset()
        e.advance(p.n_steps)
        total, _ = e.last_timing()
        n_launch = 2 * (p.n_steps // (2 * depth))
        launch_ms = total / max(n_launch, 1)
        bytes_launch = algorithmic_bytes_per_step(p) * depth
        extra = {"kernel": f"{'k_tb_tma' if kind == 3 else 'k_tb_pipe'}<{rows // 8},{depth}>", "steps_per_launch": depth,
                 "launch_ms": launch_ms,
                 "timing": "CUDA events around the run, divided by its launches"}
        tag = "k_tb_tma"
    else:  # one-step kernels: the timed run's own device time
        e.reset()
        e.advance(p.n_steps)
        total, _ = e.last_timing()
        launch_ms = total / p.n_steps
        bytes_launch = algorithmic_bytes_per_step(p)
        extra = {"kernel": "k_fused_h+k_fused_e", "steps_per_launch": 1, "launch_ms": launch_ms,
                 "timing": "CUDA events around the run, per step"}
        tag = "k_fused"
    achieved = bytes_launch / (launch_ms / 1e3) / 1e9
    traffic, traffic_src = ncu_traffic(tag)
    # "bound" names the roofline the fraction is taken against (HBM: the stencil is no
    # contraction). Temporal blocking moves a cell through HBM once per K steps, so the
    # algorithmic fraction can pass 1; "dram_frac" is the DRAM traffic ncu measured per launch
    # over the same launch time, and "limiter" what ncu shows actually limits the kernel.
    limiter, _ = profile_entry("limiter", tag)
    dram_frac = traffic / (launch_ms / 1e3) / 1e9 / peak if traffic else None
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_source": f"{peak_kind} (hbm_gbs)", "traffic": traffic, "traffic_source": traffic_src,
            "dram_frac": dram_frac, "limiter": limiter,
            "algorithmic_bytes_per_launch": bytes_launch, **extra}  # fmt: skip


def reference_kernels_line(e, p, steps: int, warmup: int = 20) -> dict:
    """Etalon's own CUDA kernels (update_te.cu, dft.cu: compiled unchanged by
    oracle/build_ref.py, launched with its CuPy backend's shapes by oracle/ref_kernels.py) on
    the same workload and GPU, one step at a time as Etalon's FDTDSolver steps them: cell-updates
    per second over ``steps`` steps timed with events on their stream after ``warmup`` steps,
    and the fields and accumulators after them against this package's engine, bit for bit."""
    from etalon_gb300 import _lib
    from oracle import ref_kernels
    from tests.ref_kernel_run import RefRun

    if not ref_kernels.available(p.precision):
        return {"unavailable": "reference kernel images missing (oracle/build_ref.py needs Etalon's tree)"}
    k = ref_kernels.RefKernels(p.precision)
    run = RefRun(k, p, warmup + steps)
    for _ in range(warmup):
        run.step()
    a, b = k.event(), k.event()
    _lib.call("etg_synchronize")
    launches0 = k.launches
    k.record(a)
    for _ in range(steps):
        run.step()
    k.record(b)
    ms = k.elapsed_ms(a, b)
    e.reset()
    e.advance(warmup + steps)
    e.synchronize()
    same = all(np.array_equal(run.field(f).view(np.uint8), e.field(f).view(np.uint8))
               for f in ("ex", "ey", "hz", "psi_ex_y", "psi_ey_x", "psi_hz_x", "psi_hz_y"))  # fmt: skip
    same = same and all(np.array_equal(run.acc(m), e.dft(m)) for m in range(len(p.samplings)))
    out = {"value": p.grid.n_cells * steps / (ms / 1e3), "unit": UNIT, "time_steps": steps,
           "ms_per_time_step": ms / steps, "kernel_launches_per_time_step": (k.launches - launches0) / steps,
           "bit_identical_to_ours": bool(same),
           "what": "Etalon's update_h_te/update_e_te/accumulate_dft, nvcc -fmad=false for sm_103a, CuPy's launch "
                   "shapes, legacy default stream, one launch per kernel per step (+ one injection scatter per "
                   "source); device time from events around the steps"}  # fmt: skip
    run.close()
    k.close()
    return out


def get_option(e, option: int) -> int:
    import ctypes as C

    from etalon_gb300 import _lib

    v = C.c_int64()
    _lib.call("etg_sim_get_option", e._h, option, C.byref(v))
    return int(v.value)


def batched_line(args, local, world=1, rank=0) -> dict:
    """64 seeded synthetic devices (bends, rings, MMIs; interiors 256-1536 cells per axis,
    12-layer CPML, one Hz source, 4 point monitors x 8 wavelengths), float32, 5000 time steps,
    stepped together by one Batch: tiles of all 64 in each launch, CUDA graphs per step block."""
    import torch

    from etalon_gb300 import autotune
    from etalon_gb300.batch import Batch
    from etalon_gb300.shard import shard
    from tests import cases

    every = cases.synthetic_batch(64, n_steps=args.batch_time_steps)
    problems = shard(every, [p.grid.n_cells for p in every], rank, world)  # no exchange between ranks
    b = Batch(problems)
    choice = autotune.tune_batch(b)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    ms, launches = [], 0
    for k in range(3):
        b.reset()
        flush.zero_()
        torch.cuda.synchronize()
        b.advance(args.batch_time_steps)
        t, n = b.last_timing()
        if k:  # the first run is the warm-up
            ms.append(t)
            launches += n
    b.close()
    t = reduce_max(world, sum(ms) / len(ms))
    cells = sum(p.grid.n_cells for p in every)
    return {"metric": "cell-updates/s (64 synthetic devices 256^2-1536^2 + CPML, fp32, one batch)",
            "value": cells * args.batch_time_steps / (t / 1e3), "unit": UNIT, "ms_per_run": t,
            "sims": len(every), "cells": cells, "time_steps": args.batch_time_steps,
            "sharding": f"{world} rank(s), devices balanced by cells, no exchange",
            "tile_rows_depth_warps": list(choice), "gpu_launches_per_run": launches // len(ms),
            "runs_timed": len(ms), "l2": "flushed before each run"}  # fmt: skip


def _gradient_once(runner, problem, eps0) -> tuple[float, np.ndarray]:
    """One gradient through the public API (simulate + backward), wall time with syncs."""
    import torch

    from etalon_gb300 import _lib
    from etalon_gb300.adjoint import point_power, simulate

    eps = eps0.clone().requires_grad_(True)
    _lib.call("etg_synchronize")
    t = time.perf_counter()
    point_power(simulate(eps, runner)[0], problem.samplings[0]).backward()
    _lib.call("etg_synchronize")
    return time.perf_counter() - t, eps.grad.numpy().copy()


def adjoint_line(args) -> dict:
    """dJ/dε of one 100×100-cell design in a 1224² grid (1200² + CPML), 20 000 steps, √N
    checkpoints, J = Σ_λ |DFT Hz|² at an output point (3 λ): gradients per second through
    simulate() + backward(), temporally blocked kernels against the one-step kernels, and the
    float32 gradient's error against the float64 one."""
    import torch

    from etalon_gb300.adjoint import AdjointRunner, DesignRegion
    from tests import cases

    n = args.adjoint_time_steps
    out = {"metric": "gradient evaluations/s (1224^2, 100x100 design, sqrt-N checkpoints, fp32)", "time_steps": n}
    grads = {}
    for name, precision, kernel, stride in (("blocked", "single", "auto", None), ("trace", "single", "auto", 0),
                                            ("one_step", "single", "plain", None), ("fp64", "double", "auto", None)):
        p, win = cases.adjoint_device(precision, n_steps=n)
        d = DesignRegion.from_box(p, win[:2], win[2:])
        eps0 = torch.as_tensor(cases.smooth_design(d.nx, d.ny, 0))
        r = AdjointRunner(p, d, stride=AdjointRunner.sqrt_stride(n) if stride is None else stride, kernel=kernel)
        reps = 1 if name == "fp64" else 2
        ts = []
        for _ in range(reps + 1):
            t, g = _gradient_once(r, p, eps0)
            ts.append(t)
        r.close()
        grads[name] = g
        out[f"{name}_s_per_gradient"] = min(ts[1:])
    out["value"] = 1.0 / out["blocked_s_per_gradient"]
    out["unit"] = "gradients/s"
    out["one_step_kernels_value"] = 1.0 / out["one_step_s_per_gradient"]
    out["trace_mode_value"] = 1.0 / out["trace_s_per_gradient"]
    ref = grads["fp64"]
    out["rel_err_vs_fp64"] = float(np.abs(grads["blocked"] - ref).max() / np.abs(ref).max())
    out["blocked_equals_one_step_bits"] = bool(np.array_equal(grads["blocked"], grads["one_step"]))
    return out


def batched_adjoint_line(args, world=1, rank=0) -> dict:
    """32 seeded design variants (regions 512-1024 cells per side + CPML, design windows 50-150
    cells, 8 λ, 10 000 steps): all forward and reverse passes run as one batch with √N
    checkpoints (the headline) and with the full trace; gradients per second against the same
    32 designs run one at a time on the single-design default path (temporally blocked kernels,
    √N checkpoints: the single-design workload's own path), and every design's float32
    gradient against its float64 gradient."""
    import torch

    from etalon_gb300 import _lib
    from etalon_gb300.adjoint import AdjointBatch, AdjointRunner, DesignRegion, point_power, simulate_batch
    from tests import cases

    n = args.batch_adjoint_time_steps
    from etalon_gb300.shard import shard

    variants = cases.adjoint_variants(32, n_steps=n)
    variants = shard(variants, [v[0].grid.n_cells for v in variants], rank, world)  # no exchange
    items, designs = [], []
    for p, win, design, seed in variants:
        d = DesignRegion.from_box(p, win[:2], win[2:])
        items.append((p, d, torch.as_tensor(cases.smooth_design(d.nx, d.ny, seed))))
        designs.append(design)
    S = AdjointRunner.sqrt_stride(n)
    out = {"metric": "gradient evaluations/s (32 designs 512^2-1024^2, 50^2-150^2 windows, 8 wavelengths, fp32, "
                     "sqrt-N checkpoints)",
           "unit": "gradients/s", "time_steps": n, "checkpoint_stride": S}  # fmt: skip

    def batched(items, stride, reps):
        runners = [AdjointRunner(p, d, stride=stride) for p, d, _ in items]
        b = AdjointBatch(runners)
        ts = []
        for _ in range(reps):
            eps = [e.clone().requires_grad_(True) for _, _, e in items]
            _lib.call("etg_synchronize")
            t = time.perf_counter()
            outs = simulate_batch(eps, b)
            sum(point_power(o[0], it[0].samplings[0]) for o, it in zip(outs, items)).backward()
            _lib.call("etg_synchronize")
            ts.append(time.perf_counter() - t)
        grads = [e.grad.numpy().copy() for e in eps]
        b.close()
        for r in runners:
            r.close()
        return min(ts[1:]) if reps > 1 else ts[0], grads

    grads = {}
    for name, stride in (("checkpoints", S), ("trace", 0)):
        t, grads[name] = batched(items, stride, 3)
        out[f"batched_{name}_s"] = reduce_max(world, t)
    # the baseline: one design at a time on the single-design default path, one untimed
    # gradient per design first (graph capture, tuning), then one timed gradient
    total, one = 0.0, []
    for p, d, e0 in items:
        r = AdjointRunner(p, d, stride=S)
        _gradient_once(r, p, e0)
        t, g = _gradient_once(r, p, e0)
        total += t
        one.append(g)
        r.close()
    total = reduce_max(world, total)
    out["one_at_a_time_s"] = total
    out["one_at_a_time_path"] = "single-design default (temporally blocked kernels, sqrt-N checkpoints)"
    out["designs"] = 32
    out["sharding"] = f"{world} rank(s), designs balanced by cells, no exchange"
    out["value"] = 32 / out["batched_checkpoints_s"]
    out["trace_value"] = 32 / out["batched_trace_s"]
    out["one_at_a_time_value"] = 32 / total
    out["speedup_vs_one_at_a_time"] = total / out["batched_checkpoints_s"]
    out["trace_speedup_vs_one_at_a_time"] = total / out["batched_trace_s"]
    out["batched_equals_one_at_a_time_bits"] = bool(
        all(np.array_equal(a, b) and np.array_equal(a, c) for a, b, c in zip(grads["checkpoints"], grads["trace"], one)))
    # float64 gradients of every design, as one float64 batch with the same checkpoints
    items64 = []
    for (p, d, e0), design in zip(items, designs):
        p64, win = cases.adjoint_device("double", n_steps=n, region=p.grid.nx - 24, design=design, n_wavelengths=8)
        items64.append((p64, DesignRegion.from_box(p64, win[:2], win[2:]), e0))
    t64, g64s = batched(items64, S, 1)
    out["fp64_batched_s"] = t64
    errs = [float(np.abs(g32 - g64).max() / np.abs(g64).max())
            for g32, g64 in zip(grads["checkpoints"], g64s) if np.abs(g64).max() > 0]  # fmt: skip
    # (a run too short for the pulse to reach the objective has no gradient to compare)
    out["rel_err_vs_fp64"] = max(errs) if errs else None
    out["rel_err_vs_fp64_median"] = float(np.median(errs)) if errs else None
    out["rel_err_designs"] = len(errs)
    return out


def fp64_line(args, local) -> dict:
    """The same workload in float64 (GB300's FP64 pipe bounds it, not HBM), the kernel chosen as
    for the headline; its fields and coefficients (about 300 MB) exceed L2."""
    import torch

    from etalon_gb300 import _lib, autotune
    from etalon_gb300.engine import TEEngine

    p = workload("double", args.time_steps)
    e = TEEngine(p, kernel="auto" if args.kernel == "tuned" else args.kernel)
    choice = list(autotune.tune(e)) if args.kernel == "tuned" else [args.kernel]
    tuned_ms = autotune.timings(e) if args.kernel == "tuned" else None
    e.set_option(_lib.OPT_TIMING, 1)
    e.advance(p.n_steps)
    ms = []
    for _ in range(2):
        e.reset()
        torch.cuda.synchronize()
        e.advance(p.n_steps)
        ms.append(e.last_timing()[0])
    e.close()
    t = sum(ms) / len(ms)
    return {"value": p.grid.n_cells * p.n_steps / (t / 1e3), "unit": UNIT, "ms_per_step": t, "kernel_choice": choice,
            "autotune_ms": tuned_ms}


def tm_line(args) -> dict:
    """The 2D TM mode on the headline grid: 2000² + 12-layer CPML, the Si strip along x in oxide,
    an Ez point current in the core, 3 point monitors × 16 wavelengths, fp32, 2000 steps; the
    dual TE run on the temporally blocked kernels (their TM variant, 40×128 tiles, K = 8, column
    segments), device time per step."""
    import torch

    from etalon_gb300 import _lib
    from etalon_gb300 import physics as ph
    from etalon_gb300 import tm
    from tests import cases

    steps = 2000
    wl = list(np.linspace(1.5, 1.6, 16))
    p = tm.tm_problem(
        size=(40.0, 40.0), dl=0.02, background_eps=cases.EPS_OXIDE,
        boxes=[ph.Box((0.0, 0.0, 0.0), (42.0, 0.5, 0.22), cases.EPS_SILICON)], pml=ph.PMLSpec(layers=12),
        sources=[tm.TMPointSource((-15.0, 0.0, 0.0), ph.GaussianPulse(1.55, 0.5))],
        monitors=[ph.DFTMonitor(f"m{k}", wl, center=(x, 0.0, 0.0)) for k, x in enumerate((-5.0, 5.0, 15.0))],
        n_steps=steps, precision="single",
    )  # fmt: skip
    e = tm.TMEngine(p)
    e.te.set_option(_lib.OPT_TB_DEPTH, 8)  # the depth the tuner takes for the TE run of this grid
    e.te.set_option(_lib.OPT_TIMING, 1)
    e.advance(200)
    ms = []
    for _ in range(2):
        e.reset()
        torch.cuda.synchronize()
        e.advance(steps)
        ms.append(e.te.last_timing()[0])
    e.close()
    t = min(ms)
    return {"value": p.grid.n_cells * steps / (t / 1e3), "unit": UNIT, "time_steps": steps,
            "grid": [p.grid.nx, p.grid.ny],
            "path": "dual TE run, temporally blocked kernels (TM variant: per-node Ez coefficient), K = 8, column segments"}  # fmt: skip


def yee3d_line(args) -> dict:
    """3D Yee on Etalon's planned 3D performance cell (docs/mvp-spec.md:109): 10 × 10 × 3 µm at
    20 nm with 12-layer CPML on every face (524 × 524 × 174 cells), a 0.5 × 0.22 µm Si strip
    along x in oxide, an Ey point current in the core (x = -4 µm), 3 point monitors × 16
    wavelengths (x = -2, 0, 2 µm) on all six components, fp32. ``--yee3d-cell`` scales the cell
    (source and monitors at the same fractions of its length). Device time of the steps (fields
    1.1 GB: past L2, no flush needed) with the default step, an H and an E kernel (each timed
    alone; the E kernel has the roofline entry: it reads six fields and three cb and writes three
    fields, 48 algorithmic B per cell; the H kernel 36 B); then the same run continued with the
    fused step (one kernel over two buffer sets, 60 B per cell)."""
    from etalon_gb300 import physics as ph
    from etalon_gb300 import yee3d
    from tests import cases

    steps, warm, timed = args.yee3d_steps, 20, 10
    wl = list(np.linspace(1.5, 1.6, 16))
    cell = tuple(float(v) for v in args.yee3d_cell.split(","))
    p = yee3d.yee3d_problem(
        cell, 0.02, background_eps=cases.EPS_OXIDE,
        boxes=[ph.Box((0.0, 0.0, 0.0), (12.0, 0.5, 0.22), cases.EPS_SILICON)], layers=12,
        sources=[ph.PointSource((-0.4 * cell[0], 0.0, 0.0), "Ey", ph.GaussianPulse(1.55, 0.5))],
        monitors=[ph.DFTMonitor(f"m{k}", wl, center=(f * cell[0], 0.0, 0.0)) for k, f in enumerate((-0.2, 0.0, 0.2))],
        n_steps=warm + 3 * steps + 2 * timed, precision="single",
    )  # fmt: skip
    g = p.grid
    e = yee3d.Yee3DEngine(p)  # the default step: an H and an E kernel per step
    e.advance(warm)
    e.synchronize()
    ms = []
    for _ in range(2):
        e.advance(steps)
        e.synchronize()
        ms.append(e.last_timing()[0])
    launches = e.last_timing()[1]
    ms_h, ms_e = e.kernel_timing(timed)
    e.set_fused(True)  # the same run continued with the fused step (one kernel, two buffer sets)
    e.advance(steps)
    e.synchronize()
    ms_fused = e.last_timing()[0]
    ms_f, _ = e.kernel_timing(timed)
    e.close()
    t = min(ms)
    cells = g.n_cells
    peak, peak_kind = hbm_peak()
    achieved = 48 * cells / (ms_e / 1e3) / 1e9
    per_cell, src = profile_entry("traffic_bytes_per_cell", "k3_update_e_f32")
    traffic = float(per_cell.split()[0]) * cells if per_cell else None
    limiter, _ = profile_entry("limiter", "k3_update_e_f32")
    return {
        "value": cells * steps / (t / 1e3), "unit": UNIT, "time_steps": steps, "ms_per_step": t / steps,
        "grid": [g.nx, g.ny, g.nz], "dtype": "f32", "gpu_launches_per_step": launches / steps,
        "kernels_ms": {"update_h": ms_h, "update_e": ms_e},
        "fused_step": {"value": cells * steps / (ms_fused / 1e3), "ms_per_step": ms_fused / steps,
                       "kernel_ms": ms_f, "frac": 60 * cells / (ms_f / 1e3) / 1e9 / peak},
        "roofline": {"kernel": "k3_update_e<float>", "bound": "hbm", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                     "algorithmic_bytes_per_launch": 48 * cells,
                     "traffic": traffic, "traffic_source": f"{src}, DRAM bytes per cell x cells" if src else None,
                     "dram_frac": traffic / (ms_e / 1e3) / 1e9 / peak if traffic else None, "limiter": limiter,
                     "h_kernel_frac": 36 * cells / (ms_h / 1e3) / 1e9 / peak},
    }  # fmt: skip


def _studio_energy(state, xp, dt, db, cell_area):
    """Etalon Studio's progress energy (etalon/studio/runner.py:258-281) on any array module."""

    def weighted(field, coefficient):
        values = field.astype(xp.float64)
        return float(xp.sum(values * values / coefficient))

    hz = state["hz"].astype(xp.float64)
    electric = dt * (weighted(state["ex"], state["cb_ex"]) + weighted(state["ey"], state["cb_ey"]))
    magnetic = dt / float(db) * float(xp.sum(hz * hz))
    return float(0.5 * cell_area * (electric + magnetic))


def _studio_downsample(field, xp, max_nodes=256):
    """Etalon Studio's snapshot of a field (etalon/studio/runner.py:284-291)."""
    n_x, n_y = field.shape
    sx = max(1, -(-n_x // max_nodes))
    sy = max(1, -(-n_y // max_nodes))
    mx, my = n_x // sx, n_y // sy
    return field[: mx * sx, : my * sy].reshape(mx, sx, my, sy).mean(axis=(1, 3)).astype(xp.float32)


def studio_line(e, p, frames: int = 20) -> dict:
    """One Studio progress frame (energy + 256-node Hz snapshot) on the final state of the
    headline run: on device arrays through the backend's ``xp`` (a few numbers and a small
    image cross the link) against NumPy after copying the fields and cb to the host."""
    import torch

    from etalon_gb300 import physics as ph
    from etalon_gb300.backend import Gb300Backend

    backend = Gb300Backend(p.precision)
    c = ph.cast_coefficients(p)
    host = {f: e.field(f) for f in ("ex", "ey", "hz")}
    host["cb_ex"], host["cb_ey"] = c.cb_ex, c.cb_ey
    dev = {k: backend.to_device(v) for k, v in host.items()}
    g = p.grid
    args = (g.dt, c.db, g.dx * g.dy * ph.UM**2)

    def device_frame():
        energy = _studio_energy(dev, backend.xp, *args)
        image = backend.to_host(_studio_downsample(dev["hz"], backend.xp))
        return energy, image

    def host_frame():
        state = {k: backend.to_host(v) for k, v in dev.items()}
        return _studio_energy(state, np, *args), _studio_downsample(state["hz"], np)

    out = {}
    for name, fn in (("device", device_frame), ("host_copy", host_frame)):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(frames):
            res = fn()
        out[f"{name}_ms_per_frame"] = 1e3 * (time.perf_counter() - t0) / frames
        out[name] = res
    (ed, imd), (eh, imh) = out.pop("device"), out.pop("host_copy")
    out.update({
        "frames": frames, "grid": [g.nx, g.ny], "snapshot": list(imd.shape),
        "energy_rel_diff": abs(ed - eh) / abs(eh) if eh else abs(ed - eh),
        "snapshot_max_rel_diff": float(np.max(np.abs(imd.astype(np.float64) - imh.astype(np.float64)))
                                       / max(float(np.max(np.abs(imh))), 1e-300)),
        "speedup": out["host_copy_ms_per_frame"] / out["device_ms_per_frame"],
        "what": "etalon/studio/runner.py:258-291 expressions; device: float64 sums and block means on the GPU",
    })  # fmt: skip
    return out


def rasterize_line(e, p, reps: int = 5) -> dict:
    """ε staircase + cb of the headline grid for 64 boxes (a design sweep's geometry): on the
    device (etg_sim_rasterize_cb) against the host path (permittivity_on_nodes, the float64 cb
    and cast, the upload), and whether the two give the same bits."""
    from etalon_gb300 import physics as ph

    g = p.grid
    rng = np.random.default_rng(7)
    lx, ly = g.nx * g.dx, g.ny * g.dy
    boxes = [ph.Box((g.x_min + float(rng.uniform(0, lx)), g.y_min + float(rng.uniform(0, ly)), 0.0),
                    (float(rng.uniform(0.5, 8.0)), float(rng.uniform(0.2, 8.0)), 0.22),
                    float(rng.choice([2.085, 12.11]))) for _ in range(64)]  # fmt: skip
    c = ph.cast_coefficients(p)

    def host():
        eps = ph.permittivity_on_nodes(g, p.background_eps, boxes)
        cb_ex = np.ascontiguousarray(g.dt / (ph.EPSILON_0 * eps["Ex"]), dtype=p.real)
        cb_ey = np.ascontiguousarray(g.dt / (ph.EPSILON_0 * eps["Ey"]), dtype=p.real)
        c.cb_ex, c.cb_ey = cb_ex, cb_ey
        e.set_coefficients(c)
        return cb_ex, cb_ey

    def device():
        e.rasterize(boxes, p.background_eps)
        e.synchronize()

    out = {}
    for name, fn in (("host", host), ("device", device)):
        res = fn()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        out[f"{name}_ms"] = 1e3 * (time.perf_counter() - t0) / reps
        if name == "host":
            want = res
    same = all(np.array_equal(e.cb(w).view(np.uint8), r.view(np.uint8)) for w, r in zip(("ex", "ey"), want))
    out.update({"boxes": len(boxes), "grid": [g.nx, g.ny], "bit_identical": bool(same),
                "speedup": out["host_ms"] / out["device_ms"],
                "host_path": "permittivity_on_nodes + dt/(eps0 eps) + cast + upload of the coefficients"})  # fmt: skip
    return out


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="single", choices=["single", "double"])
    ap.add_argument("--time-steps", type=int, default=10000)
    ap.add_argument("--kernel", default="tuned", choices=["auto", "tuned", "plain", "tb", "pipe"],
                    help="tuned: the autotuner picks kernel, tile rows, depth and warps (before timing)")
    ap.add_argument("--tile-rows", type=int, default=0, help="with a fixed --kernel: tile rows (0: its default)")
    ap.add_argument("--warps", type=int, default=0, help="with a fixed --kernel: warps per tile (0: 8)")
    ap.add_argument("--depth", type=int, default=0, help="with a fixed --kernel: steps per launch (0: its default)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the 64-device batched line")
    ap.add_argument("--batch-time-steps", type=int, default=5000)
    ap.add_argument("--no-adjoint", action="store_true", help="skip the gradient lines")
    ap.add_argument("--adjoint-time-steps", type=int, default=20000)
    ap.add_argument("--batch-adjoint-time-steps", type=int, default=10000)
    ap.add_argument("--no-fp64", action="store_true", help="skip the float64 line of the same workload")
    ap.add_argument("--no-studio", action="store_true", help="skip the live-view and rasterisation lines")
    ap.add_argument("--no-ref-kernels", action="store_true", help="skip timing Etalon's own CUDA kernels")
    ap.add_argument("--no-yee3d", action="store_true", help="skip the 3D Yee line")
    ap.add_argument("--yee3d-steps", type=int, default=200)
    ap.add_argument("--yee3d-cell", default="10,10,3", help="3D line: region size in µm (x,y,z), 20 nm cells")
    ap.add_argument("--ref-kernel-steps", type=int, default=1000)
    args = ap.parse_args()
    os.environ["ETG_BENCH_IMPL"] = args.impl
    world, rank, local = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
