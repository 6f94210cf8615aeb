"""Build recipe: the reference's own CUDA kernels, compiled from its sources into oracle/_ref/.

TEST AND BENCH INFRASTRUCTURE ONLY. Etalon's CuPy backend compiles
``etalon/fdtd/backends/cuda/update_te.cu`` and ``cuda/dft.cu`` at run time with NVRTC,
``#define REAL float|double`` and ``--fmad=false`` (etalon/fdtd/backends/cupy_backend.py:42-49).
This recipe compiles the same two files, unchanged, where they lie in the Etalon source tree,
with nvcc and the same definitions for sm_103a, into device images (a cubin and a PTX file per
file and precision) under oracle/_ref/ — nothing else is written, and no source is copied. The
images hold device code only, so the ones built here load on any host architecture; the GPU
machine, which has no Etalon tree, uses the prebuilt files. ``oracle/ref_kernels.py`` loads
them through the CUDA driver API.

    python oracle/build_ref.py [--src ETALON_TREE]
"""

from __future__ import annotations

import argparse
import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
DEFAULT_TREE = "/root/reference"
SOURCES = ("update_te", "dft")
REALS = {"f32": "float", "f64": "double"}
ARCH = "sm_103a"


def kernel_dir(tree: str | os.PathLike) -> Path:
    return Path(tree) / "etalon" / "fdtd" / "backends" / "cuda"


def images(tag: str) -> dict[str, Path]:
    """The built image of each source for a precision tag ("f32" or "f64")."""
    return {name: OUT / f"{name}_{tag}.cubin" for name in SOURCES}


def build(tree: str | os.PathLike | None = None, quiet: bool = True) -> bool:
    """Compile every image whose source is newer; False when the Etalon tree is absent."""
    tree = tree or os.environ.get("ETALON_SRC") or DEFAULT_TREE
    src_dir = kernel_dir(tree)
    if not all((src_dir / f"{n}.cu").exists() for n in SOURCES):
        return False
    nvcc = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    OUT.mkdir(exist_ok=True)
    for tag, real in REALS.items():
        for name in SOURCES:
            src = src_dir / f"{name}.cu"
            for kind in ("cubin", "ptx"):
                out = OUT / f"{name}_{tag}.{kind}"
                if out.exists() and out.stat().st_mtime >= src.stat().st_mtime:
                    continue
                arch = f"-arch={ARCH}" if kind == "cubin" else "-arch=compute_103a"
                cmd = [nvcc, f"--{kind}", arch, "-O3", "-fmad=false", f"-DREAL={real}", "-o", str(out), str(src)]
                res = subprocess.run(cmd, capture_output=True, text=True)
                if res.returncode != 0:
                    raise RuntimeError(f"nvcc failed on {src.name} ({tag}):\n{res.stdout}\n{res.stderr}")
                if not quiet:
                    print("built", out.name)
    return True


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--src", default=None, help="Etalon's source tree (default: $ETALON_SRC or the local checkout)")
    args = ap.parse_args()
    print("built" if build(args.src, quiet=False) else "Etalon's CUDA sources not found")
