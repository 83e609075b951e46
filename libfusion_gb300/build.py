"""Build libgbfusion.so in-tree for sm_103a with nvcc (no cmake, no pip).

Each translation unit is compiled in parallel, then linked into
``libfusion_gb300/_build/libgbfusion.so``.  ``-fmad=false`` keeps every float
operation rounded as written, matching the oracle's ``-ffp-contract=off``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libgbfusion.so"
SOURCES = ["runtime.cu", "ingest.cu", "mapping.cu", "raycast.cu", "tracking.cu", "mesh.cu", "synth.cu", "persist.cu", "render.cu", "gc.cu", "snapshot.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-fvisibility=hidden,-O2", "-I", str(PKG.parent / "include"),
]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgbfusion")
    return exe


def _compile(src: Path, obj: Path, extra: list[str]) -> None:
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*")) + [PKG.parent / "include" / "gbfusion.h", Path(__file__)]
    return all(p.stat().st_mtime <= t for p in deps if p.is_file())


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> Path:
    """Compile the CUDA sources and link the shared library; returns its path."""
    if not force and up_to_date():
        return LIB
    OUT.mkdir(exist_ok=True)
    extra = extra or []
    objs = [OUT / (Path(s).stem + ".o") for s in SOURCES]
    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        futs = [ex.submit(_compile, CSRC / s, o, extra) for s, o in zip(SOURCES, objs)]
        for f in futs:
            f.result()
    tmp = OUT / "libgbfusion.so.tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
