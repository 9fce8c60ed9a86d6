"""Build recipe of the CUDA library ``libdgswe.so`` (in-tree, next to this
file): nvcc for sm_103a only, the translation units compiled in parallel.

Host code is compiled with ``-ffp-contract=off`` so that the geometry and
the tables are the same bits on x86-64 and on aarch64 (where GCC would
otherwise contract multiply-adds)."""

from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
LIB = HERE / "libdgswe.so"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libdgswe")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile libdgswe.so if a source is newer than it (or ``force``)."""
    sources = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    deps = sources + sorted(CSRC.glob("*.h*")) + sorted(CSRC.glob("*.cuh")) + [
        HERE.parent / "include" / "dgswe.h"
    ]
    if LIB.exists() and not force:
        newest = max(p.stat().st_mtime for p in deps)
        if LIB.stat().st_mtime >= newest:
            return LIB
    cc = nvcc()
    obj_dir = HERE / "_build"
    obj_dir.mkdir(exist_ok=True)
    host = "-Xcompiler=-fPIC,-fopenmp,-ffp-contract=off,-O2"
    common = [cc, ARCH, "-O3", "-lineinfo", "-std=c++17", host, "-I", str(CSRC)]
    jobs = []
    for src in sources:
        obj = obj_dir / (src.stem + ".o")
        if src.suffix == ".cpp":
            cmd = [
                shutil.which("g++") or "g++", "-std=c++17", "-O2", "-fPIC", "-fopenmp",
                "-ffp-contract=off", "-I", str(CSRC), "-c", str(src), "-o", str(obj),
            ]
        else:
            fmad = "-fmad=false" if src.stem == "kernels_exact" else "-fmad=true"
            cmd = common + [fmad, "-c", str(src), "-o", str(obj)]
        jobs.append((cmd, obj))
    workers = min(len(jobs), os.cpu_count() or 4)
    with concurrent.futures.ThreadPoolExecutor(max_workers=workers) as pool:
        list(pool.map(lambda job: _run(job[0]), jobs))
    tmp = LIB.with_suffix(".so.tmp")
    _run([cc, ARCH, "-shared", "-Xcompiler=-fopenmp", "-o", str(tmp)]
         + [str(o) for _, o in jobs] + ["-lgomp"])
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(force=True, verbose=True)
