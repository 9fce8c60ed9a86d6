"""Build recipe of the oracle — test infrastructure only: the CPU
restatement of the reference path, compiled with every multiply and add
separately rounded (-ffp-contract=off) and OpenMP element loops, into
oracle/liboracle.so. Used by the tests, the smoke check and the bench's
CPU-baseline leg; never by the product."""

from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"


def build(force: bool = False) -> Path:
    srcs = [HERE / "oracle.cpp", HERE / "pointwise.hpp", HERE / "oracle.h",
            HERE.parent / "include" / "dgswe.h"]
    if LIB.exists() and not force and LIB.stat().st_mtime >= max(p.stat().st_mtime for p in srcs):
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [shutil.which("g++") or "g++", "-std=c++17", "-O3", "-ffp-contract=off",
           "-fno-fast-math", "-fopenmp", "-fPIC", "-shared", "-o", str(tmp), str(HERE / "oracle.cpp")]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{proc.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
