"""Build recipe of the oracle — test infrastructure only: the CPU
restatement of the reference path, with OpenMP element loops, into two
libraries:

- ``oracle/liboracle.so``: every multiply and add separately rounded
  (-ffp-contract=off), as the reference's Rust release build computes (Rust
  never contracts a multiply and an add on its own), tuned for the host CPU
  (the reference builds with target-cpu=native). The tests, the smoke check
  and the bench's reference arm use it.
- ``oracle/liboracle_contract.so``: the same source with multiply-adds
  contracted into FMAs (-ffp-contract=fast) — a faster build whose results
  differ in the last bits; the bench times it as a second CPU figure only.

Never used by the product."""

from __future__ import annotations

import os
import platform
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
LIB_CONTRACT = HERE / "liboracle_contract.so"


def native_flags() -> list[str]:
    """The compiler's flag for the host CPU (-mcpu on Arm, -march on x86)."""
    machine = platform.machine().lower()
    if machine in ("aarch64", "arm64"):
        return ["-mcpu=native"]
    if machine in ("x86_64", "amd64"):
        return ["-march=native"]
    return []


def _compile(out: Path, contract: str) -> None:
    tmp = out.with_suffix(".so.tmp")
    cmd = [shutil.which("g++") or "g++", "-std=c++17", "-O3", f"-ffp-contract={contract}",
           "-fno-fast-math", *native_flags(), "-fopenmp", "-fPIC", "-shared", "-o", str(tmp),
           str(HERE / "oracle.cpp")]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{proc.stderr}")
    os.replace(tmp, out)


def build(force: bool = False, contract: bool = False) -> Path:
    """Compile the oracle (``contract``: the FMA-contracted build) if a source
    is newer than it (or ``force``); returns the library's path."""
    out = LIB_CONTRACT if contract else LIB
    srcs = [HERE / "oracle.cpp", HERE / "pointwise.hpp", HERE / "oracle.h", HERE / "build.py",
            HERE.parent / "include" / "dgswe.h"]
    if out.exists() and not force and out.stat().st_mtime >= max(p.stat().st_mtime for p in srcs):
        return out
    _compile(out, "fast" if contract else "off")
    return out


def build_all(force: bool = False) -> None:
    build(force)
    build(force, contract=True)


if __name__ == "__main__":
    build_all(force=True)
    print(LIB, LIB_CONTRACT)
