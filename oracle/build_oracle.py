"""Compiles the CPU oracle (sgw_oracle.c) into oracle/build/libsgw_oracle.so.

Test infrastructure: the library gives the tests their expected answers and
the benchmark its CPU baseline; it is never part of the engine.
"""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "sgw_oracle.c"
OUT = HERE / "build" / "libsgw_oracle.so"


def build_oracle(force: bool = False) -> Path:
    if not force and OUT.exists() and OUT.stat().st_mtime >= SRC.stat().st_mtime:
        return OUT
    OUT.parent.mkdir(exist_ok=True)
    tmp = OUT.with_suffix(".so.tmp")
    subprocess.run(["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp", str(SRC),
                    "-o", str(tmp), "-lm"], check=True)
    tmp.replace(OUT)
    return OUT


if __name__ == "__main__":
    print(build_oracle(force=True))
