"""Build recipe for the oracle (test infrastructure): oracle/liboracle.so.

gcc, -ffp-contract=off so that the float instance performs exactly the IEEE
operations written in oracle_impl.h; OpenMP for the multi-threaded CPU timing.
"""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

ORACLE_DIR = Path(__file__).resolve().parent
LIB = ORACLE_DIR / "liboracle.so"
SRC = [ORACLE_DIR / "svox2_oracle.c"]
HDR = [ORACLE_DIR / "oracle_impl.h"]
FLAGS = ["-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
         "-Wall", "-Wno-unused-function"]


def build(force: bool = False) -> Path:
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("no C compiler (gcc) for the oracle")
    if not force and LIB.exists() and all(LIB.stat().st_mtime >= p.stat().st_mtime for p in SRC + HDR):
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    res = subprocess.run([cc, *FLAGS, *map(str, SRC), "-o", str(tmp), "-lm"], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    tmp.replace(LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
