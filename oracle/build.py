"""Build recipe of the CPU oracle (test infrastructure): gcc on the oracle's own
C files into oracle/_build/liboracle.so.  Nothing under oracle/ is part of the
product; only tests, the smoke check and the CPU-baseline leg of bench.py load it."""
from __future__ import annotations

import os
import pathlib
import shutil
import subprocess

HERE = pathlib.Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"
SOURCES = ["d3q27_oracle.c", "d3q39_oracle.c"]


def build(verbose: bool = False) -> pathlib.Path:
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        raise RuntimeError("no C compiler for the oracle")
    BUILD.mkdir(exist_ok=True)
    srcs = [HERE / s for s in SOURCES if (HERE / s).exists()]
    newest = max(s.stat().st_mtime for s in srcs)
    if LIB.exists() and LIB.stat().st_mtime > newest:
        return LIB
    # -ffp-contract=off: plain IEEE double arithmetic, no fused multiply-add
    cmd = [cc, "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-o", str(LIB) + ".tmp",
           *map(str, srcs), "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(str(LIB) + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
