"""Build recipe of libelbm_gb300.so: nvcc for sm_103a, one object per .cu file,
compiled in parallel, linked in-tree next to this file.  No CMake, no torch."""
from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess

HERE = pathlib.Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIB = HERE / "libelbm_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "--expt-relaxed-constexpr",
    "-Xcompiler",
    "-fPIC",
    "-Xcompiler",
    "-O2",
]


# Per-file flags: the GGM tags and the surface marking keep separately rounded
# multiply and add (no contraction), so that they match their host and CPU
# counterparts bit for bit.
FILE_FLAGS = {"ggm.cu": ["-fmad=false"],
              "geometry.cu": ["-fmad=false", "-Xcompiler", "-ffp-contract=off"]}


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libelbm_gb300")


def sources() -> list[pathlib.Path]:
    return sorted(CSRC.glob("*.cu"))


def build(verbose: bool = False, force: bool = False) -> pathlib.Path:
    """Compile every csrc/*.cu for sm_103a and link libelbm_gb300.so."""
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    srcs = sources()
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list((HERE.parent / "include").glob("*.h"))
    newest_header = max((h.stat().st_mtime for h in headers), default=0.0)

    def compile_one(src: pathlib.Path) -> pathlib.Path:
        obj = BUILD / (src.stem + ".o")
        if not force and obj.exists() and obj.stat().st_mtime > max(src.stat().st_mtime, newest_header):
            return obj
        cmd = [nvcc, *NVFLAGS, *FILE_FLAGS.get(src.name, []), "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)
        return obj

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 1))) as ex:
        objs = list(ex.map(compile_one, srcs))
    newest_obj = max(o.stat().st_mtime for o in objs)
    if force or not LIB.exists() or LIB.stat().st_mtime < newest_obj:
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
