"""Build libprismq_md.so (sm_103a) in-tree.

Each translation unit is compiled in parallel with nvcc; the integrator and
the neighbour/control kernels are compiled with --fmad=false so that their
floating-point results match the CPU oracle bit for bit, the force kernels
with --fmad=false and explicit FMAs so that no launch shape can fuse them
differently, and with -ftz=true (subnormal FP32 operands and results flush
to zero; divisions and square roots stay IEEE-rounded for normal values, so
the bond terms still match the reference's bit for bit, and the force
kernel runs ≈1 % faster), and host code is
compiled with -ffp-contract=off for the same reason (gcc contracts a*b+c into
FMA by default on aarch64).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess
import sys

HERE = pathlib.Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIB = HERE / "libprismq_md.so"
INCLUDE = HERE.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-DNDEBUG", f"-I{INCLUDE}", f"-I{CSRC}",
          "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math"]

UNITS = {
    "engine.cu": [],
    "force.cu": ["--fmad=false", "-ftz=true"],
    "integrate.cu": ["--fmad=false"],
    "nbr.cu": ["--fmad=false"],
    "noalloc.cu": ["--fmad=false"],
    "topology.cpp": [],
    "server.cpp": [],
    "prep_json.cpp": [],
}


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _compile(src: str, extra: list[str], verbose_ptxas: bool) -> pathlib.Path:
    out = BUILD / (src + ".o")
    cmd = [_nvcc(), *ARCH, *COMMON, *extra, "-c", str(CSRC / src), "-o", str(out)]
    if src.endswith(".cpp"):
        cmd = [_nvcc(), "-x", "c++", *COMMON, "-c", str(CSRC / src), "-o", str(out)]
    elif verbose_ptxas:
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    if verbose_ptxas and res.stderr:
        (BUILD / (src + ".ptxas.txt")).write_text(res.stderr)
    return out


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*")) + [INCLUDE / "prismq_md.h", pathlib.Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, verbose_ptxas: bool = False) -> pathlib.Path:
    if not force and not _stale():
        return LIB
    BUILD.mkdir(exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        futs = [ex.submit(_compile, s, e, verbose_ptxas) for s, e in UNITS.items()]
        objs = [f.result() for f in futs]
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [_nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-Xcompiler", "-fPIC"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv)
    print(LIB)
