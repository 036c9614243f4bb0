"""Build the reference-kernel harness — test infrastructure (oracle side).

Compiles oracle/ref_harness.cu, which includes the reference's own CUDA source
from where it lies in the reference tree (crates/prism-gpu/src/kernels/
nhs_amber_fused.cu and the headers beside it), into device-only cubins for
sm_103a:

  oracle/_ref/ref_harness.cubin        the reference's own nvcc flags
                                       (crates/prism-gpu/build.rs:339-355:
                                       -std=c++17 -lineinfo
                                       --expt-relaxed-constexpr -O3, FMA
                                       contraction on)
  oracle/_ref/ref_harness_nofma.cubin  the same with --fmad=false, for
                                       operation-by-operation comparison with
                                       the oracle (built without contraction)

A cubin is device code only, so the files load on any host architecture with
the CUDA driver (oracle/ref_kernels.py).  The reference tree is read here, at
build time, and nowhere else; without it the build is skipped and the tests
that need the cubins skip with that reason.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess

HERE = pathlib.Path(__file__).resolve().parent
OUT = HERE / "_ref"
SRC = HERE / "ref_harness.cu"
REF_KERNELS = pathlib.Path(os.environ.get("PRISMQ_REFERENCE_ROOT", "/root/reference")) / "crates/prism-gpu/src/kernels"
CUBINS = {"ref_harness.cubin": [], "ref_harness_nofma.cubin": ["--fmad=false"]}


def available() -> bool:
    return (REF_KERNELS / "nhs_amber_fused.cu").exists()


def _nvcc() -> str:
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def _one(name: str, extra: list[str]) -> pathlib.Path:
    out = OUT / name
    cmd = [_nvcc(), "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-lineinfo",
           "--expt-relaxed-constexpr", "-O3", *extra, f"-I{REF_KERNELS}", str(SRC), "-o", str(out)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"reference harness build failed ({name}):\n{res.stderr[-4000:]}")
    return out


def build(force: bool = False) -> bool:
    """Build both cubins when the reference tree is present; True if they exist afterwards."""
    if not available():
        return all((OUT / n).exists() for n in CUBINS)
    OUT.mkdir(exist_ok=True)
    src_t = max(SRC.stat().st_mtime, (REF_KERNELS / "nhs_amber_fused.cu").stat().st_mtime)
    todo = {n: e for n, e in CUBINS.items()
            if force or not (OUT / n).exists() or (OUT / n).stat().st_mtime < src_t}
    if todo:
        with cf.ThreadPoolExecutor(max_workers=len(todo)) as ex:
            list(ex.map(lambda kv: _one(*kv), todo.items()))
    return True


if __name__ == "__main__":
    print("built" if build(force=True) else "reference tree absent: skipped")
